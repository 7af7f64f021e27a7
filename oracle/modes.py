"""FP64 CPU restatement of ceviche's waveguide mode solver -- TEST
INFRASTRUCTURE ONLY.

Restates ceviche/modes.py:10-45 (get_modes), 48-65 (insert_mode), 81-117
(filter_modes, normalize_modes): A = diag(eps) + Dxf Dxb / k0^2 with the
(N, 1)-grid derivative matrices of ceviche/derivatives.py (oracle.fdfd),
its eigenpairs nearest sigma = max(eps).  The reference gets them from
scipy's shift-invert ``eigs`` (ARPACK, random start vector); here a dense
``numpy.linalg.eig`` of A (N is a cross section, at most a few thousand)
ordered by distance to sigma, nearest first -- the order ARPACK returns.

Eigenvector phase: the reference's is ARPACK's and changes from call to
call; here each vector is scaled to unit 2-norm with its largest-magnitude
entry (first on ties) real and positive, the convention of the GPU solver.
"""
import numpy as np

from .constants import EPSILON_0, MU_0
from .fdfd import derivative_matrices

C_0 = 1 / np.sqrt(EPSILON_0 * MU_0)


def mode_matrix(eps_cross, omega, dL, npml):
    """ceviche/modes.py:24-33 (dense)."""
    N = eps_cross.size
    Dxf, Dxb, _, _ = derivative_matrices(omega, (N, 1), [npml, 0], dL)
    k0 = omega / C_0
    return np.diag(eps_cross.ravel().astype(np.complex128)) + (Dxf @ Dxb).toarray() / k0 ** 2


def fix_phase(vecs):
    vecs = vecs / np.sqrt(np.sum(np.abs(vecs) ** 2, axis=0))
    for j in range(vecs.shape[1]):
        i = int(np.argmax(np.abs(vecs[:, j]) ** 2))
        vecs[:, j] *= np.conj(vecs[i, j]) / abs(vecs[i, j])
    return vecs


def get_modes(eps_cross, omega, dL, npml, m=1, filtering=True):
    eps_cross = np.asarray(eps_cross)
    A = mode_matrix(eps_cross, omega, dL, npml)
    sigma = np.max(eps_cross)
    w, V = np.linalg.eig(A)
    order = np.argsort(np.abs(w - sigma), kind="stable")[:m]
    vals, vecs = w[order], V[:, order]
    if filtering:
        keep = np.real(vals) > 0.0
        vals, vecs = vals[keep], vecs[:, keep]
    if vals.size == 0:
        raise BaseException("Could not find any eigenmodes for this waveguide")
    return vals, fix_phase(vecs)


def insert_mode(omega, dx, x, y, epsr, target=None, npml=0, m=1, filtering=False):
    if target is None:
        target = np.zeros(epsr.shape, dtype=complex)
    _, mode_field = get_modes(epsr[x, y], omega, dx, npml, m=m, filtering=filtering)
    target[x, y] = np.atleast_2d(mode_field)[:, m - 1].squeeze()
    return target
