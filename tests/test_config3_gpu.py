"""The adjoint-gradient configuration at full size: FDFD Ez 600x600,
dL = 20 nm, npml 25, lambda 1.55 um, a 200x200 design block of
1 + 11.25 sigmoid(filtered noise), input/output waveguides, and
J = |sum(Ez conj(probe))|^2.  dJ/deps from the GPU adjoint (forward and
transposed GPU solves, gradient kernel) is checked on 20 seeded design
pixels against the restated ceviche gradient (oracle: SuperLU of the
assembled matrix, forward and adjoint) to 1e-5 relative, and on 3 pixels
against central differences with h = 1e-4 through GPU solves at a 1e-12
FP64 residual (1e-4 relative, the reference gradient tests' ratio; with
solves at 1e-10 the difference quotient carries ~1e-6 relative noise)."""
import numpy as np
import pytest
import torch

from oracle import fdfd as ofd

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def _objective(cev, p, eps_t, tol=TOL):
    F = cev.fdfd_ez(p["omega"], p["dL"], eps_t, p["npml"], tol=tol, max_iters=400000,
                    max_stall=100000)
    _, _, ez = F.solve(torch.as_tensor(p["src"], device="cuda"))
    s = (ez * torch.as_tensor(p["probe"], device="cuda").conj()).sum()
    return (s.abs() ** 2), ez


def test_config3_adjoint_gradient(cev):
    from ceviche_gb300.workloads import config3
    p = config3()
    eps0 = p["eps"]
    N = eps0.shape[0]
    rng = np.random.default_rng(33)
    lo = N // 2 - 100
    pix = [(int(i), int(j)) for i, j in rng.integers(lo, lo + 200, size=(20, 2))]
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    J, ez = _objective(cev, p, eps)
    J.backward()
    g = eps.grad.cpu().numpy()
    g_pix = np.array([g[i, j] for i, j in pix])
    # restated ceviche gradient (host SuperLU)
    A = ofd.make_A_ez(p["omega"], p["dL"], eps0, p["npml"])
    b = 1j * p["omega"] * p["src"].ravel()
    x = ofd.spsolve(A, b)
    assert np.linalg.norm(x - ez.detach().cpu().numpy().ravel()) / np.linalg.norm(x) < 1e-7
    s = np.sum(x * np.conj(p["probe"].ravel()))
    g_ez = (2 * s * p["probe"]).reshape(eps0.shape)
    zero = np.zeros_like(g_ez)
    gref = ofd.grad_eps_ez(p["omega"], p["dL"], eps0, p["npml"], p["src"], zero, zero, g_ez)
    gref_pix = np.array([gref[i, j] for i, j in pix])
    assert np.linalg.norm(g_pix - gref_pix) / np.linalg.norm(gref_pix) < 1e-5
    # central differences through GPU solves on 4 pixels
    h = 1e-4
    fd = []
    for i, j in pix[:3]:
        e1, e2 = eps0.copy(), eps0.copy()
        e1[i, j] += h
        e2[i, j] -= h
        Jp = _objective(cev, p, torch.as_tensor(e1, device="cuda"), tol=1e-12)[0].item()
        Jm = _objective(cev, p, torch.as_tensor(e2, device="cuda"), tol=1e-12)[0].item()
        fd.append((Jp - Jm) / (2 * h))
    fd = np.array(fd)
    assert np.linalg.norm(g_pix[:3] - fd) / np.linalg.norm(fd) < 1e-4
