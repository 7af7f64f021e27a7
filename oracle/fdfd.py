"""FP64 CPU restatement of ceviche's FDFD path -- TEST INFRASTRUCTURE ONLY.

Restates (own code, same arithmetic):
    * PML stretch factors       ceviche/derivatives.py:173-216
    * derivative matrices       ceviche/derivatives.py:34-124 (incl. 1D case :75-78)
    * Ez / Hz system matrices   ceviche/fdfd.py:172-185, :200-233
    * direct solve              ceviche/primitives.py:103-119 -> solvers.py:50-62
                                (scipy SuperLU ``spsolve``; PARDISO is optional
                                 and absent, so the reference takes this branch)
    * field conversions         ceviche/fdfd.py:135-162
    * reverse-mode gradients    ceviche/primitives.py:121-135 chained through
                                fdfd.py:179 (Ez) and fdfd.py:211-233 (Hz)

Gradient convention: cotangents ``g`` follow PyTorch (g = dL/dRe + i dL/dIm
for a real loss L).  HIPS-autograd's cotangent is ``conj(g)``; with a real
``eps`` both frameworks return the same real gradient.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from .constants import EPSILON_0, MU_0, ETA_0


# ---------------------------------------------------------------- PML profiles
def sig_w(l, dw, m=3, lnR=-30):
    """ceviche/derivatives.py:209-212."""
    sig_max = -(m + 1) * lnR / (2 * ETA_0 * dw)
    return sig_max * (l / dw) ** m


def s_value(l, dw, omega):
    """ceviche/derivatives.py:214-216."""
    return 1 - 1j * sig_w(l, dw) / (omega * EPSILON_0)


def sfactor(direction, omega, dL, N, npml):
    """1D stretch profile, ceviche/derivatives.py:173-207.

    'f': i <= npml -> l = dL*(npml - i + 0.5); i > N - npml -> l = dL*(i - (N - npml) - 0.5)
    'b': same with offsets 1 instead of 0.5.
    """
    s = np.ones(N, dtype=np.complex128)
    if npml == 0:
        return s
    dw = npml * dL
    off = {"f": 0.5, "b": 1.0}[direction]
    for i in range(N):  # scalar loop keeps the reference's exact float ops
        if i <= npml:
            s[i] = s_value(dL * (npml - i + off), dw, omega)
        elif i > N - npml:
            s[i] = s_value(dL * (i - (N - npml) - off), dw, omega)
    return s


# --------------------------------------------------------- derivative matrices
def _d1(direction, n, dL, phase):
    """1D difference matrix with Bloch phasor on the wrap entry
    (ceviche/derivatives.py:94-124)."""
    ph = np.exp(1j * phase)
    if direction == "f":
        D = sp.diags([-1, 1, ph], [0, 1, -n + 1], shape=(n, n), dtype=np.complex128)
    else:
        D = sp.diags([1, -1, -np.conj(ph)], [0, -1, n - 1], shape=(n, n), dtype=np.complex128)
    return (1 / dL) * D


def derivative_matrices(omega, shape, npml, dL, bloch_x=0.0, bloch_y=0.0):
    """(Dxf, Dxb, Dyf, Dyb) with the S-factors folded in as row scalings
    (ceviche/derivatives.py:34-59, 129-171).  Flat index = i*Ny + j."""
    Nx, Ny = shape
    Ix, Iy = sp.eye(Nx), sp.eye(Ny)
    out = []
    for comp, d in (("x", "f"), ("x", "b"), ("y", "f"), ("y", "b")):
        if comp == "x":
            D = sp.eye(Ny) if Nx == 1 else sp.kron(_d1(d, Nx, dL, bloch_x), Iy)
            s = sfactor(d, omega, dL, Nx, npml[0])
            S = np.repeat(1 / s, Ny)
        else:
            D = sp.eye(Nx) if Ny == 1 else sp.kron(Ix, _d1(d, Ny, dL, bloch_y))
            s = sfactor(d, omega, dL, Ny, npml[1])
            S = np.tile(1 / s, Nx)
        out.append(sp.diags(S).dot(D).tocsr())
    return tuple(out)


def eps_xx_yy(eps):
    """Hz-grid permittivity averages (ceviche/fdfd.py:200-209): xx averages
    along axis 1, yy along axis 0 (periodic roll)."""
    exx = 0.5 * (eps + np.roll(eps, 1, axis=1))
    eyy = 0.5 * (eps + np.roll(eps, 1, axis=0))
    return exx, eyy


# ------------------------------------------------------------- system matrices
def make_A_ez(omega, dL, eps, npml, bloch=(0.0, 0.0)):
    """A = -(1/mu0)(Dxf Dxb + Dyf Dyb) - eps0 w^2 diag(eps)  (ceviche/fdfd.py:172-185)."""
    Dxf, Dxb, Dyf, Dyb = derivative_matrices(omega, eps.shape, npml, dL, *bloch)
    C = -1 / MU_0 * Dxf.dot(Dxb) - 1 / MU_0 * Dyf.dot(Dyb)
    return (C + sp.diags(-EPSILON_0 * omega ** 2 * eps.ravel())).tocsr()


def make_A_hz(omega, dL, eps, npml, bloch=(0.0, 0.0)):
    """A = (1/eps0)(Dxb diag(1/(eps_yy+1e-5)) Dxf + Dyb diag(1/(eps_xx+1e-5)) Dyf)
    + mu0 w^2 I  (ceviche/fdfd.py:211-233)."""
    Dxf, Dxb, Dyf, Dyb = derivative_matrices(omega, eps.shape, npml, dL, *bloch)
    exx, eyy = eps_xx_yy(eps)
    dxx = sp.diags(1 / (exx.ravel() + 1e-5))
    dyy = sp.diags(1 / (eyy.ravel() + 1e-5))
    D = 1 / EPSILON_0 * (Dxb.dot(dyy).dot(Dxf) + Dyb.dot(dxx).dot(Dyf))
    N = eps.size
    return (D + MU_0 * omega ** 2 * sp.eye(N)).tocsr()


def make_A(pol, omega, dL, eps, npml, bloch=(0.0, 0.0)):
    return (make_A_ez if pol == "ez" else make_A_hz)(omega, dL, eps, npml, bloch)


# ------------------------------------------------------------------ solves
def spsolve(A, b):
    """Direct sparse LU, the reference's default solve (solvers.py:60-62)."""
    return spl.spsolve(A.tocsc(), b)


def solve_ez(omega, dL, eps, npml, Jz, bloch=(0.0, 0.0)):
    """Returns (Hx, Hy, Ez) grids, ceviche/fdfd.py:58-76 + 187-192 + 138-147."""
    shape = eps.shape
    A = make_A_ez(omega, dL, eps, npml, bloch)
    b = 1j * omega * Jz.ravel()
    ez = spsolve(A, b)
    _, Dxb, _, Dyb = derivative_matrices(omega, shape, npml, dL, *bloch)
    hx = -1 / 1j / omega / MU_0 * Dyb.dot(ez)
    hy = 1 / 1j / omega / MU_0 * Dxb.dot(ez)
    return hx.reshape(shape), hy.reshape(shape), ez.reshape(shape)


def solve_hz(omega, dL, eps, npml, Mz, bloch=(0.0, 0.0)):
    """Returns (Ex, Ey, Hz) grids, ceviche/fdfd.py:58-76 + 235-244 + 150-162."""
    shape = eps.shape
    A = make_A_hz(omega, dL, eps, npml, bloch)
    b = 1j * omega * Mz.ravel()
    hz = spsolve(A, b)
    Dxf, _, Dyf, _ = derivative_matrices(omega, shape, npml, dL, *bloch)
    exx, eyy = eps_xx_yy(eps)
    ex = 1 / 1j / omega / EPSILON_0 / (exx.ravel() + 1e-5) * Dyf.dot(hz)
    ey = -1 / 1j / omega / EPSILON_0 / (eyy.ravel() + 1e-5) * Dxf.dot(hz)
    return ex.reshape(shape), ey.reshape(shape), hz.reshape(shape)


def true_residual(A, x, b):
    """||A x - b|| / ||b|| in FP64."""
    return np.linalg.norm(A.dot(x) - b) / np.linalg.norm(b)


# ---------------------------------------------------------------- gradients
def _out(c, cplx):
    """Gradient from the sensitivity c (dL = Re(sum c d eps)): Re(c) for a
    real eps; conj(c) = dL/dRe + i dL/dIm (PyTorch convention) for a complex
    (lossy) eps, for which A(eps) is holomorphic."""
    return np.conj(c) if cplx else np.real(c)


def grad_eps_ez(omega, dL, eps, npml, Jz, g_hx, g_hy, g_ez, source_times_eps=False,
                bloch=(0.0, 0.0)):
    """dL/d(eps) for a real loss of (Hx, Hy, Ez) = fdfd_ez.solve(src).

    ``src = eps*Jz`` when ``source_times_eps`` (the reference gradient tests'
    set-up, test_gradients_fdfd.py:89), else ``src = Jz``.

    Restates the reference VJP chain: sp_mult x-VJP (primitives.py:81-86) for
    the H conversions, sp_solve entries/b VJPs (primitives.py:121-135) with the
    adjoint solve on transposed indices, the diagonal block of entries
    -eps0 w^2 eps (fdfd.py:179), and the real part for real eps.
    """
    shape = eps.shape
    A = make_A_ez(omega, dL, eps, npml, bloch)
    src = (eps * Jz if source_times_eps else Jz).ravel()
    b = 1j * omega * src
    x = spsolve(A, b)
    _, Dxb, _, Dyb = derivative_matrices(omega, shape, npml, dL, *bloch)
    a = 1 / 1j / omega / MU_0
    # HIPS-style cotangents v = conj(g); sp_mult x-VJP is M^T v
    v = np.conj(g_ez.ravel()) + (-a * Dyb).T.dot(np.conj(g_hx.ravel())) \
        + (a * Dxb).T.dot(np.conj(g_hy.ravel()))
    adj = spsolve(A.T, -v)                      # primitives.py:126
    cplx = np.iscomplexobj(eps)
    grad = _out(adj * x * (-EPSILON_0 * omega ** 2), cplx)   # adj[i]*x[j] on the diagonal
    if source_times_eps:
        # b-VJP (primitives.py:130-135): A^-T v = -adj, then b = 1j*w*eps*Jz
        grad = grad + _out(-adj * 1j * omega * Jz.ravel(), cplx)
    return grad.reshape(shape)


def grad_eps_hz(omega, dL, eps, npml, Mz, g_ex, g_ey, g_hz, source_times_eps=False,
                bloch=(0.0, 0.0)):
    """dL/d(eps) for a real loss of (Ex, Ey, Hz) = fdfd_hz.solve(src).

    Restates the reference chain: the field conversions (fdfd.py:150-162)
    depend on eps directly and through Hz; the system matrix depends on
    1/(eps_yy+1e-5) and 1/(eps_xx+1e-5) (fdfd.py:211-233, whose spsp_mult
    entries VJPs reduce to (Dxb^T adj) * (Dxf x) per diagonal entry); the
    averages of fdfd.py:200-209 are rolled back.
    """
    shape = eps.shape
    Nx, Ny = shape
    A = make_A_hz(omega, dL, eps, npml, bloch)
    src = (eps * Mz if source_times_eps else Mz).ravel()
    b = 1j * omega * src
    x = spsolve(A, b)
    Dxf, Dxb, Dyf, Dyb = derivative_matrices(omega, shape, npml, dL, *bloch)
    exx, eyy = eps_xx_yy(eps)
    dxx = 1 / (exx.ravel() + 1e-5)
    dyy = 1 / (eyy.ravel() + 1e-5)
    al = 1 / 1j / omega / EPSILON_0
    vex, vey, vhz = np.conj(g_ex.ravel()), np.conj(g_ey.ravel()), np.conj(g_hz.ravel())
    Dyf_x, Dxf_x = Dyf.dot(x), Dxf.dot(x)
    # direct dependence of Ex, Ey on dxx, dyy (complex sensitivities; the
    # real part is taken at the end, or the conjugate for a complex eps)
    cplx = np.iscomplexobj(eps)
    g_dxx = vex * al * Dyf_x
    g_dyy = vey * (-al) * Dxf_x
    # dependence through Hz
    v = vhz + Dyf.T.dot(al * dxx * vex) + Dxf.T.dot(-al * dyy * vey)
    adj = spsolve(A.T, -v)
    # entries VJP adj[i]*x[j] for the blocks (1/eps0) Dxb diag(dyy) Dxf, etc.
    g_dyy = g_dyy + 1 / EPSILON_0 * Dxb.T.dot(adj) * Dxf_x
    g_dxx = g_dxx + 1 / EPSILON_0 * Dyb.T.dot(adj) * Dyf_x
    g_exx = (-dxx ** 2 * g_dxx).reshape(shape)
    g_eyy = (-dyy ** 2 * g_dyy).reshape(shape)
    grad = 0.5 * (g_exx + np.roll(g_exx, -1, axis=1)) + 0.5 * (g_eyy + np.roll(g_eyy, -1, axis=0))
    grad = _out(grad, cplx)
    if source_times_eps:
        grad = grad + _out(-adj * 1j * omega * Mz.ravel(), cplx).reshape(shape)
    return grad


# ------------------------------------------------- multi-frequency (fdfd_mf_ez)
def make_A_mf_ez(omega, dL, eps, npml, omega_mod, delta, phi, Nsb, bloch=(0.0, 0.0)):
    """Coupled sideband system of ceviche/fdfd.py:289-326: block-diagonal
    Ez operators at the centre-frequency derivatives with -eps0 W_m^2 eps on the
    diagonal, plus -eps0/2 W_m^2 delta_k exp(+-1j phi_k) coupling to sidebands
    m +- (k+1)."""
    M = 2 * Nsb + 1
    N = eps.size
    W = omega + np.arange(-Nsb, Nsb + 1) * omega_mod
    Dxf, Dxb, Dyf, Dyb = derivative_matrices(omega, eps.shape, npml, dL, *bloch)
    C = -1 / MU_0 * Dxf.dot(Dxb) - 1 / MU_0 * Dyf.dot(Dyb)
    A = sp.kron(sp.eye(M), C) + sp.diags(-EPSILON_0 * np.kron(W ** 2, eps.ravel()))
    A = A.tolil()
    nfreq = delta.shape[0]
    dmat = delta.reshape(nfreq, N)
    pmat = phi.reshape(nfreq, N)
    A = A.tocsr()
    blocks = []
    for k in range(nfreq):
        mod_p = -0.5 * EPSILON_0 * dmat[k] * np.exp(1j * pmat[k])
        mod_m = -0.5 * EPSILON_0 * dmat[k] * np.exp(-1j * pmat[k])
        ent_p = np.kron(W[:-k - 1] ** 2, mod_p)
        rows_p = np.arange((M - k - 1) * N)
        blocks.append(sp.coo_matrix((ent_p, (rows_p, rows_p + (k + 1) * N)), shape=(M * N, M * N)))
        ent_m = np.kron(W[k + 1:] ** 2, mod_m)
        rows_m = np.arange((k + 1) * N, M * N)
        blocks.append(sp.coo_matrix((ent_m, (rows_m, rows_m - (k + 1) * N)), shape=(M * N, M * N)))
    for blk in blocks:
        A = A + blk
    return A.tocsr()


def solve_mf_ez(omega, dL, eps, npml, omega_mod, delta, phi, Nsb, Jz, bloch=(0.0, 0.0)):
    """(Hx, Hy, Ez), each (M, Nx, Ny): fdfd_mf_ez.solve (fdfd.py:262-283, 328-359)."""
    M = 2 * Nsb + 1
    shape = eps.shape
    W = omega + np.arange(-Nsb, Nsb + 1) * omega_mod
    A = make_A_mf_ez(omega, dL, eps, npml, omega_mod, delta, phi, Nsb, bloch)
    b = 1j * (W[:, None] * Jz.reshape(M, -1)).ravel()
    ez = spsolve(A, b).reshape(M, -1)
    _, Dxb, _, Dyb = derivative_matrices(omega, shape, npml, dL, *bloch)
    hx = np.stack([-1 / 1j / MU_0 / W[m] * Dyb.dot(ez[m]) for m in range(M)])
    hy = np.stack([1 / 1j / MU_0 / W[m] * Dxb.dot(ez[m]) for m in range(M)])
    r = lambda a: a.reshape((M,) + shape)
    return r(hx), r(hy), r(ez)
