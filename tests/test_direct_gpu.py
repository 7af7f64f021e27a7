"""Nested-dissection direct preconditioner (CEV_PRECOND_DIRECT) on the GPU.

The factorisation has no reference counterpart; it stands where ceviche
factors the assembled matrix with SuperLU (ceviche/solvers.py:50-62).  Checks:

* apply: z = M^-1 v against scipy's sparse solve of M = A' without the
  periodic wrap entries (complex128), for Ez/Hz, A and A^T, real and complex
  eps, shift 0 and 0.5.  Tolerance 2e-4 relative L2: the factors are
  complex64, so the error is about cond(M) * 6e-8.
* solves: flexible GMRES with it reaches the FP64 true residual tol in a few
  iterations; the returned fields match the oracle's direct solve (1e-5 at
  tol 1e-8) and their residual, recomputed on the host with the oracle's
  assembled matrix, is below the tolerance.
* gradients through the transposed (adjoint) solve match the oracle's 1e-5.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl
import torch

from oracle import fdfd as ofd

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def _nowrap(A, nx, ny):
    """A without its periodic wrap entries (|di| > 1 or |dj| > 1)."""
    C = A.tocoo()
    ri, rj = np.divmod(C.row, ny)
    ci, cj = np.divmod(C.col, ny)
    keep = (np.abs(ri - ci) <= 1) & (np.abs(rj - cj) <= 1)
    return sp.csr_matrix((C.data[keep], (C.row[keep], C.col[keep])), shape=A.shape)


def _shifted(pol, omega, dL, eps, npml, beta, bloch=(0.0, 0.0)):
    """The operator with its mass term times (1 - i beta), SI units."""
    if pol == "ez":
        return ofd.make_A_ez(omega, dL, eps * (1 - 1j * beta), npml, bloch)
    A = ofd.make_A_hz(omega, dL, eps, npml, bloch)
    return A - 1j * beta * ofd.MU_0 * omega ** 2 * sp.eye(A.shape[0])


CASES = [
    # nx, ny, npml, complex eps
    (13, 11, [3, 2], False),
    (40, 36, [6, 6], False),
    (97, 80, [10, 8], False),
    (64, 48, [8, 8], True),
    (150, 131, [12, 10], False),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("pol", ["ez", "hz"])
@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("beta", [0.0, 0.5])
def test_apply_matches_sparse_solve(cev, case, pol, transpose, beta):
    from ceviche_gb300 import primitives as P
    nx, ny, npml, cplx = case
    rng = np.random.default_rng(nx * 100 + ny)
    dL = 40e-9
    omega = 2 * np.pi * 3e8 / 1.55e-6
    eps = 1 + 5 * rng.random((nx, ny))
    if cplx:
        eps = eps + 0.3j * rng.random((nx, ny))
    plan = P.get_plan(pol, (nx, ny), dL, [omega], npml)
    e = torch.as_tensor(eps, device="cuda")
    dp = P.DirectPrecond(plan, e, transpose=transpose, shift=beta)
    v = (rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny)))
    z = dp.apply(torch.as_tensor(v.astype(np.complex64), device="cuda")).cpu().numpy()
    A = _shifted(pol, omega, dL, eps, npml, beta) * plan.scale
    M = _nowrap(A, nx, ny)
    if transpose:
        M = M.T.tocsr()
    ref = spl.spsolve(M.tocsc(), v.ravel())
    assert _rel(z, ref) < 2e-4


def test_analysis_counts(cev):
    """The tree eliminates every cell once; factor sizes grow like n log n."""
    import ctypes as C
    from ceviche_gb300 import _lib
    lib = _lib.load()
    for nx, ny in ((7, 5), (200, 200), (256, 256), (97, 1024)):
        nn, fe, nd = C.c_size_t(), C.c_size_t(), C.c_size_t()
        d, fl, cov = C.c_int(), C.c_double(), (C.c_longlong * 2)()
        assert lib.cev_nd_analyse(nx, ny, C.byref(nn), C.byref(d), C.byref(fe), C.byref(fl),
                                  C.byref(nd), cov) == 0
        assert cov[0] == 0 and cov[1] == 0


def test_config1_direct_solve_matches_reference(cev):
    """200x200 Ez (the CPU-runnable configuration): converged in a few
    iterations, fields within 1e-5 of the oracle's SuperLU solve."""
    from ceviche_gb300 import workloads as W
    p = W.config1()
    F = cev.fdfd_ez(p["omega"], p["dL"], p["eps"], p["npml"], tol=1e-8, precond="direct")
    hx, hy, ez = F.solve(p["src"])
    _, _, ez_ref = ofd.solve_ez(p["omega"], p["dL"], p["eps"], p["npml"], p["src"])
    assert _rel(ez, ez_ref) < 1e-5
    info = F.last_info[0]
    assert info["code"] == 0 and info["iterations"] <= 10


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_config4_batch_reaches_1e6(cev, pol):
    """Config-4 problems (256x256, binary eps 1/12.25, dL = 1.55um/20): plain
    GMRES does not reach 1e-6 within 20,000 iterations; with the direct
    preconditioner every problem of the batch does in a few.  The FP64
    residual is recomputed on the host with the oracle's assembled matrix."""
    from ceviche_gb300 import primitives as P
    from ceviche_gb300 import workloads as W
    probs = [W.config4_problem(i) for i in range(4)]
    eps = np.stack([q["eps"] for q in probs])
    oms = [q["omega"] for q in probs]
    b = np.stack([1j * q["omega"] * q["src"] for q in probs])
    plan = P.Plan(pol, eps.shape[1:], probs[0]["dL"], oms, probs[0]["npml"])
    x, info = P.solve(plan, torch.as_tensor(eps, device="cuda"), torch.as_tensor(b, device="cuda"),
                      precond="direct", tol=1e-6, strict=True)
    xs = x.cpu().numpy()
    for k, q in enumerate(probs):
        assert info[k]["residual"] <= 1e-6 and info[k]["iterations"] <= 12
        A = ofd.make_A(pol, q["omega"], q["dL"], q["eps"], q["npml"])
        r = np.linalg.norm(A @ xs[k].ravel() - b[k].ravel()) / np.linalg.norm(b[k])
        assert r <= 1.2e-6


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_gradient_through_direct_solve(cev, pol):
    """dJ/d eps with the direct preconditioner on the forward and the
    transposed solve matches the oracle's restated gradient to 1e-5."""
    rng = np.random.default_rng(7)
    nx, ny, npml, dL = 60, 52, [8, 8], 30e-9
    omega = 2 * np.pi * 3e8 / 1.3e-6
    eps0 = 1 + 6 * rng.random((nx, ny))
    src = np.zeros((nx, ny))
    src[15, 20:30] = 1.0
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    F = cls(omega, dL, eps, npml, tol=1e-10, precond="direct")
    f1, f2, fz = F.solve(torch.as_tensor(src, device="cuda"))
    J = (f1.abs() ** 2).sum() + (f2.abs() ** 2).sum() + (fz.abs() ** 2).sum()
    J.backward()
    g = eps.grad.cpu().numpy()
    fo = (ofd.solve_ez if pol == "ez" else ofd.solve_hz)(omega, dL, eps0, npml, src)
    gref = (ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz)(
        omega, dL, eps0, npml, src, *[2 * c for c in fo])
    assert _rel(g, gref) < 1e-5


def test_shifted_laplacian_converges(cev):
    """CEV_PRECOND_SHIFTED_LAPLACIAN (exact inverse of the shifted operator,
    beta 0.5) converges on a small PML problem; it needs more iterations
    than the direct factors of the operator itself."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(3)
    nx, ny, npml, dL = 80, 72, [10, 10], 40e-9
    omega = 2 * np.pi * 3e8 / 1.55e-6
    eps = 1 + 3 * rng.random((nx, ny))
    b = np.zeros((nx, ny), complex)
    b[20, 30] = 1j * omega
    plan = P.Plan("ez", (nx, ny), dL, [omega], npml)
    et, bt = torch.as_tensor(eps, device="cuda"), torch.as_tensor(b, device="cuda")
    _, i_sl = P.solve(plan, et, bt, precond="shifted_laplacian", mg_shift=0.5, strict=True)
    _, i_d = P.solve(plan, et, bt, precond="direct", strict=True)
    assert i_sl[0]["residual"] <= 1e-6 and i_d[0]["residual"] <= 1e-6
    assert i_d[0]["iterations"] < i_sl[0]["iterations"]


def test_periodic_bloch_without_pml(cev):
    """With npml = 0 and Bloch phases the dropped wrap entries are part of
    the operator; the solve still reaches tol (a few more iterations)."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(5)
    nx, ny, dL = 48, 40, 50e-9
    omega = 2 * np.pi * 3e8 / 1.55e-6
    eps = 1 + 2 * rng.random((nx, ny))
    b = (rng.standard_normal((nx, ny)) + 1j * rng.standard_normal((nx, ny)))
    plan = P.Plan("ez", (nx, ny), dL, [omega], [0, 0], bloch=(0.3, -0.2))
    x, info = P.solve(plan, torch.as_tensor(eps, device="cuda"), torch.as_tensor(b, device="cuda"),
                      precond="direct", strict=True)
    A = ofd.make_A_ez(omega, dL, eps, [0, 0], (0.3, -0.2))
    r = np.linalg.norm(A @ x.cpu().numpy().ravel() - b.ravel()) / np.linalg.norm(b)
    assert r <= 1.2e-6
