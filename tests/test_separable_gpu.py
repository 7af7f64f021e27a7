"""The separable preconditioner (CEV_PRECOND_SEPARABLE): flexible GMRES
with the exact inverse of the constant-eps stretched operator, applied by
dense GEMMs.  Checks: the exported 1D axis operators rebuild the plan's
system matrix (1e-12); with a truly constant eps the preconditioner is the
exact inverse (FGMRES converges in a few iterations, forward and transposed,
Ez and Hz, a two-frequency batch); on the 200x200 Ez workload it reaches the
1e-6 FP64 residual in far fewer iterations than plain GMRES with the same
field; gradients through preconditioned forward and adjoint solves match the
oracle (1e-5)."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import fdfd as ofd

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def _axis(plan, b, axis, tr):
    import ctypes as C
    from ceviche_gb300 import _lib
    n = plan.nx if axis == 0 else plan.ny
    T = np.zeros((n, n), np.complex128)
    assert _lib.load().cev_fdfd_axis_matrix(plan.handle, b, axis, int(tr),
                                            T.ctypes.data_as(C.c_void_p)) == 0
    return T


@pytest.mark.parametrize("pol", ["ez", "hz"])
@pytest.mark.parametrize("tr", [False, True])
def test_axis_matrices_rebuild_operator(cev, pol, tr):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.constants import EPSILON_0, MU_0
    rng = np.random.default_rng(2)
    Nx, Ny, dL, npml, om = 23, 19, 40e-9, [4, 3], 2 * np.pi * 3e8 / 1.5e-6
    plan = P.get_plan(pol, (Nx, Ny), dL, [om], npml, (0.4, -0.2))
    eps = rng.uniform(1, 3, (Nx, Ny)) if pol == "ez" else np.full((Nx, Ny), 2.5)
    Tx, Ty = _axis(plan, 0, 0, tr), _axis(plan, 0, 1, tr)
    k2 = EPSILON_0 * MU_0 * om ** 2 * dL ** 2
    L = np.kron(Tx, np.eye(Ny)) + np.kron(np.eye(Nx), Ty)
    if pol == "ez":
        A = -L - k2 * np.diag(eps.ravel())
    else:
        A = L / (2.5 + 1e-5) + k2 * np.eye(Nx * Ny)
    x = rng.standard_normal((Nx, Ny)) + 1j * rng.standard_normal((Nx, Ny))
    y = P.apply(plan, torch.as_tensor(eps), torch.as_tensor(x), transpose=tr,
                si_units=False).cpu().numpy()
    assert _rel(A @ x.ravel(), y) < 1e-12


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_exact_for_constant_eps(cev, pol):
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(4)
    Nx, Ny, dL, npml = 64, 48, 40e-9, [8, 6]
    oms = 2 * np.pi * 3e8 / np.array([1.45e-6, 1.6e-6])
    plan = P.get_plan(pol, (Nx, Ny), dL, oms, npml)
    eps = torch.full((Nx, Ny), 2.2, dtype=torch.float64)
    b = torch.as_tensor(rng.standard_normal((2, Nx, Ny)) + 1j * rng.standard_normal((2, Nx, Ny)))
    for tr in (False, True):
        x, info = P.solve(plan, eps, b, transpose=tr, tol=1e-8, precond="separable", strict=True)
        for k, w in enumerate(oms):
            A = ofd.make_A(pol, w, dL, eps.numpy(), npml)
            A = A.T if tr else A
            assert ofd.true_residual(A, x[k].cpu().numpy().ravel(), b[k].numpy().ravel()) < 1e-8
            assert info[k]["iterations"] <= 12, info


def test_config1_far_fewer_iterations(cev):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config1
    p = config1()
    plan = P.get_plan("ez", p["eps"].shape, p["dL"], [p["omega"]], p["npml"])
    b = torch.as_tensor(1j * p["omega"] * p["src"])
    e = torch.as_tensor(p["eps"])
    xs, isep = P.solve(plan, e, b, tol=1e-6, precond="separable", strict=True)
    xp, iplain = P.solve(plan, e, b, tol=1e-6, strict=True)
    assert isep[0]["iterations"] * 5 < iplain[0]["iterations"], (isep, iplain)
    A = ofd.make_A_ez(p["omega"], p["dL"], p["eps"], p["npml"])
    ref = ofd.spsolve(A, b.numpy().ravel())
    assert ofd.true_residual(A, xs.cpu().numpy().ravel(), b.numpy().ravel()) <= 1e-6
    assert _rel(xs.cpu().numpy().ravel(), ref) <= 1e-5


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_gradient_through_preconditioned_solves(cev, pol):
    rng = np.random.default_rng(8)
    Nx, Ny, omega, dL, npml = 30, 26, 2 * np.pi * 200e12, 1e-6, [6, 5]
    eps0 = 1 + rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[15, 13] = 1.0
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps0, npml, tol=1e-10, precond="separable")
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    F.eps_r = eps
    f1, f2, fz = F.solve(torch.as_tensor(src, device="cuda"))
    L = (fz.abs() ** 2).sum() + (f1.abs() ** 2).sum() + (f2.abs() ** 2).sum()
    L.backward()
    fo = (ofd.solve_ez if pol == "ez" else ofd.solve_hz)(omega, dL, eps0, npml, src)
    gref = (ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz)(
        omega, dL, eps0, npml, src, *[2 * c for c in fo])
    assert _rel(eps.grad.cpu().numpy(), gref) < 1e-5
    for got, ref in zip((f1, f2, fz), fo):
        assert _rel(got.detach().cpu().numpy(), ref) < 1e-7
