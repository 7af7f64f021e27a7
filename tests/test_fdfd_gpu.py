"""FDFD parity on the GPU: operator, solve, fields and eps gradients against
the CPU oracle (pinned to reference fixtures) and the reference fixtures
themselves.  Tolerances: complex128 operator 1e-13 relative; complex64
operator 2e-6; solved fields 1e-5 relative L2 at 1e-6 FP64 residual (the
200x200 Ez gate); gradients 1e-5 relative."""
import os

import numpy as np
import pytest
import torch

from oracle import fdfd as ofd
from tests.conftest import GOLDEN

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


def _case(k):
    d = np.load(os.path.join(GOLDEN, "stencil_ops.npz"))
    Nx, Ny, px, py, bx, by, om, dL = d[f"c{k}_meta"]
    return d, int(Nx), int(Ny), [int(px), int(py)], (bx, by), om, dL


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("pol", ["ez", "hz"])
@pytest.mark.parametrize("transpose", [False, True])
def test_operator_c128_matches_reference(cev, k, pol, transpose):
    from ceviche_gb300 import primitives as P
    d, Nx, Ny, npml, bloch, om, dL = _case(k)
    plan = P.get_plan(pol, (Nx, Ny), dL, om, npml, bloch)
    eps = torch.as_tensor(d[f"c{k}_eps"], device="cuda")
    x = torch.as_tensor(d[f"c{k}_x"].reshape(Nx, Ny), device="cuda")
    y = P.apply(plan, eps, x, transpose=transpose).cpu().numpy().ravel()
    ref = d[f"c{k}_{pol}_{'ATx' if transpose else 'Ax'}"]
    assert _rel(y, ref) < 1e-13


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_operator_c64_matches_reference(cev, k, pol):
    from ceviche_gb300 import primitives as P
    d, Nx, Ny, npml, bloch, om, dL = _case(k)
    plan = P.get_plan(pol, (Nx, Ny), dL, om, npml, bloch)
    eps = torch.as_tensor(d[f"c{k}_eps"], device="cuda")
    x = torch.as_tensor(d[f"c{k}_x"].reshape(Nx, Ny), device="cuda")
    for tr, key in ((False, "Ax"), (True, "ATx")):
        y = P.apply(plan, eps, x, transpose=tr, precision="c64").cpu().numpy().ravel()
        assert _rel(y, d[f"c{k}_{pol}_{key}"]) < 2e-6


def test_operator_batch_omegas(cev):
    """A batch of omegas on one plan equals per-omega plans (oracle A@x)."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(5)
    Nx, Ny, dL, npml = 33, 17, 30e-9, [4, 3]
    oms = 2 * np.pi * 3e8 / np.array([1.3e-6, 1.55e-6, 1.8e-6])
    eps = rng.uniform(1, 5, (Nx, Ny))
    x = rng.standard_normal((3, Nx, Ny)) + 1j * rng.standard_normal((3, Nx, Ny))
    for pol in ("ez", "hz"):
        plan = P.get_plan(pol, (Nx, Ny), dL, oms, npml)
        y = P.apply(plan, torch.as_tensor(eps), torch.as_tensor(x)).cpu().numpy()
        for b, w in enumerate(oms):
            A = ofd.make_A(pol, w, dL, eps, npml)
            assert _rel(y[b].ravel(), A.dot(x[b].ravel())) < 1e-13


@pytest.mark.parametrize("name", ["t30", "w60"])
@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_solve_matches_reference_fields(cev, name, pol):
    d = np.load(os.path.join(GOLDEN, "fdfd_fields.npz"))
    px, py, bx, by, omega, dL = d[f"{name}_meta"]
    eps, src = d[f"{name}_eps"], d[f"{name}_src"]
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps, [int(px), int(py)], bloch_phases=(bx, by), tol=1e-9)
    out = F.solve(src)
    for got, ref in zip(out, d[f"{name}_{pol}"]):
        assert _rel(got, ref) < 1e-6


def test_config1_field_gate(cev):
    """The 200x200 Ez workload: GPU field vs sparse LU <= 1e-5 rel-L2 at
    an FP64 true residual <= 1e-6."""
    from ceviche_gb300.workloads import config1
    p = config1()
    F = cev.fdfd_ez(p["omega"], p["dL"], p["eps"], p["npml"], tol=1e-6)
    hx, hy, ez = F.solve(p["src"])
    A = ofd.make_A_ez(p["omega"], p["dL"], p["eps"], p["npml"])
    b = 1j * p["omega"] * p["src"].ravel()
    assert ofd.true_residual(A, ez.ravel(), b) <= 1e-6
    ref = ofd.spsolve(A, b)
    assert _rel(ez, ref) <= 1e-5


def test_solve_batch_and_transpose(cev):
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(11)
    Nx, Ny, dL, npml = 40, 36, 40e-9, [6, 6]
    oms = 2 * np.pi * 3e8 / np.array([1.4e-6, 1.6e-6])
    eps = rng.uniform(1, 4, (Nx, Ny))
    b = rng.standard_normal((2, Nx, Ny)) + 1j * rng.standard_normal((2, Nx, Ny))
    for pol in ("ez", "hz"):
        plan = P.get_plan(pol, (Nx, Ny), dL, oms, npml)
        for tr in (False, True):
            x, info = P.solve(plan, torch.as_tensor(eps), torch.as_tensor(b), transpose=tr,
                              tol=1e-8)
            x = x.cpu().numpy()
            for k, w in enumerate(oms):
                A = ofd.make_A(pol, w, dL, eps, npml)
                A = A.T if tr else A
                assert ofd.true_residual(A, x[k].ravel(), b[k].ravel()) < 1e-8
                assert info[k]["code"] == 0


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_gradient_matches_reference(cev, pol):
    """Reverse-mode d/d eps through the GPU adjoint vs the restated ceviche
    gradient (oracle) on the full grid and the reference's central FD pins."""
    d = np.load(os.path.join(GOLDEN, "grad_fd.npz"))
    eps0, src, pix = d["fdfd_eps"], d["fdfd_src"], d["fdfd_pix"]
    omega, dL, npml = 2 * np.pi * 200e12, 1e-6, [10, 10]
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps0, npml, tol=1e-10)
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    F.eps_r = eps
    f1, f2, fz = F.solve(eps * torch.as_tensor(src, device="cuda"))
    J = (f1.abs() ** 2).sum() + (f2.abs() ** 2).sum() + (fz.abs() ** 2).sum()
    J.backward()
    g = eps.grad.cpu().numpy()
    fo = (ofd.solve_ez if pol == "ez" else ofd.solve_hz)(omega, dL, eps0, npml, eps0 * src)
    gref = (ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz)(
        omega, dL, eps0, npml, src, *[2 * c for c in fo], source_times_eps=True)
    assert _rel(g, gref) < 1e-5
    assert _rel(g.ravel()[pix], d[f"fdfd_{pol}_grad"]) < 1e-5
    assert abs(J.item() - float(d[f"fdfd_{pol}_J"])) / float(d[f"fdfd_{pol}_J"]) < 1e-8


def test_jacobian_modes(cev):
    """jacobian(reverse) vs jacobian(numerical) with the reference test's 1e-4
    norm-ratio criterion (test_gradients_fdfd.py:24, 61-73), on a small grid."""
    rng = np.random.default_rng(3)
    Nx = Ny = 14
    omega, dL, npml = 2 * np.pi * 200e12, 1e-6, [4, 4]
    eps0 = rng.random((Nx, Ny)) + 1
    src = np.zeros((Nx, Ny))
    src[7, 7] = 1.0
    F = cev.fdfd_ez(omega, dL, eps0, npml, tol=1e-11)
    srct = torch.as_tensor(src, device="cuda")

    def J(e):
        F.eps_r = e.reshape(Nx, Ny)
        hx, hy, ez = F.solve(F.eps_r * srct)
        return (ez.abs() ** 2).sum() + (hx.abs() ** 2).sum() + (hy.abs() ** 2).sum()

    gr = cev.jacobian(J, mode="reverse")(eps0.ravel())
    gn = cev.jacobian(J, mode="numerical", step_size=1e-6)(eps0.ravel())
    assert gr.shape == (1, Nx * Ny)
    assert np.linalg.norm(gn - gr) / np.linalg.norm(gn) < 1e-4


def test_solver_reports_nonconvergence(cev):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config1
    p = config1()
    plan = P.get_plan("ez", p["eps"].shape, p["dL"], p["omega"], p["npml"])
    b = 1j * p["omega"] * torch.as_tensor(p["src"])
    with pytest.warns(P.SolverWarning):
        _, info = P.solve(plan, torch.as_tensor(p["eps"]), b, max_iters=5, restart=5)
    assert info[0]["code"] == 1
    with pytest.raises(Exception):
        P.solve(plan, torch.as_tensor(p["eps"]), b, max_iters=5, restart=5, strict=True)


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_forward_mode_jacobian(cev, pol):
    """jacobian(mode='forward') through the GPU tangent solve equals reverse
    mode and numerical differences (test_gradients_fdfd.py:106-132, 164-190)."""
    rng = np.random.default_rng(4)
    Nx, Ny = 12, 10
    omega, dL, npml = 2 * np.pi * 200e12, 1e-6, [3, 3]
    eps0 = rng.random((Nx, Ny)) + 1
    src = np.zeros((Nx, Ny))
    src[6, 5] = 1.0
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps0, npml, tol=1e-11)
    srct = torch.as_tensor(src, device="cuda")

    def J(e):
        F.eps_r = e.reshape(Nx, Ny)
        f1, f2, fz = F.solve(F.eps_r * srct)
        return torch.stack([(fz.abs() ** 2).sum(), (f1.abs() ** 2).sum() + (f2.abs() ** 2).sum()])

    gf = cev.jacobian(J, mode="forward")(eps0.ravel())
    gr = cev.jacobian(J, mode="reverse")(eps0.ravel())
    gn = cev.jacobian(J, mode="numerical", step_size=1e-6)(eps0.ravel())
    assert gf.shape == gr.shape == (2, Nx * Ny)
    assert np.linalg.norm(gf - gr) / np.linalg.norm(gr) < 1e-8
    assert np.linalg.norm(gn - gf) / np.linalg.norm(gn) < 1e-4


@pytest.mark.parametrize("pol", ["ez", "hz"])
@pytest.mark.parametrize("mag", [1e-30, 1e20])
def test_solve_extreme_rhs_magnitudes(cev, pol, mag):
    """Right-hand sides far outside float32 range after non-dimensionalisation
    (e.g. adjoint cotangents of tiny fields) still solve to tolerance."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(8)
    Nx, Ny, dL, npml, om = 24, 20, 1e-6, [4, 4], 2 * np.pi * 200e12
    eps = 1 + rng.random((Nx, Ny))
    b = mag * (rng.standard_normal((Nx, Ny)) + 1j * rng.standard_normal((Nx, Ny)))
    plan = P.get_plan(pol, (Nx, Ny), dL, om, npml)
    for tr in (False, True):
        x, info = P.solve(plan, torch.as_tensor(eps), torch.as_tensor(b), transpose=tr, tol=1e-9)
        A = ofd.make_A(pol, om, dL, eps, npml)
        A = A.T if tr else A
        assert info[0]["code"] == 0
        assert ofd.true_residual(A, x.cpu().numpy().ravel(), b.ravel()) < 1e-9


@pytest.mark.parametrize("pol", ["ez", "hz"])
@pytest.mark.parametrize("reorth", [0, 1])
@pytest.mark.parametrize("shape,blocks", [((90, 77), None), ((61, 300), None), ((70, 40), "5"),
                                          ((45, 37), None)])
def test_fused_cycle_matches_multikernel(cev, pol, reorth, shape, blocks, monkeypatch):
    """The single-launch restart cycle (one problem) against the per-iteration
    launch path: both reach the FP64 tolerance (1e-7), the iterates agree to
    1e-5 relative and the iteration counts within 10%.  Shapes cover one and two
    column tiles, (CEV_FUSED_BLOCKS=5) blocks looping over several units, and an
    odd cell count (45x37: the launch path's one-cell loads)."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(17)
    Nx, Ny = shape
    dL, npml = 40e-9, [8, 7]
    om = 2 * np.pi * 3e8 / 1.5e-6
    eps = torch.as_tensor(rng.uniform(1, 5, (Nx, Ny)))
    b = torch.as_tensor(rng.standard_normal((Nx, Ny)) + 1j * rng.standard_normal((Nx, Ny)))
    plan = P.get_plan(pol, (Nx, Ny), dL, [om], npml)
    if blocks:
        monkeypatch.setenv("CEV_FUSED_BLOCKS", blocks)
    out = {}
    for mode in ("fused", "multi"):
        if mode == "multi":
            monkeypatch.setenv("CEV_FUSED_CYCLE", "0")
        for tr in (False, True):
            x, info = P.solve(plan, eps, b, transpose=tr, tol=1e-7, reorth=reorth, strict=True)
            A = ofd.make_A(pol, om, dL, eps.numpy(), npml)
            A = A.T if tr else A
            assert ofd.true_residual(A, x.cpu().numpy().ravel(), b.numpy().ravel()) < 1e-7
            out[mode, tr] = (x.cpu().numpy(), info[0]["iterations"])
    for tr in (False, True):
        (xf, itf), (xm, itm) = out["fused", tr], out["multi", tr]
        assert _rel(xf, xm) < 1e-5, (itf, itm)
        assert abs(itf - itm) <= 0.1 * itm + 2, (itf, itm)


@pytest.mark.parametrize("shared_eps", [True, False])
def test_fused_cycle_batch(cev, shared_eps, monkeypatch):
    """A batch of 5 problems through the fused cycle (one block group per
    problem, problems converging at different iterations) against the
    per-iteration launch path."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(23)
    Nx, Ny, dL, npml = 64, 52, 40e-9, [8, 8]
    oms = 2 * np.pi * 3e8 / np.array([1.3e-6, 1.45e-6, 1.55e-6, 1.7e-6, 1.9e-6])
    B = len(oms)
    eps = rng.uniform(1, 5, (Nx, Ny)) if shared_eps else rng.uniform(1, 5, (B, Nx, Ny))
    b = rng.standard_normal((B, Nx, Ny)) + 1j * rng.standard_normal((B, Nx, Ny))
    plan = P.get_plan("ez", (Nx, Ny), dL, oms, npml)
    out = {}
    for mode in ("fused", "multi"):
        if mode == "multi":
            monkeypatch.setenv("CEV_FUSED_CYCLE", "0")
        x, info = P.solve(plan, torch.as_tensor(eps), torch.as_tensor(b), tol=1e-8, strict=True)
        out[mode] = (x.cpu().numpy(), [i["iterations"] for i in info])
        for k, w in enumerate(oms):
            A = ofd.make_A("ez", w, dL, eps if shared_eps else eps[k], npml)
            assert ofd.true_residual(A, out[mode][0][k].ravel(), b[k].ravel()) < 1e-8
    (xf, itf), (xm, itm) = out["fused"], out["multi"]
    assert _rel(xf, xm) < 1e-6, (itf, itm)
    assert len(set(itf)) > 1  # the problems really finish at different iterations
    for a_, b_ in zip(itf, itm):
        assert abs(a_ - b_) <= 0.1 * b_ + 2, (itf, itm)


@pytest.mark.parametrize("pol", ["ez", "hz"])
@pytest.mark.parametrize("shape,bloch", [((40, 132), (0.0, 0.0)), ((40, 132), (0.7, -1.1)),
                                         ((16, 8), (0.3, 0.5)), ((33, 256), (0.0, 0.4))])
def test_tma_matvec_matches_column_sweep(cev, pol, shape, bloch, monkeypatch):
    """The TMA-staged Arnoldi matvec (Ez and Hz, real eps, ny % 4 == 0) against the
    column-sweep kernel in the per-iteration GMRES path: partial row and
    column tiles, Bloch phases on the periodic wrap, forward and transposed
    solves, a two-frequency batch; both reach the FP64 tolerance (1e-7)
    against the oracle matrix and agree to 1e-5."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(29)
    Nx, Ny = shape
    dL, npml = 40e-9, [5, 4]
    oms = 2 * np.pi * 3e8 / np.array([1.5e-6, 1.7e-6])
    eps = rng.uniform(1, 5, (2, Nx, Ny))
    b = rng.standard_normal((2, Nx, Ny)) + 1j * rng.standard_normal((2, Nx, Ny))
    plan = P.get_plan(pol, (Nx, Ny), dL, oms, npml, bloch=bloch)
    monkeypatch.setenv("CEV_FUSED_CYCLE", "0")
    out = {}
    for tma in ("1", "0"):
        monkeypatch.setenv("CEV_TMA_MATVEC", tma)
        for tr in (False, True):
            x, info = P.solve(plan, torch.as_tensor(eps), torch.as_tensor(b), transpose=tr, tol=1e-7,
                              strict=True)
            for k, w in enumerate(oms):
                A = ofd.make_A(pol, w, dL, eps[k], npml, bloch)
                A = A.T if tr else A
                assert ofd.true_residual(A, x[k].cpu().numpy().ravel(), b[k].ravel()) < 1e-7
            out[tma, tr] = x.cpu().numpy()
    for tr in (False, True):
        assert _rel(out["1", tr], out["0", tr]) < 1e-5
