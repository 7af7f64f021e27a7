"""Complex (lossy) permittivity on the GPU path: ceviche's fdfd accepts a
complex eps_r (fdfd.py:40-44) and its enabled complex tests run forward-mode
jacobians through it (tests/test_gradients_fdfd_complex.py:106-132, 164-190).
Pinned to the reference's own outputs (tests/golden/complex_eps.npz):
operators 1e-13 (complex128) / 2e-6 (complex64), fields 1e-6 at a 1e-10
solve, forward-mode dJ/dc 1e-4 (the reference tests' ratio); reverse-mode
dL/d(eps) (PyTorch convention dL/dRe + i dL/dIm) against the oracle 1e-6."""
import os

import numpy as np
import pytest
import torch

from oracle import fdfd as ofd
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def _case(k):
    d = np.load(os.path.join(GOLDEN, "complex_eps.npz"))
    omega, dL, px, py, bx, by = d[f"meta{k}"]
    return d, omega, dL, [int(px), int(py)], (bx, by)


@pytest.mark.parametrize("k", range(2))
@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_operator_and_fields(cev, k, pol):
    from ceviche_gb300 import primitives as P
    d, omega, dL, npml, bloch = _case(k)
    eps, x, src = d[f"eps{k}"], d[f"x{k}"], d[f"src{k}"]
    Nx, Ny = eps.shape
    plan = P.get_plan(pol, (Nx, Ny), dL, [omega], npml, bloch)
    et = torch.as_tensor(eps)
    xt = torch.as_tensor(x.reshape(Nx, Ny))
    for tr, key in ((False, "Ax"), (True, "ATx")):
        y = P.apply(plan, et, xt, transpose=tr).cpu().numpy()
        assert _rel(y, d[f"{pol}_{key}{k}"]) < 1e-13
        y32 = P.apply(plan, et, xt, transpose=tr, precision="c64").cpu().numpy()
        assert _rel(y32, d[f"{pol}_{key}{k}"]) < 2e-6
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps, npml, bloch_phases=list(bloch), tol=1e-10)
    for got, ref in zip(F.solve(eps * src), d[f"{pol}_fields{k}"]):
        assert _rel(got, ref) < 1e-6


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_forward_mode_like_reference(cev, pol):
    """test_gradients_fdfd_complex.py's enabled tests: J(c) with
    eps = c*eps_r and source = c*eps_r*J, jacobian(mode='forward') at c=1."""
    d, omega, dL, npml, _ = _case(1)
    eps, src = d["eps1"], d["src1"]
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps, npml, tol=1e-11)
    et = torch.as_tensor(eps, device="cuda")
    st = torch.as_tensor(src, device="cuda")

    def J(c):
        F.eps_r = c * et
        f1, f2, fz = F.solve(c * et * st)
        return (fz.abs() ** 2).sum() + (f1.abs() ** 2).sum() + (f2.abs() ** 2).sum()

    gf = np.ravel(cev.jacobian(J, mode="forward")(np.array([1.0])))
    ref = float(d[f"{pol}_dJdc1"])
    assert abs(gf[0] - ref) / abs(ref) < 1e-4
    assert abs(J(torch.tensor(1.0, device="cuda", dtype=torch.float64)).item()
               - float(d[f"{pol}_J1"])) / float(d[f"{pol}_J1"]) < 1e-8


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_reverse_gradient_vs_oracle(cev, pol):
    rng = np.random.default_rng(31)
    Nx, Ny, omega, dL, npml = 26, 21, 2 * np.pi * 200e12, 1e-6, [5, 4]
    eps0 = (rng.random((Nx, Ny)) + 1) + 0.3j * (rng.random((Nx, Ny)) + 0.5)
    Jz = np.zeros((Nx, Ny))
    Jz[13, 10] = 1.0
    Jz[6, 15] = -0.4
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps0, npml, tol=1e-11)
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    F.eps_r = eps
    f1, f2, fz = F.solve(eps * torch.as_tensor(Jz, device="cuda"))
    L = (fz.abs() ** 2).sum() + 0.5 * (f1.abs() ** 2).sum() + 2.0 * (f2.abs() ** 2).sum()
    L.backward()
    g = eps.grad.cpu().numpy()
    assert np.iscomplexobj(g)
    fo = (ofd.solve_ez if pol == "ez" else ofd.solve_hz)(omega, dL, eps0, npml, eps0 * Jz)
    gref = (ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz)(
        omega, dL, eps0, npml, Jz, 2 * 0.5 * fo[0], 2 * 2.0 * fo[1], 2 * fo[2],
        source_times_eps=True)
    assert _rel(g, gref) < 1e-6


def test_fused_and_batched_complex(cev, monkeypatch):
    """Complex eps through the fused cycle (batch of 3 frequencies) and the
    per-iteration launch path agree and solve the complex system."""
    from ceviche_gb300 import primitives as P
    rng = np.random.default_rng(5)
    Nx, Ny, dL, npml = 40, 33, 40e-9, [6, 6]
    oms = 2 * np.pi * 3e8 / np.array([1.4e-6, 1.55e-6, 1.7e-6])
    eps = (1 + 3 * rng.random((Nx, Ny))) + 0.2j * rng.random((Nx, Ny))
    b = rng.standard_normal((3, Nx, Ny)) + 1j * rng.standard_normal((3, Nx, Ny))
    out = {}
    for pol in ("ez", "hz"):
        plan = P.get_plan(pol, (Nx, Ny), dL, oms, npml)
        for mode in ("1", "0"):
            monkeypatch.setenv("CEV_FUSED_CYCLE", mode)
            x, info = P.solve(plan, torch.as_tensor(eps), torch.as_tensor(b), tol=1e-9, strict=True)
            out[pol, mode] = x.cpu().numpy()
            for k, w in enumerate(oms):
                A = ofd.make_A(pol, w, dL, eps, npml)
                assert ofd.true_residual(A, out[pol, mode][k].ravel(), b[k].ravel()) < 1e-9
        assert _rel(out[pol, "1"], out[pol, "0"]) < 1e-6
