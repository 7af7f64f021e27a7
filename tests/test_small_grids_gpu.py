"""Small and odd grids that exercise launch-shape edges (partial column
tiles, row chunks of one, grids smaller than a time-blocked tile region):
FDFD solve / fields / eps gradient and FDTD steps / runner against the FP64
oracle.  Tolerances as in the main suites."""
import numpy as np
import pytest
import torch

from oracle import fdfd as ofd
from oracle import fdtd as oft

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


SHAPES = [(7, 5), (5, 7), (33, 17), (17, 33), (3, 260), (130, 3)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_fdfd_small_grids(cev, shape, pol):
    rng = np.random.default_rng(sum(shape))
    Nx, Ny = shape
    omega, dL = 2 * np.pi * 200e12, 1e-6
    npml = [min(2, Nx // 3), min(2, Ny // 3)]
    eps0 = 1 + rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[Nx // 2, Ny // 2] = 1.0
    cls = cev.fdfd_ez if pol == "ez" else cev.fdfd_hz
    F = cls(omega, dL, eps0, npml, tol=1e-10)
    got = F.solve(src)
    ref = (ofd.solve_ez if pol == "ez" else ofd.solve_hz)(omega, dL, eps0, npml, src)
    for g, r in zip(got, ref):
        assert _rel(g, r) < 1e-7
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    F.eps_r = eps
    f1, f2, fz = F.solve(torch.as_tensor(src, device="cuda"))
    L = (fz.abs() ** 2).sum() + (f1.abs() ** 2).sum() + (f2.abs() ** 2).sum()
    L.backward()
    gref = (ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz)(
        omega, dL, eps0, npml, src, *[2 * c for c in ref])
    assert _rel(eps.grad.cpu().numpy(), gref) < 1e-6


@pytest.mark.parametrize("shape", SHAPES)
def test_fdtd_small_grids(cev, shape):
    rng = np.random.default_rng(3 + sum(shape))
    Nx, Ny = shape
    eps = 1 + 3 * rng.random((Nx, Ny))
    npml = [min(2, Nx // 3), min(2, Ny // 3), 0]
    src = np.zeros((Nx, Ny))
    src[Nx // 2, Ny // 2] = 1.0
    amps = np.exp(-((np.arange(40) - 10) / 4.0) ** 2)
    F = cev.fdtd(eps, 5e-8, npml, precision="float64")
    O = oft.FDTD2D(eps, 5e-8, npml)
    for a in amps:
        f = F.forward(Jz=src * a)
        O.forward(Jz=src * a)
    assert _rel(f["Ez"].cpu().numpy()[:, :, 0], O.f["Ez"]) < 1e-11
    R = cev.fdtd(eps, 5e-8, npml, precision="float64")
    R.run(len(amps), src, amps)
    assert _rel(R.fields["Ez"].cpu().numpy()[:, :, 0], O.f["Ez"]) < 1e-11
