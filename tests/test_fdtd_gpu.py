"""FDTD parity on the GPU against the reference fixtures and the FP64 oracle.

Tolerances: float64 kernels 1e-11 relative L2 (pure FP64 recurrence, only
re-association differs); float32 kernels 2e-5 relative L2 over a few hundred
steps; the time-blocked runner 1e-6 vs the per-step kernels (same
arithmetic); config 2 (400x400, 2000 steps, float32 vs FP64) rel-L2 of Ez
every 100 steps <= 1e-3."""
import os

import numpy as np
import pytest
import torch

from oracle import fdtd as oft
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


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("precision,tol", [("float64", 1e-11), ("float32", 2e-5)])
def test_tm_steps_match_reference(cev, precision, tol):
    d = np.load(os.path.join(GOLDEN, "fdtd_fields.npz"))
    px, py, dL, dt = d["tm_meta"]
    F = cev.fdtd(d["tm_eps"][:, :, None], dL, [int(px), int(py), 0], precision=precision)
    assert F.dt == dt
    prof, amps = d["tm_prof"], d["tm_amps"]
    k = 0
    for t in range(len(amps)):
        f = F.forward(Jz=prof * amps[t])
        if (t + 1) % 50 == 0:
            assert _rel(_np(f["Ez"])[:, :, 0], d["tm_Ez_snaps"][k]) < tol
            k += 1
    for key in ("Hx", "Hy", "Dz", "Ez"):
        assert _rel(_np(f[key])[:, :, 0], d[f"tm_final_{key}"]) < tol
    for key in ("Ex", "Ey", "Hz"):
        assert np.all(_np(f[key]) == 0)


@pytest.mark.parametrize("precision,tol", [("float64", 1e-11), ("float32", 2e-5)])
def test_te_and_tm_steps_match_reference(cev, precision, tol):
    d = np.load(os.path.join(GOLDEN, "fdtd_fields.npz"))
    px, py, dL, dt = d["tm_meta"]
    F = cev.fdtd(d["tm_eps"], dL, [int(px), int(py), 0], precision=precision)
    p, a = d["tm_prof"], d["tm_amps"]
    for t in range(200):
        f = F.forward(Jx=p * a[t], Jy=-0.5 * p * a[t], Jz=0.25 * p * a[t])
    for key in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz"):
        assert _rel(_np(f[key])[:, :, 0], d[f"te_final_{key}"]) < tol, key


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("shape", [(96, 80), (131, 77)])
def test_blocked_runner_matches_steps(cev, precision, shape):
    """Time-blocked TM runner == per-step kernels (sources, probes, PML, odd sizes)."""
    rng = np.random.default_rng(7)
    Nx, Ny = shape
    eps = 1 + 5 * rng.random((Nx, Ny))
    dL, npml, steps = 25e-9, [10, 7, 0], 57
    src = np.zeros((Nx, Ny))
    src[Nx // 2, Ny // 3] = 1.0
    src[3, Ny - 2] = -0.5  # inside the PML, near the periodic wrap
    amps = np.sin(0.2 * np.arange(steps)) * np.exp(-((np.arange(steps) - 20) / 10.0) ** 2)
    probes = [(Nx // 2, Ny // 3), (0, 0), (Nx - 1, Ny - 1), (40, 41)]
    A = cev.fdtd(eps, dL, npml, precision=precision)
    series = _np(A.run(steps, src, amps, probes))
    B = cev.fdtd(eps, dL, npml, precision=precision)
    ref = []
    for t in range(steps):
        f = B.forward(Jz=src * amps[t])
        ez = _np(f["Ez"])[:, :, 0]
        ref.append([ez[i, j] for i, j in probes])
    tol = 1e-6 if precision == "float32" else 1e-13
    assert _rel(series, np.array(ref)) < tol
    assert _rel(_np(A.fields["Ez"]), _np(B.fields["Ez"])) < tol
    assert _rel(_np(A.fields["Hx"]), _np(B.fields["Hx"])) < tol


def test_config2_parity(cev):
    """The 400x400 TM workload (2000 steps): float32 GPU vs FP64 oracle,
    rel-L2 of Ez every 100 steps."""
    from ceviche_gb300.workloads import config2
    p = config2()
    F = cev.fdtd(p["eps"], p["dL"], p["npml"], precision="float32")
    O = oft.FDTD2D(p["eps"], p["dL"], p["npml"])
    worst = 0.0
    for k in range(20):
        F.run(100, p["src"], p["amps"][k * 100:(k + 1) * 100])
        for t in range(k * 100, (k + 1) * 100):
            O.forward(Jz=p["src"] * p["amps"][t])
        worst = max(worst, _rel(_np(F.fields["Ez"])[:, :, 0], O.f["Ez"]))
    assert worst <= 1e-3, worst


@pytest.mark.parametrize("precision,tol", [("float64", 1e-8), ("float32", 1e-4)])
def test_adjoint_matches_reference_fd(cev, precision, tol):
    """Reverse-time adjoint with checkpoints vs the reference's central FD on
    its gradient-test geometry (8x8, 500 steps, sum of E over all steps)."""
    d = np.load(os.path.join(GOLDEN, "grad_fd.npz"))
    eps0, prof, amps = d["fdtd_eps"], d["fdtd_prof"], d["fdtd_amps"]
    Nx, Ny = eps0.shape
    probes = [(i, j) for i in range(Nx) for j in range(Ny)]
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    series = cev.fdtd_probe_series(eps, 5e-8, [2, 2, 0], len(amps), prof, amps, probes,
                                   precision=precision, ckpt_every=64)
    S = series.sum()
    S.backward()
    assert abs(S.item() - float(d["fdtd_S"])) / abs(float(d["fdtd_S"])) < (1e-12 if precision == "float64" else 1e-5)
    assert _rel(_np(eps.grad).ravel(), d["fdtd_grad"]) < tol


def test_adjoint_matches_oracle_with_pml_and_probe(cev):
    rng = np.random.default_rng(9)
    Nx, Ny, steps = 50, 44, 300
    eps0 = 1 + 4 * rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[25, 20] = 1.0
    amps = np.exp(-((np.arange(steps) - 60) / 15.0) ** 2) * np.cos(0.4 * np.arange(steps))
    probes = [(30, 30), (8, 36), (45, 5)]
    wts = rng.standard_normal((steps, len(probes)))
    eps = torch.tensor(eps0, device="cuda", requires_grad=True)
    s = cev.fdtd_probe_series(eps, 25e-9, [8, 6, 0], steps, src, amps, probes,
                              precision="float64", ckpt_every=37)
    (s * torch.as_tensor(wts, device="cuda")).sum().backward()
    probe = np.zeros((Nx, Ny))
    g = np.zeros((Nx, Ny))
    for k, (i, j) in enumerate(probes):
        probe[:] = 0
        probe[i, j] = 1
        g += oft.adjoint_tm(eps0, 25e-9, [8, 6, 0], src, amps, probe, wts[:, k])
    assert _rel(_np(eps.grad), g) < 1e-10


@pytest.mark.parametrize("tile", range(6))  # every entry of TILE_CFGS in csrc/fdtd.cu
def test_every_tile_configuration(cev, tile, monkeypatch):
    """Each time-blocked tile shape (forced through CEV_FDTD_TILE) matches the
    per-step kernels on an odd-sized grid with PML, a source and probes."""
    monkeypatch.setenv("CEV_FDTD_TILE", str(tile))
    rng = np.random.default_rng(12)
    Nx, Ny = 141, 133
    eps = 1 + 5 * rng.random((Nx, Ny))
    dL, npml, steps = 25e-9, [12, 9, 0], 37
    src = np.zeros((Nx, Ny))
    src[70, 40] = 1.0
    src[2, 131] = 0.3
    amps = np.cos(0.3 * np.arange(steps)) * np.exp(-((np.arange(steps) - 15) / 8.0) ** 2)
    probes = [(70, 40), (0, 0), (140, 132), (66, 100)]
    A = cev.fdtd(eps, dL, npml)
    series = _np(A.run(steps, src, amps, probes))
    monkeypatch.delenv("CEV_FDTD_TILE")
    B = cev.fdtd(eps, dL, npml)
    ref = []
    for t in range(steps):
        ez = _np(B.forward(Jz=src * amps[t])["Ez"])[:, :, 0]
        ref.append([ez[i, j] for i, j in probes])
    assert _rel(series, np.array(ref)) < 1e-6
    for k in ("Ez", "Hx", "Hy", "Dz"):
        assert _rel(_np(A.fields[k]), _np(B.fields[k])) < 1e-6


@pytest.mark.parametrize("cfg", range(4))  # every entry of PERSIST_CFGS in csrc/fdtd.cu
@pytest.mark.parametrize("shape,steps", [((141, 133), 85), ((141, 133), 93), ((70, 70), 61)])
def test_every_persistent_configuration(cev, cfg, shape, steps, monkeypatch):
    """The single-launch runner (forced through CEV_FDTD_PERSIST; tiles keep
    their region resident and exchange K-wide rings through flags) matches the
    per-step kernels: odd grids with PML, sources and probes, an odd and an
    even number of K-step blocks, and a 70x70 grid whose last tile row holds
    two real rows (its ring wraps across two tile rows)."""
    monkeypatch.setenv("CEV_FDTD_PERSIST", str(cfg + 1))
    rng = np.random.default_rng(31)
    Nx, Ny = shape
    eps = 1 + 5 * rng.random((Nx, Ny))
    dL, npml = 25e-9, [12, 9, 0]
    src = np.zeros((Nx, Ny))
    src[Nx // 2, 40] = 1.0
    src[2, Ny - 2] = 0.3
    amps = np.cos(0.3 * np.arange(steps)) * np.exp(-((np.arange(steps) - 15) / 8.0) ** 2)
    probes = [(Nx // 2, 40), (0, 0), (Nx - 1, Ny - 1), (Nx // 2 - 4, Ny - 33)]
    A = cev.fdtd(eps, dL, npml)
    series = _np(A.run(steps, src, amps, probes))
    for fld in (A, ):  # a second run continues from the first run's state
        series2 = _np(fld.run(steps, src, amps, probes))
    monkeypatch.setenv("CEV_FDTD_PERSIST", "0")
    B = cev.fdtd(eps, dL, npml)
    ref = []
    for rep in range(2):
        for t in range(steps):
            ez = _np(B.forward(Jz=src * amps[t])["Ez"])[:, :, 0]
            ref.append([ez[i, j] for i, j in probes])
    assert _rel(np.concatenate([series, series2]), np.array(ref)) < 1e-6
    for k in ("Ez", "Hx", "Hy", "Dz"):
        assert _rel(_np(A.fields[k]), _np(B.fields[k])) < 1e-6


@pytest.mark.parametrize("cfg", range(6))  # every entry of STRIP_CFGS in csrc/fdtd.cu
@pytest.mark.parametrize("shape,steps", [((141, 133), 85), ((141, 133), 93), ((70, 70), 61)])
def test_every_strip_configuration(cev, cfg, shape, steps, monkeypatch):
    """The register-strip runner (forced through CEV_FDTD_STRIP; state in
    registers, neighbours by warp shuffle, single launch with the ring
    exchange) matches the per-step kernels: odd grids with PML, two sources
    and four probes (two at the same cell), an odd and an even number of
    K-step blocks, a 70x70 grid with a partial last tile row, and a second
    run continuing from the first."""
    monkeypatch.setenv("CEV_FDTD_STRIP", str(cfg + 1))
    rng = np.random.default_rng(41)
    Nx, Ny = shape
    eps = 1 + 5 * rng.random((Nx, Ny))
    dL, npml = 25e-9, [12, 9, 0]
    src = np.zeros((Nx, Ny))
    src[Nx // 2, 40] = 1.0
    src[2, Ny - 2] = 0.3
    amps = np.cos(0.3 * np.arange(steps)) * np.exp(-((np.arange(steps) - 15) / 8.0) ** 2)
    probes = [(Nx // 2, 40), (0, 0), (Nx - 1, Ny - 1), (Nx // 2, 40)]
    A = cev.fdtd(eps, dL, npml)
    series = _np(A.run(steps, src, amps, probes))
    series2 = _np(A.run(steps, src, amps, probes))
    monkeypatch.setenv("CEV_FDTD_STRIP", "0")
    monkeypatch.setenv("CEV_FDTD_PERSIST", "0")
    B = cev.fdtd(eps, dL, npml)
    ref = []
    for rep in range(2):
        for t in range(steps):
            ez = _np(B.forward(Jz=src * amps[t])["Ez"])[:, :, 0]
            ref.append([ez[i, j] for i, j in probes])
    assert _rel(np.concatenate([series, series2]), np.array(ref)) < 1e-6
    for k in ("Ez", "Hx", "Hy", "Dz"):
        assert _rel(_np(A.fields[k]), _np(B.fields[k])) < 1e-6


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("shape", [(96, 80), (131, 77), (40, 36)])
def test_te_runner_matches_steps(cev, precision, shape):
    """Time-blocked TE runner (cev_fdtd_run_te; per-step kernels below one
    tile region, 40x36) == per-step TE kernels with dense Jx, Jy (sources in
    the PML and near the periodic wrap, probes, two runs in a row)."""
    rng = np.random.default_rng(17)
    Nx, Ny = shape
    eps = 1 + 5 * rng.random((Nx, Ny))
    dL, npml, steps = 25e-9, [10, 7, 0], 45
    sx = np.zeros((Nx, Ny))
    sy = np.zeros((Nx, Ny))
    sx[Nx // 2, Ny // 3] = 1.0
    sy[Nx // 2, Ny // 3] = -0.4
    sy[3, Ny - 2] = 0.7
    amps = np.sin(0.2 * np.arange(steps)) * np.exp(-((np.arange(steps) - 20) / 10.0) ** 2)
    probes = [(Nx // 2, Ny // 3), (0, 0), (Nx - 1, Ny - 1), (20, 21)]
    A = cev.fdtd(eps, dL, npml, precision=precision)
    series = np.concatenate([_np(A.run_te(steps, sx, sy, amps, probes)) for _ in range(2)])
    B = cev.fdtd(eps, dL, npml, precision=precision)
    ref = []
    for rep in range(2):
        for t in range(steps):
            f = B.forward(Jx=sx * amps[t], Jy=sy * amps[t])
            hz = _np(f["Hz"])[:, :, 0]
            ref.append([hz[i, j] for i, j in probes])
    tol = 1e-6 if precision == "float32" else 1e-13
    assert _rel(series, np.array(ref)) < tol
    for k in ("Hz", "Dx", "Dy", "Ex", "Ey"):
        assert _rel(_np(A.fields[k]), _np(B.fields[k])) < tol, k


@pytest.mark.parametrize("precision,tol", [("float64", 1e-8), ("float32", 2e-4)])
def test_per_step_autograd_like_reference_test(cev, precision, tol):
    """The reference gradient test pattern (test_gradients_fdtd.py:66-88):
    jacobian over a Python loop of F.forward(Jz=...) summing E each step,
    against the reference's central differences."""
    d = np.load(os.path.join(GOLDEN, "grad_fd.npz"))
    eps0, prof, amps = d["fdtd_eps"], d["fdtd_prof"], d["fdtd_amps"]
    Nx, Ny = eps0.shape
    F = cev.fdtd(eps0[:, :, None], dL=5e-8, npml=[2, 2, 0], precision=precision)
    src = torch.as_tensor(prof[:, :, None], device="cuda")

    def objective(eps_arr):
        F.eps_r = eps_arr.reshape((Nx, Ny, 1))
        S = 0.0
        for t in range(len(amps)):
            fields = F.forward(Jz=src * float(amps[t]))
            S = S + torch.sum(fields["Ex"] + fields["Ey"] + fields["Ez"])
        return S

    jac = cev.jacobian(objective, mode="reverse")(eps0.ravel())
    assert jac.shape == (1, Nx * Ny)
    assert _rel(jac.ravel(), d["fdtd_grad"]) < tol
