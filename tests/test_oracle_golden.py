"""Pins the CPU oracle to fixtures produced by the unmodified reference
(tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

from oracle import fdfd as ofd
from oracle import fdtd as oft
from tests.conftest import GOLDEN


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_operator_matches_reference(k, pol):
    d = _load("stencil_ops.npz")
    Nx, Ny, px, py, bx, by, omega, dL = d[f"c{k}_meta"]
    A = ofd.make_A(pol, omega, dL, d[f"c{k}_eps"], [int(px), int(py)], (bx, by))
    x = d[f"c{k}_x"]
    assert _rel(A.dot(x), d[f"c{k}_{pol}_Ax"]) < 1e-13
    assert _rel(A.T.dot(x), d[f"c{k}_{pol}_ATx"]) < 1e-13


@pytest.mark.parametrize("name", ["t30", "w60"])
def test_fields_match_reference(name):
    d = _load("fdfd_fields.npz")
    px, py, bx, by, omega, dL = d[f"{name}_meta"]
    eps, src = d[f"{name}_eps"], d[f"{name}_src"]
    ez = ofd.solve_ez(omega, dL, eps, [int(px), int(py)], src, (bx, by))
    hz = ofd.solve_hz(omega, dL, eps, [int(px), int(py)], src, (bx, by))
    for got, ref in zip(ez, d[f"{name}_ez"]):
        assert _rel(got, ref) < 1e-10
    for got, ref in zip(hz, d[f"{name}_hz"]):
        assert _rel(got, ref) < 1e-10


def test_fdtd_tm_matches_reference():
    d = _load("fdtd_fields.npz")
    px, py, dL, dt = d["tm_meta"]
    assert oft.time_step(dL) == dt
    F, snaps = oft.run_tm(d["tm_eps"], dL, [int(px), int(py), 0], d["tm_prof"], d["tm_amps"],
                          record_every=50)
    for s, r in zip(snaps, d["tm_Ez_snaps"]):
        assert _rel(s, r) < 1e-12
    for k in ("Hx", "Hy", "Dz", "Ez", "Ex", "Ey", "Hz"):
        ref = d[f"tm_final_{k}"]
        if np.all(ref == 0):
            assert np.all(F.f[k] == 0)
        else:
            assert _rel(F.f[k], ref) < 1e-12


def test_fdtd_te_matches_reference():
    d = _load("fdtd_fields.npz")
    px, py, dL, dt = d["tm_meta"]
    F = oft.FDTD2D(d["tm_eps"], dL, [int(px), int(py), 0])
    p, a = d["tm_prof"], d["tm_amps"]
    for t in range(200):
        F.forward(Jx=p * a[t], Jy=-0.5 * p * a[t], Jz=0.25 * p * a[t])
    for k in oft.FDTD2D.FIELDS:
        assert _rel(F.f[k], d[f"te_final_{k}"]) < 1e-12, k


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_fdfd_adjoint_matches_reference_fd(pol):
    """Restated reverse-mode gradient vs central differences of the reference."""
    d = _load("grad_fd.npz")
    eps, src, pix = d["fdfd_eps"], d["fdfd_src"], d["fdfd_pix"]
    omega, dL, npml = 2 * np.pi * 200e12, 1e-6, [10, 10]
    solve = ofd.solve_ez if pol == "ez" else ofd.solve_hz
    f = solve(omega, dL, eps, npml, eps * src)
    # J = sum |f|^2 over the three components -> torch cotangent g = 2 f
    g = [2 * c for c in f]
    gradf = ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz
    grad = gradf(omega, dL, eps, npml, src, *g, source_times_eps=True)
    ref = d[f"fdfd_{pol}_grad"]
    assert _rel(grad.ravel()[pix], ref) < 1e-8


def test_fdtd_adjoint_matches_reference_fd():
    d = _load("grad_fd.npz")
    eps, prof, amps = d["fdtd_eps"], d["fdtd_prof"], d["fdtd_amps"]
    grad = oft.adjoint_tm(eps, 5e-8, [2, 2, 0], prof, amps, np.ones_like(eps), np.ones(len(amps)))
    assert _rel(grad.ravel(), d["fdtd_grad"]) < 1e-6


def test_mf_operator_and_fields_match_reference():
    d = _load("fdfd_mf.npz")
    Nsb, nfreq, omega, omega_mod, dL, px, py = d["meta"]
    Nsb = int(Nsb)
    npml = [int(px), int(py)]
    A = ofd.make_A_mf_ez(omega, dL, d["eps"], npml, omega_mod, d["delta"], d["phi"], Nsb)
    assert _rel(A.dot(d["x"]), d["Ax"]) < 1e-13
    assert _rel(A.T.dot(d["x"]), d["ATx"]) < 1e-13
    f = ofd.solve_mf_ez(omega, dL, d["eps"], npml, omega_mod, d["delta"], d["phi"], Nsb, d["src"])
    for got, ref in zip(f, d["fields"]):
        assert _rel(got, ref) < 1e-10


def test_measure_fields_matches_reference():
    """oracle.fdtd.measure_fields vs the reference's utils.measure_fields."""
    d = np.load(os.path.join(GOLDEN, "measure.npz"))
    dL, px, py = d["meta"]
    F = oft.FDTD2D(d["eps"], dL, [int(px), int(py), 0])
    src = lambda t: d["prof"] * d["amps"][t]  # noqa: E731
    probes = list(d["probes"])
    steps = len(d["amps"])
    for comp in ("Ez", "Hx"):
        m = oft.measure_fields(F, src, steps, probes, component=comp)
        assert np.linalg.norm(m - d[comp]) <= 1e-12 * np.linalg.norm(d[comp]), comp
    m = oft.measure_fields(F, src, steps, d["probes"][1], component="Ez")
    assert np.linalg.norm(m - d["Ez_single"]) <= 1e-12 * np.linalg.norm(d["Ez_single"])


def _same_up_to_phase(a, b, clusters=()):
    """Columns of a and b equal up to a unit phase; column groups listed in
    clusters (near-degenerate eigenvalues) compared as subspaces."""
    done = set()
    for grp in clusters:
        qa, qb = np.linalg.qr(a[:, grp])[0], np.linalg.qr(b[:, grp])[0]
        s = np.linalg.svd(qa.conj().T @ qb, compute_uv=False)  # principal angle cosines
        assert np.all(np.abs(s - 1) < 1e-8), s
        done |= set(grp)
    for j in range(a.shape[1]):
        if j not in done:
            assert abs(abs(np.vdot(a[:, j], b[:, j])) - 1) < 1e-10, j


def test_modes_match_reference():
    """oracle.modes.get_modes vs the reference's ARPACK get_modes."""
    from oracle import modes as om
    d = np.load(os.path.join(GOLDEN, "modes.npz"))
    for c in range(4):
        omega, dL, npml, m = d[f"meta{c}"]
        vals, vecs = om.get_modes(d[f"eps{c}"], omega, dL, int(npml), int(m), filtering=False)
        ref_v = d[f"vals{c}"]
        clusters = [(0, 1)] if c == 2 else []  # even/odd pair split by 3e-11
        assert np.max(np.abs(np.sort_complex(vals) - np.sort_complex(ref_v))) < 1e-9
        _same_up_to_phase(vecs, d[f"vecs{c}"], clusters)
    src = om.insert_mode(omega=2 * np.pi * om.C_0 / 1.55e-6, dx=50e-9, x=10, y=slice(5, 85),
                         epsr=d["ins_epsr"], m=2)
    ref = d["ins_src"]
    assert abs(abs(np.vdot(src[10, 5:85], ref[10, 5:85])) - 1) < 1e-10
    assert np.all(src[np.arange(40) != 10] == 0)


@pytest.mark.parametrize("k", range(2))
@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_complex_eps_operator_and_fields_match_reference(k, pol):
    """Complex (lossy) eps: the restated system matrices and solves against
    the reference's (fdfd.py accepts a complex eps_r)."""
    d = _load("complex_eps.npz")
    omega, dL, px, py, bx, by = d[f"meta{k}"]
    eps, x, src = d[f"eps{k}"], d[f"x{k}"], d[f"src{k}"]
    npml, bloch = [int(px), int(py)], (bx, by)
    A = ofd.make_A(pol, omega, dL, eps, npml, bloch)
    assert _rel(A.dot(x), d[f"{pol}_Ax{k}"]) < 1e-13
    assert _rel(A.T.dot(x), d[f"{pol}_ATx{k}"]) < 1e-13
    solve = ofd.solve_ez if pol == "ez" else ofd.solve_hz
    for got, ref in zip(solve(omega, dL, eps, npml, eps * src, bloch), d[f"{pol}_fields{k}"]):
        assert _rel(got, ref) < 1e-10


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_complex_eps_oracle_gradient_vs_central_differences(pol):
    """The oracle's complex-eps gradient (conj of the holomorphic sensitivity:
    dL/dRe + i dL/dIm) against complex central differences of the oracle
    objective, source proportional to eps as in the reference tests."""
    rng = np.random.default_rng(8)
    Nx, Ny, omega, dL, npml = 14, 11, 2 * np.pi * 200e12, 1e-6, [3, 3]
    eps = (rng.random((Nx, Ny)) + 1) + 0.05j * (rng.random((Nx, Ny)) + 1)
    Jz = np.zeros((Nx, Ny))
    Jz[7, 5] = 1.0
    solve = ofd.solve_ez if pol == "ez" else ofd.solve_hz
    gradf = ofd.grad_eps_ez if pol == "ez" else ofd.grad_eps_hz

    def L(e):
        f = solve(omega, dL, e, npml, e * Jz)
        return sum(np.sum(np.abs(c) ** 2) for c in f)

    f = solve(omega, dL, eps, npml, eps * Jz)
    g = gradf(omega, dL, eps, npml, Jz, *[2 * c for c in f], source_times_eps=True)
    assert np.iscomplexobj(g)
    h = 1e-4
    pix = [(7, 5), (8, 5), (6, 7), (9, 3)]
    nums = []
    for i, j in pix:
        num = 0j
        for unit, part in ((1.0, 1.0), (1j, 1j)):
            ep, em = eps.copy(), eps.copy()
            ep[i, j] += unit * h
            em[i, j] -= unit * h
            num += part * (L(ep) - L(em)) / (2 * h)
        nums.append(num)
    nums, gp = np.array(nums), np.array([g[i, j] for i, j in pix])
    # the reference gradient tests' criterion (norm ratio, ALLOWED_RATIO 1e-4)
    assert np.linalg.norm(nums - gp) / np.linalg.norm(nums) <= 1e-4, (nums, gp)
