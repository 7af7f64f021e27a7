"""Generate the golden fixtures in this directory by running the UNMODIFIED
ceviche 0.1.3 reference (forward code only) through the forward-only
autograd/matplotlib stand-in in ``refshim/``.

Usage (needs a checkout of the reference; not run by the test suite):
    python tests/golden/make_golden.py /path/to/ceviche-checkout

Fixtures (all small, seeded):
    stencil_ops.npz     A@x and A^T@x of the assembled Ez/Hz system matrices
                        (fdfd.py:172-233 via _make_A + utils.make_sparse)
    fdfd_fields.npz     fdfd_ez / fdfd_hz .solve outputs (fdfd.py:58-76)
    fdtd_fields.npz     fdtd.forward fields after TM and TE runs (fdtd.py:74-144)
    grad_fd.npz         central finite differences of reference objectives
                        (gradient pins for the FDFD and FDTD adjoints)
    fdfd_mf.npz         fdfd_mf_ez system products and solve outputs
                        (fdfd.py:247-359), plus central differences of a
                        reference objective w.r.t. eps, delta and phi
    measure.npz         utils.measure_fields time series (utils.py:316-332)
                        of Ez and Hx at three probes
    complex_eps.npz     complex (lossy) eps: A@x, A^T@x of the Ez/Hz system
                        matrices, solve outputs, and central differences of
                        the objective of test_gradients_fdfd_complex.py
                        (eps = c*eps_r, source = c*eps_r*J) in c
    modes.npz           modes.get_modes eigenvalues and eigenvectors
                        (modes.py:10-45; ARPACK phase, compare up to phase)
                        and an insert_mode source (modes.py:48-65)
"""
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(ref_root):
    sys.path.insert(0, os.path.join(HERE, "refshim"))
    sys.path.insert(0, ref_root)
    warnings.simplefilter("ignore")
    import ceviche  # noqa: E402
    from ceviche import utils, constants  # noqa: E402
    return ceviche, utils, constants


def system_matrix(F, eps, utils):
    entries, indices = F._make_A(eps.ravel())
    return utils.make_sparse(entries, indices, shape=(F.N, F.N))


def stencil_cases():
    # (Nx, Ny, npml, bloch, omega_scale, dL)
    return [
        (37, 29, [5, 4], (0.3, -0.7), 1.0, 25e-9),
        (16, 12, [3, 0], None, 1.3, 40e-9),
        (30, 30, [10, 10], None, 1.0, 1e-6),
        (9, 7, [0, 0], (1.1, 0.0), 0.8, 50e-9),
    ]
    # 1D grids (Nx or Ny == 1) are left out: the reference's own solve fails
    # there (utils.get_entries_indices on a dia-format derivative matrix).


def main(ref_root):
    ceviche, utils, constants = load_reference(ref_root)
    C_0 = constants.C_0
    rng = np.random.default_rng(20261203)
    out = {}

    # ---------------------------------------------------------------- operators
    for k, (Nx, Ny, npml, bloch, osc, dL) in enumerate(stencil_cases()):
        omega = osc * 2 * np.pi * C_0 / 1.55e-6
        if dL == 1e-6:
            omega = 2 * np.pi * 200e12
        eps = rng.uniform(1.0, 12.25, size=(Nx, Ny))
        x = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
        for pol, cls in (("ez", ceviche.fdfd_ez), ("hz", ceviche.fdfd_hz)):
            F = cls(omega, dL, eps, npml, bloch_phases=bloch)
            A = system_matrix(F, eps, utils)
            out[f"c{k}_{pol}_Ax"] = A.dot(x)
            out[f"c{k}_{pol}_ATx"] = A.T.dot(x)
        out[f"c{k}_eps"] = eps
        out[f"c{k}_x"] = x
        out[f"c{k}_meta"] = np.array([Nx, Ny, npml[0], npml[1],
                                      0.0 if bloch is None else bloch[0],
                                      0.0 if bloch is None else bloch[1], omega, dL])
    np.savez_compressed(os.path.join(HERE, "stencil_ops.npz"), **out)

    # ------------------------------------------------------------------ fields
    out = {}
    cases = [
        ("t30", 30, 30, [10, 10], None, 2 * np.pi * 200e12, 1e-6, 1.0, 2.0),
        ("w60", 60, 48, [8, 6], (0.4, 0.0), 2 * np.pi * C_0 / 1.55e-6, 25e-9, 1.0, 12.25),
    ]
    for name, Nx, Ny, npml, bloch, omega, dL, lo, hi in cases:
        eps = rng.uniform(lo, hi, size=(Nx, Ny))
        src = np.zeros((Nx, Ny))
        src[Nx // 2, Ny // 2] = 1.0
        src[npml[0] + 2, Ny // 3:Ny // 3 + 4] = 0.5
        Fe = ceviche.fdfd_ez(omega, dL, eps, npml, bloch_phases=bloch)
        Fh = ceviche.fdfd_hz(omega, dL, eps, npml, bloch_phases=bloch)
        out[f"{name}_eps"] = eps
        out[f"{name}_src"] = src
        out[f"{name}_meta"] = np.array([npml[0], npml[1], 0.0 if bloch is None else bloch[0],
                                        0.0 if bloch is None else bloch[1], omega, dL])
        out[f"{name}_ez"] = np.stack(Fe.solve(src))
        out[f"{name}_hz"] = np.stack(Fh.solve(src))
    np.savez_compressed(os.path.join(HERE, "fdfd_fields.npz"), **out)

    # -------------------------------------------------------------------- FDTD
    out = {}
    Nx, Ny, npml, dL = 24, 20, [4, 3, 0], 25e-9
    eps = rng.uniform(1.0, 6.0, size=(Nx, Ny))
    F = ceviche.fdtd(eps[:, :, None], dL, npml)
    prof = np.zeros((Nx, Ny, 1))
    prof[11, 9, 0] = 1.0
    prof[6, 14, 0] = -0.4
    steps, t0, sg = 300, 60, 15
    amps = np.exp(-(np.arange(steps) - t0) ** 2 / 2 / sg ** 2) * np.cos(0.3 * np.arange(steps))
    snaps = []
    for t in range(steps):
        f = F.forward(Jz=prof * amps[t])
        if (t + 1) % 50 == 0:
            snaps.append(f["Ez"][:, :, 0].copy())
    out["tm_eps"], out["tm_prof"], out["tm_amps"] = eps, prof[:, :, 0], amps
    out["tm_meta"] = np.array([npml[0], npml[1], dL, F.dt])
    out["tm_Ez_snaps"] = np.stack(snaps)
    for k in ("Hx", "Hy", "Dz", "Ez", "Ex", "Ey", "Hz"):
        out[f"tm_final_{k}"] = f[k][:, :, 0].copy()
    # TE run (Jx, Jy sources) plus a simultaneous Jz
    F = ceviche.fdtd(eps[:, :, None], dL, npml)
    for t in range(200):
        f = F.forward(Jx=prof * amps[t], Jy=-0.5 * prof * amps[t], Jz=0.25 * prof * amps[t])
    for k in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz"):
        out[f"te_final_{k}"] = f[k][:, :, 0].copy()
    np.savez_compressed(os.path.join(HERE, "fdtd_fields.npz"), **out)

    # ------------------------------------------------------- gradient pins (FD)
    out = {}
    # FDFD, the reference gradient-test geometry (test_gradients_fdfd.py:34-59),
    # seeded eps, objective J = sum|Fz|^2 + |Fx|^2 + |Fy|^2, source = eps*point
    Nx = Ny = 30
    omega, dL, npml = 2 * np.pi * 200e12, 1e-6, [10, 10]
    eps0 = rng.random((Nx, Ny)) + 1
    src = np.zeros((Nx, Ny))
    src[15, 15] = 1.0
    pix = rng.choice(Nx * Ny, size=12, replace=False)
    pix = np.unique(np.concatenate([pix, [15 * Ny + 15, 14 * Ny + 15, 15 * Ny + 16]]))
    h = 1e-5
    for pol, cls in (("ez", ceviche.fdfd_ez), ("hz", ceviche.fdfd_hz)):
        Fo = cls(omega, dL, eps0, npml)

        def J(e):
            Fo.eps_r = e
            a, b, c = Fo.solve(e * src)
            return np.sum(np.abs(a) ** 2) + np.sum(np.abs(b) ** 2) + np.sum(np.abs(c) ** 2)

        g = []
        for p in pix:
            ep, em = eps0.copy(), eps0.copy()
            ep.flat[p] += h
            em.flat[p] -= h
            g.append((J(ep) - J(em)) / (2 * h))
        out[f"fdfd_{pol}_grad"] = np.array(g)
        out[f"fdfd_{pol}_J"] = np.array(J(eps0))
    out["fdfd_eps"], out["fdfd_src"], out["fdfd_pix"] = eps0, src, pix

    # FDTD, the reference gradient-test geometry (test_gradients_fdtd.py:28-50)
    Nx = Ny = 8
    dL, npml = 5e-8, [2, 2, 0]
    steps, t0, sg = 500, 300, 20
    eps0 = rng.random((Nx, Ny)) + 1
    prof = np.zeros((Nx, Ny, 1))
    prof[Nx // 2, Ny // 2, 0] = 1.0
    amps = np.exp(-(np.arange(steps) - t0) ** 2 / 2 / sg ** 2)

    def S(e):
        Fd = ceviche.fdtd(e[:, :, None], dL, npml)
        s = 0.0
        for t in range(steps):
            f = Fd.forward(Jz=prof * amps[t])
            s += np.sum(f["Ex"] + f["Ey"] + f["Ez"])
        return s

    h = 1e-4
    g = np.zeros(Nx * Ny)
    for p in range(Nx * Ny):
        ep, em = eps0.copy(), eps0.copy()
        ep.flat[p] += h
        em.flat[p] -= h
        g[p] = (S(ep) - S(em)) / (2 * h)
    out["fdtd_eps"], out["fdtd_prof"], out["fdtd_amps"] = eps0, prof[:, :, 0], amps
    out["fdtd_grad"], out["fdtd_S"] = g, np.array(S(eps0))
    np.savez_compressed(os.path.join(HERE, "grad_fd.npz"), **out)
    make_mf(ceviche, utils, constants, np.random.default_rng(424242))
    make_measure(ceviche, utils, np.random.default_rng(515151))
    make_modes(ceviche, constants, np.random.default_rng(616161))
    make_complex(ceviche, utils, np.random.default_rng(717171))
    print("fixtures written to", HERE)


def make_mf(ceviche, utils, constants, rng):
    out = {}
    Nx, Ny, Nsb, nfreq = 22, 18, 2, 2
    omega, omega_mod, dL, npml = 2 * np.pi * 200e12, 2 * np.pi * 4e12, 1e-6, [5, 4]
    eps = rng.random((Nx, Ny)) + 1
    delta = 0.3 * rng.random((nfreq, Nx, Ny))
    phi = 2 * np.pi * rng.random((nfreq, Nx, Ny))
    M = 2 * Nsb + 1
    F = ceviche.fdfd_mf_ez(omega, dL, eps, omega_mod, delta, phi, Nsb, npml)
    entries, indices = F._make_A(eps.ravel(), delta.reshape(nfreq, -1), phi.reshape(nfreq, -1))
    A = utils.make_sparse(entries, indices, shape=(M * Nx * Ny, M * Nx * Ny))
    x = rng.standard_normal(M * Nx * Ny) + 1j * rng.standard_normal(M * Nx * Ny)
    src = np.zeros((M, Nx, Ny))
    src[Nsb, Nx // 2, Ny // 2] = 1.0
    src[Nsb + 1, 7, 5] = 0.4
    out.update(eps=eps, delta=delta, phi=phi, x=x, Ax=A.dot(x), ATx=A.T.dot(x), src=src,
               meta=np.array([Nsb, nfreq, omega, omega_mod, dL, npml[0], npml[1]]))
    out["fields"] = np.stack(F.solve(src))

    def J(e, d, p):
        G = ceviche.fdfd_mf_ez(omega, dL, e, omega_mod, d, p, Nsb, npml)
        hx, hy, ez = G.solve(src)
        return np.sum(np.abs(ez) ** 2) + np.sum(np.abs(hx) ** 2) + 0.5 * np.sum(np.abs(hy) ** 2)

    h = 1e-5
    pix = rng.choice(Nx * Ny, size=8, replace=False)
    ge, gd, gp = [], [], []
    for q in pix:
        e1, e2 = eps.copy(), eps.copy()
        e1.flat[q] += h
        e2.flat[q] -= h
        ge.append((J(e1, delta, phi) - J(e2, delta, phi)) / (2 * h))
        d1, d2 = delta.copy(), delta.copy()
        d1[1].flat[q] += h
        d2[1].flat[q] -= h
        gd.append((J(eps, d1, phi) - J(eps, d2, phi)) / (2 * h))
        p1, p2 = phi.copy(), phi.copy()
        p1[0].flat[q] += h
        p2[0].flat[q] -= h
        gp.append((J(eps, delta, p1) - J(eps, delta, p2)) / (2 * h))
    out.update(pix=pix, grad_eps=np.array(ge), grad_delta1=np.array(gd), grad_phi0=np.array(gp),
               J=np.array(J(eps, delta, phi)))
    np.savez_compressed(os.path.join(HERE, "fdfd_mf.npz"), **out)


def make_measure(ceviche, utils, rng):
    """measure_fields on a 34x28 grid with rods, a pulsed line source and
    three probes (a point, a weighted line, a random patch)."""
    import contextlib
    import io
    Nx, Ny, steps = 34, 28, 160
    eps = 1 + 3 * rng.random((Nx, Ny, 1))
    prof = np.zeros((Nx, Ny, 1))
    prof[10, 8:16, 0] = 1.0
    t = np.arange(steps)
    amps = np.exp(-((t - 40) / 12.0) ** 2) * np.cos(0.35 * t)
    probes = [np.zeros((Nx, Ny, 1)) for _ in range(3)]
    probes[0][20, 14, 0] = 1.0
    probes[1][25, 4:24, 0] = np.linspace(-1, 2, 20)
    probes[2][3:9, 18:26, 0] = rng.standard_normal((6, 8))
    out = dict(eps=eps[:, :, 0], prof=prof[:, :, 0], amps=amps,
               probes=np.stack([p[:, :, 0] for p in probes]), meta=np.array([5e-8, 6, 5]))
    F = ceviche.fdtd(eps, dL=5e-8, npml=[6, 5, 0])
    src = lambda k: prof * amps[k]  # noqa: E731
    with contextlib.redirect_stdout(io.StringIO()):  # the reference prints progress
        out["Ez"] = utils.measure_fields(F, src, steps, probes, component="Ez")
        out["Hx"] = utils.measure_fields(F, src, steps, probes, component="Hx")
        out["Ez_single"] = utils.measure_fields(F, src, steps, probes[1], component="Ez")
    np.savez_compressed(os.path.join(HERE, "measure.npz"), **out)


def mode_cases(rng):
    """(eps_cross, lambda, dL, npml, m): slab guides, a coupled pair, PML."""
    cases = []
    e = np.ones(120)
    e[50:70] = 12.25
    e[30:36] = 4.0
    cases.append((e, 1.55e-6, 50e-9, 0, 4))
    cases.append((e, 1.55e-6, 50e-9, 10, 3))
    e2 = np.ones(160)
    e2[40:52] = 9.0
    e2[100:112] = 9.0  # two identical guides: near-degenerate even/odd pair
    cases.append((e2, 1.3e-6, 40e-9, 12, 4))
    e3 = 1 + 2 * rng.random(64)
    e3[20:40] += 8.0
    cases.append((e3, 1.8e-6, 60e-9, 5, 2))
    return cases


def make_modes(ceviche, constants, rng):
    from ceviche import modes
    out = {}
    for c, (e, lam, dL, npml, m) in enumerate(mode_cases(rng)):
        omega = 2 * np.pi * constants.C_0 / lam
        vals, vecs = modes.get_modes(e, omega, dL, npml, m=m, filtering=False)
        out[f"eps{c}"], out[f"vals{c}"], out[f"vecs{c}"] = e, vals, vecs
        out[f"meta{c}"] = np.array([omega, dL, npml, m])
    # insert_mode on a 2D permittivity: m = 2 profile across a slice
    epsr = np.ones((40, 90))
    epsr[:, 38:50] = 12.25
    omega = 2 * np.pi * constants.C_0 / 1.55e-6
    out["ins_epsr"] = epsr
    out["ins_src"] = modes.insert_mode(omega, 50e-9, 10, slice(5, 85), epsr, m=2)
    np.savez_compressed(os.path.join(HERE, "modes.npz"), **out)


def make_complex(ceviche, utils, rng):
    out = {}
    cases = [(37, 29, [5, 4], (0.3, -0.7), 2 * np.pi * 200e12, 1e-6),
             (30, 30, [10, 10], None, 2 * np.pi * 200e12, 1e-6)]
    for c, (Nx, Ny, npml, bloch, omega, dL) in enumerate(cases):
        eps = (rng.random((Nx, Ny)) + 1) + 1j * (rng.random((Nx, Ny)) + 1)
        x = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
        src = np.zeros((Nx, Ny), dtype=complex)
        src[Nx // 2, Ny // 2] = 1e-8
        src[Nx // 3, Ny // 4] = 0.5e-8j
        out[f"eps{c}"], out[f"x{c}"], out[f"src{c}"] = eps, x, src
        out[f"meta{c}"] = np.array([omega, dL, npml[0], npml[1],
                                    *(bloch if bloch else (0.0, 0.0))])
        for pol, cls in (("ez", ceviche.fdfd_ez), ("hz", ceviche.fdfd_hz)):
            F = cls(omega, dL, eps, npml, bloch_phases=list(bloch) if bloch else None)
            A = system_matrix(F, eps, utils)
            out[f"{pol}_Ax{c}"], out[f"{pol}_ATx{c}"] = A.dot(x), A.T.dot(x)
            out[f"{pol}_fields{c}"] = np.stack(F.solve(eps * src))

            def J(cc):
                G = cls(omega, dL, cc * eps, npml, bloch_phases=list(bloch) if bloch else None)
                f1, f2, fz = G.solve(cc * eps * src)
                return np.sum(np.abs(fz) ** 2 + np.abs(f1) ** 2 + np.abs(f2) ** 2)

            h = 1e-6
            out[f"{pol}_J{c}"] = np.array(J(1.0))
            out[f"{pol}_dJdc{c}"] = np.array((J(1.0 + h) - J(1.0 - h)) / (2 * h))
    np.savez_compressed(os.path.join(HERE, "complex_eps.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CEVICHE_REF", ""))
