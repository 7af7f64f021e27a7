"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (all inputs generated; no dataset is involved).

config k uses seed 1000 + k; problem i of a batch uses seed (1000 + k)*100000 + i.
"""
import numpy as np

from .constants import C_0


def _rng(seed):
    return np.random.default_rng(seed)


def config1(seed=1001):
    """Plain FDFD Ez, 200x200, dL=25 nm, npml 20, lambda 1.55 um: eps 1, a
    10-cell eps=12.25 waveguide (j in [95,105) along x), a 40x40 central
    design block eps ~ U[1, 12.25], a 10-cell line source at i = npml+10."""
    rng = _rng(seed)
    Nx = Ny = 200
    npml = 20
    eps = np.ones((Nx, Ny))
    eps[:, 95:105] = 12.25
    eps[80:120, 80:120] = rng.uniform(1.0, 12.25, size=(40, 40))
    src = np.zeros((Nx, Ny))
    src[npml + 10, 95:105] = 1.0
    return dict(omega=2 * np.pi * C_0 / 1.55e-6, dL=25e-9, eps=eps, npml=[npml, npml], src=src)


def rods_eps(Nx, Ny, npml, n_rods, rng):
    """eps 1 plus n_rods circular rods (radius 4..12 cells, eps ~ U[2, 12.25])
    centred in the non-PML interior; later rods overwrite earlier ones."""
    eps = np.ones((Nx, Ny))
    for _ in range(n_rods):
        ci = rng.uniform(npml, Nx - npml)
        cj = rng.uniform(npml, Ny - npml)
        r = rng.integers(4, 13)
        e = rng.uniform(2.0, 12.25)
        # only the rod's bounding window can satisfy the disc test
        i0, i1 = max(0, int(np.floor(ci - r))), min(Nx, int(np.ceil(ci + r)) + 1)
        j0, j1 = max(0, int(np.floor(cj - r))), min(Ny, int(np.ceil(cj + r)) + 1)
        I, J = np.meshgrid(np.arange(i0, i1), np.arange(j0, j1), indexing="ij")
        win = eps[i0:i1, j0:j1]
        win[(I - ci) ** 2 + (J - cj) ** 2 <= r * r] = e
    return eps


def config2(seed=1002, N=400, steps=2000):
    """FDTD TM 400x400, dL=25 nm, npml [20, 20, 0], 30 seeded rods, Gaussian
    pulse Jz point source at the centre (200 THz, sigma 20 fs, t0 24 fs).
    ``N`` scales the grid (rod count scaled by area) for the HBM-bound runs."""
    from .fdtd_util import fdtd_dt
    rng = _rng(seed)
    npml = 20
    n_rods = int(round(30 * (N / 400) ** 2))
    eps = rods_eps(N, N, npml, n_rods, rng)
    dL = 25e-9
    dt = fdtd_dt(dL)
    t = np.arange(steps) * dt
    sigma, t0, f0 = 20e-15, 24e-15, 200e12
    amps = np.exp(-(t - t0) ** 2 / (2 * sigma ** 2)) * np.cos(2 * np.pi * f0 * t)
    src = np.zeros((N, N))
    src[N // 2, N // 2] = 1.0
    return dict(eps=eps, dL=dL, npml=[npml, npml, 0], src=src, amps=amps, steps=steps, dt=dt)


def binary_design(Nx, Ny, block, sigma, rng):
    """eps in {1, 12.25}: Gaussian-filtered U[0,1) noise thresholded at 0.5
    inside a centred block x block region."""
    from scipy.ndimage import gaussian_filter
    eps = np.ones((Nx, Ny))
    noise = gaussian_filter(rng.random((block, block)), sigma=sigma, mode="wrap")
    # the filtered field concentrates near 0.5; threshold at its median so the
    # fill factor stays near one half
    design = np.where(noise > np.median(noise), 12.25, 1.0)
    i0, j0 = (Nx - block) // 2, (Ny - block) // 2
    eps[i0:i0 + block, j0:j0 + block] = design
    return eps


def config3(seed=1003):
    """Adjoint FDFD Ez 600x600, dL=20 nm, npml 25, lambda 1.55 um; 200x200
    design eps = 1 + 11.25 sigmoid(gaussian_filter(N(0,1), 3)); 12-cell input
    and output waveguides (eps 12.25); line source at i = npml+10; Gaussian
    probe (12 cells) at i = Nx-npml-10.  J = |sum(Ez conj(probe))|^2."""
    from scipy.ndimage import gaussian_filter
    rng = _rng(seed)
    N, npml, block = 600, 25, 200
    eps = np.ones((N, N))
    c = N // 2
    eps[:, c - 6:c + 6] = 12.25
    z = gaussian_filter(rng.standard_normal((block, block)), sigma=3)
    z = z / z.std()
    i0 = c - block // 2
    eps[i0:i0 + block, i0:i0 + block] = 1 + 11.25 / (1 + np.exp(-z))
    src = np.zeros((N, N))
    src[npml + 10, c - 6:c + 6] = 1.0
    probe = np.zeros((N, N))
    jj = np.arange(N)
    probe[N - npml - 10, :] = np.exp(-((jj - c) / 6.0) ** 2) * (np.abs(jj - c) < 6)
    return dict(omega=2 * np.pi * C_0 / 1.55e-6, dL=20e-9, eps=eps, npml=[npml, npml],
                src=src, probe=probe)


def config4_problem(i, seed=1004):
    """One 256x256 learned-preconditioner problem: dL = 1.55um/20, npml 16,
    binary eps over a 160x160 block, lambda ~ U[1.3, 1.8] um, a point or line
    source outside the block."""
    rng = _rng(seed * 100000 + i)
    N, npml, block = 256, 16, 160
    dL = 1.55e-6 / 20
    eps = binary_design(N, N, block, 4, rng)
    lam = rng.uniform(1.3e-6, 1.8e-6)
    src = np.zeros((N, N))
    lo = npml + 2
    side = rng.integers(0, 4)
    pos = rng.integers(lo, N - lo)
    depth = rng.integers(lo, (N - block) // 2 - 2)
    ii, jj = [(depth, pos), (N - 1 - depth, pos), (pos, depth), (pos, N - 1 - depth)][side]
    if rng.random() < 0.5:
        src[ii, jj] = 1.0
    else:
        if side < 2:
            src[ii, max(lo, jj - 8):min(N - lo, jj + 8)] = 1.0
        else:
            src[max(lo, ii - 8):min(N - lo, ii + 8), jj] = 1.0
    return dict(omega=2 * np.pi * C_0 / lam, dL=dL, eps=eps, npml=[npml, npml], src=src)


def config5(seed=1005, n_omega=16, N=2048, block=1600, npml=40):
    """Large scale: 2048x2048, dL=15 nm, npml 40, binary eps over a 1600x1600
    block, 16 omegas with lambda ~ U[1.3, 1.8] um, one line source."""
    rng = _rng(seed)
    dL = 15e-9
    eps = binary_design(N, N, block, 4, rng)
    lams = rng.uniform(1.3e-6, 1.8e-6, size=n_omega)
    src = np.zeros((N, N))
    c = N // 2
    src[npml + 20, c - 20:c + 20] = 1.0
    return dict(omegas=2 * np.pi * C_0 / lams, dL=dL, eps=eps, npml=[npml, npml], src=src)
