"""FP64 CPU restatement of ceviche's 2D FDTD -- TEST INFRASTRUCTURE ONLY.

Restates (own code, same arithmetic and operation order):
    * time step          ceviche/fdtd.py:213-222   (3D Courant limit x 0.5)
    * PML sigmas         ceviche/fdtd.py:224-263   (2X-grid loop, same write order)
    * update coefficients ceviche/fdtd.py:265-316
    * eps averaging      ceviche/utils.py:153-176  (xx along axis 0, yy along axis 1)
    * one step           ceviche/fdtd.py:74-144 with the curls of
                         ceviche/derivatives.py:16-30 (periodic roll)

The reference stores (Nx, Ny, 1) arrays; with Nz == 1 every roll along z is
the identity, so the z-differences are exactly zero and the arrays here are
(Nx, Ny).  npml_z must be 0 (the reference raises IndexError otherwise).

TE fields (Hz, Ex, Ey, Dx, Dy) are computed only once a Jx/Jy source has been
seen: before that every one of their updates multiplies exact zeros, so
skipping them does not change any value.

``adjoint_tm`` restates the reverse-mode derivative that autograd would tape
through ``forward`` (used by test_gradients_fdtd.py:66-165) for the TM fields.
"""
import numpy as np

from .constants import EPSILON_0, C_0


def time_step(dL, stability_factor=0.5):
    """ceviche/fdtd.py:213-222."""
    dL_sum = 3 / dL ** 2
    dL_avg = 1 / np.sqrt(dL_sum)
    return dL_avg / C_0 * stability_factor


def sigma_profiles(Nx, Ny, npml, dt):
    """1D sigma samples on the Yee grid (ceviche/fdtd.py:224-263).

    Returns dict with sxH (sigHx along i), sxD (sigDx along i), syH, syD.
    sigHx = sigx2[1::2], sigDx = sigx2[::2] along x; sigHy = sigy2[1::2],
    sigDy = sigy2[::2] along y.
    """
    def prof(N, n):
        s2 = np.zeros(2 * N)
        for k in range(2 * n):
            k1 = 2 * n - k + 1
            k2 = 2 * N - 2 * n + k
            s2[k1] = (0.5 * EPSILON_0 / dt) * (k / 2 / n) ** 3
            s2[k2] = (0.5 * EPSILON_0 / dt) * (k / 2 / n) ** 3
        return s2

    sx2 = prof(Nx, npml[0])
    sy2 = prof(Ny, npml[1])
    return dict(sxH=sx2[1::2], sxD=sx2[::2], syH=sy2[1::2], syD=sy2[::2])


def coefficients(eps, dt, sig):
    """Update coefficients of ceviche/fdtd.py:265-316 on (Nx, Ny) grids (mu_r = 1,
    sigma_z = 0)."""
    Nx, Ny = eps.shape
    e0 = EPSILON_0
    Z = np.zeros((Nx, Ny))
    sHx = sig["sxH"][:, None] + Z
    sHy = sig["syH"][None, :] + Z
    sDx = sig["sxD"][:, None] + Z
    sDy = sig["syD"][None, :] + Z
    sHz = Z
    sDz = Z
    c = {}

    def block(pref, sa, sb, sself, m2sign, m3sign):
        # pref x: (sa, sb) = (sigy, sigz); sself = sigx
        m0 = 1 / dt + (sa + sb) / 2 / e0 + sa * sb * dt / 4 / e0 ** 2
        m1 = 1 / m0 * (1 / dt - (sa + sb) / 2 / e0 - sa * sb * dt / 4 / e0 ** 2)
        return m0, m1

    for comp, (sa, sb, ss) in dict(Hx=(sHy, sHz, sHx), Hy=(sHx, sHz, sHy), Hz=(sHx, sHy, sHz)).items():
        m0, m1 = block(comp, sa, sb, ss, -1, -1)
        c["m" + comp + "1"] = m1
        c["m" + comp + "2"] = -1 / m0 * C_0 / 1.0
        c["m" + comp + "3"] = -1 / m0 * C_0 * dt * ss / e0 / 1.0
        c["m" + comp + "4"] = -1 / m0 * dt * sa * sb / e0 ** 2
    for comp, (sa, sb, ss) in dict(Dx=(sDy, sDz, sDx), Dy=(sDx, sDz, sDy), Dz=(sDx, sDy, sDz)).items():
        m0, m1 = block(comp, sa, sb, ss, 1, 1)
        c["m" + comp + "1"] = m1
        c["m" + comp + "2"] = 1 / m0 * C_0
        c["m" + comp + "3"] = 1 / m0 * C_0 * dt * ss / e0
        c["m" + comp + "4"] = -1 / m0 * dt * sa * sb / e0 ** 2
    exx = (eps + np.roll(eps, 1, axis=0)) / 2
    eyy = (eps + np.roll(eps, 1, axis=1)) / 2
    ezz = (eps + eps) / 2
    c["mEx1"], c["mEy1"], c["mEz1"] = 1 / exx, 1 / eyy, 1 / ezz
    return c


class FDTD2D:
    """Stateful FP64 2D FDTD with the reference's step semantics."""

    FIELDS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz")

    def __init__(self, eps, dL, npml):
        eps = np.asarray(eps, dtype=np.float64)
        if eps.ndim == 3:
            assert eps.shape[2] == 1
            eps = eps[:, :, 0]
        npml = list(npml) + [0] * (3 - len(npml))
        assert npml[2] == 0, "2D grids need npml_z == 0"
        self.eps, self.dL, self.npml = eps, dL, npml
        self.Nx, self.Ny = eps.shape
        self.dt = time_step(dL)
        self.sig = sigma_profiles(self.Nx, self.Ny, npml, self.dt)
        self.c = coefficients(eps, self.dt, self.sig)
        self.reset()

    def reset(self):
        z = lambda: np.zeros((self.Nx, self.Ny))
        self.t_index = 0
        self.f = {k: z() for k in self.FIELDS}
        self.aux = {k: z() for k in ("ICEx", "ICEy", "ICEz", "IHx", "IHy", "IHz",
                                     "ICHx", "ICHy", "ICHz", "IDx", "IDy", "IDz")}
        self.te_active = False

    def forward(self, Jx=None, Jy=None, Jz=None):
        """One step, ceviche/fdtd.py:74-144."""
        f, a, c, dL = self.f, self.aux, self.c, self.dL
        self.t_index += 1
        if Jx is not None or Jy is not None:
            self.te_active = True
        Ex, Ey, Ez = f["Ex"], f["Ey"], f["Ez"]
        roll = np.roll
        # curl E (derivatives.py:16-22); z-rolls are the identity for Nz == 1
        CEx = (roll(Ez, -1, axis=1) - Ez) / dL - (Ey - Ey) / dL
        CEy = (Ex - Ex) / dL - (roll(Ez, -1, axis=0) - Ez) / dL
        a["ICEx"] = a["ICEx"] + CEx
        a["ICEy"] = a["ICEy"] + CEy
        a["IHx"] = a["IHx"] + f["Hx"]
        a["IHy"] = a["IHy"] + f["Hy"]
        Hx = c["mHx1"] * f["Hx"] + c["mHx2"] * CEx + c["mHx3"] * a["ICEx"] + c["mHx4"] * a["IHx"]
        Hy = c["mHy1"] * f["Hy"] + c["mHy2"] * CEy + c["mHy3"] * a["ICEy"] + c["mHy4"] * a["IHy"]
        if self.te_active:
            CEz = (roll(Ey, -1, axis=0) - Ey) / dL - (roll(Ex, -1, axis=1) - Ex) / dL
            a["ICEz"] = a["ICEz"] + CEz
            a["IHz"] = a["IHz"] + f["Hz"]
            f["Hz"] = c["mHz1"] * f["Hz"] + c["mHz2"] * CEz + c["mHz3"] * a["ICEz"] + c["mHz4"] * a["IHz"]
        f["Hx"], f["Hy"] = Hx, Hy
        Hz = f["Hz"]
        # curl H (derivatives.py:24-30)
        CHz = (Hy - roll(Hy, 1, axis=0)) / dL - (Hx - roll(Hx, 1, axis=1)) / dL
        a["ICHz"] = a["ICHz"] + CHz
        a["IDz"] = a["IDz"] + f["Dz"]
        Dz = c["mDz1"] * f["Dz"] + c["mDz2"] * CHz + c["mDz3"] * a["ICHz"] + c["mDz4"] * a["IDz"]
        if Jz is not None:
            Dz = Dz + np.reshape(Jz, Dz.shape)
        f["Dz"] = Dz
        if self.te_active:
            CHx = (Hz - roll(Hz, 1, axis=1)) / dL - (Hy - Hy) / dL
            CHy = (Hx - Hx) / dL - (Hz - roll(Hz, 1, axis=0)) / dL
            a["ICHx"] = a["ICHx"] + CHx
            a["ICHy"] = a["ICHy"] + CHy
            a["IDx"] = a["IDx"] + f["Dx"]
            a["IDy"] = a["IDy"] + f["Dy"]
            Dx = c["mDx1"] * f["Dx"] + c["mDx2"] * CHx + c["mDx3"] * a["ICHx"] + c["mDx4"] * a["IDx"]
            Dy = c["mDy1"] * f["Dy"] + c["mDy2"] * CHy + c["mDy3"] * a["ICHy"] + c["mDy4"] * a["IDy"]
            if Jx is not None:
                Dx = Dx + np.reshape(Jx, Dx.shape)
            if Jy is not None:
                Dy = Dy + np.reshape(Jy, Dy.shape)
            f["Dx"], f["Dy"] = Dx, Dy
            f["Ex"] = c["mEx1"] * Dx
            f["Ey"] = c["mEy1"] * Dy
        f["Ez"] = c["mEz1"] * Dz
        return f


def run_tm(eps, dL, npml, src_profile, amps, record_every=None):
    """Run len(amps) TM steps with Jz(t) = src_profile * amps[t]; returns the
    final fields dict and, if ``record_every``, the list of Ez snapshots taken
    after steps record_every, 2*record_every, ..."""
    F = FDTD2D(eps, dL, npml)
    snaps = []
    for t, a in enumerate(amps):
        f = F.forward(Jz=src_profile * a)
        if record_every and (t + 1) % record_every == 0:
            snaps.append(f["Ez"].copy())
    return F, snaps


def measure_fields(F, source, steps, probes, component="Ez"):
    """ceviche/utils.py:316-332 on an FDTD2D: reset, then per step
    F.forward(Jz=source(t)) and sum(field * probe) for each probe."""
    F.reset()
    if not isinstance(probes, list):
        probes = [probes]
    measured = np.zeros((steps, len(probes)))
    for t in range(steps):
        f = F.forward(Jz=source(t))
        for k, p in enumerate(probes):
            measured[t, k] = np.sum(f[component] * np.reshape(p, f[component].shape))
    return measured


def adjoint_tm(eps, dL, npml, src_profile, amps, probe, weights):
    """dL/d(eps) for L = sum_t weights[t] * sum(probe * Ez_t), with the TM
    recurrence of ``FDTD2D.forward`` (Jz = src_profile * amps[t], eps-independent).

    Restated reverse-mode sweep (all states kept in memory; small grids only).
    With sigma_z = 0, mHx4 = mHy4 = mDz3 = 0 exactly, so IHx, IHy and ICHz do
    not influence any output and carry no adjoint.
    """
    F = FDTD2D(eps, dL, npml)
    c = F.c
    Dz_hist = [F.f["Dz"].copy()]
    for a in amps:
        F.forward(Jz=src_profile * a)
        Dz_hist.append(F.f["Dz"].copy())
    T = len(amps)
    z = np.zeros_like(F.eps)
    aHx, aHy, aDz, aICEx, aICEy, aIDz = z.copy(), z.copy(), z.copy(), z.copy(), z.copy(), z.copy()
    aEz_next = z.copy()    # adjoint of Ez^n contributed by step n+1's curls
    grad = z.copy()
    inv_eps = c["mEz1"]
    roll = np.roll
    for n in range(T, 0, -1):
        # total adjoint of Ez^n and Dz^n
        aEz = weights[n - 1] * probe + aEz_next
        aDz = aDz + aEz * inv_eps
        grad += aEz * (-Dz_hist[n] * inv_eps ** 2)
        # reverse of step n
        aDz_prev = c["mDz1"] * aDz
        aCHz = c["mDz2"] * aDz
        aIDz = aIDz + c["mDz4"] * aDz
        aDz_prev = aDz_prev + aIDz
        aHy_t = aHy + (aCHz - roll(aCHz, -1, axis=0)) / dL
        aHx_t = aHx - (aCHz - roll(aCHz, -1, axis=1)) / dL
        aHx = c["mHx1"] * aHx_t
        aCEx = c["mHx2"] * aHx_t
        aICEx = aICEx + c["mHx3"] * aHx_t
        aCEx = aCEx + aICEx
        aHy = c["mHy1"] * aHy_t
        aCEy = c["mHy2"] * aHy_t
        aICEy = aICEy + c["mHy3"] * aHy_t
        aCEy = aCEy + aICEy
        # CEx = (Ez[i,j+1]-Ez)/dL ; CEy = -(Ez[i+1,j]-Ez)/dL  (of Ez^{n-1})
        aEz_next = (roll(aCEx, 1, axis=1) - aCEx) / dL - (roll(aCEy, 1, axis=0) - aCEy) / dL
        aDz = aDz_prev
    # Ez^0 = 0 and does not depend on eps (Dz^0 = 0)
    return grad
