"""Drop-in ``fdfd_ez`` / ``fdfd_hz`` (ceviche/fdfd.py:11-244) on the GPU.

Same constructor, ``eps_r`` setter and ``solve(source) -> (F1, F2, Fz)``
contract.  numpy inputs give numpy complex128 outputs; torch inputs give
device tensors that are differentiable with respect to ``eps_r`` and the
source (reverse mode through the transposed GPU solve).

Extensions: ``omega`` may be a 1D array (a batch of frequencies solved
together) and ``eps_r``/``source`` may carry a leading batch dimension;
solver options (``tol``, ``restart``, ``precond``, ...) are keyword arguments.
"""
import numpy as np
import torch

from . import primitives as prim


def _to_tensor(a, dtype):
    if torch.is_tensor(a):
        t = a
        if not t.is_cuda:
            t = t.cuda()
        return t.to(dtype) if t.dtype != dtype else t
    return torch.as_tensor(np.asarray(a), dtype=dtype, device="cuda")


def _eps_tensor(eps):
    """eps_r on the device: float64, or complex128 for a complex (lossy) eps."""
    cplx = eps.is_complex() if torch.is_tensor(eps) else np.iscomplexobj(eps)
    return _to_tensor(eps, torch.complex128 if cplx else torch.float64)


class fdfd:
    """Base class (ceviche/fdfd.py:11-162)."""

    pol = None

    def __init__(self, omega, dL, eps_r, npml, bloch_phases=None, **solver_opts):
        self.omega = omega
        self.dL = dL
        self.npml = npml
        self._setup_bloch_phases(bloch_phases)
        self.eps_r = eps_r
        self.solver_opts = dict(solver_opts)
        self.last_info = None

    # -- eps_r property (fdfd.py:35-44)
    @property
    def eps_r(self):
        return self._eps_r

    @eps_r.setter
    def eps_r(self, new_eps):
        self._save_shape(new_eps)
        self._eps_r = new_eps

    def _save_shape(self, grid):
        shape = tuple(grid.shape)
        if len(shape) not in (2, 3):
            raise ValueError(f"eps_r must be (Nx, Ny) or (batch, Nx, Ny), got {shape}")
        self.shape = shape[-2:]
        self.Nx, self.Ny = self.shape
        self.N = self.Nx * self.Ny

    def _setup_bloch_phases(self, bloch_phases):
        """ceviche/fdfd.py:101-112."""
        self.bloch_x = 0.0
        self.bloch_y = 0.0
        self.bloch_z = 0.0
        if bloch_phases is not None:
            self.bloch_x = bloch_phases[0]
            if len(bloch_phases) > 1:
                self.bloch_y = bloch_phases[1]
            if len(bloch_phases) > 2:
                self.bloch_z = bloch_phases[2]

    def _vec_to_grid(self, vec):
        return vec.reshape(self.shape)

    def _grid_to_vec(self, grid):
        return grid.flatten()

    # -- plan / operator access
    def _plan(self):
        return prim.get_plan(self.pol, self.shape, self.dL, self.omega, self.npml,
                             (self.bloch_x, self.bloch_y))

    def A(self, x, transpose=False):
        """Matrix-free system matrix product A x (SI units), x of grid shape."""
        eps = _eps_tensor(self.eps_r)
        xt = _to_tensor(x, torch.complex128)
        y = prim.apply(self._plan(), eps, xt, transpose=transpose)
        return y.reshape(xt.shape)

    def solve(self, source_z):
        """Solve for the fields of this polarisation (ceviche/fdfd.py:58-76)."""
        numpy_out = not torch.is_tensor(self.eps_r) and not torch.is_tensor(source_z)
        eps = _eps_tensor(self.eps_r)
        src = source_z if torch.is_tensor(source_z) else np.asarray(source_z)
        src_dtype = torch.complex128 if (torch.is_tensor(src) and src.is_complex()) or \
            (not torch.is_tensor(src) and np.iscomplexobj(src)) else torch.float64
        src = _to_tensor(src, src_dtype)
        plan = self._plan()
        f1, f2, fz = prim.FDFDSolve.apply(eps, src, plan, self.solver_opts)
        self.last_info = getattr(prim, "_last_info", None)
        squeeze = np.ndim(self.omega) == 0 and eps.dim() == 2 and src.dim() == 2
        out = []
        for f in (f1, f2, fz):
            f = f[0] if squeeze else f
            out.append(f.detach().cpu().numpy() if numpy_out else f)
        return tuple(out)


class fdfd_ez(fdfd):
    """Ez polarisation: A = -(1/mu0)(Dxf Dxb + Dyf Dyb) - eps0 w^2 eps
    (ceviche/fdfd.py:166-192).  solve(Jz) -> (Hx, Hy, Ez).

    Solves default to ``precond="direct"`` (complex64 nested-dissection
    factors preconditioning flexible GMRES to the FP64 tolerance), the GPU
    counterpart of the direct solve ceviche performs; ``precond="none"``
    selects plain restarted GMRES."""

    pol = "ez"

    def __init__(self, omega, dL, eps_r, npml, bloch_phases=None, **solver_opts):
        solver_opts.setdefault("precond", "direct")
        super().__init__(omega, dL, eps_r, npml, bloch_phases=bloch_phases, **solver_opts)


class fdfd_hz(fdfd):
    """Hz polarisation: A = (1/eps0)(Dxb/eps_yy Dxf + Dyb/eps_xx Dyf) + mu0 w^2
    (ceviche/fdfd.py:194-244).  solve(Mz) -> (Ex, Ey, Hz).  Solves default to
    ``precond="direct"`` as for fdfd_ez."""

    pol = "hz"

    def __init__(self, omega, dL, eps_r, npml, bloch_phases=None, **solver_opts):
        solver_opts.setdefault("precond", "direct")
        super().__init__(omega, dL, eps_r, npml, bloch_phases=bloch_phases, **solver_opts)


class fdfd_mf_ez(fdfd):
    """Multi-frequency (time-modulated) Ez FDFD, ceviche/fdfd.py:247-359.

    fdfd_mf_ez(omega, dL, eps_r, omega_mod, delta, phi, Nsb, npml,
    bloch_phases=None); delta, phi: (Nfreq, Nx, Ny) modulation depth and
    phase of each harmonic.  solve(source) with source (2*Nsb+1, Nx, Ny)
    returns (Hx, Hy, Ez), each (2*Nsb+1, Nx, Ny); differentiable in eps_r,
    delta, phi and the source when those are torch tensors.
    """

    pol = "ez"

    def __init__(self, omega, dL, eps_r, omega_mod, delta, phi, Nsb, npml, bloch_phases=None,
                 **solver_opts):
        super().__init__(omega, dL, eps_r, npml, bloch_phases=bloch_phases, **solver_opts)
        self.omega_mod = omega_mod
        self.delta = delta
        self.phi = phi
        self.Nsb = Nsb

    def _vec_to_grid(self, vec):
        return vec.reshape((2 * self.Nsb + 1,) + tuple(self.shape))

    def solve(self, source_z):
        tens = [torch.is_tensor(a) for a in (self.eps_r, self.delta, self.phi, source_z)]
        numpy_out = not any(tens)
        if (self.eps_r.is_complex() if torch.is_tensor(self.eps_r)
                else np.iscomplexobj(self.eps_r)):
            raise NotImplementedError("fdfd_mf_ez takes a real eps_r")
        eps = _to_tensor(self.eps_r, torch.float64)
        delta = _to_tensor(self.delta, torch.float64)
        phi = _to_tensor(self.phi, torch.float64)
        cpl = delta * torch.exp(1j * phi)
        src = source_z if torch.is_tensor(source_z) else np.asarray(source_z)
        cplx = (torch.is_tensor(src) and src.is_complex()) or \
            (not torch.is_tensor(src) and np.iscomplexobj(src))
        src = _to_tensor(src, torch.complex128 if cplx else torch.float64)
        plan = prim.get_mf_plan(self.shape, self.dL, self.omega, self.omega_mod, self.Nsb,
                                self.npml, (self.bloch_x, self.bloch_y))
        out = prim.FDFDMFSolve.apply(eps, cpl, src, plan, self.solver_opts)
        if numpy_out:
            return tuple(f.detach().cpu().numpy() for f in out)
        return out
