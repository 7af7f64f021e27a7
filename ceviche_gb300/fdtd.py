"""Drop-in ``fdtd`` (ceviche/fdtd.py:10-316) on the GPU, plus a time-blocked
bulk runner and a checkpointed reverse-time adjoint.

``forward(Jx=None, Jy=None, Jz=None)`` advances one step with the reference's
semantics and returns the fields dict.  Field values are device tensors of
shape (Nx, Ny, 1): E fields are fresh tensors each step; H and D entries
alias the live state (clone them to keep a history).

``run(steps, source, amps, probes)`` advances many TM steps with a sparse
source J(t) = source * amps[t] in time-blocked kernels and records Ez at probe
cells.  ``fdtd_probe_series`` is its differentiable form (d/d eps_r through
``cev_fdtd_adjoint_tm``).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, stream_ptr

_TM = ("hx", "hy", "dz", "icex", "icey", "idz")
_TE = ("hz", "dx", "dy", "ihz", "ichx", "ichy")


def _reshape3(arr):
    """ceviche/utils.py:206-214 reshape_to_ND(N=3)."""
    shape = tuple(arr.shape)
    if len(shape) > 3:
        raise ValueError("array is larger than 3 dimensional, given shape {}".format(shape))
    return arr.reshape(shape + (1,) * (3 - len(shape)))


class fdtd:
    """FDTD object: fdtd(eps_r, dL, npml, precision='float32')."""

    def __init__(self, eps_r, dL, npml, precision="float32"):
        if precision not in ("float32", "float64"):
            raise ValueError("precision must be 'float32' or 'float64'")
        self.precision = precision
        self.dtype = torch.float32 if precision == "float32" else torch.float64
        self._plan_h = None
        eps_r = _reshape3(eps_r)
        self.Nx, self.Ny, self.Nz = self.grid_shape = tuple(eps_r.shape)
        self._dL = dL
        self._npml = list(npml)
        self.eps_r = eps_r

    def __repr__(self):
        return "FDTD(eps_r.shape={}, dL={}, NPML={})".format(self.grid_shape, self.dL, self.npml)

    def __str__(self):
        return "FDTD object:\n\tdomain size = {}\n\tdL = {}\n\tNPML = {}".format(
            self.grid_shape, self.dL, self.npml)

    def __del__(self):
        self._destroy()

    def _destroy(self):
        if getattr(self, "_plan_h", None) is not None and getattr(_lib, "_lib", None) is not None:
            _lib._lib.cev_fdtd_plan_destroy(self._plan_h)
            self._plan_h = None

    # -- setters that rebuild coefficients (fdtd.py:36-72)
    @property
    def dL(self):
        return self._dL

    @dL.setter
    def dL(self, v):
        self._dL = v
        self._rebuild()

    @property
    def npml(self):
        return self._npml

    @npml.setter
    def npml(self, v):
        self._npml = list(v)
        self._rebuild()

    @property
    def eps_r(self):
        return self._eps_r

    @eps_r.setter
    def eps_r(self, new_eps):
        new_eps = _reshape3(new_eps)
        self._eps_r = new_eps
        self.grid_shape = self.Nx, self.Ny, self.Nz = tuple(new_eps.shape)
        self.N = self.Nx * self.Ny * self.Nz
        self._rebuild()

    def _rebuild(self):
        if not hasattr(self, "_eps_r"):
            return
        if self.Nz != 1:
            raise NotImplementedError("only 2D grids (Nz == 1) are supported")
        npml = list(self._npml) + [0] * (3 - len(self._npml))
        if npml[2] != 0:
            raise ValueError("npml[2] must be 0 for a 2D grid (Nz == 1)")
        if not torch.cuda.is_available():
            raise _lib.CevError("ceviche_gb300 needs a CUDA device (sm_103a)")
        lib = _lib.load()
        self._destroy()
        e = self._eps_r
        eps = (e.detach() if torch.is_tensor(e) else torch.as_tensor(np.asarray(e)))
        self._eps_dev = eps.to(device="cuda", dtype=torch.float64).reshape(self.Nx, self.Ny).contiguous()
        h = C.c_void_p()
        prec = _lib.PREC_C64 if self.precision == "float32" else _lib.PREC_C128
        check(lib.cev_fdtd_plan_create(C.byref(h), self.Nx, self.Ny, float(self._dL), npml[0],
                                       npml[1], prec, ptr(self._eps_dev), stream_ptr()),
              "fdtd_plan_create")
        self._plan_h = h
        self.dt = lib.cev_fdtd_dt(h)
        self.initialize_fields()

    def initialize_fields(self):
        """Zero fields and PML integrals (fdtd.py:147-211)."""
        self.t_index = 0
        # one zeroed block (one allocation, one fill) holds the TM state and
        # the zero field every key starts from
        z = torch.zeros((len(_TM) + 1, self.Nx, self.Ny), dtype=self.dtype, device="cuda")
        self._st = {k: z[i] for i, k in enumerate(_TM)}
        self._te = None
        zero3 = z[len(_TM)].view(self.Nx, self.Ny, 1)
        self.fields = {k: zero3 for k in ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz")}

    def _iez(self):
        ez = torch.empty((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
        one = torch.ones((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
        st = _lib.FDTDState()
        st.dz = one.data_ptr()
        check(_lib.load().cev_fdtd_e_fields(self._plan_h, C.byref(st), None, None, ptr(ez),
                                            stream_ptr()), "fdtd_e_fields")
        return ez

    def _state(self):
        s = _lib.FDTDState()
        for k, v in self._st.items():
            setattr(s, k, v.data_ptr())
        if self._te is not None:
            for k, v in self._te.items():
                setattr(s, k, v.data_ptr())
        return s

    def _src(self, J):
        if J is None:
            return None
        t = J if torch.is_tensor(J) else torch.as_tensor(np.asarray(J))
        t = t.to(device="cuda", dtype=self.dtype).reshape(self.Nx, self.Ny).contiguous()
        return t

    def _differentiable(self, *srcs):
        e = self._eps_r
        need = (torch.is_tensor(e) and e.requires_grad) or any(
            torch.is_tensor(j) and j.requires_grad for j in srcs if j is not None)
        return need and torch.is_grad_enabled()

    def forward(self, Jx=None, Jy=None, Jz=None):
        """One time step of FDTD (ceviche/fdtd.py:74-144).

        When eps_r (or Jz) is a tensor that requires grad, the TM step is
        recorded for autograd (state advanced out of place; backward is the
        per-step adjoint kernel), so objectives summed over steps can be
        differentiated as in the reference's gradient tests.
        """
        lib = _lib.load()
        if self._differentiable(Jx, Jy, Jz):
            if Jx is not None or Jy is not None:
                raise NotImplementedError("differentiable steps support the TM (Jz) source only")
            return self._forward_autograd(Jz)
        self.t_index += 1
        jx, jy, jz = self._src(Jx), self._src(Jy), self._src(Jz)
        if (jx is not None or jy is not None) and self._te is None:
            self._te = {k: torch.zeros((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
                        for k in _TE}
        st = self._state()
        check(lib.cev_fdtd_step(self._plan_h, C.byref(st), ptr(jx), ptr(jy), ptr(jz),
                                int(self._te is not None), stream_ptr()), "fdtd_step")
        ez = torch.empty((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
        ex = ey = None
        if self._te is not None:
            ex = torch.empty_like(ez)
            ey = torch.empty_like(ez)
        check(lib.cev_fdtd_e_fields(self._plan_h, C.byref(st), ptr(ex), ptr(ey), ptr(ez),
                                    stream_ptr()), "fdtd_e_fields")
        f = self.fields
        v3 = lambda t: t.view(self.Nx, self.Ny, 1)
        f["Hx"], f["Hy"], f["Dz"], f["Ez"] = v3(self._st["hx"]), v3(self._st["hy"]), \
            v3(self._st["dz"]), v3(ez)
        if self._te is not None:
            f["Hz"], f["Dx"], f["Dy"] = v3(self._te["hz"]), v3(self._te["dx"]), v3(self._te["dy"])
            f["Ex"], f["Ey"] = v3(ex), v3(ey)
        return f

    def _forward_autograd(self, Jz):
        self.t_index += 1
        eps = self._eps_r
        jz = None
        if Jz is not None:
            jz = Jz if torch.is_tensor(Jz) else torch.as_tensor(np.asarray(Jz))
            jz = jz.to(device="cuda", dtype=self.dtype).reshape(self.Nx, self.Ny)
        st = [self._st[k] for k in _TM]
        out = _TMStep.apply(eps, jz, self, *st)
        for k, v in zip(_TM, out[:6]):
            self._st[k] = v
        v3 = lambda t: t.view(self.Nx, self.Ny, 1)
        f = self.fields
        f["Hx"], f["Hy"], f["Dz"], f["Ez"] = v3(out[0]), v3(out[1]), v3(out[2]), v3(out[6])
        return f

    # -- bulk TM runner
    def _io(self, source, amps, probes, steps):
        """Sparse source + probe arrays on the device; returns (FDTDIO, keepalive)."""
        keep = []
        io = _lib.FDTDIO()
        if source is not None:
            prof = source if torch.is_tensor(source) else torch.as_tensor(np.asarray(source))
            prof = prof.detach().to("cpu", torch.float64).reshape(-1)
            idx = torch.nonzero(prof).reshape(-1)
            w = prof[idx]
            a = amps if torch.is_tensor(amps) else torch.as_tensor(np.asarray(amps))
            a = a.detach().to("cuda", self.dtype).reshape(-1).contiguous()
            if a.numel() < steps:
                raise ValueError(f"amps has {a.numel()} entries, need {steps}")
            # cell indices and weights travel in one host-to-device copy: the
            # weights first (8- or 4-byte aligned), then the int32 indices
            ns, wb = int(idx.numel()), torch.finfo(self.dtype).bits // 8
            host = torch.empty(ns * (wb + 4), dtype=torch.uint8)
            host[: ns * wb] = w.to(self.dtype).view(torch.uint8)
            host[ns * wb:] = idx.to(torch.int32).view(torch.uint8)
            dev = host.to("cuda")
            w_d = dev[: ns * wb].view(self.dtype)
            idx_d = dev[ns * wb:].view(torch.int32)
            keep += [dev, a]
            io.n_src = int(idx.numel())
            io.src_idx, io.src_w, io.amps = idx_d.data_ptr(), w_d.data_ptr(), a.data_ptr()
        out = None
        if probes is not None and len(probes) > 0:
            pidx = torch.as_tensor([int(i) * self.Ny + int(j) for i, j in probes],
                                   dtype=torch.int32, device="cuda")
            out = torch.zeros((steps, len(probes)), dtype=self.dtype, device="cuda")
            keep += [pidx, out]
            io.n_probe = len(probes)
            io.probe_idx, io.probe_out = pidx.data_ptr(), out.data_ptr()
        return io, keep, out

    def run(self, steps, source=None, amps=None, probes=None):
        """Advance ``steps`` TM steps with Jz(t) = source * amps[t]; returns the
        (steps, n_probe) series of Ez at ``probes`` [(i, j), ...] (or None)."""
        lib = _lib.load()
        io, keep, out = self._io(source, amps, probes, steps)
        st = self._state()
        check(lib.cev_fdtd_run_tm(self._plan_h, C.byref(st), int(steps), C.byref(io),
                                  stream_ptr()), "fdtd_run_tm")
        self.t_index += steps
        ez = torch.empty((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
        check(lib.cev_fdtd_e_fields(self._plan_h, C.byref(st), None, None, ptr(ez), stream_ptr()),
              "fdtd_e_fields")
        v3 = lambda t: t.view(self.Nx, self.Ny, 1)
        self.fields.update(Hx=v3(self._st["hx"]), Hy=v3(self._st["hy"]), Dz=v3(self._st["dz"]),
                           Ez=v3(ez))
        return out


    def run_te(self, steps, source_x=None, source_y=None, amps=None, probes=None):
        """Advance ``steps`` TE steps with Jx(t) = source_x * amps[t] and
        Jy(t) = source_y * amps[t] (time-blocked, cev_fdtd_run_te); returns
        the (steps, n_probe) series of Hz at ``probes`` (or None).  The TM
        fields do not change (Nz = 1: the polarisations are independent)."""
        lib = _lib.load()
        if self._te is None:
            self._te = {k: torch.zeros((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
                        for k in _TE}
        keep = []
        io = _lib.FDTDIOTE()
        if source_x is not None or source_y is not None:
            def prof(src):
                if src is None:
                    return torch.zeros(self.Nx * self.Ny, dtype=torch.float64)
                t = src if torch.is_tensor(src) else torch.as_tensor(np.asarray(src))
                return t.detach().to("cpu", torch.float64).reshape(-1)
            px, py = prof(source_x), prof(source_y)
            idx = torch.nonzero((px != 0) | (py != 0)).reshape(-1)
            a = amps if torch.is_tensor(amps) else torch.as_tensor(np.asarray(amps))
            a = a.detach().to("cuda", self.dtype).reshape(-1).contiguous()
            if a.numel() < steps:
                raise ValueError(f"amps has {a.numel()} entries, need {steps}")
            idx_d = idx.to("cuda", torch.int32).contiguous()
            wx = px[idx].to("cuda", self.dtype).contiguous()
            wy = py[idx].to("cuda", self.dtype).contiguous()
            keep += [idx_d, wx, wy, a]
            io.n_src = int(idx.numel())
            io.src_idx, io.src_wx, io.src_wy, io.amps = (idx_d.data_ptr(), wx.data_ptr(),
                                                         wy.data_ptr(), a.data_ptr())
        out = None
        if probes is not None and len(probes) > 0:
            pidx = torch.as_tensor([int(i) * self.Ny + int(j) for i, j in probes],
                                   dtype=torch.int32, device="cuda")
            out = torch.zeros((steps, len(probes)), dtype=self.dtype, device="cuda")
            keep += [pidx, out]
            io.n_probe = len(probes)
            io.probe_idx, io.probe_out = pidx.data_ptr(), out.data_ptr()
        st = self._state()
        check(lib.cev_fdtd_run_te(self._plan_h, C.byref(st), int(steps), C.byref(io),
                                  stream_ptr()), "fdtd_run_te")
        self.t_index += steps
        ex = torch.empty((self.Nx, self.Ny), dtype=self.dtype, device="cuda")
        ey = torch.empty_like(ex)
        check(lib.cev_fdtd_e_fields(self._plan_h, C.byref(st), ptr(ex), ptr(ey), None,
                                    stream_ptr()), "fdtd_e_fields")
        v3 = lambda t: t.view(self.Nx, self.Ny, 1)
        self.fields.update(Hz=v3(self._te["hz"]), Dx=v3(self._te["dx"]), Dy=v3(self._te["dy"]),
                           Ex=v3(ex), Ey=v3(ey))
        del keep
        return out


class _TMStep(torch.autograd.Function):
    """One TM step, out of place: (eps, jz, state) -> (new state, Ez)."""

    @staticmethod
    def forward(ctx, eps, jz, F, hx, hy, dz, icex, icey, idz):
        lib = _lib.load()
        new = [t.clone() for t in (hx, hy, dz, icex, icey, idz)]
        st = _lib.FDTDState()
        for k, v in zip(_TM, new):
            setattr(st, k, v.data_ptr())
        jzc = None if jz is None else jz.detach().contiguous()
        check(lib.cev_fdtd_step(F._plan_h, C.byref(st), None, None, ptr(jzc), 0, stream_ptr()),
              "fdtd_step")
        ez = torch.empty_like(new[2])
        check(lib.cev_fdtd_e_fields(F._plan_h, C.byref(st), None, None, ptr(ez), stream_ptr()),
              "fdtd_e_fields")
        ctx.F = F
        ctx.eps_shape = eps.shape if torch.is_tensor(eps) else None
        ctx.has_jz = jz is not None
        ctx.save_for_backward(dz, new[2])
        return (*new, ez)

    @staticmethod
    def backward(ctx, ghx, ghy, gdz, gicex, gicey, gidz, gez):
        F = ctx.F
        lib = _lib.load()
        dz_in, dz_out = ctx.saved_tensors
        z = lambda g: torch.zeros_like(dz_in) if g is None else g.detach().contiguous().clone()
        adj = [z(g) for g in (ghx, ghy, gdz, gicex, gicey, gidz)]
        gjz = None
        if ctx.has_jz and ctx.needs_input_grad[1]:
            gjz = adj[2] + (0 if gez is None else gez * F._iez())
        st = _lib.FDTDState()
        for k, v in zip(_TM, adj):
            setattr(st, k, v.data_ptr())
        scratch = torch.empty(4 * F.Nx * F.Ny, dtype=F.dtype, device="cuda")
        geps = torch.zeros((F.Nx, F.Ny), dtype=torch.float64, device="cuda")
        gezc = None if gez is None else gez.detach().contiguous()
        check(lib.cev_fdtd_step_adjoint_tm(F._plan_h, ptr(dz_in.contiguous()), ptr(dz_out),
                                           ptr(gezc), C.byref(st), ptr(scratch), ptr(geps),
                                           stream_ptr()), "fdtd_step_adjoint_tm")
        ge = None
        if ctx.eps_shape is not None and ctx.needs_input_grad[0]:
            ge = geps.reshape(ctx.eps_shape)
        return (ge, gjz, None, *adj)


class _ProbeSeries(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps, F, steps, source, amps, probes, ckpt_every):
        out = F.run(steps, source, amps, probes)
        ctx.F, ctx.args = F, (steps, source, amps, probes, ckpt_every)
        ctx.eps_shape = eps.shape
        return out.to(eps.dtype) if eps.dtype != out.dtype else out

    @staticmethod
    def backward(ctx, g):
        F = ctx.F
        steps, source, amps, probes, ck = ctx.args
        lib = _lib.load()
        io, keep, _ = F._io(source, amps, probes, steps)
        w = g.detach().to("cuda", F.dtype).contiguous()
        geps = torch.zeros((F.Nx, F.Ny), dtype=torch.float64, device="cuda")
        nbytes = lib.cev_fdtd_adjoint_workspace_size(F._plan_h, int(steps), int(ck))
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        check(lib.cev_fdtd_adjoint_tm(F._plan_h, int(steps), int(ck), C.byref(io), ptr(w),
                                      ptr(geps), ptr(ws), nbytes, stream_ptr()), "fdtd_adjoint_tm")
        return geps.reshape(ctx.eps_shape).to(g.dtype if g.dtype.is_floating_point else
                                              torch.float64), None, None, None, None, None, None


def fdtd_probe_series(eps_r, dL, npml, steps, source, amps, probes, precision="float32",
                      ckpt_every=64):
    """Ez(t) at ``probes`` for a TM run from zero fields, differentiable in eps_r.

    eps_r: torch tensor (Nx, Ny); source: (Nx, Ny) profile; amps: (steps,)."""
    eps_t = eps_r if torch.is_tensor(eps_r) else torch.as_tensor(np.asarray(eps_r))
    F = fdtd(eps_t.detach().cpu().numpy(), dL, npml, precision=precision)
    return _ProbeSeries.apply(eps_t, F, int(steps), source, amps, list(probes), int(ckpt_every))
