"""Device-side FDFD primitives over the C ABI, and their autograd rules.

Replaces ceviche/primitives.py: ``sp_mult`` (the matrix-free operator
``apply``), ``sp_solve`` (``solve``, a GPU Krylov solve instead of the sparse
LU of ceviche/solvers.py:50-62) and their reverse/forward derivatives
(primitives.py:74-148), specialised to the Yee system matrices so no sparse
entries/indices ever exist.

Gradient convention: PyTorch's (g = dL/dRe + i dL/dIm).  For a real loss and
real eps the gradients equal ceviche/HIPS-autograd's.
"""
import ctypes as C
import warnings

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, stream_ptr
from .constants import EPSILON_0, MU_0

_DEFAULT_OPTS = dict(tol=1e-6, inner_rtol=1e-4, max_iters=20000, restart=30, precond="none",
                     reorth=0, max_stall=20, mg_levels=0, mg_shift=0.5, sep_shift=0.0)


_last_info = None  # infos of the latest solve (read by fdfd.solve as last_info)


class SolverWarning(UserWarning):
    """A solve finished without reaching its tolerance."""


def _require_cuda():
    if not torch.cuda.is_available():
        raise _lib.CevError("ceviche_gb300 needs a CUDA device (sm_103a); none is available")


class Plan:
    """Owns a cev_fdfd_plan: PML stencil tables for a batch of omegas on one grid."""

    def __init__(self, pol, shape, dL, omegas, npml, bloch=(0.0, 0.0)):
        _require_cuda()
        lib = _lib.load()
        self.pol = {"ez": _lib.POL_EZ, "hz": _lib.POL_HZ}[pol]
        self.pol_name = pol
        self.nx, self.ny = int(shape[0]), int(shape[1])
        self.omegas = np.atleast_1d(np.asarray(omegas, dtype=np.float64)).copy()
        self.batch = len(self.omegas)
        self.dL = float(dL)
        self.npml = (int(npml[0]), int(npml[1]))
        self.bloch = (float(bloch[0]), float(bloch[1]))
        self.device = torch.device("cuda", torch.cuda.current_device())
        h = C.c_void_p()
        om = self.omegas.ctypes.data_as(C.POINTER(C.c_double))
        check(lib.cev_fdfd_plan_create(C.byref(h), self.pol, self.nx, self.ny, self.batch,
                                       self.dL, om, self.npml[0], self.npml[1],
                                       self.bloch[0], self.bloch[1]), "plan_create")
        self.handle = h
        self.scale = lib.cev_fdfd_plan_scale(h)
        self.omega_t = torch.tensor(self.omegas, dtype=torch.float64, device=self.device)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and getattr(_lib, "_lib", None) is not None:
            _lib._lib.cev_fdfd_plan_destroy(h)
            self.handle = None

    @property
    def shape(self):
        return (self.nx, self.ny)


_plan_cache = {}


def get_plan(pol, shape, dL, omegas, npml, bloch=(0.0, 0.0)):
    om = tuple(float(w) for w in np.atleast_1d(omegas))
    key = (pol, int(shape[0]), int(shape[1]), float(dL), om, int(npml[0]), int(npml[1]),
           float(bloch[0]), float(bloch[1]), torch.cuda.current_device())
    p = _plan_cache.get(key)
    if p is None:
        if len(_plan_cache) > 64:
            _plan_cache.clear()
        p = _plan_cache[key] = Plan(pol, shape, dL, om, npml, bloch)
    return p


_CPLX = {torch.float64: torch.complex128, torch.float32: torch.complex64}


def _eps_arg(plan, eps, dtype, like=None):
    """eps as a contiguous (1 or batch, nx, ny) device tensor; returns (eps, shared).

    A complex eps (lossy media) is passed as interleaved complex of the
    matching precision and switches the plan to complex eps; a tangent or
    gradient array (``like`` = the eps it belongs to) follows that eps."""
    cplx = (like if like is not None else eps).is_complex()
    if like is None:
        check(_lib.load().cev_fdfd_plan_set_eps_complex(plan.handle, int(cplx)), "set_eps_complex")
    e = eps.to(device=plan.device, dtype=_CPLX[dtype] if cplx else dtype)
    e = e.resolve_conj().resolve_neg().contiguous()
    if e.dim() == 2:
        e = e.unsqueeze(0)
    if e.shape[-2:] != (plan.nx, plan.ny):
        raise ValueError(f"eps shape {tuple(e.shape)} does not match grid {plan.shape}")
    if e.shape[0] not in (1, plan.batch):
        raise ValueError(f"eps batch {e.shape[0]} must be 1 or {plan.batch}")
    return e, int(e.shape[0] == 1 and plan.batch >= 1)


def _field_arg(plan, x, dtype):
    t = x.to(device=plan.device, dtype=dtype)
    if t.dim() == 2:
        t = t.unsqueeze(0)
    if t.shape != (plan.batch, plan.nx, plan.ny):
        if t.shape[0] == 1 and plan.batch > 1:
            t = t.expand(plan.batch, plan.nx, plan.ny)
        else:
            raise ValueError(f"field shape {tuple(t.shape)} does not match "
                             f"({plan.batch}, {plan.nx}, {plan.ny})")
    return t.resolve_conj().resolve_neg().contiguous()


def apply(plan, eps, x, transpose=False, precision="c128", si_units=True):
    """y = A x (or A^T x) on the GPU; x complex (batch, nx, ny)."""
    lib = _lib.load()
    if precision == "c128":
        e, sh = _eps_arg(plan, eps, torch.float64)
        xt = _field_arg(plan, x, torch.complex128)
        prec = _lib.PREC_C128
    else:
        e, sh = _eps_arg(plan, eps, torch.float32)
        xt = _field_arg(plan, x, torch.complex64)
        prec = _lib.PREC_C64
    y = torch.empty_like(xt)
    check(lib.cev_fdfd_apply(plan.handle, ptr(e), sh, ptr(xt), ptr(y), int(bool(transpose)), prec,
                             int(bool(si_units)), stream_ptr()), "apply")
    return y


def make_opts(**kw):
    o = dict(_DEFAULT_OPTS)
    for k, v in kw.items():
        if v is None:
            continue
        if k not in o and k not in ("transpose", "use_x0", "learned", "separable", "direct"):
            raise TypeError(f"unknown solver option {k!r}")
        o[k] = v
    s = _lib.SolveOpts()
    _lib.load().cev_solve_opts_default(C.byref(s))
    s.tol = float(o["tol"])
    s.inner_rtol = float(o["inner_rtol"])
    s.max_iters = int(o["max_iters"])
    s.restart = int(o["restart"])
    s.precond = _lib.PRECOND[o["precond"]] if isinstance(o["precond"], str) else int(o["precond"])
    s.transpose = int(bool(o.get("transpose", 0)))
    s.use_x0 = int(bool(o.get("use_x0", 0)))
    s.reorth = int(o["reorth"])
    s.max_stall = int(o["max_stall"])
    s.mg_levels = int(o["mg_levels"])
    s.mg_shift = float(o["mg_shift"])
    lp = o.get("learned")
    s.learned = None if lp is None else C.c_void_p(lp.handle_ptr())
    sp = o.get("separable")
    s.separable = None if sp is None else sp.handle
    dp = o.get("direct")
    s.direct = None if dp is None else dp.handle
    return s


def _workspace(nbytes, device):
    buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
    off = (-buf.data_ptr()) % 256
    return buf, buf.data_ptr() + off


class SolveResult(list):
    """Per-problem solve records (status, iterations, cycles, residual)."""


def solve(plan, eps, b, transpose=False, x0=None, strict=False, fallback=True, **opts):
    """Solve A x = b (A^T x = b) for every problem; b complex (batch, nx, ny) in SI units.

    Returns (x complex128, infos).  Non-convergence warns (or raises with strict).
    ``precond="direct"`` preconditions with complex64 nested-dissection
    factors of the operator (``DirectPrecond``, cached per plan and eps), the
    GPU counterpart of the sparse LU behind ceviche's solve; it converges in a
    few iterations where plain GMRES needs thousands.
    ``precond="shifted_laplacian"`` uses the same factorisation of the
    shifted operator (mass term times 1 - i*mg_shift).
    With a preconditioner (``precond`` "learned" or "separable") and
    ``fallback``, a solve that stops short of ``tol`` (stagnation of the
    flexible GMRES) continues with plain GMRES from its iterate for the rest of
    the ``max_iters`` budget; the infos then count both phases and record the
    preconditioned iterations as ``precond_iterations``.  ``max_stall`` sets
    when the preconditioned phase hands over (a small value gives a hybrid:
    the network for the first cycles, plain GMRES after); the plain phase
    keeps at least the default stall limit.
    """
    global _last_info
    x, res, rc, tol = _solve_once(plan, eps, b, transpose, x0, **opts)
    if rc > 0 and fallback and opts.get("precond", "none") not in ("none", 0):
        left = int(opts.get("max_iters", _DEFAULT_OPTS["max_iters"])) - max(r["iterations"] for r in res)
        if left > 0:
            plain = {k: v for k, v in opts.items()
                     if k not in ("precond", "learned", "separable", "direct")}
            plain["max_iters"] = left
            # the stall limit decides when to leave the preconditioned phase; the
            # plain phase keeps at least the default patience
            plain["max_stall"] = max(int(opts.get("max_stall", _DEFAULT_OPTS["max_stall"])),
                                     _DEFAULT_OPTS["max_stall"])
            x, res2, rc, tol = _solve_once(plan, eps, b, transpose, x, **plain)
            for r, r2 in zip(res, res2):
                r2["precond_iterations"] = r["iterations"]
                r2["iterations"] += r["iterations"]
                r2["cycles"] += r["cycles"]
            res = res2
    if rc > 0:
        msg = (f"FDFD solve did not reach tol={tol:g}: "
               + ", ".join(f"[{k}] {r['status']} res={r['residual']:.3g} it={r['iterations']}"
                           for k, r in enumerate(res) if r["code"] != 0))
        if strict:
            raise _lib.CevError(msg)
        warnings.warn(msg, SolverWarning, stacklevel=2)
    _last_info = res
    return x, res


def _solve_once(plan, eps, b, transpose, x0, **opts):
    """One cev_fdfd_solve call: (x, infos, status, tol)."""
    lib = _lib.load()
    e, sh = _eps_arg(plan, eps, torch.float64)
    bt = _field_arg(plan, b, torch.complex128)
    keep = None
    if opts.get("precond") == "separable" and opts.get("separable") is None:
        keep = SeparablePrecond(plan, e, shift=opts.get("sep_shift", 0.0), transpose=transpose)
        opts = dict(opts, separable=keep)
        e, sh = _eps_arg(plan, eps, torch.float64)  # re-assert the eps kind on the plan
    if opts.get("precond") in ("direct", "shifted_laplacian") and opts.get("direct") is None:
        shift = 0.0 if opts["precond"] == "direct" else float(opts.get("mg_shift", 0.5))
        keep = direct_precond(plan, e, transpose=transpose, shift=shift)
        opts = dict(opts, direct=keep)
    s = make_opts(transpose=transpose, use_x0=x0 is not None, **opts)
    if x0 is not None:
        x = _field_arg(plan, x0, torch.complex128).clone()
    else:
        x = torch.empty_like(bt)
    nbytes = lib.cev_fdfd_solve_workspace_size(plan.handle, C.byref(s))
    if nbytes == 0:
        raise ValueError("invalid solver options")
    ws, wptr = _workspace(nbytes, plan.device)
    infos = (_lib.SolveInfo * plan.batch)()
    rc = lib.cev_fdfd_solve(plan.handle, ptr(e), sh, ptr(bt), ptr(x), C.byref(s), infos,
                            C.c_void_p(wptr), nbytes, stream_ptr())
    check(rc, "solve")
    res = SolveResult(dict(status=_lib.STATUS_NAMES.get(i.status, i.status), code=i.status,
                           iterations=i.iterations, cycles=i.cycles, residual=i.residual)
                      for i in infos)
    del ws
    return x, res, rc, s.tol


def fields(plan, eps, fz):
    """Secondary field components (f1, f2) from the solved component (SI, complex128)."""
    lib = _lib.load()
    e, sh = _eps_arg(plan, eps, torch.float64)
    z = _field_arg(plan, fz, torch.complex128)
    f1 = torch.empty_like(z)
    f2 = torch.empty_like(z)
    check(lib.cev_fdfd_fields(plan.handle, ptr(e), sh, ptr(z), ptr(f1), ptr(f2), stream_ptr()),
          "fields")
    return f1, f2


def fields_adjoint(plan, eps, fz, g1, g2, gz, geps):
    """gz += M1^H g1 + M2^H g2 (in place); geps += direct eps term (Hz)."""
    lib = _lib.load()
    e, sh = _eps_arg(plan, eps, torch.float64)
    z = _field_arg(plan, fz, torch.complex128)
    a = _field_arg(plan, g1, torch.complex128)
    b = _field_arg(plan, g2, torch.complex128)
    check(lib.cev_fdfd_fields_adjoint(plan.handle, ptr(e), sh, ptr(z), ptr(a), ptr(b), ptr(gz),
                                      ptr(geps), stream_ptr()), "fields_adjoint")


def jvp_rhs(plan, eps, deps, x, rhs):
    """rhs += -(dA/d eps . deps) x (in place)."""
    lib = _lib.load()
    e, sh = _eps_arg(plan, eps, torch.float64)
    de, _ = _eps_arg(plan, deps, torch.float64, like=e)
    if de.shape != e.shape:
        de = de.expand_as(e).contiguous()
    xt = _field_arg(plan, x, torch.complex128)
    check(lib.cev_fdfd_jvp_rhs(plan.handle, ptr(e), sh, ptr(de), ptr(xt), ptr(rhs), stream_ptr()),
          "jvp_rhs")


def fields_jvp(plan, eps, deps, fz, df1, df2):
    """(df1, df2) += direct eps tangent of the secondary fields (Hz only)."""
    lib = _lib.load()
    e, sh = _eps_arg(plan, eps, torch.float64)
    de, _ = _eps_arg(plan, deps, torch.float64, like=e)
    if de.shape != e.shape:
        de = de.expand_as(e).contiguous()
    z = _field_arg(plan, fz, torch.complex128)
    check(lib.cev_fdfd_fields_jvp(plan.handle, ptr(e), sh, ptr(de), ptr(z), ptr(df1), ptr(df2),
                                  stream_ptr()), "fields_jvp")


def grad_eps(plan, eps, x, mu, geps):
    """geps += system-matrix part of dL/d(eps) given x and mu = A^-T conj(g_x)."""
    lib = _lib.load()
    e, sh = _eps_arg(plan, eps, torch.float64)
    xt = _field_arg(plan, x, torch.complex128)
    m = _field_arg(plan, mu, torch.complex128)
    check(lib.cev_fdfd_grad_eps(plan.handle, ptr(e), sh, ptr(xt), ptr(m), ptr(geps), stream_ptr()),
          "grad_eps")


def _sep_factors(plan, transpose):
    """Eigendecompositions of the plan's 1D axis operators (cached per plan and
    transpose flag): device complex128 Vx, Vx^-1 [B][nx][nx], Vy, Vy^-1
    [B][ny][ny] and the eigenvalues (complex128 [B][n])."""
    cache = plan.__dict__.setdefault("_sep_cache", {})
    key = bool(transpose)
    if key in cache:
        return cache[key]
    lib = _lib.load()
    out = {}
    for axis, n, name in ((0, plan.nx, "x"), (1, plan.ny, "y")):
        V, Vi, L = [], [], []
        for b in range(plan.batch):
            T = np.zeros((n, n), dtype=np.complex128)
            check(lib.cev_fdfd_axis_matrix(plan.handle, b, axis, int(key),
                                           T.ctypes.data_as(C.c_void_p)), "axis_matrix")
            lam, vec = np.linalg.eig(T)
            V.append(vec)
            Vi.append(np.linalg.inv(vec))
            L.append(lam)
        dev = plan.device
        out["v" + name] = torch.as_tensor(np.stack(V), dtype=torch.complex128, device=dev).contiguous()
        out["vi" + name] = torch.as_tensor(np.stack(Vi), dtype=torch.complex128, device=dev).contiguous()
        out["l" + name] = torch.as_tensor(np.stack(L), dtype=torch.complex128, device=dev)
    cache[key] = out
    return out


class SeparablePrecond:
    """CEV_PRECOND_SEPARABLE for a plan and an eps: the exact inverse of the
    stretched operator with eps replaced by its mean c per problem (times
    1 + i*shift), applied as dense GEMMs on the device.  The 1D
    eigendecompositions are host LAPACK work, O(n^3) per axis and problem,
    cached on the plan; the per-eps part is the table 1/d."""

    def __init__(self, plan, eps, shift=0.0, transpose=False):
        lib = _lib.load()
        f = _sep_factors(plan, transpose)
        e = eps if eps.dim() == 3 else eps.unsqueeze(0)
        c = e.reshape(e.shape[0], -1).mean(dim=1).to(torch.complex128) * (1 + 1j * shift)
        if c.numel() == 1 and plan.batch > 1:
            c = c.expand(plan.batch)
        k2 = (EPSILON_0 * MU_0 * plan.dL ** 2) * plan.omega_t ** 2
        lam = f["lx"][:, :, None] + f["ly"][:, None, :]
        if plan.pol_name == "ez":
            d = -lam - (k2 * c).view(-1, 1, 1)
        else:
            d = lam / (c + 1e-5).view(-1, 1, 1) + k2.view(-1, 1, 1)
        self.dinv = (1.0 / d).to(torch.complex128).contiguous()
        self._keep = (f["vx"], f["vix"], f["vy"], f["viy"])
        h = C.c_void_p()
        check(lib.cev_sep_precond_create(C.byref(h), plan.handle, int(bool(transpose)),
                                         ptr(f["vx"]), ptr(f["vix"]), ptr(f["vy"]),
                                         ptr(f["viy"]), ptr(self.dinv)), "sep_precond_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and getattr(_lib, "_lib", None) is not None:
            _lib._lib.cev_sep_precond_destroy(h)
            self.handle = None


class DirectPrecond:
    """cev_nd_precond for a plan and an eps: complex64 nested-dissection
    factors of the plan's operator (A or A^T), or of the shifted operator with
    ``shift`` > 0.  The factorisation runs on the GPU when the object is made;
    ``factor_bytes`` and ``factor_cmacs`` report its size and work."""

    def __init__(self, plan, eps, transpose=False, shift=0.0):
        lib = _lib.load()
        e, sh = _eps_arg(plan, eps, torch.float64)
        h = C.c_void_p()
        check(lib.cev_nd_precond_create(C.byref(h), plan.handle, ptr(e), sh, int(bool(transpose)),
                                        float(shift), stream_ptr()), "nd_precond_create")
        self.handle = h
        self.plan = plan  # the handle reads the plan's tables; keep it alive
        nb, fl, nd = C.c_size_t(), C.c_double(), C.c_int()
        check(lib.cev_nd_precond_info(h, C.byref(nb), C.byref(fl), C.byref(nd)), "nd_precond_info")
        self.factor_bytes, self.factor_cmacs, self.depths = nb.value, fl.value, nd.value
        self.transpose, self.shift = bool(transpose), float(shift)

    def apply(self, v):
        """z = M^-1 v for complex64 (batch, nx, ny) device tensors."""
        vt = _field_arg(self.plan, v, torch.complex64)
        z = torch.empty_like(vt)
        check(_lib.load().cev_nd_precond_apply(self.handle, ptr(vt), ptr(z), stream_ptr()),
              "nd_precond_apply")
        return z

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and getattr(_lib, "_lib", None) is not None:
            _lib._lib.cev_nd_precond_destroy(h)
            self.handle = None


def direct_precond(plan, eps, transpose=False, shift=0.0):
    """The DirectPrecond of (plan, eps, transpose, shift), reused while eps is
    unchanged (one factorisation kept per plan, transpose flag and shift)."""
    cache = plan.__dict__.setdefault("_nd_cache", {})
    key = (bool(transpose), float(shift))
    hit = cache.get(key)
    e = eps.detach()
    if hit is not None and hit[0].shape == e.shape and hit[0].dtype == e.dtype \
            and torch.equal(hit[0], e):
        return hit[1]
    cache.pop(key, None)  # free the old factors before making new ones
    dp = DirectPrecond(plan, e, transpose=transpose, shift=shift)
    cache[key] = (e.clone(), dp)
    return dp


class FDFDSolve(torch.autograd.Function):
    """(eps, src) -> (F1, F2, Fz) of ceviche's fdfd.solve with b = 1j*omega*src.

    Backward: the transposed GPU solve of primitives.py:121-135 plus the eps
    chain of fdfd.py:179 (Ez) / 211-233 (Hz) and of the field conversions.
    """

    @staticmethod
    def forward(ctx, eps, src, plan, opts):
        om = plan.omega_t.view(-1, 1, 1)
        s = _field_arg(plan, src, torch.complex128)
        b = 1j * om * s
        x, info = solve(plan, eps, b, **opts)
        f1, f2 = fields(plan, eps, x)
        ctx.plan, ctx.opts = plan, opts
        ctx.src_real = not src.is_complex()
        ctx.src_shape = src.shape
        ctx.eps_shape = eps.shape
        ctx.save_for_backward(eps, x)
        ctx.save_for_forward(eps, x)
        ctx.info = info
        return f1, f2, x

    @staticmethod
    def backward(ctx, g1, g2, gz):
        plan = ctx.plan
        eps, x = ctx.saved_tensors
        e, sh = _eps_arg(plan, eps, torch.float64)
        zeros = lambda: torch.zeros_like(x)
        g1 = zeros() if g1 is None else g1.to(torch.complex128).contiguous()
        g2 = zeros() if g2 is None else g2.to(torch.complex128).contiguous()
        gx = zeros() if gz is None else gz.to(torch.complex128).contiguous().clone()
        geps = torch.zeros_like(e)
        fields_adjoint(plan, e, x, g1, g2, gx, geps if plan.pol_name == "hz" else None)
        geps_out = grad_src = None
        mu, _ = solve(plan, e, gx.conj().resolve_conj(), transpose=True, **ctx.opts)
        if ctx.needs_input_grad[0]:
            grad_eps(plan, e, x, mu, geps)
            geps_out = geps.reshape(ctx.eps_shape) if geps.numel() == int(np.prod(ctx.eps_shape)) \
                else geps
        if ctx.needs_input_grad[1]:
            lam = mu.conj()
            gs = -1j * plan.omega_t.view(-1, 1, 1) * lam
            if len(ctx.src_shape) == 2:
                gs = gs.sum(0)
            grad_src = gs.real if ctx.src_real else gs
            grad_src = grad_src.reshape(ctx.src_shape)
        return geps_out, grad_src, None, None

    @staticmethod
    def jvp(ctx, deps, dsrc, _plan, _opts):
        """Tangent solve A dx = 1j w dsrc - dA x (primitives.py:139-146)."""
        plan = ctx.plan
        eps, x = ctx.saved_tensors
        rhs = torch.zeros_like(x)
        if dsrc is not None:
            rhs += 1j * plan.omega_t.view(-1, 1, 1) * _field_arg(plan, dsrc, torch.complex128)
        if deps is not None:
            jvp_rhs(plan, eps, deps, x, rhs)
        dx, _ = solve(plan, eps, rhs, **ctx.opts)
        df1, df2 = fields(plan, eps, dx)
        if deps is not None:
            fields_jvp(plan, eps, deps, x, df1, df2)
        return df1, df2, dx


# ---------------------------------------------------- multi-frequency (mf) Ez
class MFPlan:
    """Owns a multi-frequency Ez plan: M = 2*Nsb+1 sidebands W_m sharing the
    centre-frequency PML tables (ceviche/fdfd.py:247-359)."""

    pol_name = "ez"

    def __init__(self, shape, dL, omega, omega_mod, nsb, npml, bloch=(0.0, 0.0)):
        _require_cuda()
        lib = _lib.load()
        self.nx, self.ny = int(shape[0]), int(shape[1])
        self.nsb = int(nsb)
        self.batch = 2 * self.nsb + 1
        self.device = torch.device("cuda", torch.cuda.current_device())
        h = C.c_void_p()
        check(lib.cev_fdfd_mf_plan_create(C.byref(h), self.nx, self.ny, float(dL), float(omega),
                                          float(omega_mod), self.nsb, int(npml[0]), int(npml[1]),
                                          float(bloch[0]), float(bloch[1])), "mf_plan_create")
        self.handle = h
        self.scale = lib.cev_fdfd_plan_scale(h)
        W = omega + np.arange(-self.nsb, self.nsb + 1) * omega_mod
        self.omega_t = torch.tensor(W, dtype=torch.float64, device=self.device)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and getattr(_lib, "_lib", None) is not None:
            _lib._lib.cev_fdfd_plan_destroy(h)
            self.handle = None

    @property
    def shape(self):
        return (self.nx, self.ny)


_mf_cache = {}


def get_mf_plan(shape, dL, omega, omega_mod, nsb, npml, bloch=(0.0, 0.0)):
    key = (int(shape[0]), int(shape[1]), float(dL), float(omega), float(omega_mod), int(nsb),
           int(npml[0]), int(npml[1]), float(bloch[0]), float(bloch[1]),
           torch.cuda.current_device())
    p = _mf_cache.get(key)
    if p is None:
        if len(_mf_cache) > 16:
            _mf_cache.clear()
        p = _mf_cache[key] = MFPlan(shape, dL, omega, omega_mod, nsb, npml, bloch)
    return p


def _cpl_arg(plan, cpl):
    if cpl is None or cpl.numel() == 0:
        return torch.zeros((0, plan.nx, plan.ny), dtype=torch.complex128, device=plan.device), 0
    c = cpl.to(device=plan.device, dtype=torch.complex128).reshape(-1, plan.nx, plan.ny)
    c = c[: 2 * plan.nsb].contiguous()  # harmonics k >= 2*Nsb couple no sideband pair
    return c, int(c.shape[0])


def mf_apply(plan, eps, cpl, x, transpose=False):
    lib = _lib.load()
    e = eps.to(device=plan.device, dtype=torch.float64).reshape(plan.nx, plan.ny).contiguous()
    c, nf = _cpl_arg(plan, cpl)
    xt = _field_arg(plan, x, torch.complex128)
    y = torch.empty_like(xt)
    check(lib.cev_fdfd_mf_apply(plan.handle, ptr(e), nf, ptr(c), ptr(xt), ptr(y),
                                int(bool(transpose)), stream_ptr()), "mf_apply")
    return y


def mf_solve(plan, eps, cpl, b, transpose=False, strict=False, **opts):
    lib = _lib.load()
    e = eps.to(device=plan.device, dtype=torch.float64).reshape(plan.nx, plan.ny).contiguous()
    c, nf = _cpl_arg(plan, cpl)
    bt = _field_arg(plan, b, torch.complex128)
    s = make_opts(transpose=transpose, **opts)
    x = torch.empty_like(bt)
    nbytes = lib.cev_fdfd_mf_solve_workspace_size(plan.handle, nf, C.byref(s))
    if nbytes == 0:
        raise ValueError("invalid solver options")
    ws, wptr = _workspace(nbytes, plan.device)
    info = (_lib.SolveInfo * 1)()
    rc = lib.cev_fdfd_mf_solve(plan.handle, ptr(e), nf, ptr(c), ptr(bt), ptr(x), C.byref(s), info,
                               C.c_void_p(wptr), nbytes, stream_ptr())
    check(rc, "mf_solve")
    del ws
    r = dict(status=_lib.STATUS_NAMES.get(info[0].status, info[0].status), code=info[0].status,
             iterations=info[0].iterations, cycles=info[0].cycles, residual=info[0].residual)
    if rc > 0:
        msg = f"multi-frequency FDFD solve did not reach tol={s.tol:g}: {r}"
        if strict:
            raise _lib.CevError(msg)
        warnings.warn(msg, SolverWarning, stacklevel=2)
    return x, r


class FDFDMFSolve(torch.autograd.Function):
    """(eps, c, src) -> (Hx, Hy, Ez) of fdfd_mf_ez.solve with b_m = 1j W_m src_m
    (ceviche/fdfd.py:328-337); c_k = delta_k exp(1j phi_k).  Backward: the
    transposed coupled solve plus cev_fdfd_mf_grad."""

    @staticmethod
    def forward(ctx, eps, cpl, src, plan, opts):
        W = plan.omega_t.view(-1, 1, 1)
        b = 1j * W * _field_arg(plan, src, torch.complex128)
        x, info = mf_solve(plan, eps, cpl, b, **opts)
        f1, f2 = fields(plan, eps.reshape(plan.nx, plan.ny), x)
        ctx.plan, ctx.opts = plan, opts
        ctx.src_real = not src.is_complex()
        ctx.save_for_backward(eps, cpl, x)
        ctx.info = info
        return f1, f2, x

    @staticmethod
    def backward(ctx, g1, g2, gz):
        plan = ctx.plan
        eps, cpl, x = ctx.saved_tensors
        lib = _lib.load()
        e = eps.reshape(plan.nx, plan.ny)
        zeros = lambda: torch.zeros_like(x)
        g1 = zeros() if g1 is None else g1.to(torch.complex128).contiguous()
        g2 = zeros() if g2 is None else g2.to(torch.complex128).contiguous()
        gx = zeros() if gz is None else gz.to(torch.complex128).contiguous().clone()
        fields_adjoint(plan, e, x, g1, g2, gx, None)
        mu, _ = mf_solve(plan, eps, cpl, gx.conj().resolve_conj(), transpose=True, **ctx.opts)
        c, nf = _cpl_arg(plan, cpl)
        geps = torch.zeros((plan.nx, plan.ny), dtype=torch.float64, device=plan.device)
        gcpl = torch.zeros_like(c)
        check(lib.cev_fdfd_mf_grad(plan.handle, nf, ptr(x), ptr(mu), ptr(geps), ptr(gcpl),
                                   stream_ptr()), "mf_grad")
        g_eps = geps.reshape(eps.shape) if ctx.needs_input_grad[0] else None
        g_cpl = None
        if ctx.needs_input_grad[1]:
            g_cpl = torch.zeros_like(cpl, dtype=torch.complex128).reshape(-1, plan.nx, plan.ny)
            g_cpl[:nf] = gcpl
            g_cpl = g_cpl.reshape(cpl.shape)
        g_src = None
        if ctx.needs_input_grad[2]:
            gs = -1j * plan.omega_t.view(-1, 1, 1) * mu.conj()
            g_src = gs.real if ctx.src_real else gs
        return g_eps, g_cpl, g_src, None, None
