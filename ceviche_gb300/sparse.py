"""Generic sparse primitives ``sp_mult`` / ``sp_solve`` on the GPU
(ceviche/primitives.py:58-148): the entries/indices interface for matrices
that are not a Yee stencil, over the CSR entry points of include/cevgpu.h.

Gradient conventions follow PyTorch (g = dL/dRe + i dL/dIm).  Reverse mode
restates the reference VJPs (primitives.py:74-88, 121-137): for y = A x,
grad_x = A^H g and grad_entries[k] = g[i_k] conj(x[j_k]); for x = A^{-1} b,
lambda = A^{-H} g (a transposed GPU solve), grad_b = lambda and
grad_entries[k] = -lambda[i_k] conj(x[j_k]).  Forward mode restates the JVPs
(primitives.py:90-98, 139-148): d(Ax) = A dx + dA x, d(A^{-1}b) = A^{-1}(db - dA x).
"""
import ctypes as C
import warnings

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, stream_ptr
from .primitives import SolverWarning, _require_cuda, _workspace, make_opts


class CSR:
    """COO entries/indices (duplicates summed) as device CSR, plus its transpose."""

    def __init__(self, entries, indices, n):
        _require_cuda()
        self.n = int(n)
        idx = torch.as_tensor(np.asarray(indices) if not torch.is_tensor(indices) else indices)
        self.idx = idx.to("cuda", torch.int64).reshape(2, -1)
        self.perm = None
        self._t = None
        self._build(self.idx)
        self.set_values(entries)

    def _build(self, idx):
        key = idx[0] * self.n + idx[1]
        order = torch.argsort(key, stable=True)
        ks = key[order]
        uniq, inv = torch.unique_consecutive(ks, return_inverse=True)
        self.perm, self.inv, self.nnz = order, inv, int(uniq.numel())
        self.rows_u = uniq // self.n
        self.cols_u = uniq % self.n
        self.col = self.cols_u.to(torch.int32).contiguous()
        counts = torch.bincount(self.rows_u, minlength=self.n)
        self.row_ptr = torch.zeros(self.n + 1, dtype=torch.int32, device="cuda")
        self.row_ptr[1:] = torch.cumsum(counts, 0).to(torch.int32)

    def csr_values(self, entries):
        """Entry vector (COO order) -> summed CSR values (complex128)."""
        e = entries if torch.is_tensor(entries) else torch.as_tensor(np.asarray(entries))
        e = e.to("cuda", torch.complex128).reshape(-1)
        v = torch.zeros(self.nnz, dtype=torch.complex128, device="cuda")
        v.index_add_(0, self.inv, e[self.perm])
        return v

    def set_values(self, entries):
        self.val = self.csr_values(entries).resolve_conj().resolve_neg().contiguous()
        amax = float(self.val.abs().max()) if self.nnz else 1.0
        self.scale = 1.0 / amax if amax > 0 else 1.0
        self._t = None

    def transpose(self):
        """CSR of A^T (built once from A's summed entries)."""
        if self._t is None:
            self._t = CSR(self.val, torch.stack([self.cols_u, self.rows_u]), self.n)
        return self._t

    def apply(self, x, values=None):
        lib = _lib.load()
        xv = x.to("cuda", torch.complex128).reshape(-1).resolve_conj().resolve_neg().contiguous()
        y = torch.empty_like(xv)
        val = self.val if values is None else values
        check(lib.cev_csr_apply(self.n, self.nnz, ptr(self.row_ptr), ptr(self.col), ptr(val),
                                ptr(xv), ptr(y), stream_ptr()), "csr_apply")
        return y

    def solve(self, b, strict=False, **opts):
        lib = _lib.load()
        bv = b.to("cuda", torch.complex128).reshape(-1).resolve_conj().resolve_neg().contiguous()
        x = torch.empty_like(bv)
        s = make_opts(**opts)
        nbytes = lib.cev_csr_solve_workspace_size(self.n, self.nnz, C.byref(s))
        ws, wptr = _workspace(nbytes, torch.device("cuda"))
        info = (_lib.SolveInfo * 1)()
        rc = lib.cev_csr_solve(self.n, self.nnz, ptr(self.row_ptr), ptr(self.col), ptr(self.val),
                               self.scale, ptr(bv), ptr(x), C.byref(s), info, C.c_void_p(wptr),
                               nbytes, stream_ptr())
        check(rc, "csr_solve")
        del ws
        if rc > 0:
            msg = (f"sparse solve did not reach tol={s.tol:g}: residual "
                   f"{info[0].residual:.3g} after {info[0].iterations} iterations")
            if strict:
                raise _lib.CevError(msg)
            warnings.warn(msg, SolverWarning, stacklevel=2)
        return x


def _gather_grad(g_rows, x_cols, indices, real):
    gi = g_rows[indices[0]] * x_cols[indices[1]].conj()
    return gi.real if real else gi


class _SpMult(torch.autograd.Function):
    @staticmethod
    def forward(ctx, entries, x, indices, n, opts):
        A = CSR(entries.detach(), indices, n)
        y = A.apply(x.detach())
        ctx.A, ctx.idx = A, A.idx
        ctx.e_real, ctx.x_real = not entries.is_complex(), not x.is_complex()
        ctx.save_for_backward(entries, x)
        ctx.save_for_forward(entries, x)
        return y

    @staticmethod
    def backward(ctx, g):
        entries, x = ctx.saved_tensors
        g = g.to(torch.complex128)
        xc = x.to("cuda", torch.complex128).reshape(-1)
        ge = gx = None
        if ctx.needs_input_grad[0]:
            ge = _gather_grad(g, xc, ctx.idx, ctx.e_real)
        if ctx.needs_input_grad[1]:
            gx = ctx.A.transpose().apply(g.conj()).conj()
            gx = gx.real if ctx.x_real else gx
            gx = gx.reshape(x.shape)
        return ge, gx, None, None, None

    @staticmethod
    def jvp(ctx, de, dx, _i, _n, _o):
        entries, x = ctx.saved_tensors
        out = torch.zeros(ctx.A.n, dtype=torch.complex128, device="cuda")
        if dx is not None:
            out = out + ctx.A.apply(dx)
        if de is not None:
            out = out + ctx.A.apply(x, values=ctx.A.csr_values(de))
        return out


class _SpSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, entries, b, indices, n, opts):
        A = CSR(entries.detach(), indices, n)
        x = A.solve(b.detach(), **opts)
        ctx.A, ctx.idx, ctx.opts = A, A.idx, opts
        ctx.e_real, ctx.b_real = not entries.is_complex(), not b.is_complex()
        ctx.save_for_backward(x)
        ctx.save_for_forward(x)
        ctx.b_shape = b.shape
        return x

    @staticmethod
    def backward(ctx, g):
        x, = ctx.saved_tensors
        mu = ctx.A.transpose().solve(g.to(torch.complex128).conj(), **ctx.opts)
        lam = mu.conj()
        ge = gb = None
        if ctx.needs_input_grad[0]:
            ge = _gather_grad(-lam, x, ctx.idx, ctx.e_real)
        if ctx.needs_input_grad[1]:
            gb = (lam.real if ctx.b_real else lam).reshape(ctx.b_shape)
        return ge, gb, None, None, None

    @staticmethod
    def jvp(ctx, de, db, _i, _n, _o):
        x, = ctx.saved_tensors
        rhs = torch.zeros_like(x)
        if db is not None:
            rhs = rhs + db.to(torch.complex128).reshape(-1)
        if de is not None:
            rhs = rhs - ctx.A.apply(x, values=ctx.A.csr_values(de))
        return ctx.A.solve(rhs, **ctx.opts)


def _t(a):
    if torch.is_tensor(a):
        return a.to("cuda")
    return torch.as_tensor(np.asarray(a), device="cuda")


def sp_mult(entries, indices, x, **opts):
    """y = A x with A = sparse(entries, indices) of shape (x.size, x.size)."""
    numpy_out = not torch.is_tensor(entries) and not torch.is_tensor(x)
    e, xv = _t(entries), _t(x)
    y = _SpMult.apply(e, xv, indices, xv.numel(), opts)
    return y.detach().cpu().numpy() if numpy_out else y


def sp_solve(entries, indices, b, **opts):
    """x = A^{-1} b with A = sparse(entries, indices) of shape (b.size, b.size)."""
    numpy_out = not torch.is_tensor(entries) and not torch.is_tensor(b)
    e, bv = _t(entries), _t(b)
    opts = dict(dict(tol=1e-10), **opts)
    x = _SpSolve.apply(e, bv, indices, bv.numel(), opts)
    return x.detach().cpu().numpy() if numpy_out else x
