"""Learned right preconditioner for the GPU flexible GMRES (precond="learned").

A 4-level convolutional encoder-decoder (csrc/learned.cu: bf16 tensor-core
convolutions with fp32 accumulation, forward and backward) maps a Krylov
basis vector v of a single-frequency Ez problem to z ~ A'^-1 v, where A' is
the non-dimensional operator the solver iterates on.  It has no counterpart
in ceviche; it serves the iterative solve that replaces ceviche's direct
``spsolve`` (ceviche/solvers.py:37-62, primitives.py:103-119).

Training is physics-informed and runs on the GPU through the library's own
kernels: for residual vectors r that the plain solver produces on the
training problems, the loss is

    L = mean_b ||A' z_b - r_b||^2 / ||r_b||^2,   z = f(r),

its gradient dL/dz = 2 A'^H (A' z - r) / (B ||r||^2) comes from the stencil
kernels (cev_fdfd_apply, transposed and conjugated), and dL/dparams from the
network's backward kernels; Adam is one more kernel.  Parameters, gradients
and the Adam moments are fp32 device tensors owned here.

    net = LearnedPreconditioner(256, 256, max_batch=16)
    net.fit(problems, steps=2000)
    x, info = primitives.solve(plan, eps, b, precond="learned", learned=net)
"""
import ctypes as C
import warnings

import numpy as np
import torch

from . import _lib
from . import primitives as P
from ._lib import check, ptr, stream_ptr


def param_count(c0):
    n = C.c_size_t()
    check(_lib.load().cev_learned_param_count(int(c0), C.byref(n)), "learned_param_count")
    return n.value


def init_params(c0, seed=0):
    """He-normal conv weights, zero biases, a small head (float32 numpy);
    layout: per conv layer W[cout][cin][3][3] then b[cout], then head W[2][c0], b[2]."""
    c1, c2, c3, c4 = c0, 2 * c0, 4 * c0, 8 * c0
    specs = [(8, c1), (c1, c2), (c2, c3), (c3, c4), (c4, c4), (c4, c3), (c3, c3), (c3, c2),
             (c2, c2), (c2, c1), (c1, c1)]
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co in specs:
        parts.append(rng.standard_normal(co * ci * 9) * np.sqrt(2.0 / (9 * ci)))
        parts.append(np.zeros(co))
    parts.append(rng.standard_normal(2 * c0) * (0.01 / np.sqrt(c0)))
    parts.append(np.zeros(2))
    return np.concatenate(parts).astype(np.float32)


class LearnedPreconditioner:
    """The network, its parameters and its Adam state on one device."""

    def __init__(self, nx, ny, max_batch=16, c0=32, seed=0, params=None):
        P._require_cuda()
        lib = _lib.load()
        self.nx, self.ny, self.max_batch, self.c0 = int(nx), int(ny), int(max_batch), int(c0)
        self.nparam = param_count(c0)
        dev = torch.device("cuda", torch.cuda.current_device())
        p = init_params(c0, seed) if params is None else np.asarray(params, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters, got {p.size}")
        self.params = torch.as_tensor(p, device=dev).contiguous()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.step = 0
        h = C.c_void_p()
        check(lib.cev_learned_create(C.byref(h), self.nx, self.ny, self.max_batch, self.c0),
              "learned_create")
        self.handle = h
        self._packed = False
        self.history = []

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and getattr(_lib, "_lib", None) is not None:
            _lib._lib.cev_learned_destroy(h)
            self.handle = None

    # ------------------------------------------------------------ parameters
    def _pack(self):
        if not self._packed:
            check(_lib.load().cev_learned_set_params(self.handle, ptr(self.params), stream_ptr()),
                  "learned_set_params")
            self._packed = True

    def handle_ptr(self):
        """The C handle for cev_solve_opts.learned (parameters packed first)."""
        self._pack()
        return self.handle.value

    def state_dict(self):
        return {"nx": self.nx, "ny": self.ny, "c0": self.c0, "params": self.params.cpu(),
                "step": self.step}

    def load_state_dict(self, sd):
        if (sd["nx"], sd["ny"], sd["c0"]) != (self.nx, self.ny, self.c0):
            raise ValueError("state is for another grid or width")
        self.params.copy_(sd["params"].to(self.params.device))
        self.step = int(sd.get("step", 0))
        self._packed = False

    # ---------------------------------------------------------- forward/backward
    def forward(self, plan, eps, r):
        """z = f(r) for every problem of the plan (complex64 (batch, nx, ny))."""
        self._pack()
        e, sh = P._eps_arg(plan, eps, torch.float32)
        rt = P._field_arg(plan, r, torch.complex64)
        z = torch.empty_like(rt)
        check(_lib.load().cev_learned_forward(self.handle, plan.handle, ptr(e), sh, ptr(rt), ptr(z),
                                              stream_ptr()), "learned_forward")
        return z

    def backward(self, gz):
        """Accumulate dL/dparams into self.grad for dL/dz = gz (after forward)."""
        g = gz.to(torch.complex64).contiguous()
        check(_lib.load().cev_learned_backward(self.handle, ptr(g), ptr(self.grad), stream_ptr()),
              "learned_backward")
        return self.grad

    def loss_and_grad(self, plan, eps, r):
        """Physics loss mean_b ||A' f(r_b) - r_b||^2/||r_b||^2 and its parameter gradient."""
        z = self.forward(plan, eps, r)
        rt = P._field_arg(plan, r, torch.complex64)
        w = P.apply(plan, eps, z, precision="c64", si_units=False) - rt
        B = rt.shape[0]
        rn = (rt.abs() ** 2).reshape(B, -1).sum(1).clamp_min(1e-30)
        per = (w.abs() ** 2).reshape(B, -1).sum(1) / rn
        aw = P.apply(plan, eps, w.conj().resolve_conj(), transpose=True, precision="c64",
                     si_units=False).conj()
        gz = (2.0 / B) * aw / rn.view(B, 1, 1)
        self.grad.zero_()
        self.backward(gz)
        return per.mean(), per

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        check(_lib.load().cev_adam_step(ptr(self.params), ptr(self.grad), ptr(self.m), ptr(self.v),
                                        self.nparam, lr, beta1, beta2, eps, self.step, stream_ptr()),
              "adam_step")
        self._packed = False

    def train_step(self, plan, eps, r, lr=1e-3):
        loss, _ = self.loss_and_grad(plan, eps, r)
        self.adam(lr)
        return loss

    def fit(self, samples, steps, lr=1e-3, lr_final=None, seed=0, log_every=0):
        """Adam on (plan, eps, r) samples drawn uniformly; cosine decay to lr_final."""
        rng = np.random.default_rng(seed)
        lr_final = lr * 0.05 if lr_final is None else lr_final
        for k in range(steps):
            plan, eps, r = samples[rng.integers(len(samples))]
            a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * k / max(1, steps)))
            loss = self.train_step(plan, eps, r, lr=float(a))
            if log_every and (k % log_every == 0 or k == steps - 1):
                self.history.append((k, float(loss)))
        return self.history


def residual_samples(plan, eps, b, iters=(0, 10, 30, 90)):
    """Training inputs from the plain GPU solver: for each k in ``iters`` the
    residuals b - A x_k of its iterate after k iterations (k = 0 gives b).
    Returns complex64 tensors (batch, nx, ny)."""
    out = []
    bt = P._field_arg(plan, b, torch.complex128)
    x = None
    done = 0
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", P.SolverWarning)
        for k in sorted(iters):
            if k > done:
                x, _ = P.solve(plan, eps, bt, x0=x, tol=1e-14, max_iters=k - done,
                               max_stall=10 ** 6)
                done = k
            r = bt if x is None else bt - P.apply(plan, eps, x)
            out.append(r.to(torch.complex64))
    return out


def on_policy_samples(net, plan, eps, b, iters=(30, 90, 270)):
    """Residuals b - A x_k of flexible GMRES *with the network* after k
    iterations: the vectors on which the preconditioned solver stalls.  One
    round of training on these (with the plain-solver samples) lowers the
    residual the preconditioned solver reaches."""
    bt = P._field_arg(plan, b, torch.complex128)
    out = []
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", P.SolverWarning)
        for k in iters:
            x, _ = P.solve(plan, eps, bt, tol=1e-14, max_iters=k, max_stall=10 ** 6,
                           precond="learned", learned=net)
            out.append((bt - P.apply(plan, eps, x)).to(torch.complex64))
    return out
