"""``jacobian`` (ceviche/jacobians.py:16-91) over PyTorch.

Objectives are written with torch operations; the wrapped argument is passed
as a float64 CUDA tensor.  The result is a numpy array of shape
(n_outputs, n_inputs), as in the reference.

* reverse   -- one torch.autograd VJP per output element
               (jacobians.py:29-35); FDFD solves differentiate through the
               transposed GPU solve.
* forward   -- one forward-mode JVP per input element
               (torch.autograd.forward_ad; jacobians.py:38-51); FDFD solves
               propagate tangents through one extra GPU solve each
               (primitives.py:139-146).  Complex inputs follow jacobians.py:47-50.
* numerical -- forward differences with ``step_size`` on the flattened input,
               exactly as jacobians.py:54-73.
"""
import numpy as np
import torch


def _as_input(x):
    if torch.is_tensor(x):
        t = x.detach()
    else:
        t = torch.as_tensor(np.asarray(x))
    dt = torch.complex128 if t.is_complex() else torch.float64
    return t.to(device="cuda" if torch.cuda.is_available() else "cpu", dtype=dt)


def _to_numpy(v):
    if torch.is_tensor(v):
        return v.detach().cpu().numpy()
    return np.asarray(v)


def jacobian(fun, argnum=0, mode="reverse", step_size=1e-6):
    """Jacobian of ``fun`` with respect to argument ``argnum``."""
    if mode == "reverse":
        return _jacobian_reverse(fun, argnum)
    elif mode == "forward":
        return _jacobian_forward(fun, argnum)
    elif mode == "numerical":
        return _jacobian_numerical(fun, argnum, step_size=step_size)
    else:
        raise ValueError("'mode' kwarg must be either 'reverse' or 'forward' or 'numerical', "
                         "given {}".format(mode))


def _jacobian_reverse(fun, argnum):
    def jac(*args):
        x = _as_input(args[argnum]).requires_grad_(True)
        a = list(args)
        a[argnum] = x
        out = fun(*a)
        out = out if torch.is_tensor(out) else torch.as_tensor(out)
        flat = out.reshape(-1)
        if flat.is_complex():
            raise TypeError("reverse-mode jacobian needs a real-valued function")
        rows = []
        for k in range(flat.numel()):
            g, = torch.autograd.grad(flat[k], x, retain_graph=k + 1 < flat.numel(),
                                     allow_unused=True)
            rows.append(torch.zeros_like(x).reshape(-1) if g is None else g.reshape(-1))
        return _to_numpy(torch.stack(rows)).reshape(flat.numel(), x.numel())
    return jac


def _jacobian_forward(fun, argnum):
    import torch.autograd.forward_ad as fwAD

    def jac(*args):
        x = _as_input(args[argnum])
        n_in = x.numel()
        a = list(args)

        def column(t):
            with fwAD.dual_level():
                a[argnum] = fwAD.make_dual(x, t.reshape(x.shape))
                out = fun(*a)
                out = out if torch.is_tensor(out) else torch.as_tensor(out)
                tan = fwAD.unpack_dual(out).tangent
                if tan is None:
                    tan = torch.zeros_like(out)
                return tan.reshape(-1).detach()

        cols = []
        for i in range(n_in):
            t = torch.zeros(n_in, dtype=x.dtype, device=x.device)
            if x.is_complex():
                t[i] = 1.0
                re = column(t)
                t[i] = 1j
                im = column(t)
                cols.append(re - 1j * im)
            else:
                t[i] = 1.0
                cols.append(column(t))
        J = torch.stack(cols, dim=1)
        return _to_numpy(J)
    return jac


def _jacobian_numerical(fun, argnum, step_size=1e-7):
    def jac(*args):
        x = _as_input(args[argnum])
        in_array = x.reshape(-1).clone()
        a = list(args)

        def call(v):
            a[argnum] = v
            with torch.no_grad():
                return np.atleast_1d(_to_numpy(fun(*a))).reshape(-1)

        out0 = call(in_array)
        m, n = in_array.numel(), out0.size
        J = np.zeros((n, m), dtype=np.result_type(out0.dtype, np.float64))
        for i in range(m):
            xi = in_array.clone()
            xi[i] += step_size
            J[:, i] = (call(xi) - out0) / step_size
        return J
    return jac
