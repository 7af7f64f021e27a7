"""CPU float32 restatement of the learned preconditioner's network -- TEST
INFRASTRUCTURE ONLY.

The network has no counterpart in ceviche (it is the right preconditioner of
the flexible GMRES that stands in for ceviche's direct solve,
ceviche/solvers.py:37-62), so this oracle is the plain PyTorch float32
reference of the same maths, run on the CPU: the same architecture,
parameter layout and input features as the CUDA kernels, with bf16 rounding
applied where the GPU stores bf16 (input features, conv/pool/upsample
outputs, conv weights).  Gradients come from torch autograd on this graph.

Parameter layout (one flat float32 vector): per conv layer W[cout][cin][3][3]
then b[cout]; then the 1x1 head W[2][c0] and b[2].
"""
import numpy as np
import torch
import torch.nn.functional as F

CIN0 = 8


def layer_specs(c0):
    """(cin, cout, level) of the 11 conv layers."""
    c1, c2, c3, c4 = c0, 2 * c0, 4 * c0, 8 * c0
    return [(CIN0, c1, 0), (c1, c2, 1), (c2, c3, 2), (c3, c4, 3), (c4, c4, 3), (c4, c3, 3),
            (c3, c3, 2), (c3, c2, 2), (c2, c2, 1), (c2, c1, 1), (c1, c1, 0)]


def param_count(c0):
    return sum(co * ci * 9 + co for ci, co, _ in layer_specs(c0)) + 2 * c0 + 2


def unpack(params, c0):
    """Views of the flat parameter vector: [(W, b)] * 11, (Wh, bh)."""
    out, off = [], 0
    for ci, co, _ in layer_specs(c0):
        W = params[off:off + co * ci * 9].view(co, ci, 3, 3)
        off += co * ci * 9
        b = params[off:off + co]
        off += co
        out.append((W, b))
    Wh = params[off:off + 2 * c0].view(2, c0)
    bh = params[off + 2 * c0:off + 2 * c0 + 2]
    return out, (Wh, bh)


def init_params(c0, seed=0):
    """He-normal conv weights, zero biases, a small head (numpy float32)."""
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co, _ in layer_specs(c0):
        parts.append(rng.standard_normal(co * ci * 9) * np.sqrt(2.0 / (9 * ci)))
        parts.append(np.zeros(co))
    parts.append(rng.standard_normal(2 * c0) * (0.01 / np.sqrt(c0)))
    parts.append(np.zeros(2))
    return np.concatenate(parts).astype(np.float32)


def _bf(x, on):
    return x.to(torch.bfloat16).to(x.dtype) if on else x


def features(r, eps, k2, npml):
    """Input channels (B, 8, nx, ny) and the per-problem RMS of r.

    r complex (B, nx, ny); eps real (B, nx, ny); k2 (B,) non-dimensional
    eps0*mu0*omega^2*dL^2; npml (npml_x, npml_y)."""
    B, nx, ny = r.shape
    nrm = torch.sqrt((r.real ** 2 + r.imag ** 2).reshape(B, -1).mean(1))
    inv = torch.where(nrm > 0, 1.0 / nrm, torch.zeros_like(nrm)).view(B, 1, 1)
    i = torch.arange(nx).view(-1, 1)
    j = torch.arange(ny).view(1, -1)
    px, py = npml
    pml = ((i < px) | (i >= nx - px) | (j < py) | (j >= ny - py)).to(torch.float32)
    k2 = k2.view(B, 1, 1).to(torch.float32)
    X = torch.zeros(B, CIN0, nx, ny, dtype=torch.float32)
    X[:, 0] = (r.real * inv).to(torch.float32)
    X[:, 1] = (r.imag * inv).to(torch.float32)
    X[:, 2] = k2 * eps.to(torch.float32)
    X[:, 3] = pml
    X[:, 4] = torch.sqrt(k2).expand(B, nx, ny)
    return X, nrm.to(torch.float32)


def network(params, c0, X, round_bf16=True):
    """Output channels (B, 2, nx, ny) of the encoder-decoder for features X."""
    convs, (Wh, bh) = unpack(params, c0)
    bf = lambda t: _bf(t, round_bf16)

    def conv(x, l):
        W, b = convs[l]
        return bf(F.relu(F.conv2d(x, bf(W), b, padding=1)))

    def pool(x):
        return bf(F.avg_pool2d(x, 2))

    def up_add(x, s):
        return bf(F.interpolate(x, scale_factor=2, mode="nearest") + s)

    X = bf(X)
    A1 = conv(X, 0)
    A2 = conv(pool(A1), 1)
    A3 = conv(pool(A2), 2)
    A4 = conv(pool(A3), 3)
    A5 = conv(A4, 4)
    A6 = conv(A5, 5)
    A7 = conv(up_add(A6, A3), 6)
    A8 = conv(A7, 7)
    A9 = conv(up_add(A8, A2), 8)
    A10 = conv(A9, 9)
    A11 = conv(up_add(A10, A1), 10)
    return torch.einsum("bchw,oc->bohw", A11, Wh) + bh.view(1, 2, 1, 1)


def apply(params, c0, r, eps, k2, npml, round_bf16=True):
    """z = |r| * f(r/|r|, eps, k2) as complex (B, nx, ny)."""
    X, nrm = features(r, eps, k2, npml)
    o = network(params, c0, X, round_bf16)
    s = nrm.view(-1, 1, 1)
    return torch.complex(s * o[:, 0], s * o[:, 1])


def param_grad(params, c0, r, eps, k2, npml, gz, round_bf16=True):
    """dL/dparams for dL/dz = gz (PyTorch complex cotangent convention)."""
    p = params.detach().clone().requires_grad_(True)
    z = apply(p, c0, r, eps, k2, npml, round_bf16)
    L = (gz.real * z.real + gz.imag * z.imag).sum()
    L.backward()
    return p.grad.detach()
