"""Waveguide modes on the GPU: ``get_modes`` / ``insert_mode``
(ceviche/modes.py:10-65) over ``cev_mode_solve``, plus ``get_modes_batch``
for many cross sections (or frequencies) in one launch.

``get_modes(eps_cross, omega, dL, npml, m=1, filtering=True)`` returns
``(vals, vecs)`` like the reference: ``vals`` the m eigenvalues (n_eff^2) of
diag(eps) + Dxf Dxb / k0^2 nearest max(eps), nearest first; ``vecs`` an
(N, m) array of unit-norm profiles.  The reference's eigenvector phase is
that of ARPACK's random start vector; here the largest-magnitude entry of
each profile is real and positive.  Non-convergence raises (ARPACK raises
ArpackNoConvergence).  ``filter_modes`` / ``normalize_modes`` mirror
modes.py:81-117 on the returned host arrays.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, stream_ptr
from .primitives import _require_cuda, _workspace


def get_modes_batch(eps_cross, omega, dL, npml, m=1, tol=1e-10, max_iters=1000):
    """eps_cross: (B, N) real permittivities.  Returns device tensors vals
    (B, m) and vecs (B, N, m), complex128, and the iteration counts (B,)."""
    _require_cuda()
    e = eps_cross if torch.is_tensor(eps_cross) else torch.as_tensor(np.asarray(eps_cross))
    if e.is_complex():
        raise TypeError("the GPU mode solver takes a real permittivity")
    e = e.detach().to("cuda", torch.float64)
    if e.dim() == 1:
        e = e.reshape(1, -1)
    e = e.reshape(e.shape[0], -1).contiguous()
    B, N = e.shape
    lib = _lib.load()
    nbytes = lib.cev_mode_workspace_size(B, N, int(m))
    if nbytes == 0:
        raise ValueError(f"unsupported sizes: batch={B}, N={N}, m={m} (N >= 3, m <= min(N, 24))")
    ws, wptr = _workspace(nbytes, e.device)
    vals = torch.empty((B, m), dtype=torch.complex128, device="cuda")
    vecs = torch.empty((B, m, N), dtype=torch.complex128, device="cuda")
    iters = torch.empty(B, dtype=torch.int32, device="cuda")
    status = torch.empty(B, dtype=torch.int32, device="cuda")
    check(lib.cev_mode_solve(B, N, ptr(e), float(omega), float(dL), int(npml), int(m), float(tol),
                             int(max_iters), ptr(vals), ptr(vecs), ptr(iters), ptr(status),
                             C.c_void_p(wptr), nbytes, stream_ptr()), "mode_solve")
    del ws
    st = status.cpu().numpy()
    if np.any(st != 0):
        bad = int(np.flatnonzero(st)[0])
        why = "singular shift" if st[bad] == 2 else f"no convergence in {max_iters} iterations"
        raise _lib.CevError(f"mode solve of cross section {bad}: {why}")
    return vals, vecs.transpose(1, 2), iters


def filter_modes(values, vectors, filters=None):
    """ceviche/modes.py:81-106."""
    if filters is None:
        return values, vectors
    keep = np.ones(values.shape, dtype=bool)
    for f in filters:
        keep = np.logical_and(keep, f(values))
    idx = np.where(keep)[0]
    return values[idx], vectors[:, idx]


def normalize_modes(vectors):
    """ceviche/modes.py:109-117: unit 2-norm columns."""
    return vectors / np.sqrt(np.sum(np.square(np.abs(vectors)), axis=0))


def get_modes(eps_cross, omega, dL, npml, m=1, filtering=True):
    """ceviche/modes.py:10-45 on the GPU."""
    eps = np.asarray(eps_cross)
    vals, vecs, _ = get_modes_batch(eps.reshape(1, -1), omega, dL, npml, m=m)
    vals, vecs = vals[0].cpu().numpy(), vecs[0].cpu().numpy()
    if filtering:
        vals, vecs = filter_modes(vals, vecs, filters=[lambda v: np.real(v) > 0.0])
    if vals.size == 0:
        raise BaseException("Could not find any eigenmodes for this waveguide")
    return vals, normalize_modes(vecs)


def insert_mode(omega, dx, x, y, epsr, target=None, npml=0, m=1, filtering=False):
    """ceviche/modes.py:48-65: the m-th mode of the cross section epsr[x, y]
    written into target[x, y] (a new complex array by default)."""
    if target is None:
        target = np.zeros(epsr.shape, dtype=complex)
    _, mode_field = get_modes(epsr[x, y], omega, dx, npml, m=m, filtering=filtering)
    target[x, y] = np.atleast_2d(mode_field)[:, m - 1].squeeze()
    return target
