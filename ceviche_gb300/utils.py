"""``measure_fields`` (ceviche/utils.py:316-332) with on-device probe sums.

The reference steps ``F.forward(Jz=source(t))`` and takes
``np.sum(fields[component] * probe)`` for each probe on the host every step.
Here every step's probe sums are reduced on the GPU by ``cev_probe_measure``
into a device buffer that is read back once.  When ``source`` is given as a
separable ``(profile, amps)`` pair (Jz(t) = profile * amps[t]) and the
component is Ez of a TM run, the time-blocked runner records the probes'
cells and the same kernel combines them, so no per-step launch is needed.

Probes are arrays with one entry per cell, shaped like the fields ((Nx, Ny, 1)
as in the reference's examples, or (Nx, Ny)).  The reference prints its
progress every ``steps // 20`` steps (and divides by zero below 20 steps);
here ``verbose=True`` prints the same lines every ``max(steps // 20, 1)``
steps and the default is quiet.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, stream_ptr

_MAX_ROWS = 65535
_COMPONENTS = ("Ex", "Ey", "Ez", "Dx", "Dy", "Dz", "Hx", "Hy", "Hz")


class ProbeSet:
    """Probe masks as a device CSR of their non-zero cells (FP64 weights)."""

    def __init__(self, probes, Nx, Ny):
        self.n_cells = Nx * Ny
        cells, weights, pptr = [], [], [0]
        for p in probes:
            a = p.detach().cpu().numpy() if torch.is_tensor(p) else np.asarray(p)
            if a.size != self.n_cells:
                raise ValueError(f"probe has {a.size} entries, the grid has {self.n_cells} cells")
            if np.iscomplexobj(a):
                raise ValueError("probes must be real (the FDTD fields are real)")
            a = a.reshape(-1).astype(np.float64)
            nz = np.flatnonzero(a)
            cells.append(nz)
            weights.append(a[nz])
            pptr.append(pptr[-1] + nz.size)
        self.n_probe = len(pptr) - 1
        cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
        self.cells_np = cat(cells, np.int64)
        self.ptr = torch.as_tensor(np.asarray(pptr, np.int32), device="cuda")
        self.cell = torch.as_tensor(cat(cells, np.int32), device="cuda")
        self.w = torch.as_tensor(cat(weights, np.float64), device="cuda")

    def measure(self, field, out, row0=0, nrows=1, stride=0, cell=None):
        """out[row0 + t, p] = sum_q w_q field[t*stride + cell_q] for t < nrows."""
        lib = _lib.load()
        f = field.detach().contiguous()
        if f.dtype not in (torch.float32, torch.float64):
            raise TypeError(f"field dtype {f.dtype} is not float32/float64")
        cell = self.cell if cell is None else cell
        for r in range(0, nrows, _MAX_ROWS):
            nr = min(_MAX_ROWS, nrows - r)
            check(lib.cev_probe_measure(self.n_probe, ptr(self.ptr), ptr(cell), ptr(self.w),
                                        C.c_void_p(f.data_ptr() + r * stride * f.element_size()),
                                        int(f.dtype == torch.float64), nr, stride,
                                        C.c_void_p(out[row0 + r:].data_ptr()), out.stride(0),
                                        stream_ptr()), "probe_measure")


def _separable(source):
    return isinstance(source, tuple) and len(source) == 2 and not callable(source[0])


def measure_fields(F, source, steps, probes, component="Ez", verbose=False):
    """(steps, n_probe) float64 array of sum(fields[component] * probe) after
    each step of F driven by Jz = source(t) (or profile * amps[t])."""
    if component not in _COMPONENTS:
        raise KeyError(component)
    F.initialize_fields()
    if not isinstance(probes, list):
        probes = [probes]
    ps = ProbeSet(probes, F.Nx, F.Ny)
    out = torch.zeros((steps, ps.n_probe), dtype=torch.float64, device="cuda")
    if steps == 0 or ps.n_probe == 0:
        return out.cpu().numpy()
    if _separable(source) and component == "Ez" and F._te is None:
        profile, amps = source
        cells, local = np.unique(ps.cells_np, return_inverse=True)
        if cells.size == 0:
            F.run(steps, profile, amps)
            return out.cpu().numpy()
        series = F.run(steps, profile, amps, [(int(c) // F.Ny, int(c) % F.Ny) for c in cells])
        local_d = torch.as_tensor(local.astype(np.int32), device="cuda")
        ps.measure(series, out, nrows=steps, stride=cells.size, cell=local_d)
        return out.cpu().numpy()
    if _separable(source):
        profile, amps = source
        source = lambda t: profile * amps[t]  # noqa: E731
    every = max(steps // 20, 1)
    for t in range(steps):
        if verbose and t % every == 0:
            print("{:.2f} % done".format(float(t) / steps * 100.0))
        fields = F.forward(Jz=source(t))
        ps.measure(fields[component], out, row0=t)
    return out.cpu().numpy()
