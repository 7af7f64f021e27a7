"""cev_fdtd_run_tm_noalloc: the allocation-free TM runner for callers that
cannot allocate device memory (a host framework that owns every device
allocation, or a real-time loop where cudaMalloc/cudaFree are off limits).

It is called here through the C ABI and must reproduce cev_fdtd_run_tm (the
plan-based runner that allocates its own shadow state) on the same inputs,
within the float32 tolerance the FDTD runner tests use (1e-6 relative), on two
calls in a row -- the second call continues from the first call's state and
runs after the shared static scratch holds the first call's leftovers.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from ceviche_gb300 import _lib

TOL = 1e-6


def _rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _lib_loaded():
    from ceviche_gb300 import build
    build.build()
    return _lib.load()


def _state(nx, ny):
    ts = {k: torch.zeros((nx, ny), dtype=torch.float32, device="cuda")
          for k in ("hx", "hy", "dz", "icex", "icey", "idz")}
    st = _lib.FDTDState()
    for k, v in ts.items():
        setattr(st, k, v.data_ptr())
    return ts, st


def _io(nx, ny, steps, rng):
    src = torch.tensor([(nx // 2) * ny + ny // 3, 3 * ny + ny - 2], dtype=torch.int32, device="cuda")
    w = torch.tensor([1.0, -0.5], dtype=torch.float32, device="cuda")
    t = np.arange(steps)
    amps = torch.as_tensor(np.sin(0.21 * t) * np.exp(-((t - 30) / 14.0) ** 2),
                           dtype=torch.float32, device="cuda")
    probes = [(nx // 2, ny // 3), (0, 0), (nx - 1, ny - 1), (17, 40)]
    pidx = torch.tensor([i * ny + j for i, j in probes], dtype=torch.int32, device="cuda")
    out = torch.zeros((steps, len(probes)), dtype=torch.float32, device="cuda")
    io = _lib.FDTDIO()
    io.n_src, io.src_idx, io.src_w, io.amps = 2, src.data_ptr(), w.data_ptr(), amps.data_ptr()
    io.n_probe, io.probe_idx, io.probe_out = len(probes), pidx.data_ptr(), out.data_ptr()
    return io, out, (src, w, amps, pidx)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(128, 112), (40, 36), (512, 512), (8192, 32), (32, 8192)])
def test_noalloc_runner_matches_plan_runner(shape):
    """(512, 512) fills the static scratch to its cell limit; (8192, 32) and
    (32, 8192) fill the axis tables to their per-dimension limit.  The
    runner builds its PML tables on the device, the plan runner on the host:
    agreement to 1e-6 also checks the tables."""
    lib = _lib_loaded()
    nx, ny = shape
    dL, npml = 25e-9, (9, 7)
    rng = np.random.default_rng(21)
    eps = torch.as_tensor(1 + 5 * rng.random((nx, ny)), dtype=torch.float64, device="cuda")
    stream = _lib.stream_ptr()

    plan = C.c_void_p()
    _lib.check(lib.cev_fdtd_plan_create(C.byref(plan), nx, ny, dL, npml[0], npml[1],
                                        _lib.PREC_C64, _lib.ptr(eps), stream), "plan")
    ref_fields, ref_st = _state(nx, ny)
    new_fields, new_st = _state(nx, ny)
    try:
        for call, steps in enumerate((70, 45)):  # two calls in a row
            io_r, out_r, keep_r = _io(nx, ny, steps, rng)
            io_n, out_n, keep_n = _io(nx, ny, steps, rng)
            _lib.check(lib.cev_fdtd_run_tm(plan, C.byref(ref_st), steps, C.byref(io_r), stream),
                       "run_tm")
            _lib.check(lib.cev_fdtd_run_tm_noalloc(nx, ny, dL, npml[0], npml[1], _lib.ptr(eps),
                                                   C.byref(new_st), steps, C.byref(io_n), stream),
                       "run_tm_noalloc")
            torch.cuda.synchronize()
            assert _rel(out_n.cpu().numpy(), out_r.cpu().numpy()) < TOL, f"probes, call {call}"
            for k in ref_fields:
                assert _rel(new_fields[k].cpu().numpy(), ref_fields[k].cpu().numpy()) < TOL, \
                    f"{k}, call {call}"
            assert float(out_r.abs().max()) > 0
    finally:
        lib.cev_fdtd_plan_destroy(plan)


def test_noalloc_rejects_oversize_grid():
    """Grids above the static scratch limit fail with a clear error before any
    CUDA call (so this check runs without a GPU)."""
    lib = _lib_loaded()
    st = _lib.FDTDState()
    rc = lib.cev_fdtd_run_tm_noalloc(1024, 1024, 25e-9, 10, 10, C.c_void_p(16), C.byref(st), 10,
                                     None, None)
    assert rc == _lib.CEV_ERR_INVALID
    assert b"exceeds the allocation-free runner's limit" in lib.cev_last_error_string()
