"""The C-ABI library loads and exports every entry point include/cevgpu.h
declares (no CUDA call is made).  CPU only."""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "cevgpu.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"CEV_API\s+[\w\s\*]+?\b(cev_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib_path():
    from ceviche_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = _declared()
    assert "cev_fdfd_solve" in names and "cev_fdtd_run_tm" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib_path):
    from ceviche_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == _declared()
    lib = _lib.load(lib_path)
    assert lib.cev_version() >= 100


def test_validation_errors_without_gpu(lib_path):
    """Host-side argument checks fail synchronously with a message."""
    from ceviche_gb300 import _lib
    lib = _lib.load(lib_path)
    h = ctypes.c_void_p()
    om = (ctypes.c_double * 1)(1e15)
    rc = lib.cev_fdfd_plan_create(ctypes.byref(h), 0, 1, 20, 1, 25e-9, om, 0, 4, 0.0, 0.0)
    assert rc == _lib.CEV_ERR_INVALID
    assert b"1D grids" in lib.cev_last_error_string()
    rc = lib.cev_fdfd_plan_create(ctypes.byref(h), 7, 20, 20, 1, 25e-9, om, 0, 4, 0.0, 0.0)
    assert rc == _lib.CEV_ERR_INVALID
    opts = _lib.SolveOpts()
    lib.cev_solve_opts_default(ctypes.byref(opts))
    assert opts.tol == 1e-6 and opts.restart == 30
