"""cev_dense_eig (the mode solver's Rayleigh-Ritz eigensolver, host side)
against numpy.linalg.eig on random, Hermitian, triangular and defective-ish
small matrices.  CPU only: the function makes no CUDA call."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from ceviche_gb300 import _lib, build
    build.build()
    return _lib.load()


def _eig(lib, H):
    k = H.shape[0]
    h = np.ascontiguousarray(H, dtype=np.complex128)
    w = np.zeros(k, np.complex128)
    v = np.zeros((k, k), np.complex128)
    rc = lib.cev_dense_eig(k, h.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                           v.ctypes.data_as(C.c_void_p))
    return rc, w, v


@pytest.mark.parametrize("k", [1, 2, 3, 7, 12, 24])
def test_random_complex(lib, k):
    rng = np.random.default_rng(k)
    for kind in ("general", "hermitian", "triangular", "scaled"):
        H = rng.standard_normal((k, k)) + 1j * rng.standard_normal((k, k))
        if kind == "hermitian":
            H = H + H.conj().T
        elif kind == "triangular":
            H = np.triu(H)
        elif kind == "scaled":
            H = H * 1e12
        rc, w, v = _eig(lib, H)
        assert rc == 0
        nrm = np.linalg.norm(H, 2)
        # eigen-residuals and agreement of the spectrum with numpy
        assert np.linalg.norm(H @ v - v * w[None, :], 2) <= 1e-11 * nrm, kind
        assert np.allclose(np.linalg.norm(v, axis=0), 1)
        ref = np.linalg.eigvals(H)
        for x in w:
            assert np.min(np.abs(ref - x)) <= 1e-10 * nrm, kind


def test_rejects_bad_k(lib):
    from ceviche_gb300 import _lib
    rc, _, _ = _eig(lib, np.zeros((1, 1)))
    assert rc == 0
    h = np.zeros(2 * 25 * 25)
    w = np.zeros(50)
    assert lib.cev_dense_eig(25, h.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                             h.ctypes.data_as(C.c_void_p)) == _lib.CEV_ERR_INVALID
