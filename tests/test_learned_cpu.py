"""Learned preconditioner, host side (no GPU): the library's parameter count
and the package's initialisation agree with the oracle's layout, the oracle
network is scale-equivariant (z(a r) = a z(r) for a > 0, as the solver
assumes), and invalid widths are rejected."""
import ctypes as C

import numpy as np
import torch

from oracle import learned as OL


def test_param_layout_matches_oracle():
    from ceviche_gb300 import _lib
    from ceviche_gb300 import learned as LM
    for c0 in (8, 16, 32):
        n = C.c_size_t()
        assert _lib.load().cev_learned_param_count(c0, C.byref(n)) == 0
        assert n.value == OL.param_count(c0) == LM.param_count(c0)
        assert np.array_equal(LM.init_params(c0, 4), OL.init_params(c0, 4))
    n = C.c_size_t()
    assert _lib.load().cev_learned_param_count(12, C.byref(n)) == _lib.CEV_ERR_INVALID


def test_oracle_scale_equivariance():
    rng = np.random.default_rng(0)
    B, nx, ny, c0 = 2, 16, 24, 8
    p = torch.as_tensor(OL.init_params(c0, 1))
    r = torch.as_tensor(rng.standard_normal((B, nx, ny)) + 1j * rng.standard_normal((B, nx, ny)),
                        dtype=torch.complex64)
    eps = torch.as_tensor(rng.uniform(1, 12, (B, nx, ny)), dtype=torch.float32)
    k2 = torch.tensor([0.05, 0.08])
    z1 = OL.apply(p, c0, r, eps, k2, (3, 3), round_bf16=False)
    z2 = OL.apply(p, c0, 7.5 * r, eps, k2, (3, 3), round_bf16=False)
    assert torch.allclose(z2, 7.5 * z1, rtol=1e-5, atol=1e-6)
