"""Waveguide modes on the GPU (ceviche/modes.py:10-65) against the
reference's ARPACK results (tests/golden/modes.npz) and the dense FP64
oracle.  Eigenvalues to 1e-9 absolute (the reference's own ARPACK accuracy
is ~1e-11); eigenvectors up to a unit phase to 1e-9 (the reference's phase is
random), the near-degenerate even/odd pair of case 2 (split by 3e-11) as a
subspace; against the oracle, which uses the same phase convention, vectors
directly to 1e-8."""
import os

import numpy as np
import pytest

from oracle import modes as om
from tests.conftest import GOLDEN
from tests.test_oracle_golden import _same_up_to_phase

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def test_get_modes_matches_reference_and_oracle(cev):
    from ceviche_gb300 import modes
    d = np.load(os.path.join(GOLDEN, "modes.npz"))
    for c in range(4):
        omega, dL, npml, m = d[f"meta{c}"]
        args = (d[f"eps{c}"], omega, dL, int(npml), int(m))
        vals, vecs = modes.get_modes(*args, filtering=False)
        assert vals.shape == (int(m),) and vecs.shape == (d[f"eps{c}"].size, int(m))
        ref_v = d[f"vals{c}"]
        assert np.max(np.abs(np.sort_complex(vals) - np.sort_complex(ref_v))) < 1e-9, c
        clusters = [(0, 1)] if c == 2 else []
        _same_up_to_phase(vecs, d[f"vecs{c}"], clusters)
        ov, oV = om.get_modes(*args, filtering=False)
        if c != 2:
            assert np.max(np.abs(vals - ov)) < 1e-9
            assert np.max(np.abs(vecs - oV)) < 1e-8, c


def test_insert_mode_matches_reference(cev):
    from ceviche_gb300 import modes
    d = np.load(os.path.join(GOLDEN, "modes.npz"))
    omega = 2 * np.pi * om.C_0 / 1.55e-6
    src = modes.insert_mode(omega, 50e-9, 10, slice(5, 85), d["ins_epsr"], m=2)
    ref = d["ins_src"]
    assert src.dtype == np.complex128 and src.shape == ref.shape
    assert abs(abs(np.vdot(src[10, 5:85], ref[10, 5:85])) - 1) < 1e-9
    assert np.all(src[np.arange(40) != 10] == 0)


def test_batch_equals_single(cev):
    """A batch of cross sections (one CTA each) equals one-by-one solves."""
    from ceviche_gb300 import modes
    rng = np.random.default_rng(5)
    N, B = 90, 6
    eps = np.ones((B, N))
    for b in range(B):
        w0 = 30 + 3 * b
        eps[b, w0:w0 + 8 + b] = 4 + 8 * rng.random()
    omega = 2 * np.pi * om.C_0 / 1.55e-6
    vals, vecs, iters = modes.get_modes_batch(eps, omega, 50e-9, 8, m=2)
    for b in range(B):
        v1, V1 = modes.get_modes(eps[b], omega, 50e-9, 8, m=2, filtering=False)
        assert np.max(np.abs(vals[b].cpu().numpy() - v1)) < 1e-10
        assert np.max(np.abs(vecs[b].cpu().numpy() - V1)) < 1e-8
    assert int(iters.max()) < 1000


def test_filtering_and_errors(cev):
    from ceviche_gb300 import modes
    eps = np.ones(40)
    eps[15:25] = 12.25
    omega = 2 * np.pi * om.C_0 / 1.55e-6
    vals, vecs = modes.get_modes(eps, omega, 50e-9, 0, m=3)  # filtering=True keeps Re > 0
    assert np.all(vals.real > 0)
    with pytest.raises(ValueError):
        modes.get_modes(np.ones(2), omega, 50e-9, 0, m=1)
    with pytest.raises(TypeError):
        modes.get_modes_batch(np.ones((1, 10), complex), omega, 50e-9, 0, m=1)
