"""GB300-native (sm_103a) implementation of ceviche's Yee-stencil hot path.

Drop-in API of ceviche 0.1.3 (ceviche/__init__.py:6-12) for the parts on that
path: ``fdfd_ez``, ``fdfd_hz``, ``fdtd`` and ``jacobian``.  All compute runs
in hand-written CUDA kernels behind the C ABI of include/cevgpu.h
(libcevgpu.so, loaded on first use).  Importing the package needs no GPU.
"""
__version__ = "0.1.3+gb300"

from .fdfd import fdfd_ez, fdfd_hz, fdfd_mf_ez  # noqa: F401
from .fdtd import fdtd, fdtd_probe_series  # noqa: F401
from .jacobians import jacobian  # noqa: F401
from .sparse import sp_mult, sp_solve  # noqa: F401
from . import constants, primitives  # noqa: F401
