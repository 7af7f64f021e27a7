"""Forward-only stand-in for HIPS autograd, used ONLY to import the ceviche
reference in the fixture-generation script (tests/golden/make_golden.py).

ceviche's forward solvers need nothing from autograd beyond the
``primitive``/``defvjp``/``defjvp`` names existing, so ``primitive`` is the
identity and the derivative registrations are no-ops.  No gradient is ever
computed through this module.
"""
from . import extend  # noqa: F401
from . import numpy  # noqa: F401


def primitive(f):
    return f


def grad(*args, **kwargs):  # pragma: no cover - never called by the forward path
    raise NotImplementedError("forward-only autograd stand-in")


def checkpoint(f):  # pragma: no cover
    return f
