"""Placeholders so ``from autograd.core import make_vjp, make_jvp`` imports."""


def make_vjp(*args, **kwargs):  # pragma: no cover
    raise NotImplementedError("forward-only autograd stand-in")


def make_jvp(*args, **kwargs):  # pragma: no cover
    raise NotImplementedError("forward-only autograd stand-in")
