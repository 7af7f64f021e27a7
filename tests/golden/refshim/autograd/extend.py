"""No-op derivative registration for the forward-only autograd stand-in."""


def primitive(f):
    return f


def defvjp(*args, **kwargs):
    return None


def defjvp(*args, **kwargs):
    return None


def vspace(x):  # pragma: no cover - only used by reverse/forward jacobians
    raise NotImplementedError("forward-only autograd stand-in")
