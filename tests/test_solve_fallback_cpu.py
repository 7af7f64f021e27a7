"""Host logic of primitives.solve's fallback (no GPU): a preconditioned solve
that stops short of tol continues with plain GMRES from its iterate for the
rest of the iteration budget; infos add up both phases; a converged or
unpreconditioned solve makes no second call; fallback=False keeps the first
result."""
import warnings

import pytest
import torch


def _info(code, it, cyc=1, res=1e-3):
    return dict(status="x", code=code, iterations=it, cycles=cyc, residual=res)


@pytest.fixture
def fake(monkeypatch):
    from ceviche_gb300 import primitives as P
    calls = []

    def once(plan, eps, b, transpose, x0, **opts):
        calls.append((x0, dict(opts)))
        if opts.get("precond", "none") != "none":
            return torch.full((1, 2, 2), 1.0), [_info(2, 300, 10, 0.5)], 2, 1e-6
        return torch.full((1, 2, 2), 2.0), [_info(0, 120, 4, 1e-7)], 0, 1e-6

    monkeypatch.setattr(P, "_solve_once", once)
    return P, calls


def test_fallback_continues_with_plain(fake):
    P, calls = fake
    x, res = P.solve(None, None, None, precond="learned", learned=object(), max_iters=1000)
    assert len(calls) == 2
    x0, opts = calls[1]
    assert "precond" not in opts and "learned" not in opts and opts["max_iters"] == 700
    assert opts["max_stall"] == 20  # default patience for the plain phase
    assert torch.equal(x0, torch.full((1, 2, 2), 1.0))  # continues from the first iterate
    assert torch.equal(x, torch.full((1, 2, 2), 2.0))
    assert res[0]["iterations"] == 420 and res[0]["precond_iterations"] == 300
    assert res[0]["cycles"] == 14 and res[0]["code"] == 0


def test_hybrid_stall_limit_only_governs_the_handover(fake):
    P, calls = fake
    P.solve(None, None, None, precond="learned", learned=object(), max_stall=1, max_iters=1000)
    assert calls[0][1]["max_stall"] == 1 and calls[1][1]["max_stall"] == 20
    P.solve(None, None, None, precond="learned", learned=object(), max_stall=50, max_iters=1000)
    assert calls[3][1]["max_stall"] == 50


def test_no_fallback_without_preconditioner_or_when_disabled(fake):
    P, calls = fake
    P.solve(None, None, None, max_iters=1000)
    assert len(calls) == 1
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        _, res = P.solve(None, None, None, precond="separable", fallback=False, max_iters=1000)
    assert len(calls) == 2 and res[0]["code"] == 2


def test_no_fallback_when_budget_is_spent(fake):
    P, calls = fake
    with pytest.warns(P.SolverWarning):
        _, res = P.solve(None, None, None, precond="learned", learned=object(), max_iters=300)
    assert len(calls) == 1 and res[0]["iterations"] == 300
