"""Generic entries/indices primitives on the GPU (ceviche/primitives.py:58-148)
against scipy (the reference's make_sparse + dot / spsolve) and against
complex central differences, as tests/test_primitives.py does (there with
assert_almost_equal to 3 decimals; here 1e-6 relative)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl
import torch

pytestmark = pytest.mark.gpu


def _problem(N=8, M=44, seed=2):
    rng = np.random.default_rng(seed)
    ent = (rng.random(M) - 0.5) + 1j * (rng.random(M) - 0.5)
    idx = rng.integers(0, N, size=(2, M))
    # a well-conditioned diagonal keeps the random system solvable
    ent = np.concatenate([ent, 4.0 + 0j * np.arange(N)])
    idx = np.concatenate([idx, np.vstack([np.arange(N), np.arange(N)])], axis=1)
    A = sp.coo_matrix((ent, idx), shape=(N, N)).tocsr()
    return rng, ent, idx, A


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_sp_mult_and_solve_match_scipy():
    from ceviche_gb300.sparse import sp_mult, sp_solve
    for N, M in ((8, 44), (300, 2000)):
        rng, ent, idx, A = _problem(N, M, seed=N)
        x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        assert _rel(sp_mult(ent, idx, x), A.dot(x)) < 1e-13
        b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        xs = sp_solve(ent, idx, b)
        assert _rel(A.dot(xs), b) < 1e-9
        assert _rel(xs, spl.spsolve(A.tocsc(), b)) < 1e-8


def _num_grad(f, z, h=1e-6):
    """Complex central differences, d/dRe + i d/dIm (torch convention)."""
    g = np.zeros(z.size, dtype=np.complex128)
    for k in range(z.size):
        for unit, part in ((1.0, 1.0), (1j, 1j)):
            zp, zm = z.copy(), z.copy()
            zp[k] += unit * h
            zm[k] -= unit * h
            g[k] += part * (f(zp) - f(zm)) / (2 * h)
    return g


@pytest.mark.parametrize("which", ["mult", "solve"])
def test_reverse_gradients(which):
    from ceviche_gb300.sparse import sp_mult, sp_solve
    rng, ent, idx, A = _problem()
    N = A.shape[0]
    v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    w = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    fn = sp_mult if which == "mult" else sp_solve

    def loss_np(e, vv):
        y = fn(e, idx, vv)
        return float(np.sum(np.abs(y * w) ** 2))

    e_t = torch.tensor(ent, device="cuda", requires_grad=True)
    v_t = torch.tensor(v, device="cuda", requires_grad=True)
    y = fn(e_t, idx, v_t)
    L = (torch.abs(y * torch.as_tensor(w, device="cuda")) ** 2).sum()
    L.backward()
    ge = _num_grad(lambda e: loss_np(e, v), ent)
    gv = _num_grad(lambda vv: loss_np(ent, vv), v)
    # central differences through a solve at tol 1e-10 carry ~1e-10/h noise
    tol = 1e-6 if which == "mult" else 1e-5
    assert _rel(e_t.grad.cpu().numpy(), ge) < tol
    assert _rel(v_t.grad.cpu().numpy(), gv) < tol


@pytest.mark.parametrize("which", ["mult", "solve"])
def test_forward_mode_matches_reverse(which):
    import torch.autograd.forward_ad as fwAD
    from ceviche_gb300.sparse import sp_mult, sp_solve
    rng, ent, idx, A = _problem()
    N = A.shape[0]
    v = torch.as_tensor(rng.standard_normal(N) + 1j * rng.standard_normal(N), device="cuda")
    fn = sp_mult if which == "mult" else sp_solve
    e0 = torch.tensor(ent, device="cuda")
    de = torch.as_tensor(rng.standard_normal(ent.size) + 1j * rng.standard_normal(ent.size),
                         device="cuda")
    dv = torch.as_tensor(rng.standard_normal(N) + 1j * rng.standard_normal(N), device="cuda")
    with fwAD.dual_level():
        y = fn(fwAD.make_dual(e0, de), idx, fwAD.make_dual(v, dv))
        tan = fwAD.unpack_dual(y).tangent.cpu().numpy()
    h = 1e-7
    yp = fn((e0 + h * de).cpu().numpy(), idx, (v + h * dv).cpu().numpy())
    ym = fn((e0 - h * de).cpu().numpy(), idx, (v - h * dv).cpu().numpy())
    assert _rel(tan, (yp - ym) / (2 * h)) < (1e-6 if which == "mult" else 1e-5)
