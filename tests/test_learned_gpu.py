"""Learned preconditioner (csrc/learned.cu, ceviche_gb300/learned.py).

The network has no counterpart in ceviche, so its oracle is the CPU float32
PyTorch restatement in oracle/learned.py.  Checks:
  * forward: z matches the oracle; its error against the unrounded fp32
    oracle is no larger than that of the bf16-rounding oracle;
  * backward: per-layer parameter gradients, same criterion, for a
    structured (z) and a random cotangent;
  * the training gradient (physics loss through the stencil) against torch
    autograd of the same loss with the dense non-dimensional operator;
  * Adam against its formula;
  * training on the GPU lowers the held-out loss, and flexible GMRES with the
    trained network reaches a lower residual in 30 and 90 iterations than
    plain GMRES (by 5% or more) and than the untrained network (by 2x) on
    held-out 256x256 problems;
  * invalid uses fail loudly.
"""
import numpy as np
import pytest
import torch

from oracle import fdfd as ofd
from oracle import learned as OL

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(torch.linalg.norm((a - b).ravel()) / torch.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def _case(nx, ny, B, c0, seed=1):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.constants import EPSILON_0, MU_0
    rng = np.random.default_rng(seed)
    dL = 50e-9
    oms = 2 * np.pi * 3e8 / rng.uniform(1.3e-6, 1.8e-6, B)
    plan = P.get_plan("ez", (nx, ny), dL, oms, (4, 4))
    eps = torch.as_tensor(rng.uniform(1, 12, (B, nx, ny)))
    r = torch.as_tensor(rng.standard_normal((B, nx, ny)) + 1j * rng.standard_normal((B, nx, ny)))
    p = OL.init_params(c0, seed + 2)
    p[p == 0] = rng.standard_normal(int((p == 0).sum())) * 0.1  # non-zero biases
    k2 = torch.as_tensor(EPSILON_0 * MU_0 * dL ** 2 * oms ** 2, dtype=torch.float32)
    return plan, eps, r, p, k2, rng


@pytest.mark.parametrize("shape", [(32, 32, 2, 8), (64, 48, 3, 32)])
def test_forward_and_gradients_match_oracle(cev, shape):
    from ceviche_gb300.learned import LearnedPreconditioner
    nx, ny, B, c0 = shape
    plan, eps, r, p, k2, rng = _case(nx, ny, B, c0)
    net = LearnedPreconditioner(nx, ny, max_batch=4, c0=c0, params=p)
    pt, r64, e32 = torch.as_tensor(p), r.to(torch.complex64), eps.float()
    z = net.forward(plan, eps, r).cpu()
    zb = OL.apply(pt, c0, r64, e32, k2, (4, 4))
    zf = OL.apply(pt, c0, r64, e32, k2, (4, 4), round_bf16=False)
    assert _rel(z, zb) < 5e-3
    assert _rel(z, zf) <= 2 * _rel(zb, zf) + 1e-6
    for kind in ("z", "random"):
        gz = z if kind == "z" else torch.as_tensor(
            rng.standard_normal((B, nx, ny)) + 1j * rng.standard_normal((B, nx, ny))).to(torch.complex64)
        net.grad.zero_()
        g = net.backward(gz.cuda()).cpu()
        gb = OL.param_grad(pt, c0, r64, e32, k2, (4, 4), gz)
        gf = OL.param_grad(pt, c0, r64, e32, k2, (4, 4), gz, round_bf16=False)
        off = 0
        for l, (ci, co, _) in enumerate(OL.layer_specs(c0)):
            n = co * ci * 9 + co
            e_gpu, e_ref = _rel(g[off:off + n], gf[off:off + n]), _rel(gb[off:off + n], gf[off:off + n])
            assert e_gpu <= 1.5 * e_ref + 2e-3, (kind, l, e_gpu, e_ref)
            off += n
        e_gpu, e_ref = _rel(g[off:], gf[off:]), _rel(gb[off:], gf[off:])
        assert e_gpu <= 1.5 * e_ref + 1e-4, (kind, "head", e_gpu, e_ref)


def test_conv_paths_agree(cev):
    """The tcgen05 convs (default: persistent for single-slab layers; and
    without the persistent variant) and the mma.sync conv give the same forward
    and backward up to accumulation order, and no bounded wait ran out."""
    import ctypes as C
    from ceviche_gb300 import _lib
    from ceviche_gb300.learned import LearnedPreconditioner
    lib = _lib.load()
    nx, ny, B, c0 = 64, 48, 3, 32
    plan, eps, r, p, k2, rng = _case(nx, ny, B, c0, seed=7)
    net = LearnedPreconditioner(nx, ny, max_batch=4, c0=c0, params=p)
    gz = torch.as_tensor(rng.standard_normal((B, nx, ny)) + 1j * rng.standard_normal((B, nx, ny)),
                         dtype=torch.complex64).cuda()
    out = {}
    try:
        for impl in (0, 1, 2):
            assert lib.cev_learned_set_conv_impl(impl) == 0
            z = net.forward(plan, eps, r).cpu()
            net.grad.zero_()
            out[impl] = (z, net.backward(gz).cpu().clone())
    finally:
        lib.cev_learned_set_conv_impl(1)
    fault = C.c_int(-1)
    assert lib.cev_learned_tc_fault(C.byref(fault)) == 0 and fault.value == 0
    for impl in (1, 2):  # tcgen05 (persistent single-slab layers), tcgen05 (not persistent)
        assert _rel(out[impl][0], out[0][0]) < 2e-3
        assert _rel(out[impl][1], out[0][1]) < 2e-2


def test_training_gradient_through_stencil(cev):
    """loss_and_grad (network backward fed by the stencil adjoint) against
    torch autograd of the same physics loss with the dense A' and the
    oracle network."""
    from ceviche_gb300 import _lib
    from ceviche_gb300.learned import LearnedPreconditioner
    nx, ny, B, c0 = 32, 24, 2, 8
    plan, eps, r, p, k2, _ = _case(nx, ny, B, c0, seed=5)
    net = LearnedPreconditioner(nx, ny, max_batch=2, c0=c0, params=p)
    loss, _ = net.loss_and_grad(plan, eps, r)
    g = net.grad.cpu()
    scale = _lib.load().cev_fdfd_plan_scale(plan.handle)
    Ad = [torch.as_tensor((scale * ofd.make_A_ez(w, plan.dL, eps[b].numpy(), plan.npml)).toarray(),
                          dtype=torch.complex64) for b, w in enumerate(plan.omegas)]
    r64 = r.to(torch.complex64)

    def physics_loss(params, round_bf16):
        z = OL.apply(params, c0, r64, eps.float(), k2, (4, 4), round_bf16)
        per = []
        for b in range(B):
            w = Ad[b] @ z[b].reshape(-1) - r64[b].reshape(-1)
            per.append((w.abs() ** 2).sum() / (r64[b].abs() ** 2).sum())
        return torch.stack(per).mean()

    grads = {}
    for rb in (True, False):
        q = torch.as_tensor(p).clone().requires_grad_(True)
        L = physics_loss(q, rb)
        L.backward()
        grads[rb] = (float(L.detach()), q.grad)
    assert abs(float(loss) - grads[False][0]) <= 1e-2 * grads[False][0]
    e_gpu, e_ref = _rel(g, grads[False][1]), _rel(grads[True][1], grads[False][1])
    assert e_gpu <= 1.5 * e_ref + 5e-3, (e_gpu, e_ref)


def test_adam_matches_formula(cev):
    from ceviche_gb300 import _lib
    from ceviche_gb300._lib import ptr, stream_ptr
    rng = np.random.default_rng(0)
    n = 10007
    p0, g = (torch.as_tensor(rng.standard_normal(n), dtype=torch.float32) for _ in range(2))
    m0 = torch.as_tensor(rng.standard_normal(n), dtype=torch.float32) * 0.1
    v0 = torch.as_tensor(rng.random(n), dtype=torch.float32) * 0.1
    p, m, v, gg = (t.clone().cuda() for t in (p0, m0, v0, g))
    step, lr, b1, b2, e = 7, 1e-3, 0.9, 0.999, 1e-8
    assert _lib.load().cev_adam_step(ptr(p), ptr(gg), ptr(m), ptr(v), n, lr, b1, b2, e, step,
                                     stream_ptr()) == 0
    mm = b1 * m0 + (1 - b1) * g
    vv = b2 * v0 + (1 - b2) * g * g
    ref = p0 - lr * (mm / (1 - b1 ** step)) / (torch.sqrt(vv / (1 - b2 ** step)) + e)
    assert torch.allclose(p.cpu(), ref, rtol=1e-5, atol=1e-7)
    # float32 (1 - beta) against float64 in the reference: a few ulp where the terms cancel
    assert torch.allclose(m.cpu(), mm, rtol=1e-5, atol=1e-7)
    assert torch.allclose(v.cpu(), vv, rtol=1e-5, atol=1e-7)


def _group(ids):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config4_problem
    pr = [config4_problem(i) for i in ids]
    om = np.array([q["omega"] for q in pr])
    pl = P.get_plan("ez", (256, 256), pr[0]["dL"], om, pr[0]["npml"])
    ep = torch.as_tensor(np.stack([q["eps"] for q in pr])).cuda()
    bb = torch.stack([torch.as_tensor(1j * q["omega"] * q["src"]) for q in pr]).cuda()
    return pl, ep, bb


def test_trained_network_gains_over_plain(cev):
    """Train on 64 config-4 problems (256x256, binary eps, lambda in
    [1.3, 1.8] um) from the plain solver's residuals, then compare on 8
    held-out problems at equal iteration counts."""
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.learned import LearnedPreconditioner, residual_samples
    iters = (0, 10, 30, 90, 270)
    samples = []
    for g0 in range(0, 64, 16):
        pl, ep, bb = _group(range(g0, g0 + 16))
        samples += [(pl, ep, r) for r in residual_samples(pl, ep, bb, iters=iters)]
    pl, ep, bb = _group(range(1000, 1008))
    held = residual_samples(pl, ep, bb, iters=(0, 30))
    untrained = LearnedPreconditioner(256, 256, max_batch=16, c0=32, seed=0)
    before = [float(untrained.loss_and_grad(pl, ep, r)[0]) for r in held]
    net = LearnedPreconditioner(256, 256, max_batch=16, c0=32, seed=0)
    net.fit(samples, steps=3000, lr=5e-4)
    after = [float(net.loss_and_grad(pl, ep, r)[0]) for r in held]
    assert after[0] < 0.2 * before[0] and after[1] < 0.9 * before[1], (before, after)

    def median_res(k, **kw):
        _, info = P.solve(pl, ep, bb, tol=1e-12, max_iters=k, max_stall=10 ** 6, **kw)
        return float(np.median([i["residual"] for i in info]))

    for k in (30, 90):
        plain = median_res(k)
        learned = median_res(k, precond="learned", learned=net)
        raw = median_res(k, precond="learned", learned=untrained)
        # measured: 0.20 vs 0.23 at 30 iterations after 3000 steps (0.14 vs 0.24 after 6000
        # steps on 128 problems); the gain is real but small
        assert learned < 0.95 * plain and learned < 0.5 * raw, (k, plain, learned, raw)


def test_invalid_uses_fail(cev):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300._lib import CevError
    from ceviche_gb300.learned import LearnedPreconditioner
    with pytest.raises(CevError):
        LearnedPreconditioner(36, 36, max_batch=1, c0=8)  # not divisible by 8
    net = LearnedPreconditioner(32, 32, max_batch=1, c0=8)
    eps = torch.ones(32, 32, dtype=torch.float64)
    b = torch.zeros(1, 32, 32, dtype=torch.complex128)
    b[0, 16, 16] = 1.0
    hz = P.get_plan("hz", (32, 32), 50e-9, [1.2e15], (4, 4))
    with pytest.raises(CevError):
        P.solve(hz, eps, b, precond="learned", learned=net)
    two = P.get_plan("ez", (32, 32), 50e-9, [1.2e15, 1.3e15], (4, 4))
    with pytest.raises(CevError):
        P.solve(two, eps, b.expand(2, 32, 32), precond="learned", learned=net)  # batch > max


def test_dropin_class_with_learned_preconditioner(cev):
    """fdfd_ez(..., precond="learned") with an untrained network: flexible
    GMRES stagnates and the solver falls back to plain GMRES from its iterate;
    the field and the eps-gradient (adjoint solve, same fallback) match the
    oracle's."""
    from ceviche_gb300.learned import LearnedPreconditioner
    rng = np.random.default_rng(11)
    nx, ny, npml, dL = 40, 32, 6, 40e-9
    omega = 2 * np.pi * 3e8 / 1.5e-6
    eps = rng.uniform(1, 4, (nx, ny))
    src = np.zeros((nx, ny))
    src[10, 12:20] = 1.0
    net = LearnedPreconditioner(nx, ny, max_batch=1, c0=8, seed=3)
    F = cev.fdfd_ez(omega, dL, torch.as_tensor(eps, device="cuda"), [npml, npml], tol=1e-10,
                    precond="learned", learned=net)
    e = torch.tensor(eps, device="cuda", requires_grad=True)
    F.eps_r = e
    _, _, ez = F.solve(torch.as_tensor(src, device="cuda"))
    A = ofd.make_A_ez(omega, dL, eps, [npml, npml])
    ref = ofd.spsolve(A, 1j * omega * src.ravel())
    assert np.linalg.norm(ez.detach().cpu().numpy().ravel() - ref) <= 1e-8 * np.linalg.norm(ref)
    probe = np.zeros((nx, ny))
    probe[30, 10:22] = 1.0
    J = (ez * torch.as_tensor(probe, device="cuda")).sum().abs() ** 2
    J.backward()
    s = np.sum(ref * probe.ravel())
    g_ez = 2 * np.conj(s) * probe  # dJ/dRe + i dJ/dIm of |sum(Ez * probe)|^2
    zeros = np.zeros((nx, ny))
    g_ref = ofd.grad_eps_ez(omega, dL, eps, [npml, npml], src, zeros, zeros, g_ez.conj())
    g = e.grad.cpu().numpy()
    assert np.linalg.norm(g - g_ref) <= 1e-6 * np.linalg.norm(g_ref), np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
