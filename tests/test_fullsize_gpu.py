"""Full-size parity of the two configurations whose GPU paths were
otherwise checked only at small sizes.

* FDTD reverse-time adjoint at 400x400, 4000 steps, checkpoints every 64
  steps (the adjoint FDTD workload): the float64 adjoint gradient of a probe
  objective L = sum_t sum_p w[t, p] Ez_t(p) against central differences
  (h = 1e-4) of the float64 forward at three pixels (relative 1e-5), and the
  float32 gradient against the float64 one (relative L2 5e-3 over the grid).
  This replaces the autograd tape over ceviche/fdtd.py:74-144 that the
  reference's tests/test_gradients_fdtd.py:66-165 differentiate.
* FDFD 2048x2048 with 16 omegas (the large-scale workload), Ez and Hz, solved
  with the nested-dissection direct preconditioner to 1e-6: every problem
  reports convergence, and the FP64 residual ||A x - b|| / ||b|| of four
  returned fields is recomputed on the host with the oracle's assembled
  matrix (ceviche/fdfd.py:172-233) and must be <= 1.2e-6.
"""
import numpy as np
import pytest
import torch

from oracle import fdfd as ofd

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cev():
    import ceviche_gb300
    from ceviche_gb300 import build
    build.build()
    return ceviche_gb300


def _rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_fdtd_adjoint_400x400_4000_steps(cev):
    from ceviche_gb300.workloads import config2
    p = config2(steps=4000)
    probes = [(300, 200), (200, 300), (120, 120)]
    rng = np.random.default_rng(33)
    w = rng.standard_normal((4000, len(probes)))
    wt = {}

    def loss(eps_t, precision):
        series = cev.fdtd_probe_series(eps_t, p["dL"], p["npml"], 4000, p["src"], p["amps"],
                                       probes, precision=precision, ckpt_every=64)
        key = str(series.dtype)
        if key not in wt:
            wt[key] = torch.as_tensor(w, dtype=series.dtype, device=series.device)
        return (series * wt[key]).sum()

    grads = {}
    for precision in ("float64", "float32"):
        eps = torch.tensor(p["eps"], device="cuda", requires_grad=True)
        loss(eps, precision).backward()
        grads[precision] = eps.grad.detach().cpu().numpy()
    g64 = grads["float64"]
    h = 1e-4
    for (i, j) in [(250, 200), (210, 205), (200, 260)]:
        vals = []
        for s in (+1, -1):
            e = p["eps"].copy()
            e[i, j] += s * h
            with torch.no_grad():
                vals.append(float(loss(torch.as_tensor(e, device="cuda"), "float64")))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(g64[i, j] - fd) <= 1e-5 * max(abs(fd), 1e-12 * np.abs(g64).max()), (i, j, g64[i, j], fd)
    assert _rel(grads["float32"], g64) < 5e-3


@pytest.mark.parametrize("pol", ["ez", "hz"])
def test_config5_direct_solve_residual_on_host(cev, pol):
    from ceviche_gb300 import primitives as P
    from ceviche_gb300.workloads import config5
    q = config5()
    n = q["eps"].shape[0]
    plan = P.Plan(pol, (n, n), q["dL"], q["omegas"], q["npml"])
    eps = torch.as_tensor(q["eps"], device="cuda")
    b = np.stack([1j * w * q["src"] for w in q["omegas"]])
    x, info = P.solve(plan, eps, torch.as_tensor(b, device="cuda"), precond="direct", tol=1e-6,
                      strict=True)
    assert all(r["code"] == 0 and r["residual"] <= 1e-6 for r in info)
    for k in (0, 5, 10, 15):
        A = ofd.make_A(pol, q["omegas"][k], q["dL"], q["eps"], q["npml"])
        xk = x[k].cpu().numpy().ravel()
        r = np.linalg.norm(A @ xk - b[k].ravel()) / np.linalg.norm(b[k])
        assert r <= 1.2e-6, (k, r)
