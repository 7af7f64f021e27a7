"""Multi-frequency FDFD (fdfd_mf_ez, ceviche/fdfd.py:247-359) on the GPU
against fixtures from the reference: the coupled operator (1e-13 relative),
solved fields (1e-6 at tol 1e-10) and gradients w.r.t. eps, delta and phi
against the reference's central differences (1e-5 relative)."""
import os

import numpy as np
import pytest
import torch

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def fx():
    from ceviche_gb300 import build
    build.build()
    d = np.load(os.path.join(GOLDEN, "fdfd_mf.npz"))
    Nsb, nfreq, omega, omega_mod, dL, px, py = d["meta"]
    return d, int(Nsb), omega, omega_mod, dL, [int(px), int(py)]


def test_mf_operator(fx):
    from ceviche_gb300 import primitives as P
    d, Nsb, omega, omega_mod, dL, npml = fx
    Nx, Ny = d["eps"].shape
    plan = P.get_mf_plan((Nx, Ny), dL, omega, omega_mod, Nsb, npml)
    cpl = torch.as_tensor(d["delta"] * np.exp(1j * d["phi"]))
    x = torch.as_tensor(d["x"].reshape(2 * Nsb + 1, Nx, Ny))
    eps = torch.as_tensor(d["eps"])
    for tr, key in ((False, "Ax"), (True, "ATx")):
        y = P.mf_apply(plan, eps, cpl, x, transpose=tr).cpu().numpy()
        assert _rel(y, d[key]) < 1e-13


def test_mf_fields(fx):
    import ceviche_gb300 as cev
    d, Nsb, omega, omega_mod, dL, npml = fx
    F = cev.fdfd_mf_ez(omega, dL, d["eps"], omega_mod, d["delta"], d["phi"], Nsb, npml, tol=1e-10)
    out = F.solve(d["src"])
    for got, ref in zip(out, d["fields"]):
        assert got.shape == ref.shape
        assert _rel(got, ref) < 1e-6


def test_mf_gradients(fx):
    import ceviche_gb300 as cev
    d, Nsb, omega, omega_mod, dL, npml = fx
    eps = torch.tensor(d["eps"], device="cuda", requires_grad=True)
    delta = torch.tensor(d["delta"], device="cuda", requires_grad=True)
    phi = torch.tensor(d["phi"], device="cuda", requires_grad=True)
    F = cev.fdfd_mf_ez(omega, dL, eps, omega_mod, delta, phi, Nsb, npml, tol=1e-11)
    hx, hy, ez = F.solve(torch.as_tensor(d["src"], device="cuda"))
    J = (ez.abs() ** 2).sum() + (hx.abs() ** 2).sum() + 0.5 * (hy.abs() ** 2).sum()
    J.backward()
    pix = d["pix"]
    assert abs(J.item() - float(d["J"])) / float(d["J"]) < 1e-8
    assert _rel(eps.grad.cpu().numpy().ravel()[pix], d["grad_eps"]) < 1e-5
    assert _rel(delta.grad[1].cpu().numpy().ravel()[pix], d["grad_delta1"]) < 1e-5
    assert _rel(phi.grad[0].cpu().numpy().ravel()[pix], d["grad_phi0"]) < 1e-5
