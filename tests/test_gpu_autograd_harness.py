"""The adjoint behind torch.autograd (check harness only, tests/harness_autograd.py):
gradients of E0 in (t, U, eps_i) by Hellmann-Feynman against torch's central
finite differences (gradcheck, h = 1e-4, |error| < 1e-6), and the flux
curvature by a double backward through the linear-response solve against
central differences (first 1e-6, second 1e-4 relative: the round-off bound of
a second difference at h = 1e-4)."""
import pytest
import torch

from conftest import philox_uniform
from harness_autograd import ChainCfg, ChainEnergy, FluxCfg, FluxEnergy, flux_point

pytestmark = pytest.mark.gpu


def test_chain_energy_gradcheck(ed):
    cfg = ChainCfg()
    eps = philox_uniform(100, cfg.L, 6.0)
    theta = torch.tensor([-1.0, 1.0, *eps], dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda th: ChainEnergy.apply(th, cfg), (theta,), eps=1e-4, atol=1e-6,
                                    rtol=1e-6, raise_exception=True)
    # through a torch expression: d/dtheta (E0 - c)^2 = 2 (E0 - c) dE0/dtheta
    E = ChainEnergy.apply(theta, cfg)
    c = -5.0
    ((E - c) ** 2).backward()
    g = theta.grad.clone()
    theta.grad = None
    ChainEnergy.apply(theta, cfg).backward()
    assert torch.allclose(g, 2 * (E.detach() - c) * theta.grad, rtol=1e-14, atol=0)


@pytest.mark.parametrize("phi", [0.3, 1.1])
def test_flux_energy_double_backward(ed, phi):
    cfg = FluxCfg()
    p = torch.tensor(phi, dtype=torch.float64, requires_grad=True)
    E = FluxEnergy.apply(p, cfg)
    (g,) = torch.autograd.grad(E, p, create_graph=True)
    (g2,) = torch.autograd.grad(g, p)
    e0, d1, d2 = flux_point(phi, cfg)
    assert E.item() == e0 and g.item() == d1 and g2.item() == d2
    h = 1e-4
    ep = FluxEnergy.apply(torch.tensor(phi + h, dtype=torch.float64), cfg).item()
    em = FluxEnergy.apply(torch.tensor(phi - h, dtype=torch.float64), cfg).item()
    assert abs((ep - em) / (2 * h) - d1) < 1e-6
    assert abs((ep - 2 * e0 + em) / h ** 2 - d2) < 1e-4 * max(1.0, abs(d2))
