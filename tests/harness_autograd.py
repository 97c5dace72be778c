"""torch.autograd wrappers around the library's adjoint — check harness only
(the product exposes the derivatives through the C ABI; nothing in the
package imports torch.autograd).

ChainEnergy: E0 of an open Hubbard chain as a function of
theta = (t, U, eps_0 .. eps_{L-1}) (the MBL driver's Line chains,
Hubbard_EE_test.cu:102-140, with one on-site list for both spins).  Forward:
a fixed-step device Lanczos ground state.  Backward: Hellmann-Feynman
contractions on the device -- dE0/dU = sum_i <n_i,up n_i,dn> and
dE0/d eps_i = <n_i,up + n_i,dn> (ed_site_densities), dE0/dt = <H_kin>/t
(ed_op_expect on the hopping-only operator).

FluxEnergy: E0 of the twisted Kagome12 cluster as a function of the flux Phi
(Peierls phase Phi dx_b on every bond).  Its backward is dE0/dPhi through
FluxSlope, whose forward is the Hellmann-Feynman <dH/dPhi> and whose own
backward is d2E0/dPhi2 from the linear-response solve (ed_response), so a
double backward gives the Drude curvature.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch


def _pkg():
    import exact_diagonalization_for_fermionic_systems_with_gpu_gb300 as ed
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import observables as ob
    return ed, L, ob


@dataclass(frozen=True)
class ChainCfg:
    L: int = 10
    q_up: int = 5
    q_dn: int = 5
    steps: int = 300
    seed: int = 1


def _chain_ground(theta, cfg: ChainCfg):
    ed, L, _ = _pkg()
    t, U = float(theta[0]), float(theta[1])
    eps = [float(v) for v in theta[2:]]
    terms = L.chain(cfg.L, t=t, periodic=False, eps=eps)
    H = ed.Hubbard(ed.H_TBq(cfg.L, cfg.q_up).extend(terms), ed.H_TBq(cfg.L, cfg.q_dn).extend(terms), U)
    e0, v = ed.Lanczos().eigen(H, max_steps=cfg.steps, mode="fixed", seed=cfg.seed)
    return H, e0, v


class ChainEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, cfg: ChainCfg):
        if theta.numel() != 2 + cfg.L:
            raise ValueError("theta = (t, U, eps_0 .. eps_{L-1})")
        th = theta.detach().cpu().double().numpy()
        H, e0, v = _chain_ground(th, cfg)
        ed, L, ob = _pkg()
        nu, nd, dd = ob.site_densities(H, v)
        t = float(th[0])
        kin_terms = L.chain(cfg.L, t=t, periodic=False)
        K = ed.Hubbard(ed.H_TBq(cfg.L, cfg.q_up).extend(kin_terms), ed.H_TBq(cfg.L, cfg.q_dn).extend(kin_terms), 0.0)
        grad = torch.empty_like(theta.detach().double())
        grad[0] = ob.expect(K, v) / t
        grad[1] = float(dd.sum())
        grad[2:] = torch.from_numpy(nu + nd)
        K.close()
        H.close()
        ctx.save_for_backward(grad.to(theta.device, theta.dtype))
        return theta.new_tensor(e0)

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None


@dataclass(frozen=True)
class FluxCfg:
    q_up: int = 2
    q_dn: int = 2
    U: float = 4.0
    steps: int = 300
    response_steps: int = 200
    seed: int = 1


def _flux_ops(phi: float, cfg: FluxCfg):
    ed, L, _ = _pkg()
    terms = L.kagome12(flux=phi, peierls=True)
    d1t, d2t = L.kagome12_flux_derivatives(phi)
    H = ed.Hubbard(ed.H_TBq(12, cfg.q_up).extend(terms), ed.H_TBq(12, cfg.q_dn).extend(terms), cfg.U)
    dH = ed.Hubbard(ed.H_TBq(12, cfg.q_up).extend(d1t), ed.H_TBq(12, cfg.q_dn).extend(d1t), 0.0)
    d2H = ed.Hubbard(ed.H_TBq(12, cfg.q_up).extend(d2t), ed.H_TBq(12, cfg.q_dn).extend(d2t), 0.0)
    return H, dH, d2H


def flux_point(phi: float, cfg: FluxCfg):
    """(E0, dE0/dPhi, d2E0/dPhi2) from one ground state and the adjoint."""
    ed, _, ob = _pkg()
    H, dH, d2H = _flux_ops(phi, cfg)
    e0, v = ed.Lanczos().eigen(H, max_steps=cfg.steps, mode="fixed", seed=cfg.seed)
    d1, d2 = ob.response(H, dH, d2H, v, e0, steps=cfg.response_steps)
    for op in (H, dH, d2H):
        op.close()
    return e0, d1, d2


class FluxSlope(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phi, cfg: FluxCfg):
        _, d1, d2 = flux_point(float(phi), cfg)
        ctx.save_for_backward(phi.new_tensor(d2))
        return phi.new_tensor(d1)

    @staticmethod
    def backward(ctx, g):
        (d2,) = ctx.saved_tensors
        return g * d2, None


class FluxEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phi, cfg: FluxCfg):
        ed, L, _ = _pkg()
        terms = L.kagome12(flux=float(phi), peierls=True)
        H = ed.Hubbard(ed.H_TBq(12, cfg.q_up).extend(terms), ed.H_TBq(12, cfg.q_dn).extend(terms), cfg.U)
        e0, _ = ed.Lanczos().eigen(H, max_steps=cfg.steps, mode="fixed", ritz="none", seed=cfg.seed)
        H.close()
        ctx.save_for_backward(phi)
        ctx.cfg = cfg
        return phi.new_tensor(e0)

    @staticmethod
    def backward(ctx, g):
        (phi,) = ctx.saved_tensors
        return g * FluxSlope.apply(phi, ctx.cfg), None
