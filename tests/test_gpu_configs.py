"""The headline configurations at their own sizes.

C3: Kagome12 6+6, U=4, with the twist phase Phi * dx_b on every bond
(complex FP64, dim 853,776), at three of the sixteen sweep twists
Phi_k = (2 pi / 4) k / 15, against the CPU fixtures of
tests/golden/flux_kagome12_q66_U4.json (scipy eigsh of the oracle's
Kronecker-sum Hamiltonian and a projected conjugate-gradient solve of the
response equation): E0 to 1e-10 relative, dE0/dPhi and d2E0/dPhi2 to 1e-8.

C5: Lieb18 9+9, U=4 (dim 2,363,904,400, 18.9 GB per vector), 150 fixed
Lanczos steps with the Ritz vector regenerated by a second recurrence, from
two start vectors: the two E0 agree to 1e-10 relative, and each Ritz pair's
residual |H psi - E0 psi| is below 1e-7 (with the spectral gap above it, the
eigenvalue error is then of order residual^2 / gap).
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FLUX = json.loads((GOLDEN / "flux_kagome12_q66_U4.json").read_text())


@pytest.mark.parametrize("point", FLUX["points"], ids=[f"k{p['k']}" for p in FLUX["points"]])
def test_c3_flux_point_matches_cpu_fixture(ed, point):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    p = sweeps.flux_sweep([point["phi"]], steps=sweeps.FLUX_STEPS, response_steps=sweeps.FLUX_RESPONSE_STEPS)[0]
    assert abs(p.e0 - point["E0"]) < 1e-10 * abs(point["E0"]), p.e0 - point["E0"]
    assert abs(p.d1 - point["dE0_dphi"]) < 1e-8 * max(1.0, abs(point["dE0_dphi"])), p.d1 - point["dE0_dphi"]
    assert abs(p.d2 - point["d2E0_dphi2"]) < 1e-8 * max(1.0, abs(point["d2E0_dphi2"])), p.d2 - point["d2E0_dphi2"]
    assert p.min_bits >= 48


def test_c5_lieb18_two_seeds_agree(ed):
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    t = L.lieb18()
    op = ed.Hubbard(ed.H_TBq(18, 9).extend(t), ed.H_TBq(18, 9).extend(t), 4.0)
    assert op.matvec_kind == "two_pass"
    D = op.rows()
    e0s = []
    for seed in (0, 1):
        ev = torch.empty(D, dtype=torch.float64, device="cuda")
        lz = ed.Lanczos()
        e0, _ = lz.eigen(op, max_steps=150, mode="fixed", ritz="recompute", seed=seed, evec_out=ev)
        y = torch.empty_like(ev)
        op.Hubbard_mv(ev, y)
        torch.cuda.synchronize()
        y.sub_(ev, alpha=e0)
        res = float(torch.linalg.vector_norm(y))
        assert abs(float(torch.linalg.vector_norm(ev)) - 1.0) < 1e-12
        assert res < 1e-7, res
        assert lz.result.min_bits >= 48
        e0s.append(e0)
        del y, ev
        torch.cuda.empty_cache()
    assert abs(e0s[0] - e0s[1]) < 1e-10 * abs(e0s[0]), e0s
    op.close()
