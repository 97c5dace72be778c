"""Host logic of the parameter sweeps (no GPU): disorder keying, lattice
terms, row layout, the twist grid."""
import math

import numpy as np

from conftest import philox_uniform


def test_mbl_disorder_is_keyed_by_realisation(edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    eu, ed = sweeps.mbl_disorder(3, 12, 6.0, seed=0)
    x = philox_uniform(3, 24, 6.0)
    assert np.array_equal(eu, x[:12]) and np.array_equal(ed, x[12:])
    assert np.max(np.abs(np.concatenate([eu, ed]))) <= 6.0
    assert not np.array_equal(eu, sweeps.mbl_disorder(4, 12, 6.0)[0])
    assert np.array_equal(sweeps.mbl_disorder(3, 12, 6.0, seed=2)[0],
                          philox_uniform(2 * (1 << 20) + 3, 24, 6.0)[:12])


def test_mbl_chain_terms_follow_line16():
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    eps = np.arange(12) * 0.5 - 3
    terms = sweeps.mbl_chain_terms(eps)
    hops = [t for t in terms if t[0] == "H"]
    site = [t for t in terms if t[0] == "N"]
    assert [(t[1], t[2], t[3]) for t in hops] == [(i, i + 1, -1.0) for i in range(11)]
    assert [(t[1], t[3]) for t in site] == [(i, eps[i]) for i in range(12)]


def test_flux_grid_and_rows():
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, sweeps
    phis = sweeps.flux_phis(16)
    assert phis.size == 16 and phis[0] == 0.0 and abs(phis[-1] - 2 * math.pi / L.KAGOME12_LX) < 1e-15
    terms = L.kagome12(flux=0.0, peierls=True)
    assert sum(t[0] == "P" for t in terms) == 24 and all(t[4] == 0.0 for t in terms if t[0] == "P")
    pts = [sweeps.MblPoint(2, (7, 5), -1.5, 0.3, 0.4, np.arange(3.0), np.arange(3.0) + 10, 300)]
    pts[0].min_bits = 51
    rows = sweeps.mbl_rows(pts)
    assert rows[0][:11] == (2, 7, 5, -1.5, 0.3, 0.0, 1.0, 2.0, 10.0, 11.0, 12.0)
    assert rows[0][11] == 51 and math.isnan(rows[0][12])
    fp = [sweeps.FluxPoint(0.1, -2.0, 0.5, 1.5, 300, 52)]
    assert sweeps.flux_rows(fp)[0][:5] == (0.1, -2.0, 0.5, 1.5, 52)
    # errors against an oracle table are attached by key, the largest returned
    assert sweeps.attach_oracle(fp, {0.1: -2.0 + 3e-12}) == abs(-2.0 - (-2.0 + 3e-12))
    assert sweeps.flux_rows(fp)[0][5] == fp[0].err_vs_oracle
    assert sweeps.attach_oracle(pts, {(2, (7, 5)): -1.5}) == 0.0
    assert math.isnan(sweeps.attach_oracle(pts, {(3, (7, 5)): -1.5}))
