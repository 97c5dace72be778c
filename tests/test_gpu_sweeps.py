"""Parameter sweeps on the GPU against dense diagonalisation by the oracle:
disorder sweep (E0, entanglement entropy, dE0/d eps_{i,s}) on an open L=8
chain with spin-dependent disorder, twist sweep (E0, dE0/dPhi, d2E0/dPhi2)
on Kagome12 2+2."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dense_ground(orc, N, qu, qd, tu, td, U):
    H = orc.hamiltonian(N, qu, qd, tu, td, U).toarray()
    w, V = np.linalg.eigh(H)
    assert w[1] - w[0] > 1e-6
    return w, V


def test_mbl_sweep_matches_dense(ed, orc):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    N, U, W = 8, 1.0, 6.0
    sectors = ((4, 4), (5, 3))
    tm = sweeps.SweepTiming()
    pts = sweeps.mbl_sweep(realisations=(0, 5), sectors=sectors, n_sites=N, W=W, U=U, steps=200, timing=tm)
    assert len(pts) == 4 and tm.instances == 4 and tm.lanczos_steps == 800
    for p in pts:
        eu, edn = sweeps.mbl_disorder(p.realisation, N, W)
        qu, qd = p.sector
        w, V = dense_ground(orc, N, qu, qd, sweeps.mbl_chain_terms(eu), sweeps.mbl_chain_terms(edn), U)
        g = V[:, 0]
        assert abs(p.e0 - w[0]) < 1e-10 * max(1.0, abs(w[0]))
        su, sd = orc.Tables(N, qu).state, orc.Tables(N, qd).state
        P = (g * g).reshape(su.size, sd.size)
        nu = P.sum(1) @ ((su[:, None] >> np.arange(N)) & 1)
        nd = P.sum(0) @ ((sd[:, None] >> np.arange(N)) & 1)
        assert np.max(np.abs(p.n_up - nu)) < 1e-8 and np.max(np.abs(p.n_dn - nd)) < 1e-8
        svn, sref = orc.entanglement_entropy(g, N, qu, qd, list(range(N // 2)))
        assert abs(p.s_vn - svn) < 1e-8 and abs(p.s_ref - sref) < 1e-7 * max(1.0, sref)


def test_flux_sweep_matches_dense(ed, orc):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, sweeps
    N, q, U = 12, 2, 4.0
    phis = (0.3, 0.6)  # 2+2 at zero twist is triply degenerate
    pts = sweeps.flux_sweep(phis, n_up=q, n_dn=q, U=U, steps=300, response_steps=200)
    for p, phi in zip(pts, phis):
        terms = L.kagome12(flux=phi, peierls=True)
        d1t, d2t = L.kagome12_flux_derivatives(phi)
        w, V = dense_ground(orc, N, q, q, terms, terms, U)
        g = V[:, 0]
        A1 = orc.hamiltonian(N, q, q, d1t, d1t, 0.0).toarray()
        A2 = orc.hamiltonian(N, q, q, d2t, d2t, 0.0).toarray()
        m = V.conj().T @ (A1 @ g)
        exact1 = float(np.real(np.vdot(g, A1 @ g)))
        exact2 = float(np.real(np.vdot(g, A2 @ g)) - 2 * np.sum(np.abs(m[1:]) ** 2 / (w[1:] - w[0])))
        assert abs(p.e0 - w[0]) < 1e-10 * abs(w[0])
        assert abs(p.d1 - exact1) < 1e-9 * max(1.0, abs(exact1))
        assert abs(p.d2 - exact2) < 1e-8 * max(1.0, abs(exact2))


def test_mbl_sweep_batched_equals_unbatched(ed):
    """The disorder sweep with its realisations batched per sector
    (ed_lanczos_batch) returns the unbatched sweep's E0, entropies and
    densities exactly (same start vectors, bit-identical coefficients)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    kw = dict(realisations=range(5), sectors=((6, 6), (8, 4)), steps=80)
    a = sweeps.mbl_sweep(**kw)
    b = sweeps.mbl_sweep(batch=3, **kw)
    assert [(p.realisation, p.sector) for p in a] == [(p.realisation, p.sector) for p in b]
    for p, q in zip(a, b):
        assert p.e0 == q.e0 and p.s_vn == q.s_vn and p.s_ref == q.s_ref
        assert np.array_equal(p.n_up, q.n_up) and np.array_equal(p.n_dn, q.n_dn)
