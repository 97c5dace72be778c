"""Observables on the GPU against the oracle: site densities and
Hellmann-Feynman derivatives (checked by central finite differences), the
entanglement entropy, the reference's Kubo Drude weight, and the
second-order flux response against a dense sum over states."""
import math

import numpy as np
import pytest

from conftest import philox_uniform

pytestmark = pytest.mark.gpu


def ground(ed, N, qu, qd, terms, U, steps=300, seed=1, dn_terms=None):
    op = ed.Hubbard(ed.H_TBq(N, qu).extend(terms), ed.H_TBq(N, qd).extend(dn_terms or terms), U)
    e0, v = ed.Lanczos().eigen(op, max_steps=steps, mode="fixed", seed=seed)
    return op, e0, v


def numpy_densities(orc, N, qu, qd, psi):
    su = orc.Tables(N, qu).state
    sd = orc.Tables(N, qd).state
    P = np.abs(psi.reshape(su.size, sd.size)) ** 2
    bu = (su[:, None] >> np.arange(N)) & 1
    bd = (sd[:, None] >> np.arange(N)) & 1
    return P.sum(1) @ bu, P.sum(0) @ bd, np.einsum("ud,ui,di->i", P, bu, bd)


def test_site_densities(ed, orc):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    op, e0, v = ground(ed, 12, 5, 4, L.kagome12(), 4.0)
    nu, nd, dd = ob.site_densities(op, v)
    ru, rd, rdd = numpy_densities(orc, 12, 5, 4, v)
    assert np.max(np.abs(nu - ru)) < 1e-12 and np.max(np.abs(nd - rd)) < 1e-12 and np.max(np.abs(dd - rdd)) < 1e-12
    assert abs(nu.sum() - 5) < 1e-12 and abs(nd.sum() - 4) < 1e-12


def test_hellmann_feynman_matches_finite_differences(ed):
    """dE0/dU = sum_i <n_up n_dn>, dE0/d eps_i = <n_i>, dE0/dt = <H_kin>/t on
    the disordered L=12 chain, against central differences (h = 1e-4)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    eps = list(philox_uniform(100, 12, 6.0))
    U, t, h = 1.0, -1.0, 1e-4

    def e0_of(U=U, t=t, eps=eps):
        terms = L.chain(12, periodic=False, t=t, eps=eps)
        return ground(ed, 12, 6, 6, terms, U, steps=300)[1]

    op, e0, v = ground(ed, 12, 6, 6, L.chain(12, periodic=False, eps=eps), U)
    nu, nd, dd = ob.site_densities(op, v)
    d_u = (e0_of(U=U + h) - e0_of(U=U - h)) / (2 * h)
    assert abs(dd.sum() - d_u) < 1e-6
    i = 5
    ep, em = list(eps), list(eps)
    ep[i] += h
    em[i] -= h
    d_eps = (e0_of(eps=ep) - e0_of(eps=em)) / (2 * h)
    assert abs(nu[i] + nd[i] - d_eps) < 1e-6
    kin = ed.Hubbard(ed.H_TBq(12, 6).extend(L.chain(12, periodic=False, t=t)),
                     ed.H_TBq(12, 6).extend(L.chain(12, periodic=False, t=t)), 0.0)
    d_t = (e0_of(t=t + h) - e0_of(t=t - h)) / (2 * h)
    assert abs(ob.expect(kin, v) / t - d_t) < 1e-6


def test_entanglement_entropy_device(ed, orc, golden_energies):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    g = golden_energies["chain8_pbc_q44_U4"]
    op = ed.Hubbard(ed.H_TBq(8, 4).extend(L.chain(8)), ed.H_TBq(8, 4).extend(L.chain(8)), 4.0)
    e0, v = ed.Lanczos().eigen(op, max_steps=100, mode="fixed", reorth=True, seed=0)
    s_vn, s_ref = ob.entanglement_entropy(op, v, [0, 1, 2, 3])
    assert abs(s_vn - g["EE_vN_A0123"]) < 1e-8
    assert abs(s_ref - g["EE_ref_A0123"]) < 1e-8 * abs(g["EE_ref_A0123"])
    # the same psi through the oracle's dense reshape + numpy SVD
    for qu, qd, sites in ((6, 6, range(6)), (8, 4, range(6)), (7, 5, (0, 2, 4, 6, 8, 10))):
        gg = golden_energies["chain12_open_W6_seed100_q66_U1"]
        terms = L.chain(12, periodic=False, eps=gg["eps"])
        op2, e2, v2 = ground(ed, 12, qu, qd, terms, 1.0)
        a, b = ob.entanglement_entropy(op2, v2, list(sites))
        ra, rb = orc.entanglement_entropy(v2, 12, qu, qd, list(sites))
        assert abs(a - ra) < 1e-10 and abs(b - rb) < 1e-9 * max(1.0, rb)


@pytest.mark.parametrize("qu,qd", [(0, 6), (12, 6), (6, 0), (0, 0), (1, 11), (12, 12)])
def test_observables_on_degenerate_sectors(ed, orc, golden_energies, qu, qd):
    """Ground states of sectors with an empty or a full spin species (one
    block of the entanglement reshape per species) and of the one-state
    sectors: entanglement entropies of sites 0..5 against the oracle's dense
    reshape + SVD, site densities against numpy."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    gg = golden_energies["chain12_open_W6_seed100_q66_U1"]
    terms = L.chain(12, periodic=False, eps=gg["eps"])
    op = ed.Hubbard(ed.H_TBq(12, qu).extend(terms), ed.H_TBq(12, qd).extend(terms), 1.0)
    e0, v = ed.Lanczos().eigen(op, max_steps=min(300, op.rows()), mode="fixed", seed=1)
    assert abs(np.linalg.norm(v) - 1.0) < 1e-12
    a, b = ob.entanglement_entropy(op, v, list(range(6)))
    ra, rb = orc.entanglement_entropy(v, 12, qu, qd, list(range(6)))
    assert abs(a - ra) < 1e-10 and abs(b - rb) < 1e-9 * max(1.0, abs(rb)), (a, ra, b, rb)
    nu, nd, dd = ob.site_densities(op, v)
    ru, rd, rdd = numpy_densities(orc, 12, qu, qd, v)
    assert np.max(np.abs(nu - ru)) < 1e-12 and np.max(np.abs(nd - rd)) < 1e-12 and np.max(np.abs(dd - rdd)) < 1e-12
    assert abs(nu.sum() - qu) < 1e-12 and abs(nd.sum() - qd) < 1e-12
    op.close()


def test_drude_kubo_matches_oracle(ed, orc):
    """The reference's drude_weight_Jx on Kagome12 3+3 (U=4): the device
    result equals the oracle's restatement (oracle Lanczos, continued
    fraction and sums) on the same ground state."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    N, q, U = 12, 3, 4.0
    vol = 8.0 * math.sqrt(3.0)
    H, e0, v = ground(ed, N, q, q, L.kagome12(), U)
    J = ed.Hubbard(ed.H_TBq(N, q).extend(L.kagome12_current_x()), ed.H_TBq(N, q).extend(L.kagome12_current_x()), 0.0)
    K = ed.Hubbard(ed.H_TBq(N, q).extend(L.kagome12_kinetic_x()), ed.H_TBq(N, q).extend(L.kagome12_kinetic_x()), 0.0)
    D, kin, vert, sigma = ob.drude_kubo(H, J, K, v, e0, vol, want_sigma=True)
    # oracle
    tH = orc.Tables(N, q, L.kagome12())
    tJ = orc.Tables(N, q, L.kagome12_current_x())
    tK = orc.Tables(N, q, L.kagome12_kinetic_x())
    phi = orc.matvec(tJ, tJ, 0.0, v)
    _, a, b, _ = orc.lanczos(tH, tH, U, phi, 200, mode="fixed", want_evec=False)
    w = 0.004 * np.arange(1, 8001) + 0.01j
    lam = orc.continued_fraction(a, b, float(phi @ phi), e0, w)
    sig = -lam.imag / (np.pi * w.real)
    vertex = float(np.sum(sig[w.real > 0.01]) * 0.004)
    kinetic = float(v @ orc.matvec(tK, tK, 0.0, v))
    Dref = (-kinetic - 2 * vertex) / vol
    assert abs(kin - kinetic) < 1e-12 * abs(kinetic)
    assert abs(vert - vertex) < 1e-8 * abs(vertex)
    assert abs(D - Dref) < 1e-8 * max(abs(Dref), 1e-3)
    # sigma(w) itself near its 1/delta-high peaks follows the exact pole
    # positions of a 200-step Lanczos without reorthogonalisation, which
    # (ghost copies included) move with last-bit rounding, and its running
    # integral (the spectral weight below w) moves by the weight of a pole
    # times its shift over delta near such a pole; held to 2e-3 of the total
    # weight at every w (observed: up to 3e-4 near the sharpest poles), while
    # the total (the Drude weight above) is held to 1e-8
    run = np.cumsum(sigma - sig) * 0.004
    assert np.max(np.abs(run)) < 2e-3 * np.sum(np.abs(sig)) * 0.004


def test_response_subspace_of_degenerate_level_vs_dense(ed, orc):
    """Kagome12 2+2 at zero twist has a three-fold ground level.  The device
    first- and second-order matrices over it (ed_response_subspace, given
    the dense ground states in a random unitary mix) against the dense
    degenerate perturbation theory: their eigenvalues (basis independent) to
    1e-8, and the flux sweep's lowest branch at Phi = 0 (which finds the
    multiplet with Lanczos runs from further start vectors) to 1e-8."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob, sweeps
    N, q, U = 12, 2, 4.0
    terms = L.kagome12(flux=0.0, peierls=True)
    d1t, d2t = L.kagome12_flux_derivatives(0.0)
    Hd = orc.hamiltonian(N, q, q, terms, terms, U).toarray()
    A1 = orc.hamiltonian(N, q, q, d1t, d1t, 0.0).toarray()
    A2 = orc.hamiltonian(N, q, q, d2t, d2t, 0.0).toarray()
    w, V = np.linalg.eigh(Hd)
    g = int(np.sum(w - w[0] < 1e-9))
    assert g == 3
    S = V[:, :g]
    D1 = S.conj().T @ A1 @ S
    C = V[:, g:].conj().T @ (A1 @ S)
    M = S.conj().T @ A2 @ S - 2 * (C.conj().T @ (C / (w[g:] - w[0])[:, None]))
    rng = np.random.default_rng(4)
    Uq, _ = np.linalg.qr(rng.standard_normal((g, g)) + 1j * rng.standard_normal((g, g)))
    psis = torch.from_numpy(np.ascontiguousarray((S @ Uq).T)).to("cuda")
    H = ed.Hubbard(ed.H_TBq(N, q).extend(terms), ed.H_TBq(N, q).extend(terms), U)
    dH = ed.Hubbard(ed.H_TBq(N, q).extend(d1t), ed.H_TBq(N, q).extend(d1t), 0.0)
    d2H = ed.Hubbard(ed.H_TBq(N, q).extend(d2t), ed.H_TBq(N, q).extend(d2t), 0.0)
    D1g, Mg = ob.response_subspace(H, dH, d2H, psis, float(w[0]), steps=200)
    assert np.allclose(np.linalg.eigvalsh(0.5 * (D1g + D1g.conj().T)), np.linalg.eigvalsh(0.5 * (D1 + D1.conj().T)),
                       atol=1e-9, rtol=0)
    assert np.allclose(np.linalg.eigvalsh(0.5 * (Mg + Mg.conj().T)), np.linalg.eigvalsh(0.5 * (M + M.conj().T)),
                       atol=1e-8, rtol=1e-8)
    d1_ref, d2_ref = ob.lowest_branch(D1, M)
    p = sweeps.flux_sweep([0.0], n_up=q, n_dn=q, U=U)[0]
    assert abs(p.e0 - w[0]) < 1e-10 * abs(w[0])
    assert abs(p.d1 - d1_ref) < 1e-9 and abs(p.d2 - d2_ref) < 1e-8 * max(1.0, abs(d2_ref))


@pytest.mark.parametrize("flux", [0.3, 1.1])
def test_flux_response_vs_dense_sum_over_states(ed, orc, flux):
    """dE0/dPhi and d2E0/dPhi2 from the device (Hellmann-Feynman + a
    200-step linear-response Lanczos) against the dense sum over states on
    Kagome12 2+2 with Peierls phases, and against central differences."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    N, q, U = 12, 2, 4.0
    terms = L.kagome12(flux=flux)
    d1t, d2t = L.kagome12_flux_derivatives(flux)
    H, e0, v = ground(ed, N, q, q, terms, U, steps=300)
    dH = ed.Hubbard(ed.H_TBq(N, q).extend(d1t), ed.H_TBq(N, q).extend(d1t), 0.0)
    d2H = ed.Hubbard(ed.H_TBq(N, q).extend(d2t), ed.H_TBq(N, q).extend(d2t), 0.0)
    first, second = ob.response(H, dH, d2H, v, e0, steps=200)
    Hd = orc.hamiltonian(N, q, q, terms, terms, U).toarray()
    w, V = np.linalg.eigh(Hd)
    assert w[1] - w[0] > 1e-6
    g = V[:, 0]
    A1 = orc.hamiltonian(N, q, q, d1t, d1t, 0.0).toarray()
    A2 = orc.hamiltonian(N, q, q, d2t, d2t, 0.0).toarray()
    m = V.conj().T @ (A1 @ g)
    exact1 = float(np.real(np.vdot(g, A1 @ g)))
    exact2 = float(np.real(np.vdot(g, A2 @ g)) - 2 * np.sum(np.abs(m[1:]) ** 2 / (w[1:] - w[0])))
    assert abs(first - exact1) < 1e-9 * max(1.0, abs(exact1))
    assert abs(second - exact2) < 1e-8 * max(1.0, abs(exact2))
    h = 1e-4
    ep = ground(ed, N, q, q, L.kagome12(flux=flux + h), U)[1]
    em = ground(ed, N, q, q, L.kagome12(flux=flux - h), U)[1]
    assert abs((ep - em) / (2 * h) - first) < 1e-6
    assert abs((ep - 2 * e0 + em) / h ** 2 - second) < 1e-4 * max(1.0, abs(second))


@pytest.mark.parametrize("qu,qd", [(0, 3), (12, 3)])
def test_flux_response_on_degenerate_sectors(ed, orc, qu, qd):
    """The flux response of Kagome12 sectors whose up species is empty or
    full (only the down electrons carry current) against the dense sum over
    states."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    N, U, flux = 12, 4.0, 0.3
    terms = L.kagome12(flux=flux)
    d1t, d2t = L.kagome12_flux_derivatives(flux)
    H, e0, v = ground(ed, N, qu, qd, terms, U, steps=220)
    dH = ed.Hubbard(ed.H_TBq(N, qu).extend(d1t), ed.H_TBq(N, qd).extend(d1t), 0.0)
    d2H = ed.Hubbard(ed.H_TBq(N, qu).extend(d2t), ed.H_TBq(N, qd).extend(d2t), 0.0)
    first, second = ob.response(H, dH, d2H, v, e0, steps=200)
    Hd = orc.hamiltonian(N, qu, qd, terms, terms, U).toarray()
    w, V = np.linalg.eigh(Hd)
    assert w[1] - w[0] > 1e-6
    g = V[:, 0]
    A1 = orc.hamiltonian(N, qu, qd, d1t, d1t, 0.0).toarray()
    A2 = orc.hamiltonian(N, qu, qd, d2t, d2t, 0.0).toarray()
    m = V.conj().T @ (A1 @ g)
    exact1 = float(np.real(np.vdot(g, A1 @ g)))
    exact2 = float(np.real(np.vdot(g, A2 @ g)) - 2 * np.sum(np.abs(m[1:]) ** 2 / (w[1:] - w[0])))
    assert abs(e0 - w[0]) < 1e-10 * max(1.0, abs(w[0]))
    assert abs(first - exact1) < 1e-9 * max(1.0, abs(exact1))
    assert abs(second - exact2) < 1e-8 * max(1.0, abs(exact2))


@pytest.mark.parametrize("qu,qd", [(0, 6), (6, 0), (12, 6), (6, 12)])
def test_s2_on_polarised_sectors(ed, qu, qd):
    """With one species empty or full every state of the sector has the
    largest spin, S = |N_up - N_dn| / 2 = 3: S^2 = 12 and S_xy = S^2 - S_z^2
    = 3 on any vector (S_xy x = 3 x)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    t = L.chain(12, periodic=False)
    op = ed.Hubbard(ed.H_TBq(12, qu).extend(t), ed.H_TBq(12, qd).extend(t), 2.0)
    x = philox_uniform(21, op.rows())
    x /= np.linalg.norm(x)
    y = ob.s2_apply(op, x)
    assert np.max(np.abs(y - 3.0 * x)) < 1e-13
    sxy, s2 = ob.s2_expect(op, x)
    assert abs(sxy - 3.0) < 1e-12 and abs(s2 - 12.0) < 1e-12
    op.close()


@pytest.mark.parametrize("case", ["chain8_35", "kagome12_54", "kagome12_22_flux"])
def test_s2_apply_matches_oracle(ed, orc, case):
    """ed_s2_apply (TotalSpin::Hubbard::Hubbard_mv) against the restated
    S_xy on random vectors, real and complex (Peierls) operators, 1e-14 of
    the vector norms."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    N, qu, qd, t = {"chain8_35": (8, 3, 5, L.chain(8)), "kagome12_54": (12, 5, 4, L.kagome12()),
                    "kagome12_22_flux": (12, 2, 2, L.kagome12(flux=0.4))}[case]
    op = ed.Hubbard(ed.H_TBq(N, qu).extend(t), ed.H_TBq(N, qd).extend(t), 2.0)
    up, dn = orc.Tables(N, qu), orc.Tables(N, qd)
    rng = np.random.default_rng(7)
    n = op.rows()
    x = rng.standard_normal(n) + (1j * rng.standard_normal(n) if op.is_complex else 0)
    y = ob.s2_apply(op, x)
    ref = orc.sxy_matvec(up, dn, x.real) + (1j * orc.sxy_matvec(up, dn, x.imag) if op.is_complex else 0)
    assert np.linalg.norm(y - ref) < 1e-14 * np.linalg.norm(x) * 4


def test_s2_of_ground_states(ed):
    """Total spin of Lanczos ground states (ConservedTotalSpin_Kagome_
    randomHop.cu:113-116): the half-filled L=8 Hubbard ring is a singlet;
    Kagome12 5+4 has S^2 = S(S+1) with S half-integer >= 1/2."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    op = ed.Hubbard(ed.H_TBq(8, 4).extend(L.chain(8)), ed.H_TBq(8, 4).extend(L.chain(8)), 4.0)
    e0, v = ed.Lanczos().eigen(op, max_steps=100, mode="fixed", reorth=True, seed=0)
    sxy, s2 = ob.s2_expect(op, v)
    assert abs(s2) < 1e-9 and abs(sxy - s2) < 1e-15
    op2 = ed.Hubbard(ed.H_TBq(12, 5).extend(L.kagome12()), ed.H_TBq(12, 4).extend(L.kagome12()), 4.0)
    e0, v = ed.Lanczos().eigen(op2, max_steps=300, mode="fixed", reorth=True, seed=0)
    sxy, s2 = ob.s2_expect(op2, v)
    S = (-1 + math.sqrt(1 + 4 * s2)) / 2
    assert abs(s2 - (0.25 + sxy)) < 1e-14
    assert abs(2 * S - round(2 * S)) < 1e-6 and round(2 * S) % 2 == 1


def test_entanglement_cluster_bidiag_matches_gesvd(ed, monkeypatch):
    """The cluster Householder bidiagonalisation + host bidiagonal SVD
    against cusolverDnDgesvd for every block (ED_EE_METHOD=gesvd), on the
    open L=12 (6,6) and (7,5) ground states (blocks up to 400 x 400) and a
    random vector (no small singular values)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import observables as ob, sweeps
    eu, edn = sweeps.mbl_disorder(2, 12, 6.0)
    for qu, qd in ((6, 6), (7, 5)):
        op = ed.Hubbard(ed.H_TBq(12, qu).extend(sweeps.mbl_chain_terms(eu)),
                        ed.H_TBq(12, qd).extend(sweeps.mbl_chain_terms(edn)), 1.0)
        e0, v = ed.Lanczos().eigen(op, max_steps=300, mode="fixed", seed=1)
        x = ed.Lanczos().random_vector(op.rows(), 5)
        x = x / np.linalg.norm(x)
        for psi, sites in ((v, range(6)), (v, (0, 2, 4, 6, 8, 10)), (x, range(6))):
            monkeypatch.delenv("ED_EE_METHOD", raising=False)
            a = ob.entanglement_entropy(op, psi, list(sites))
            monkeypatch.setenv("ED_EE_METHOD", "gesvd")
            b = ob.entanglement_entropy(op, psi, list(sites))
            assert abs(a[0] - b[0]) < 1e-12 and abs(a[1] - b[1]) < 1e-10 * max(1.0, b[1])


@pytest.mark.parametrize("method", ["bidiag", "gesvd"])
def test_entanglement_entropy_batch_matches_single(ed, monkeypatch, method):
    """ed_entanglement_entropy_batch: every state's entropies equal its own
    single-state call bit for bit (cluster bidiagonalisation and the gesvd
    path), on the (6,6) and (8,4) sectors of the L=12 chain."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, observables as ob
    if method == "gesvd":
        monkeypatch.setenv("ED_EE_METHOD", "gesvd")
    eps = list(philox_uniform(100, 12, 6.0))
    terms = L.chain(12, periodic=False, eps=eps)
    for qu, qd in ((6, 6), (8, 4)):
        op = ed.Hubbard(ed.H_TBq(12, qu).extend(terms), ed.H_TBq(12, qd).extend(terms), 1.0)
        g = torch.Generator(device="cuda").manual_seed(qu)
        psis = torch.empty((3, op.rows()), dtype=torch.float64, device="cuda").uniform_(-1.0, 1.0, generator=g)
        psis /= psis.norm(dim=1, keepdim=True)
        svn, sref = ob.entanglement_entropy_batch(op, psis, range(6))
        for b in range(3):
            s1, r1 = ob.entanglement_entropy(op, psis[b], range(6))
            assert svn[b] == s1 and sref[b] == r1, (qu, qd, b)
        h_svn, _ = ob.entanglement_entropy_batch(op, psis.cpu().numpy(), range(6))
        assert np.array_equal(h_svn, svn)
        op.close()


def test_entropy_gesvd_pool_is_repeatable(ed, monkeypatch):
    """The cuSOLVER fallback of the entanglement entropy on eight worker
    streams (ED_EE_METHOD=gesvd, ED_EE_STREAMS=8), twenty calls on the C4
    (6,6) ground state: bit-identical entropies every time, and equal to
    the cluster bidiagonalisation's to 1e-10."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import observables as ob, sweeps
    eu, edn = sweeps.mbl_disorder(0, 12, 6.0)
    op = ed.Hubbard(ed.H_TBq(12, 6).extend(sweeps.mbl_chain_terms(eu)),
                    ed.H_TBq(12, 6).extend(sweeps.mbl_chain_terms(edn)), 1.0)
    psi = torch.empty(op.rows(), dtype=torch.float64, device="cuda")
    ed.Lanczos().eigen(op, max_steps=300, mode="fixed", seed=0, evec_out=psi)
    a_sites = list(range(6))
    ref = ob.entanglement_entropy(op, psi, a_sites)
    monkeypatch.setenv("ED_EE_METHOD", "gesvd")
    monkeypatch.setenv("ED_EE_STREAMS", "8")
    first = ob.entanglement_entropy(op, psi, a_sites)
    for _ in range(19):
        assert ob.entanglement_entropy(op, psi, a_sites) == first
    assert abs(first[0] - ref[0]) < 1e-10 and abs(first[1] - ref[1]) < 1e-10 * max(1.0, ref[1])
    op.close()
