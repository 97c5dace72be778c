"""The CPU oracle pinned against the reference's own tables and known answers.

The fixtures in tests/golden/ were produced by compiling the reference's
MBL_test/include/fermi_operator.h (oracle/Makefile `ref`) and by dense /
scipy eigensolves on those tables (tests/golden/make_golden.py).
"""
import hashlib
import math

import numpy as np
import pytest

from conftest import philox_uniform, rel_err

DENSE_E0_CHAIN8 = -4.603526299989137  # dense eigvalsh on the reference tables, L=8 PBC 4+4 U=4


def _digest(state, ax, aj):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(state, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(ax, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(aj, dtype=np.int64).tobytes())
    return h.hexdigest()


def test_oracle_tables_bit_exact_small(orc, golden_tables):
    meta, arrays = golden_tables
    for name, m in meta["small"].items():
        t = orc.Tables(m["N"], m["Q"], [tuple(x) for x in m["terms"]])
        assert not t.overflow
        assert np.array_equal(t.state, arrays[f"{name}__state"]), name
        assert np.array_equal(t.Ax, arrays[f"{name}__ax"]), name
        assert np.array_equal(t.Aj, arrays[f"{name}__aj"].astype(np.int64)), name


def test_oracle_tables_digest_large(orc, golden_tables):
    meta, _ = golden_tables
    for name, m in meta["large"].items():
        t = orc.Tables(m["N"], m["Q"], [tuple(x) for x in m["terms"]])
        assert t.count == m["count"]
        assert _digest(t.state, t.Ax, t.Aj) == m["sha256"], name


def test_oracle_live_against_reference_build(orc):
    """When the reference's table builder is built here, compare random
    term lists live (skipped where the reference checkout is absent)."""
    if not orc.REF_TABLES.exists():
        pytest.skip("oracle/_ref/ref_tables not built (no reference checkout)")
    rng = np.random.default_rng(5)
    for trial in range(12):
        N = int(rng.integers(4, 11))
        Q = int(rng.integers(1, N))
        terms = []
        for _ in range(int(rng.integers(1, 2 * N))):
            kind = ["H", "J", "N"][int(rng.integers(0, 3))]
            i, j = (int(v) for v in rng.choice(N, 2, replace=False))
            terms.append((kind, i, j, float(np.round(rng.uniform(-2, 2), 3)), 0.0))
        ref = orc.ref_tables(N, Q, terms)
        t = orc.Tables(N, Q, terms)
        if t.overflow:
            continue
        assert np.array_equal(t.state, ref[0])
        assert np.array_equal(t.Ax, ref[2]), (N, Q, terms)
        assert np.array_equal(t.Aj, ref[3]), (N, Q, terms)


def test_dense_e0_chain8(orc, golden_energies):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    g = golden_energies["chain8_pbc_q44_U4"]
    assert abs(g["E0"] - DENSE_E0_CHAIN8) < 1e-12 * abs(DENSE_E0_CHAIN8)
    t = orc.Tables(8, 4, L.chain(8))
    H = t.sparse()
    import scipy.sparse as sp
    I = sp.identity(t.count)
    st = t.state
    dbl = orc.popcount((st[:, None] & st[None, :])).ravel().astype(float)
    Hfull = (sp.kron(H, I) + sp.kron(I, H) + sp.diags(4.0 * dbl)).toarray()
    w = np.linalg.eigvalsh(Hfull)
    assert abs(w[0] - g["E0"]) < 1e-11 * abs(g["E0"])


def test_u0_closed_form(golden_energies):
    # U = 0: E0 = 2 * (sum of the 4 lowest levels of -2cos(k)), k = 2 pi n / 8
    # with antiperiodic-or-periodic boundary from the Jordan-Wigner string:
    # for 4 fermions on a ring the string makes the boundary antiperiodic.
    g = golden_energies["chain8_pbc_q44_U0"]["E0"]
    assert abs(g - (-(4 + 4 * math.sqrt(2)))) < 1e-12 * abs(g)


def test_atomic_limit(orc, golden_energies):
    g = golden_energies["atomic8_q32_U3"]
    eps = g["eps"]
    best = math.inf
    for up in range(256):
        if bin(up).count("1") != 3:
            continue
        for dn in range(256):
            if bin(dn).count("1") != 2:
                continue
            e = sum(eps[i] for i in range(8) if up >> i & 1) + sum(eps[i] for i in range(8) if dn >> i & 1)
            e += 3.0 * bin(up & dn).count("1")
            best = min(best, e)
    assert abs(best - g["E0"]) < 1e-12


def test_oracle_lanczos_matches_golden(orc, golden_energies):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    from conftest import philox_uniform
    t = orc.Tables(8, 4, L.chain(8))
    f = philox_uniform(0, 4900)
    e_fixed, a, b, v = orc.lanczos(t, t, 4.0, f, 100, mode="fixed", reorth=True)
    e_ref, a2, b2, v2 = orc.lanczos(t, t, 4.0, f, 1000, mode="reference")
    E0 = golden_energies["chain8_pbc_q44_U4"]["E0"]
    assert abs(e_fixed - E0) < 1e-12 * abs(E0)
    assert abs(e_ref - E0) < 1e-10 * abs(E0)
    assert len(a2) % 10 == 0 and len(a2) < 1000
    # the Ritz vectors are eigenvectors
    Hv = orc.matvec(t, t, 4.0, v)
    assert np.linalg.norm(Hv - e_fixed * v) < 1e-8


def test_oracle_tridiag_vs_scipy(orc):
    from scipy.linalg import eigh_tridiagonal
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 37, 300):
        a = rng.normal(size=n)
        b = np.abs(rng.normal(size=max(n - 1, 0))) + 0.1
        lam, z = orc.tridiag_lowest(a, b)
        w, V = eigh_tridiagonal(a, b)
        assert abs(lam - w[0]) < 1e-13 * max(1.0, abs(w[0]))
        assert abs(abs(np.dot(z, V[:, 0])) - 1.0) < 1e-10


def test_oracle_matvec_equals_sparse(orc):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    terms = L.kagome12()
    t = orc.Tables(12, 5, terms)
    t2 = orc.Tables(12, 4, terms)
    H = orc.hamiltonian(12, 5, 4, terms, terms, 3.0)
    x = np.random.default_rng(2).standard_normal(t.count * t2.count)
    assert rel_err(orc.matvec(t, t2, 3.0, x), H @ x) < 1e-14


def test_continued_fraction_vs_resolvent(orc):
    """g(w) from 200 Lanczos coefficients equals <phi|(w+E-H)^-1|phi> on a
    small dense problem (the reference correlator, HubMatrix_GPU.cuh:820-835)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    terms = L.chain(6)
    t = orc.Tables(6, 3, terms)
    H = orc.hamiltonian(6, 3, 3, terms, terms, 2.0).toarray()
    phi = np.random.default_rng(4).standard_normal(H.shape[0])
    norm2 = float(phi @ phi)
    _, a, b, _ = orc.lanczos(t, t, 2.0, phi, H.shape[0], mode="fixed", reorth=True, want_evec=False)
    w = np.array([0.3 + 0.05j, 1.7 + 0.05j, -0.5 + 0.2j])
    E = -1.0
    g = orc.continued_fraction(a, b, norm2, E, w)
    direct = np.array([phi @ np.linalg.solve((wk + E) * np.eye(H.shape[0]) - H, phi) for wk in w])
    assert np.max(np.abs(g - direct)) < 1e-9 * np.max(np.abs(direct))


def test_sampled_rows_match_full_matvec(orc):
    """oracle.sampled_rows (the check for vectors too large for the host)
    equals the full restated matvec on the rows it samples."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    eps = list(philox_uniform(11, 8, 2.0))
    up, dn = orc.Tables(8, 3, L.chain(8)), orc.Tables(8, 5, L.chain(8, eps=eps))
    x = philox_uniform(5, up.count * dn.count)
    y = orc.matvec(up, dn, 2.5, x, mask=0b10110111)
    idx = np.random.default_rng(0).choice(x.size, 300, replace=False)
    ys, scale = orc.sampled_rows(up, dn, 2.5, idx, lambda i: x[i], mask=0b10110111)
    assert np.all(np.abs(ys - y[idx]) <= 1e-14 * (scale + 1e-300))


def test_sxy_oracle_total_spin_multiplets(orc):
    """The restated S_xy gives S^2 = S(S+1) on exact eigenstates: two sites
    with one up and one down fermion split into a singlet (S^2 = 0) and the
    Sz = 0 member of the triplet (S^2 = 2); the half-filled Hubbard chain of
    4 sites has a singlet ground state; S^2 commutes with H."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    up, dn = orc.Tables(2, 1), orc.Tables(2, 1)
    S = np.column_stack([orc.sxy_matvec(up, dn, e) for e in np.eye(4)])
    w = np.linalg.eigvalsh(S)
    # two doublon singlets, the singlet and the Sz = 0 triplet member of the
    # singly occupied pair
    assert np.allclose(w, [0.0, 0.0, 0.0, 2.0])
    t = L.chain(4)
    Hu, Hd = orc.Tables(4, 2, t), orc.Tables(4, 2, t)
    H = orc.hamiltonian(4, 2, 2, t, t, 4.0).toarray()
    S = np.column_stack([orc.sxy_matvec(Hu, Hd, e) for e in np.eye(H.shape[0])])
    assert np.max(np.abs(H @ S - S @ H)) < 1e-12
    ev, V = np.linalg.eigh(H)
    assert abs(V[:, 0] @ S @ V[:, 0]) < 1e-10
    # every eigenvalue of S_xy (Sz = 0) is S(S+1)
    ws = np.linalg.eigvalsh(S)
    ss = (-1 + np.sqrt(1 + 4 * np.clip(ws, 0, None))) / 2
    assert np.max(np.abs(ss - np.round(ss))) < 1e-10


def test_oracle_kagome12_terms_match_the_package_lattice():
    """The CPU baseline builds Kagome12 from the oracle's own restatement of
    KagomeLattice12; it must be the term list the library is given."""
    from oracle import oracle as O
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    assert O.kagome12_terms() == L.kagome12()
    assert np.array_equal(O.philox_uniform(7, 33, 2.0), philox_uniform(7, 33, 2.0))
