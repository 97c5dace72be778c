"""Several lowest eigenpairs (ed_eigs_lowest, the Spectra::SymEigsSolver
replacement) against dense diagonalisation and scipy's ARPACK on the oracle's
Hamiltonian, and the TotalSpinExcited flow: S^2 of each eigenvector."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_eigs_lowest_matches_dense(ed, orc):
    from conftest import philox_uniform
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, spectra
    N, q, U = 8, 4, 2.0
    t = L.chain(N, periodic=False, eps=list(philox_uniform(5, N, 1.5)))
    op = ed.Hubbard(ed.H_TBq(N, q).extend(t), ed.H_TBq(N, q).extend(t), U)
    nev = 6
    info = {}
    w, v, r = spectra.eigs_lowest(op, nev, result=info)
    assert info["converged"] and info["nconv"] == nev
    wd, Vd = np.linalg.eigh(orc.hamiltonian(N, q, q, t, t, U).toarray())
    assert np.min(np.diff(wd[: nev + 1])) > 1e-6
    assert np.max(np.abs(w - wd[:nev])) < 1e-10 * np.max(np.abs(wd[:nev]))
    ov = np.abs(np.sum(v * Vd[:, :nev].T, axis=1))
    assert np.max(np.abs(ov - 1.0)) < 1e-8
    assert np.max(np.abs(v @ v.T - np.eye(nev))) < 1e-12
    assert np.all(r < 1e-10 * np.maximum(np.abs(w), 1.0))


def test_spectra_surface_lieb12_total_spin(ed, orc):
    """TotalSpinExcited_Lieb_randomHop.cu:129-157 on LiebLattice12 3+3 with
    random hoppings (X = 0.3): 4 lowest pairs, then Sxy = <V|S V> and
    S^2 = (Qup - Qdn)^2 / 4 + Sxy for each; against scipy's eigsh and the
    oracle's S_xy."""
    import scipy.sparse.linalg as sla
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import datio, lattices as L, observables as ob, spectra
    N, q, U, X, nev = 12, 3, 4.0, 0.3, 4
    r = datio.site_factors(datio.random_numbers(1, N, seed=3)[0], X)
    t = L.lieb12(r)
    H = ed.Hubbard(ed.H_TBq(N, q).extend(t), ed.H_TBq(N, q).extend(t), U)
    eigs = spectra.SymEigsSolver(H, nev, 4 * (nev + 1))
    eigs.init()
    nconv = eigs.compute(spectra.SortRule.SmallestAlge, 1000, 1e-10, spectra.SortRule.SmallestAlge)
    assert eigs.info() == spectra.CompInfo.Successful and nconv == nev
    ev, evec = eigs.eigenvalues(), eigs.eigenvectors()
    Hs = orc.hamiltonian(N, q, q, t, t, U)
    wr = np.sort(sla.eigsh(Hs, k=nev + 2, which="SA", tol=1e-13)[0])
    assert np.max(np.abs(ev - wr[:nev])) < 1e-9 * np.max(np.abs(wr))
    tu = orc.Tables(N, q, t)
    for i in range(nev):
        V = np.ascontiguousarray(evec[:, i])
        sxy, s2 = ob.s2_expect(H, V)
        ref = float(V @ orc.sxy_matvec(tu, tu, V))
        assert abs(sxy - ref) < 1e-10
        assert abs(s2 - ref) < 1e-10  # Qup = Qdn
        # S^2 = S(S+1) for an eigenvector of a spin-symmetric H
        S = (-1 + np.sqrt(1 + 4 * s2)) / 2
        assert abs(S - round(S)) < 1e-6


def test_eigs_reports_not_converged(ed):
    from conftest import philox_uniform
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, spectra
    t = L.chain(8, periodic=False, eps=list(philox_uniform(6, 8, 1.0)))
    op = ed.Hubbard(ed.H_TBq(8, 4).extend(t), ed.H_TBq(8, 4).extend(t), 2.0)
    info = {}
    spectra.eigs_lowest(op, 5, ncv=8, tol=1e-14, max_restarts=1, result=info)
    assert not info["converged"] and info["restarts"] == 1 and info["nconv"] < 5


def test_eigs_on_degenerate_sectors(ed, orc):
    """One up particle against eleven down (dim 144): the 4 lowest pairs
    against dense diagonalisation; a one-state sector cannot hold a pair
    beyond its only state and is refused."""
    from conftest import philox_uniform
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, spectra
    t = L.chain(12, periodic=False, eps=list(philox_uniform(8, 12, 2.0)))
    op = ed.Hubbard(ed.H_TBq(12, 1).extend(t), ed.H_TBq(12, 11).extend(t), 1.5)
    nev = 4
    info = {}
    w, v, r = spectra.eigs_lowest(op, nev, result=info)
    assert info["converged"]
    wd = np.linalg.eigvalsh(orc.hamiltonian(12, 1, 11, t, t, 1.5).toarray())
    assert np.min(np.diff(wd[: nev + 1])) > 1e-6
    assert np.max(np.abs(w - wd[:nev])) < 1e-10 * np.max(np.abs(wd[:nev]))
    op.close()
    one = ed.Hubbard(ed.H_TBq(12, 0).extend(t), ed.H_TBq(12, 0).extend(t), 1.5)
    with pytest.raises(Exception):
        spectra.eigs_lowest(one, 1)
    one.close()
