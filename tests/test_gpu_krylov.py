"""Krylov time evolution on the GPU against dense exp(-iHt) from the oracle's
Hamiltonian: real operator with the reference driver's product-state start
(Time_evol_test.cu:33-35), real operator with a complex start, complex
(Peierls) operator, more times than one pass of the combine kernel; and, at
the full open L=12 chain (6,6) sector, the conserved norm and energy."""
import numpy as np
import pytest
import scipy.linalg as sl

pytestmark = pytest.mark.gpu


def dense_evolve(H, psi0, times):
    w, V = np.linalg.eigh(H)
    c = V.conj().T @ psi0
    return np.stack([V @ (np.exp(-1j * w * t) * c) for t in times])


def product_state(orc, N, qu, qd, up_word, dn_word):
    su, sd = orc.Tables(N, qu).state, orc.Tables(N, qd).state
    v = np.zeros(su.size * sd.size, dtype=np.complex128)
    v[int(np.where(su == up_word)[0][0]) * sd.size + int(np.where(sd == dn_word)[0][0])] = 1.0
    return v


@pytest.mark.parametrize("case", ["chain8_product", "chain8_complex_start", "kagome12_flux"])
def test_krylov_matches_dense(ed, orc, case):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev, lattices as L
    from conftest import philox_uniform
    if case == "kagome12_flux":
        N, qu, qd, U, t = 12, 2, 2, 4.0, L.kagome12(flux=0.7)
    else:
        N, qu, qd, U, t = 8, 4, 4, 4.0, L.chain(8, periodic=False, eps=list(philox_uniform(3, 8, 2.0)))
    op = ed.Hubbard(ed.H_TBq(N, qu).extend(t), ed.H_TBq(N, qd).extend(t), U)
    Hd = orc.hamiltonian(N, qu, qd, t, t, U).toarray()
    if case == "chain8_product":
        psi0 = product_state(orc, N, qu, qd, 0b00001111, 0b11110000)
    else:
        x = philox_uniform(11, 2 * op.rows())
        psi0 = (x[0::2] + 1j * x[1::2]) * 0.3
    times = [0.0, 0.1, 0.3, 0.5, 1.0, 1.5, 2.0, 3.0, 4.0, 5.0]  # > 8: two combine passes
    info = {}
    got = ev.krylov_evolve(op, psi0, times, max_steps=250, tol=1e-12, result=info)
    ref = dense_evolve(Hd, psi0, times)
    nrm = np.linalg.norm(psi0)
    assert info["runs"] == (1 if case in ("chain8_product", "kagome12_flux") else 2)
    assert abs(info["norm"] - nrm) < 1e-14 * nrm
    for i in range(len(times)):
        assert np.linalg.norm(got[i] - ref[i]) < 1e-10 * nrm, (case, times[i])
    assert info["err_est"] < 1e-9 * nrm


@pytest.mark.parametrize("qu,qd", [(0, 0), (12, 12), (0, 6), (1, 11)])
def test_krylov_degenerate_sectors(ed, orc, qu, qd):
    """Sectors of one state (the recurrence stops after its first step) and
    with an empty spin species, against dense exp(-iHt)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev, lattices as L
    from conftest import philox_uniform
    t = L.chain(12, periodic=False, eps=list(philox_uniform(7, 12, 2.0)))
    op = ed.Hubbard(ed.H_TBq(12, qu).extend(t), ed.H_TBq(12, qd).extend(t), 1.5)
    Hd = orc.hamiltonian(12, qu, qd, t, t, 1.5)
    Hd = Hd.toarray() if hasattr(Hd, "toarray") else np.asarray(Hd)
    x = philox_uniform(13, 2 * op.rows())
    psi0 = (x[0::2] + 1j * x[1::2]) * 0.5
    times = [0.0, 0.4, 1.3, 2.0]
    info = {}
    got = ev.krylov_evolve(op, psi0, times, max_steps=250, tol=1e-12, result=info)
    ref = dense_evolve(Hd, psi0, times)
    nrm = np.linalg.norm(psi0)
    for i in range(len(times)):
        assert np.linalg.norm(got[i] - ref[i]) < 1e-10 * nrm, (qu, qd, times[i])
    op.close()


def test_krylov_stops_at_invariant_subspace(ed, orc):
    """A start in a tiny invariant subspace (2 sites, 1+1 particles: 4 states)
    stops the recurrence at beta < tol, like the reference's b < 1e-10."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev, lattices as L
    t = L.chain(2, periodic=False)
    op = ed.Hubbard(ed.H_TBq(2, 1).extend(t), ed.H_TBq(2, 1).extend(t), 2.0)
    psi0 = np.zeros(4, dtype=np.complex128)
    psi0[0] = 1.0
    info = {}
    got = ev.krylov_evolve(op, psi0, [0.3, 4.0], max_steps=50, tol=1e-10, result=info)
    assert info["steps"] <= 4
    ref = dense_evolve(orc.hamiltonian(2, 1, 1, t, t, 2.0).toarray(), psi0, [0.3, 4.0])
    assert np.max(np.abs(got - ref)) < 1e-12


def test_krylov_reference_driver_surface(ed, orc):
    """Krylov.Krylov_time_evol adds exp(-iH dt) phi0 into phi, on device tensors."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev, lattices as L
    t = L.chain(8)
    op = ed.Hubbard(ed.H_TBq(8, 3).extend(t), ed.H_TBq(8, 3).extend(t), 1.0)
    psi0 = product_state(orc, 8, 3, 3, 0b00000111, 0b00000111)
    phi0 = torch.tensor(psi0, device="cuda")
    phi = torch.zeros_like(phi0)
    kry = ev.Krylov(56, 56)
    kry.Make_tridiagonal_eigen(op, phi0)
    assert kry.steps > 10
    kry.Krylov_time_evol(op, phi0, phi, 1.5)
    ref = dense_evolve(orc.hamiltonian(8, 3, 3, t, t, 1.0).toarray(), psi0, [1.5])[0]
    assert np.max(np.abs(phi.cpu().numpy() - ref)) < 1e-11


def test_krylov_full_chain12_conserves_norm_and_energy(ed, orc):
    """Open L=12, W=6, U=1, sector (6,6) (853,776 states), start = the
    half-filled product state of the reference MBL driver (up 0..0011000000
    pattern replaced by sites 0..5 filled): |psi(t)| = |psi0| and <H>(t) =
    <H>(0) at t up to 2."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev, observables as ob, sweeps
    eu, edn = sweeps.mbl_disorder(0, 12, 6.0)
    op = ed.Hubbard(ed.H_TBq(12, 6).extend(sweeps.mbl_chain_terms(eu)),
                    ed.H_TBq(12, 6).extend(sweeps.mbl_chain_terms(edn)), 1.0)
    psi0 = product_state(orc, 12, 6, 6, 0b000000111111, 0b111111000000)
    times = [0.25, 0.5, 1.0, 2.0]
    info = {}
    out = ev.krylov_evolve(op, psi0, times, max_steps=200, tol=1e-12, result=info)
    e_start = float(np.real(np.vdot(psi0, op.matvec(psi0.real.copy()))))
    for i in range(len(times)):
        v = out[i]
        assert abs(np.linalg.norm(v) - 1.0) < 1e-10
        hv = op.matvec(np.ascontiguousarray(v.real)) + 1j * op.matvec(np.ascontiguousarray(v.imag))
        assert abs(np.real(np.vdot(v, hv)) - e_start) < 1e-9 * max(1.0, abs(e_start))
    assert info["err_est"] < 1e-8


def test_krylov_two_pass_operator_regenerates_basis(ed, monkeypatch):
    """An operator on the two-pass matvec (forced here on chain12 (7,5))
    evolves by regenerating its Krylov vectors instead of storing them; the
    result matches the stored-basis evolution of the same operator built for
    the row engine, for a real and a complex start and three times."""
    from conftest import philox_uniform
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev, sweeps
    eu, edn = sweeps.mbl_disorder(1, 12, 6.0)
    tu, td = sweeps.mbl_chain_terms(eu), sweeps.mbl_chain_terms(edn)
    op = ed.Hubbard(ed.H_TBq(12, 7).extend(tu), ed.H_TBq(12, 5).extend(td), 1.0)
    monkeypatch.setenv("ED_MATVEC", "striped")
    op2 = ed.Hubbard(ed.H_TBq(12, 7).extend(tu), ed.H_TBq(12, 5).extend(td), 1.0)
    monkeypatch.delenv("ED_MATVEC")
    n = op.rows()
    x = philox_uniform(21, 2 * n)
    for psi0 in (x[:n] + 0j, x[0::2] + 1j * x[1::2]):
        psi0 = psi0 / np.linalg.norm(psi0)
        ia, ib = {}, {}
        a = ev.krylov_evolve(op, psi0, [0.2, 0.7, 1.5], max_steps=120, tol=1e-12, result=ia)
        b = ev.krylov_evolve(op2, psi0, [0.2, 0.7, 1.5], max_steps=120, tol=1e-12, result=ib)
        assert ia["steps"] == ib["steps"] and ia["runs"] == ib["runs"]
        assert np.max(np.abs(a - b)) < 1e-13
