"""One persistent launch over Lanczos runs of different sectors, real and
complex (ed_lanczos_batch's general kernel): every run's alpha, beta, E0 and
Ritz vector equal those of its own ed_lanczos_run bit for bit; the batched
flux sweep (ground states and response solves each in one launch) equals the
unbatched sweep exactly."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ops(ed):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, sweeps
    eu, edn = sweeps.mbl_disorder(0, 12, 6.0)
    tu, td = sweeps.mbl_chain_terms(eu), sweeps.mbl_chain_terms(edn)
    ops = [ed.Hubbard(ed.H_TBq(12, qu).extend(tu), ed.H_TBq(12, qd).extend(td), 1.0)
           for qu, qd in ((6, 6), (7, 5), (8, 4))]
    k = L.kagome12(flux=0.3)
    ops.append(ed.Hubbard(ed.H_TBq(12, 5).extend(k), ed.H_TBq(12, 5).extend(k), 4.0))
    ops.append(ed.Hubbard(ed.H_TBq(12, 6).extend(L.kagome12()), ed.H_TBq(12, 6).extend(L.kagome12()), 8.0))
    eu2, edn2 = sweeps.mbl_disorder(1, 12, 6.0)
    ops.append(ed.Hubbard(ed.H_TBq(12, 7).extend(sweeps.mbl_chain_terms(eu2)),
                          ed.H_TBq(12, 5).extend(sweeps.mbl_chain_terms(edn2)), 1.0))
    return ops


@pytest.mark.parametrize("steps", [40])
def test_mixed_sector_mixed_kind_batch_equals_single_runs(ed, edlib, steps):
    import torch
    ops = _ops(ed)
    # four shapes (924^2, 792^2, 495^2 real; 792^2 complex), five table groups
    assert len({(op.dimUP, op.dimDN, op.is_complex) for op in ops}) == 4
    sizes = [op.rows() * (2 if op.is_complex else 1) for op in ops]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    starts = torch.empty(int(offs[-1]), dtype=torch.float64, device="cuda")
    for b, n in enumerate(sizes):
        assert edlib.ed_random_vector_device(int(n), 100 + b, C.c_void_p(starts[int(offs[b])].data_ptr()), None) == 0
    evecs = torch.empty_like(starts)
    results = []
    e0s, views, alpha, beta = ed.hubbard.lanczos_multi(ops, steps, starts=starts, evec_out=evecs, results=results)
    assert results[0].launches >= 1
    sh = starts.cpu().numpy()
    for b, op in enumerate(ops):
        f = sh[int(offs[b]):int(offs[b + 1])].copy()
        if op.is_complex:
            f = f.view(np.complex128)
        lz = ed.Lanczos()
        e0, v = lz.eigen(op, f=f, max_steps=steps, mode="fixed", ritz="stored")
        assert e0 == e0s[b], (b, e0, e0s[b])
        assert np.array_equal(np.array(lz.a), alpha[b]) and np.array_equal(np.array(lz.b), beta[b])
        vb = views[b].cpu().numpy()
        assert np.array_equal(vb, v), b
        assert results[b].min_bits == lz.result.min_bits
    for op in ops:
        op.close()


def test_degenerate_sector_batch_equals_single_runs(ed, edlib):
    """A batch holding one-row sectors (an empty or a full up species), a
    one-column sector (no down particle), a regular sector and a complex
    one-row sector: each run equals its own single run bit for bit."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, sweeps
    eu, edn = sweeps.mbl_disorder(2, 12, 6.0)
    tu, td = sweeps.mbl_chain_terms(eu), sweeps.mbl_chain_terms(edn)
    ops = [ed.Hubbard(ed.H_TBq(12, qu).extend(tu), ed.H_TBq(12, qd).extend(td), 1.0)
           for qu, qd in ((0, 6), (12, 6), (6, 0), (6, 6))]
    k = L.kagome12(flux=0.3)
    ops.append(ed.Hubbard(ed.H_TBq(12, 0).extend(k), ed.H_TBq(12, 6).extend(k), 4.0))
    steps = 40
    sizes = [op.rows() * (2 if op.is_complex else 1) for op in ops]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    starts = torch.empty(int(offs[-1]), dtype=torch.float64, device="cuda")
    for b, n in enumerate(sizes):
        assert edlib.ed_random_vector_device(int(n), 200 + b, C.c_void_p(starts[int(offs[b])].data_ptr()), None) == 0
    evecs = torch.empty_like(starts)
    e0s, views, alpha, beta = ed.hubbard.lanczos_multi(ops, steps, starts=starts, evec_out=evecs, results=[])
    sh = starts.cpu().numpy()
    for b, op in enumerate(ops):
        f = sh[int(offs[b]):int(offs[b + 1])].copy()
        if op.is_complex:
            f = f.view(np.complex128)
        lz = ed.Lanczos()
        e0, v = lz.eigen(op, f=f, max_steps=steps, mode="fixed", ritz="stored")
        assert e0 == e0s[b], (b, e0, e0s[b])
        assert np.array_equal(np.array(lz.a), alpha[b]) and np.array_equal(np.array(lz.b), beta[b])
        assert np.array_equal(views[b].cpu().numpy(), v), b
    for op in ops:
        op.close()


def test_homogeneous_batch_in_general_kernel_equals_specialised(ed, monkeypatch):
    """The same-sector real batch that the specialised kernel takes gives the
    same coefficients when ED_LZ_BATCH=multi routes it to the general one."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    ops = []
    for r in range(4):
        eu, edn = sweeps.mbl_disorder(r, 12, 6.0)
        ops.append(ed.Hubbard(ed.H_TBq(12, 6).extend(sweeps.mbl_chain_terms(eu)),
                              ed.H_TBq(12, 6).extend(sweeps.mbl_chain_terms(edn)), 1.0))
    a = ed.lanczos_batch(ops, 50, seed=7)
    monkeypatch.setenv("ED_LZ_BATCH", "multi")
    b = ed.lanczos_batch(ops, 50, seed=7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])
    assert np.array_equal(a[1], b[1])
    for op in ops:
        op.close()


def test_flux_sweep_batched_equals_unbatched(ed):
    """Kagome12 4+4 (complex, dim 245,025) at four twists including the
    degenerate zero twist: the batched sweep (one launch for the ground
    states, one for the response solves, the multiplet search at Phi = 0
    outside) returns the unbatched sweep's E0, dE0/dPhi, d2E0/dPhi2 exactly."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    phis = sweeps.flux_phis(16)[[0, 3, 9, 15]]
    kw = dict(n_up=4, n_dn=4, U=4.0, steps=200, response_steps=120)
    a = sweeps.flux_sweep(phis, **kw)
    b = sweeps.flux_sweep(phis, batch=4, **kw)
    for p, q in zip(a, b):
        assert (p.phi, p.e0, p.d1, p.d2) == (q.phi, q.e0, q.d1, q.d2)
        assert p.min_bits == q.min_bits
