"""GPU parity of the spin-split matvec against the CPU oracle.

Real operators are compared with the restated reference kernel
(oracle/hubbard_oracle.c, Hubbard_mv_); complex (Peierls) operators with the
oracle's independent scipy construction.  Tolerance: the GPU sums +-x
exactly in int64 fixed point and rounds once, so the normwise relative
difference to the FP64 oracle is set by the oracle's own rounding:
|y_gpu - y_oracle| / |y_oracle| < 1e-13.
"""
import numpy as np
import pytest

from conftest import philox_uniform, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-13


def make_op(ed, N, qu, qd, up_terms, dn_terms, U, dilution=None):
    hu = ed.H_TBq(N, qu).extend(up_terms)
    hd = ed.H_TBq(N, qd).extend(dn_terms)
    return ed.Hubbard(hu, hd, U, dilution=dilution)


def real_cases():
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    eps8 = list(philox_uniform(11, 8, 2.0))
    eps12 = list(philox_uniform(100, 12, 6.0))
    return [
        ("chain8_pbc_44_U4", 8, 4, 4, L.chain(8), L.chain(8), 4.0, None),
        ("chain8_pbc_35_U2.5_diluted", 8, 3, 5, L.chain(8), L.chain(8, eps=eps8), 2.5, 0b10110111),
        ("kagome12_66_U8", 12, 6, 6, L.kagome12(), L.kagome12(), 8.0, None),
        ("kagome12_54_Kx", 12, 5, 4, L.kagome12_kinetic_x(), L.kagome12_kinetic_x(), 0.0, None),
        ("kagome12_54_Jx", 12, 5, 4, L.kagome12_current_x(), L.kagome12_current_x(), 0.0, None),
        ("chain12_open_W6_66", 12, 6, 6, L.chain(12, periodic=False, eps=eps12), L.chain(12, periodic=False, eps=eps12), 1.0, None),
        ("chain12_open_W6_75", 12, 7, 5, L.chain(12, periodic=False, eps=eps12), L.chain(12, periodic=False, eps=eps12), 1.0, None),
        ("chain12_open_W6_84", 12, 8, 4, L.chain(12, periodic=False, eps=eps12), L.chain(12, periodic=False, eps=eps12), 1.0, None),
        ("lieb12_66_U4", 12, 6, 6, L.lieb12(), L.lieb12(), 4.0, None),
        ("square3x4_43_U3", 12, 4, 3, L.squared_3by4(), L.squared_3by4(), 3.0, None),
        ("atomic8_32_U3", 8, 3, 2, [("N", i, 0, eps8[i], 0.0) for i in range(8)],
         [("N", i, 0, eps8[i], 0.0) for i in range(8)], 3.0, None),
        ("random_hop10_46", 10, 4, 6, [("H", i, (i + 3) % 10, 0.3 + 0.1 * i, 0.0) for i in range(10)],
         [("H", i, (i + 1) % 10, -1.0, 0.0) for i in range(10)] + [("J", 0, 5, 0.7, 0.0)], 1.7, None),
    ]


@pytest.mark.parametrize("case", real_cases(), ids=lambda c: c[0])
def test_matvec_real_vs_oracle(ed, orc, case):
    name, N, qu, qd, ut, dt, U, dil = case
    op = make_op(ed, N, qu, qd, ut, dt, U, dil)
    tu, td = orc.Tables(N, qu, ut), orc.Tables(N, qd, dt)
    rng = np.random.default_rng(7)
    for trial in range(2):
        x = rng.standard_normal(op.rows())
        y = op.matvec(x)
        yo = orc.matvec(tu, td, U, x, mask=(orc.mask_all(N) if dil is None else dil))
        assert rel_err(y, yo) < TOL, (name, rel_err(y, yo))


def degenerate_cases():
    """Sectors with an empty or a full spin species (a one-dimensional spin
    space: one row of the product basis, or rows of one element), a sector
    with no particle at all, and a small square one: the row engine's edge
    shapes (grid larger than the row count, odd one-element rows, empty hop
    tables)."""
    return [
        ("chain8_04", 8, 0, 4), ("chain8_40", 8, 4, 0), ("chain8_84", 8, 8, 4), ("chain8_48", 8, 4, 8),
        ("chain8_00", 8, 0, 0), ("chain8_17", 8, 1, 7), ("chain12_06", 12, 0, 6),
    ]


@pytest.mark.parametrize("case", degenerate_cases(), ids=lambda c: c[0])
def test_matvec_degenerate_sectors_vs_oracle(ed, orc, case):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    name, N, qu, qd = case
    t = L.chain(N, eps=list(philox_uniform(5, N, 1.5)))
    op = make_op(ed, N, qu, qd, t, t, 4.0)
    tu, td = orc.Tables(N, qu, t), orc.Tables(N, qd, t)
    assert op.rows() == tu.count * td.count
    x = np.random.default_rng(3).standard_normal(op.rows())
    y = op.matvec(x)
    yo = orc.matvec(tu, td, 4.0, x)
    if not np.any(yo):
        assert not np.any(y), name  # the empty sector's operator is zero
    else:
        assert rel_err(y, yo) < TOL, (name, rel_err(y, yo))
    op.close()


@pytest.mark.parametrize("case", degenerate_cases(), ids=lambda c: c[0])
def test_lanczos_degenerate_sectors_vs_dense(ed, orc, case):
    """Lanczos on the same sectors (fixed steps, up to the dimension: the
    one-row sectors break down after the first step and T stops there)
    against the lowest eigenvalue of the oracle's dense Hamiltonian."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    name, N, qu, qd = case
    t = L.chain(N, eps=list(philox_uniform(5, N, 1.5)))
    op = make_op(ed, N, qu, qd, t, t, 4.0)
    e0, _ = ed.Lanczos().eigen(op, max_steps=min(200, op.rows()), mode="fixed", ritz="none", seed=0)
    H = orc.hamiltonian(N, qu, qd, t, t, 4.0)
    H = H.toarray() if hasattr(H, "toarray") else np.asarray(H)
    e_ref = float(np.linalg.eigvalsh(H)[0])
    assert abs(e0 - e_ref) < 1e-10 * max(1.0, abs(e_ref)), (name, e0, e_ref)
    op.close()


def complex_degenerate_cases():
    """Kagome12 with a Peierls twist (complex, four coefficient classes) on
    sectors with an empty or a full spin species, no particle, and one
    particle against eleven."""
    return [("k12_0_6", 0, 6), ("k12_6_0", 6, 0), ("k12_12_5", 12, 5), ("k12_5_12", 5, 12),
            ("k12_0_0", 0, 0), ("k12_1_11", 1, 11)]


@pytest.mark.parametrize("case", complex_degenerate_cases(), ids=lambda c: c[0])
def test_complex_degenerate_sectors_vs_dense(ed, orc, case):
    """Complex matvec against the oracle's dense Hamiltonian, and Lanczos E0
    (fixed steps, up to the dimension) against its lowest eigenvalue."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    name, qu, qd = case
    terms = L.kagome12(flux=0.37)
    op = make_op(ed, 12, qu, qd, terms, terms, 4.0)
    assert op.is_complex or not (0 < qu < 12 or 0 < qd < 12)
    H = orc.hamiltonian(12, qu, qd, terms, terms, 4.0)
    H = H.toarray() if hasattr(H, "toarray") else np.asarray(H)
    assert H.shape == (op.rows(), op.rows())
    rng = np.random.default_rng(7)
    x = rng.standard_normal(op.rows()) + (1j * rng.standard_normal(op.rows()) if op.is_complex else 0)
    y, yo = op.matvec(x), H @ x
    if not np.any(yo):
        assert not np.any(y), name
    else:
        assert rel_err(y, yo) < TOL, (name, rel_err(y, yo))
    e0, _ = ed.Lanczos().eigen(op, max_steps=min(200, op.rows()), mode="fixed", ritz="none", seed=0)
    e_ref = float(np.linalg.eigvalsh(H)[0])
    assert abs(e0 - e_ref) < 1e-10 * max(1.0, abs(e_ref)), (name, e0, e_ref)
    op.close()


def test_matvec_device_path_matches_host_path(ed):
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    op = make_op(ed, 12, 6, 6, L.kagome12(), L.kagome12(), 8.0)
    x = np.random.default_rng(1).standard_normal(op.rows())
    y_host = op.matvec(x)
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    op.Hubbard_mv(xt, yt)
    torch.cuda.synchronize()
    assert np.array_equal(yt.cpu().numpy(), y_host)


def test_matvec_hermitian_and_scale_invariant(ed):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    op = make_op(ed, 12, 6, 5, L.kagome12(), L.kagome12(), 4.0)
    rng = np.random.default_rng(3)
    x, z = rng.standard_normal(op.rows()), rng.standard_normal(op.rows())
    hx, hz = op.matvec(x), op.matvec(z)
    assert abs(z @ hx - x @ hz) < 1e-12 * np.linalg.norm(hx) * np.linalg.norm(z)
    # exact power-of-two scaling of the input scales the output exactly
    for k in (-900, -3, 1, 700):
        assert np.array_equal(op.matvec(x * 2.0 ** k), hx * 2.0 ** k), k
    assert np.array_equal(op.matvec(np.zeros(op.rows())), np.zeros(op.rows()))


def test_matvec_nonfinite_input_is_reported(ed):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300._capi import EdError
    op = make_op(ed, 8, 4, 4, L.chain(8), L.chain(8), 4.0)
    x = np.ones(op.rows())
    x[17] = np.nan
    with pytest.raises(EdError) as e:
        op.matvec(x)
    assert e.value.status == 6


def test_matvec_wide_dynamic_range(ed, orc):
    """Elements spanning 2^-40..1: the FX input quantisation (54 bits below
    the largest element) keeps the normwise error at FP64 level."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    op = make_op(ed, 8, 4, 4, L.chain(8), L.chain(8), 4.0)
    t = orc.Tables(8, 4, L.chain(8))
    rng = np.random.default_rng(4)
    x = rng.standard_normal(op.rows()) * 2.0 ** rng.integers(-40, 1, op.rows())
    assert rel_err(op.matvec(x), orc.matvec(t, t, 4.0, x)) < TOL


@pytest.mark.parametrize("flux", [0.0, 0.37, np.pi / 2])
def test_matvec_complex_peierls(ed, orc, flux):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    terms = L.kagome12(flux=flux) if flux else [("P",) + t[1:] if t[0] == "H" else t for t in L.kagome12()]
    op = make_op(ed, 12, 4, 3, terms, terms, 4.0)
    assert op.is_complex
    H = orc.hamiltonian(12, 4, 3, terms, terms, 4.0)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(op.rows()) + 1j * rng.standard_normal(op.rows())
    assert rel_err(op.matvec(x), H @ x) < TOL
    # Hermitian: <z, H x> = conj(<x, H z>)
    z = rng.standard_normal(op.rows()) + 1j * rng.standard_normal(op.rows())
    a, b = np.vdot(z, op.matvec(x)), np.vdot(x, op.matvec(z))
    assert abs(a - np.conj(b)) < 1e-12 * abs(a)


def test_complex_operator_zero_flux_equals_real(ed):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    real = make_op(ed, 12, 5, 5, L.kagome12(), L.kagome12(), 8.0)
    pt = [("P",) + t[1:] if t[0] == "H" else t for t in L.kagome12()]
    cplx = make_op(ed, 12, 5, 5, pt, pt, 8.0)
    x = np.random.default_rng(6).standard_normal(real.rows())
    yr = real.matvec(x)
    yc = cplx.matvec(x.astype(np.complex128))
    assert np.array_equal(yc.real, yr) and not np.any(yc.imag)


def test_basis_rank_unrank_device(ed, edlib):
    import ctypes as C
    import torch
    for N, Q in ((12, 6), (18, 9), (40, 9)):
        count = ed.binom(N, Q)
        r = torch.randint(0, count, (100000,), dtype=torch.int64, device="cuda")
        w = torch.empty_like(r)
        r2 = torch.empty_like(r)
        assert edlib.ed_basis_unrank_device(N, Q, C.c_void_p(r.data_ptr()), r.numel(), C.c_void_p(w.data_ptr()), None) == 0
        assert edlib.ed_basis_rank_device(N, Q, C.c_void_p(w.data_ptr()), w.numel(), C.c_void_p(r2.data_ptr()), None) == 0
        torch.cuda.synchronize()
        assert torch.equal(r, r2)
        host = ed.basis_unrank(N, Q, r[:2000].cpu().numpy())
        assert np.array_equal(host.view(np.int64), w[:2000].cpu().numpy())


def test_device_random_vector_matches_host(ed, edlib):
    import ctypes as C
    import torch
    n = 1_000_003
    t = torch.empty(n, dtype=torch.float64, device="cuda")
    assert edlib.ed_random_vector_device(n, 42, C.c_void_p(t.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy(), philox_uniform(42, n))


def kernel_cases():
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    eps12 = list(philox_uniform(100, 12, 6.0))
    return [
        ("kagome12_66_U8", 12, 6, 6, L.kagome12(), L.kagome12(), 8.0),
        ("kagome12_66_U0", 12, 6, 6, L.kagome12(), L.kagome12(), 0.0),
        ("kagome12_54_flux", 12, 5, 4, L.kagome12(flux=0.3), L.kagome12(flux=0.3), 4.0),
        ("kagome12_66_flux", 12, 6, 6, L.kagome12(flux=0.3), L.kagome12(flux=0.3), 4.0),
        ("kagome12_66_flux_up_only", 12, 6, 6, L.kagome12(flux=0.3), L.kagome12(), 4.0),
        ("kagome12_55_Kx_2classes", 12, 5, 5, L.kagome12_kinetic_x(), L.kagome12_kinetic_x(), 1.0),
        ("chain12_open_W6_75", 12, 7, 5, L.chain(12, periodic=False, eps=eps12), L.chain(12, periodic=False, eps=eps12), 1.0),
        # odd down dimension (495): every other row starts off a 16-byte boundary
        ("chain12_open_W6_84_odd_rows", 12, 8, 4, L.chain(12, periodic=False, eps=eps12),
         L.chain(12, periodic=False, eps=eps12), 1.0),
        ("kagome12_54_real_odd_rows", 12, 5, 4, L.kagome12(), L.kagome12(), 4.0),
        ("chain8_35", 8, 3, 5, L.chain(8), L.chain(8), 2.0),
        ("chain8_04_no_up_hops", 8, 0, 4, L.chain(8), L.chain(8), 2.0),
        ("chain2_11", 2, 1, 1, L.chain(2, periodic=False), L.chain(2, periodic=False), 3.0),
        ("chain14_75", 14, 7, 5, L.chain(14), L.chain(14), 4.0),
        # one-row sectors (an empty or a full up species) through every kernel
        ("chain14_07", 14, 0, 7, L.chain(14), L.chain(14), 4.0),
        ("chain14_147", 14, 14, 7, L.chain(14), L.chain(14), 4.0),
    ]


@pytest.mark.parametrize("case", kernel_cases(), ids=lambda c: c[0])
def test_matvec_kernels_agree_bit_for_bit(ed, monkeypatch, case):
    """The row-staged TMA kernel, the two-pass (striped) kernel over the
    permuted down index and the generic kernel compute the same exact integer
    sums: their outputs and Lanczos coefficients agree bit for bit (an
    operator a kernel does not take falls through to the next one)."""
    name, N, qu, qd, ut, dt, U = case
    ops = {}
    variants = {"auto": {}, "striped": {"ED_MATVEC": "striped"}, "generic": {"ED_MATVEC": "generic"}}
    for kind, env in variants.items():
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        ops[kind] = make_op(ed, N, qu, qd, ut, dt, U)
        for k in env:
            monkeypatch.delenv(k, raising=False)
    # the two-pass kernel takes real single-class operators with an even
    # down dimension; the others fall through
    if not ops["auto"].is_complex and "classes" not in name and ops["auto"].dimDN % 2 == 0:
        assert ops["striped"].matvec_kind == "two_pass", name
    assert ops["generic"].matvec_kind == "generic"
    rng = np.random.default_rng(11)
    n = ops["auto"].rows()
    cplx = ops["auto"].is_complex
    x = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    ys = {k: op.matvec(x) for k, op in ops.items()}
    for k in ys:
        assert np.array_equal(ys[k], ys["generic"]), k
    runs = {}
    for k, op in ops.items():
        lz = ed.Lanczos()
        e, _ = lz.eigen(op, max_steps=min(30, n), mode="fixed", ritz="none", seed=4)
        runs[k] = (lz.a, lz.b, e)
    for k in runs:
        assert runs[k] == runs["generic"], k


def test_lieb18_full_size_sampled_rows(ed, orc):
    """Lieb18 9+9 (D = 2,363,904,400; 18.9 GB per FP64 vector), which the
    reference's int-indexed kernel cannot run: y = H x on the device for a
    uniform(-1,1) x, and 20,000 output elements (plus the first and last)
    recomputed on the host from the oracle's tables, each to 1e-13 of the sum
    of its terms' magnitudes."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    t = L.lieb18()
    H = make_op(ed, 18, 9, 9, t, t, 4.0)
    D = H.rows()
    assert D == 48620 * 48620
    free, _ = torch.cuda.mem_get_info()
    if free < 64e9:
        pytest.skip("needs ~57 GB of free device memory")
    g = torch.Generator(device="cuda").manual_seed(18)
    x = torch.empty(D, dtype=torch.float64, device="cuda").uniform_(-1.0, 1.0, generator=g)
    y = torch.empty_like(x)
    H.Hubbard_mv(x, y)
    torch.cuda.synchronize()
    rng = np.random.default_rng(18)
    idx = np.concatenate([[0, D - 1], rng.integers(0, D, 20000)])
    up = orc.Tables(18, 9, t)

    def fetch(i):
        return x[torch.from_numpy(np.ascontiguousarray(i)).to("cuda")].cpu().numpy()

    ys, scale = orc.sampled_rows(up, up, 4.0, idx, fetch)
    yg = y[torch.from_numpy(idx).to("cuda")].cpu().numpy()
    assert np.all(np.abs(yg - ys) <= 1e-13 * scale + 1e-300)
    H.close()


def test_lieb18_two_pass_lanczos_matches_generic(ed, monkeypatch):
    """At full Lieb18 9+9 size the Lanczos recurrence through the two-pass
    matvec (permuted down index, L2-striped up term) gives the same alpha and
    beta, bit for bit, as through the generic kernel (4 steps each)."""
    import torch
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    free, _ = torch.cuda.mem_get_info()
    if free < 140e9:
        pytest.skip("needs ~130 GB of free device memory")
    t = L.lieb18()
    runs = {}
    for kind in ("", "generic"):
        if kind:
            monkeypatch.setenv("ED_MATVEC", kind)
        op = make_op(ed, 18, 9, 9, t, t, 4.0)
        assert op.matvec_kind == (kind or "two_pass")
        lz = ed.Lanczos()
        lz.eigen(op, max_steps=4, mode="fixed", ritz="none", seed=1)
        runs[kind or "auto"] = (lz.a, lz.b)
        op.close()
        monkeypatch.delenv("ED_MATVEC", raising=False)
    assert runs["auto"] == runs["generic"]


@pytest.mark.parametrize("case", ["chain8_35_disorder", "kagome12_22_flux", "chain8_44_U_dilute"])
def test_write_dense_matches_oracle(ed, orc, case):
    """Hubbard::Write: the dense matrix against the oracle's sparse
    Hamiltonian (real, complex Peierls, U on a subset of sites)."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    if case == "chain8_35_disorder":
        N, qu, qd, U, t, mask = 8, 3, 5, 2.0, L.chain(8, eps=list(philox_uniform(4, 8, 1.5))), None
    elif case == "kagome12_22_flux":
        N, qu, qd, U, t, mask = 12, 2, 2, 4.0, L.kagome12(flux=0.4), None
    else:
        N, qu, qd, U, t, mask = 8, 4, 4, 3.0, L.chain(8), 0b10110101
    op = make_op(ed, N, qu, qd, t, t, U, dilution=mask)
    H = op.Write()
    ref = orc.hamiltonian(N, qu, qd, t, t, U, mask=mask).toarray()
    assert H.shape == ref.shape
    assert np.max(np.abs(H - ref)) < 1e-14 * max(1.0, np.max(np.abs(ref)))
    x = philox_uniform(9, op.rows())
    if op.is_complex:
        x = x + 0j
    assert np.max(np.abs(H @ x - op.matvec(x))) < 1e-12 * np.max(np.abs(ref)) * np.sqrt(op.rows())


def test_operator_cache_same_hops_new_diagonal(ed, orc):
    """Operators whose hopping terms repeat (disorder realisations) reuse the
    cached off-diagonal tables; each one's matvec still matches the oracle,
    and rebuilding an operator gives the same outputs bit for bit."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    rng = np.random.default_rng(21)
    x = rng.standard_normal(ed.binom(10, 5) * ed.binom(10, 4))
    outs = {}
    for r in (0, 1, 0, 2):
        eu = list(philox_uniform(300 + r, 10, 6.0))
        ed_ = list(philox_uniform(400 + r, 10, 6.0))
        up, dn = L.chain(10, periodic=False, eps=eu), L.chain(10, periodic=False, eps=ed_)
        op = make_op(ed, 10, 5, 4, up, dn, 1.0)
        y = op.matvec(x)
        yo = orc.matvec(orc.Tables(10, 5, up), orc.Tables(10, 4, dn), 1.0, x, mask=orc.mask_all(10))
        assert rel_err(y, yo) < TOL, r
        if r in outs:
            assert np.array_equal(outs[r], y)
        outs[r] = y
        op.close()
