"""C-ABI library: loads, exports the header's symbols, and its host-side
functions (basis, reference ELL export, start-vector generator, argument
checks) are bit-exact against the reference fixtures.  No GPU needed."""
import hashlib
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, philox_uniform


def header_functions():
    text = (ROOT / "include" / "ed_hubbard.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ed_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_function(edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    names = header_functions()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", str(_capi.lib_path())], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (ed_[a-z0-9_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(edlib, n)
    # the binding declares every exported function
    assert set(names) == set(_capi.SIGNATURES), set(names) ^ set(_capi.SIGNATURES)


def test_status_strings(edlib):
    assert edlib.ed_status_string(0) == b"ok"
    assert b"argument" in edlib.ed_status_string(1)
    assert edlib.ed_version() >= 100


def test_rank_unrank_exhaustive(ed):
    from math import comb
    for N in range(1, 15):
        for Q in range(0, N + 1):
            words = np.array([n for n in range(1 << N) if bin(n).count("1") == Q], dtype=np.uint64)
            assert words.size == comb(N, Q) == ed.binom(N, Q)
            got = ed.basis_unrank(N, Q, np.arange(words.size))
            assert np.array_equal(got, words), (N, Q)
            assert np.array_equal(ed.basis_rank(N, Q, words), np.arange(words.size)), (N, Q)


def test_rank_unrank_large_and_64bit(ed):
    rng = np.random.default_rng(9)
    for N, Q in ((18, 9), (24, 12), (40, 7), (62, 31)):
        count = ed.binom(N, Q)
        r = rng.integers(0, count, size=2000, dtype=np.int64)
        w = ed.basis_unrank(N, Q, r)
        assert all(bin(int(x)).count("1") == Q and int(x) < (1 << N) for x in w[:200])
        assert np.array_equal(ed.basis_rank(N, Q, w), r)
        # ascending-integer order == rank order
        order = np.argsort(r)
        assert np.all(np.diff(w[order].astype(object)) > 0) or len(set(r)) < len(r)


def test_rank_rejects_wrong_popcount(ed):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300._capi import EdError
    with pytest.raises(EdError):
        ed.basis_rank(8, 4, np.array([7], dtype=np.uint64))


def test_states_match_reference_fixtures(ed, golden_tables):
    meta, arrays = golden_tables
    for name, m in meta["small"].items():
        h = ed.H_TBq(m["N"], m["Q"])
        assert np.array_equal(h.state.astype(np.int64), arrays[f"{name}__state"]), name


def test_ell_export_bit_exact(ed, golden_tables):
    meta, arrays = golden_tables
    for name, m in meta["small"].items():
        h = ed.H_TBq(m["N"], m["Q"]).extend([tuple(x) for x in m["terms"]])
        ax, aj = h.ell()
        assert np.array_equal(ax, arrays[f"{name}__ax"]), name
        assert np.array_equal(aj, arrays[f"{name}__aj"].astype(np.int64)), name


def test_ell_export_digest_large(ed, golden_tables):
    meta, _ = golden_tables
    for name, m in meta["large"].items():
        h = ed.H_TBq(m["N"], m["Q"]).extend([tuple(x) for x in m["terms"]])
        ax, aj = h.ell()
        d = hashlib.sha256()
        d.update(h.state.astype(np.int64).tobytes())
        d.update(ax.tobytes())
        d.update(aj.tobytes())
        assert d.hexdigest() == m["sha256"], name


def test_start_vector_is_philox4x64(ed):
    for seed in (0, 1, 235, 2**40 + 3):
        for n in (1, 3, 4, 1001):
            assert np.array_equal(ed.random_vector(n, seed), philox_uniform(seed, n))


def test_op_create_argument_errors(edlib):
    import ctypes as C
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    d = _capi.ed_model_desc()
    h = C.c_void_p()
    d.n_sites, d.n_up, d.n_dn = 0, 0, 0
    assert edlib.ed_op_create(C.byref(h), C.byref(d), 0) == 1
    d.n_sites, d.n_up, d.n_dn = 8, 9, 4
    assert edlib.ed_op_create(C.byref(h), C.byref(d), 0) == 1
    # a term on a site outside the lattice
    terms = (_capi.ed_term * 1)()
    terms[0].kind, terms[0].i, terms[0].j, terms[0].value = 0, 0, 8, -1.0
    d.n_sites, d.n_up, d.n_dn = 8, 4, 4
    d.up_terms, d.n_up_terms = terms, 1
    assert edlib.ed_op_create(C.byref(h), C.byref(d), 0) == 1
    # a Peierls term in a real operator
    terms[0].kind, terms[0].j = 3, 1
    assert edlib.ed_op_create(C.byref(h), C.byref(d), 0) == 1
    # null pointers
    assert edlib.ed_op_create(None, C.byref(d), 0) == 1
    assert edlib.ed_op_perform(None, None, None, 0, None) == 1
    assert edlib.ed_lanczos_run(None, None, None, 0, None, 0, None, None, None, None) == 1
    assert edlib.ed_entanglement_entropy_batch(None, 1, None, 0, 0, None, None, None) == 1
    assert edlib.ed_op_matvec_kind(None) == -1


def test_op_create_cached_tables_still_check_onsite_sites(edlib):
    """A second operator with the same hopping terms reuses the cached
    off-diagonal tables; its on-site terms are still checked (a site outside
    the lattice is an argument error, not a silent table hit)."""
    import ctypes as C
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    hops = [(0, i, (i + 1) % 8, -1.0) for i in range(8)]
    def desc(extra):
        t = hops + extra
        arr = (_capi.ed_term * len(t))()
        for k, (kind, i, j, v) in enumerate(t):
            arr[k].kind, arr[k].i, arr[k].j, arr[k].value = kind, i, j, v
        d = _capi.ed_model_desc()
        d.n_sites, d.n_up, d.n_dn = 8, 3, 3
        d.up_terms, d.n_up_terms = arr, len(t)
        d.dn_terms, d.n_dn_terms = arr, len(t)
        return d, arr
    h = C.c_void_p()
    d1, keep1 = desc([(2, 3, 0, 0.5)])
    st = edlib.ed_op_create(C.byref(h), C.byref(d1), 0)  # fills the cache (no device here: it may stop later)
    if st == 0:
        edlib.ed_op_destroy(h)
    d2, keep2 = desc([(2, 9, 0, 0.5)])  # Make_N on site 9 of 8
    assert edlib.ed_op_create(C.byref(h), C.byref(d2), 0) == 1


def test_ell_rejects_peierls(edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    terms = (_capi.ed_term * 1)()
    terms[0].kind, terms[0].i, terms[0].j, terms[0].value, terms[0].phase = 3, 0, 1, -1.0, 0.3
    assert edlib.ed_tables_ell(4, 2, terms, 1, None, None, None) == 1


def test_lattice_tables():
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    assert len(L.kagome12()) == 24 + 12
    assert len(L.lieb18()) == 24
    assert len(L.chain(8)) == 8 and len(L.chain(12, periodic=False)) == 11
    # every Kagome site has coordination 4, every Lieb18 corner 4 and edge 2
    deg = np.zeros(12, int)
    for i, j in zip(L.KAGOME12_FIRST, L.KAGOME12_SECOND):
        deg[i] += 1; deg[j] += 1
    assert set(deg) == {4}
    deg = np.zeros(18, int)
    for i, j in zip(L.LIEB18_FIRST, L.LIEB18_SECOND):
        deg[i] += 1; deg[j] += 1
    assert sorted(set(deg)) == [2, 4]


@pytest.mark.parametrize("n", [1, 2, 3, 17, 100, 301, 1000])
def test_tridiagonal_lowest_vs_scipy(edlib, n):
    """ed_tridiag_lowest (host bisection + inverse iteration, the Lanczos T
    eigensolve) against scipy's LAPACK tridiagonal solver."""
    import numpy as np
    from scipy.linalg import eigh_tridiagonal
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300.hubbard import tridiag_lowest
    rng = np.random.default_rng(n)
    a = rng.normal(size=n) * 3
    b = np.abs(rng.normal(size=max(n - 1, 0))) + 1e-3
    lam, z = tridiag_lowest(a, b)
    w, V = eigh_tridiagonal(a, b) if n > 1 else (a, np.ones((1, 1)))
    assert abs(lam - w[0]) < 1e-12 * max(1.0, np.max(np.abs(w)))
    assert abs(abs(z @ V[:, 0]) - 1.0) < 1e-9
    assert np.max(np.abs(z)) == np.max(z)  # largest component positive
