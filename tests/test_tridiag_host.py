"""The host tridiagonal eigensolver and Krylov propagator (no GPU): all
eigenpairs against scipy's eigh_tridiagonal, exp(-i T t) e_0 against
scipy.linalg.expm, on random matrices, Lanczos-like matrices with clustered
(ghost) eigenvalues, and split / tiny cases."""
import numpy as np
import pytest
import scipy.linalg as sl


def dense(a, b):
    return np.diag(a) + np.diag(b, 1) + np.diag(b, -1)


def cases():
    rng = np.random.default_rng(7)
    yield rng.standard_normal(1), np.zeros(0)
    yield np.array([1.0, -2.0]), np.array([0.5])
    yield rng.standard_normal(40), rng.standard_normal(39)
    b = rng.standard_normal(59)
    b[[10, 30]] = 0.0  # three decoupled blocks
    yield rng.standard_normal(60), b
    yield np.full(30, 2.0), np.full(29, 1e-9)  # near-degenerate
    # a plain Lanczos T on a 200-dim diagonal matrix run 150 steps: ghosts
    d = np.sort(rng.uniform(-5, 5, 200))
    q = rng.standard_normal(200)
    q /= np.linalg.norm(q)
    al, be, qp = [], [], np.zeros(200)
    bprev = 0.0
    for _ in range(150):
        w = d * q - bprev * qp
        a = q @ w
        w -= a * q
        bn = np.linalg.norm(w)
        al.append(a)
        be.append(bn)
        qp, q, bprev = q, w / bn, bn
    yield np.array(al), np.array(be[:-1])


@pytest.mark.parametrize("k", range(6))
def test_tridiag_eigen_against_scipy(edlib, k):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev
    a, b = list(cases())[k]
    w, Z = ev.tridiag_eigen(a, b)
    wr = sl.eigh_tridiagonal(a, b, eigvals_only=True) if a.size > 1 else a.copy()
    scale = max(1.0, np.max(np.abs(wr)))
    assert np.max(np.abs(w - wr)) < 1e-13 * scale * a.size
    T = dense(a, b)
    assert np.max(np.abs(Z.T @ Z - np.eye(a.size))) < 1e-13 * a.size
    assert np.max(np.abs(T @ Z - Z * w)) < 1e-13 * scale * a.size


@pytest.mark.parametrize("k", range(6))
def test_tridiag_expm_against_scipy(edlib, k):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import evolution as ev
    a, b = list(cases())[k]
    times = [0.0, 0.02, 0.7, 3.0, 25.0]
    c = ev.tridiag_expm(a, b, times)
    T = dense(a, b)
    for i, t in enumerate(times):
        ref = sl.expm(-1j * t * T)[:, 0]
        assert np.max(np.abs(c[i] - ref)) < 1e-12 * max(1.0, abs(t) * np.max(np.abs(T)))
        assert abs(np.linalg.norm(c[i]) - 1.0) < 1e-13 * a.size


def test_tridiag_bad_arguments(edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    lib = _capi.load()
    assert lib.ed_tridiag_eigen(0, None, None, None, None) == 1  # ED_ERR_ARG
    assert lib.ed_tridiag_expm(3, None, None, 1, None, None) == 1  # ED_ERR_ARG


@pytest.mark.parametrize("n", [1, 2, 7, 40])
def test_dense_sym_eigen_against_numpy(edlib, n):
    """The Rayleigh-Ritz solve of ed_eigs_lowest (cyclic Jacobi) against
    numpy's eigh, including a matrix with a repeated eigenvalue."""
    import ctypes as C
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    if n >= 7:
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        d = np.sort(rng.standard_normal(n))
        d[3] = d[2]
        A = (Q * d) @ Q.T
    a = np.asfortranarray(A)
    w = np.empty(n)
    z = np.empty((n, n), order="F")
    assert _capi.load().ed_dense_sym_eigen(n, a.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p),
                                           z.ctypes.data_as(C.c_void_p)) == 0
    wr = np.linalg.eigvalsh(A)
    assert np.max(np.abs(w - wr)) < 1e-13 * max(1.0, np.max(np.abs(wr))) * n
    assert np.max(np.abs(z.T @ z - np.eye(n))) < 1e-13 * n
    assert np.max(np.abs(A @ z - z * w)) < 1e-13 * max(1.0, np.max(np.abs(wr))) * n


def bidiag_cases():
    rng = np.random.default_rng(11)
    yield np.array([3.0]), np.zeros(0)
    yield rng.standard_normal(2), rng.standard_normal(1)
    yield rng.standard_normal(50), rng.standard_normal(49)
    d = rng.standard_normal(40)
    d[[0, 17, 39]] = 0.0  # zero diagonal entries, top / middle / bottom
    yield d, rng.standard_normal(39)
    e = rng.standard_normal(59)
    e[[5, 30]] = 0.0
    yield rng.standard_normal(60), e
    # graded: singular values over 30 decades, as a ground state's Schmidt values
    yield np.exp(-np.arange(80) * 0.9), np.exp(-np.arange(79) * 0.9) * 0.3
    # the bidiagonal of a Householder reduction of a low-rank-plus-noise block
    A = rng.standard_normal((120, 5)) @ rng.standard_normal((5, 100)) + 1e-13 * rng.standard_normal((120, 100))
    yield householder_bidiag(A)


def householder_bidiag(A):
    """(d, e) of an upper bidiagonal B with the singular values of A (m >= n),
    by alternating Householder reflections (numpy, small sizes)."""
    A = A.copy()
    m, n = A.shape
    d, e = np.zeros(n), np.zeros(max(n - 1, 0))

    def reflect(x):
        a, rest = x[0], np.linalg.norm(x[1:])
        if rest == 0.0:
            return np.zeros_like(x), 0.0, a
        b = -np.copysign(np.hypot(a, rest), a)
        v = x.copy()
        v[0] = 1.0
        v[1:] = x[1:] / (a - b)
        return v, (b - a) / b, b

    for k in range(n):
        v, tau, d[k] = reflect(A[k:, k])
        A[k:, k + 1:] -= tau * np.outer(v, v @ A[k:, k + 1:])
        if k < n - 1:
            u, tau, e[k] = reflect(A[k, k + 1:])
            A[k + 1:, k + 1:] -= tau * np.outer(A[k + 1:, k + 1:] @ u, u)
    return d, e


@pytest.mark.parametrize("k", range(7))
def test_bidiag_singular_values_against_numpy(edlib, k):
    import ctypes as C
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    d, e = list(bidiag_cases())[k]
    n = d.size
    B = np.diag(d) + (np.diag(e, 1) if n > 1 else 0)
    ref = np.linalg.svd(B, compute_uv=False)
    s = np.empty(n)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    ee = np.ascontiguousarray(e) if n > 1 else np.zeros(1)
    assert _capi.load().ed_bidiag_singular_values(n, ptr(np.ascontiguousarray(d)), ptr(ee), ptr(s)) == 0
    assert np.max(np.abs(s - ref)) < 8e-16 * n * ref[0]
    if k == 5:  # graded values keep about eps * |B| absolute accuracy
        assert np.max(np.abs(s - ref)) < 1e-15
