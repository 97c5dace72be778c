"""CPU oracle for the Hubbard ED hot path.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs may import this module; the product never does.

Two independent CPU paths are offered:
  * the C restatement of the reference (hubbard_oracle.c, built into
    _build/liboracle.so): reference ELL tables, the Hubbard_mv_ matvec,
    Lanczos::eigen, the continued fraction;
  * numpy/scipy: sparse Kronecker-sum Hamiltonians built from those tables
    (or, for Peierls phases, from the term semantics directly), dense
    eigensolves, SVD-based entanglement entropy.
Reference citations are in hubbard_oracle.c and in the docstrings below.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path
from typing import Iterable, List, Sequence, Tuple

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_TABLES = HERE / "_ref" / "ref_tables"

_lib = None


def load():
    """Load (building first if needed) the C restatement."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    lib = C.CDLL(str(LIB_PATH))
    vp, i64, dbl, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int
    sig = {
        "orc_binom": (i64, [i32, i32]),
        "orc_tbq_new": (vp, [i32, i32]),
        "orc_tbq_free": (None, [vp]),
        "orc_tbq_clear": (None, [vp]),
        "orc_make_h": (None, [vp, i32, i32, dbl]),
        "orc_make_j": (None, [vp, i32, i32, dbl]),
        "orc_make_n": (None, [vp, i32, dbl]),
        "orc_tbq_overflow": (i32, [vp]),
        "orc_tbq_count": (i64, [vp]),
        "orc_tbq_nslots": (i32, [vp]),
        "orc_tbq_ax": (vp, [vp]),
        "orc_tbq_aj": (vp, [vp]),
        "orc_tbq_state": (vp, [vp]),
        "orc_matvec": (None, [vp, vp, dbl, C.c_uint64, vp, vp]),
        "orc_matvec_z": (None, [vp, vp, dbl, C.c_uint64, vp, vp]),
        "orc_tridiag_eigval": (dbl, [i32, vp, vp, i32]),
        "orc_tridiag_eigvec": (None, [i32, vp, vp, dbl, vp]),
        "orc_lanczos": (i32, [vp, vp, dbl, C.c_uint64, vp, i32, i32, i32, vp, vp, vp, vp, vp]),
        "orc_continued_fraction": (None, [i32, vp, vp, dbl, dbl, i32, vp, vp, vp, vp]),
        "orc_num_threads": (i32, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class Tables:
    """One spin's reference tables built by the C restatement of H_TBq."""

    def __init__(self, N: int, Q: int, terms: Iterable[tuple] = ()):
        self.lib = load()
        self.N, self.Q = N, Q
        self.h = self.lib.orc_tbq_new(N, Q)
        self.count = int(self.lib.orc_tbq_count(self.h))
        self.nslots = int(self.lib.orc_tbq_nslots(self.h))
        for t in terms:
            self.add(t)

    def add(self, t: tuple) -> None:
        kind, i, j, v = t[0], t[1], t[2], t[3]
        if kind == "H":
            self.lib.orc_make_h(self.h, i, j, v)
        elif kind == "J":
            self.lib.orc_make_j(self.h, i, j, v)
        elif kind == "N":
            self.lib.orc_make_n(self.h, i, v)
        else:
            raise ValueError("the reference tables hold real Make_H/Make_J/Make_N terms only")

    @property
    def overflow(self) -> bool:
        return bool(self.lib.orc_tbq_overflow(self.h))

    def _arr(self, fn, dtype, n):
        ptr = fn(self.h)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double if dtype == np.float64 else C.c_int64)),
                                     shape=(n,)).copy()

    @property
    def Ax(self) -> np.ndarray:
        return self._arr(self.lib.orc_tbq_ax, np.float64, self.count * self.nslots).reshape(self.nslots, self.count)

    @property
    def Aj(self) -> np.ndarray:
        return self._arr(self.lib.orc_tbq_aj, np.int64, self.count * self.nslots).reshape(self.nslots, self.count)

    @property
    def state(self) -> np.ndarray:
        return self._arr(self.lib.orc_tbq_state, np.int64, self.count)

    def dense(self) -> np.ndarray:
        """Dense count x count matrix of the table (H_TBq::Write semantics,
        fermi_operator.h:227-235)."""
        M = np.zeros((self.count, self.count))
        ax, aj = self.Ax, self.Aj
        for s in range(self.nslots):
            nz = ax[s] != 0
            rows = np.nonzero(nz)[0]
            np.add.at(M, (rows, aj[s][nz]), ax[s][nz])
        return M

    def sparse(self):
        import scipy.sparse as sp
        ax, aj = self.Ax, self.Aj
        nz = ax != 0
        rows = np.broadcast_to(np.arange(self.count), ax.shape)[nz]
        return sp.csr_matrix((ax[nz], (rows, aj[nz])), shape=(self.count, self.count))

    def __del__(self):
        try:
            self.lib.orc_tbq_free(self.h)
        except Exception:
            pass


def mask_all(N: int) -> int:
    return (1 << N) - 1


# KagomeLattice12, DrudeWeight/src/drude_v2_cal_Kagome_randomHop.cu:794-808:
# Make_H(first[b], second[b], -r_i r_j) on the 24 bonds (lists :796-797), then
# Make_N(i, -2 r_i^2) on every site.  Restated here so that the CPU baseline
# builds the workload without the product package.
_KAGOME12_FIRST = (0, 1, 3, 4, 6, 7, 9, 10, 0, 2, 6, 8, 3, 5, 9, 11, 2, 1, 8, 7, 5, 4, 11, 10)
_KAGOME12_SECOND = (1, 3, 4, 0, 7, 9, 10, 6, 2, 6, 8, 0, 5, 9, 11, 3, 1, 11, 7, 5, 4, 8, 10, 2)


def kagome12_terms() -> List[tuple]:
    """The uniform (r_i = 1) KagomeLattice12 term list."""
    terms = [("H", i, j, -1.0, 0.0) for i, j in zip(_KAGOME12_FIRST, _KAGOME12_SECOND)]
    return terms + [("N", i, 0, -2.0, 0.0) for i in range(12)]


def philox_uniform(seed: int, n: int, scale: float = 1.0) -> np.ndarray:
    """scale * uniform(-1, 1) from numpy's Philox4x64-10 keyed by (seed, 0):
    the 52 high mantissa bits of each raw 64-bit word give a double in [1, 2),
    mapped to 2u - 3.  The library's counter-based start vector produces the
    same doubles."""
    bg = np.random.Philox(key=np.array([seed, 0], dtype=np.uint64))
    r = bg.random_raw(n)
    return scale * (((r >> np.uint64(12)) | np.uint64(0x3FF0000000000000)).view(np.float64) * 2.0 - 3.0)


def matvec(up: Tables, dn: Tables, U: float, x: np.ndarray, mask: int | None = None) -> np.ndarray:
    """Restated Hubbard_mv_ (HubMatrix_GPU.cuh:114-161) on the CPU."""
    lib = load()
    mask = mask_all(up.N) if mask is None else mask
    if np.iscomplexobj(x):
        xx = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(xx)
        lib.orc_matvec_z(up.h, dn.h, U, mask, _p(xx), _p(y))
    else:
        xx = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(xx)
        lib.orc_matvec(up.h, dn.h, U, mask, _p(xx), _p(y))
    return y


def lanczos(up: Tables, dn: Tables, U: float, f: np.ndarray, max_steps: int = 1000, mode: str = "reference",
            reorth: bool = False, want_evec: bool = True, mask: int | None = None):
    """Restated Lanczos::eigen (HubMatrix_GPU.cuh:561-613).  Returns
    (e0, alpha, beta, evec)."""
    lib = load()
    mask = mask_all(up.N) if mask is None else mask
    f = np.ascontiguousarray(f, dtype=np.float64)
    alpha = np.zeros(max_steps)
    beta = np.zeros(max_steps + 1)
    n = C.c_int(0)
    e0 = C.c_double(0.0)
    evec = np.zeros(f.size) if want_evec else None
    st = lib.orc_lanczos(up.h, dn.h, U, mask, _p(f), max_steps, 0 if mode == "reference" else 1, 1 if reorth else 0,
                         _p(alpha), _p(beta), C.byref(n), C.byref(e0), _p(evec) if want_evec else None)
    if st != 0:
        raise RuntimeError(f"orc_lanczos failed: {st}")
    k = n.value
    return e0.value, alpha[:k], beta[: k + 1], evec


def tridiag_lowest(alpha: Sequence[float], off: Sequence[float]) -> Tuple[float, np.ndarray]:
    lib = load()
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    b = np.ascontiguousarray(off, dtype=np.float64)
    if b.size == 0:
        b = np.zeros(1)
    lam = lib.orc_tridiag_eigval(a.size, _p(a), _p(b), 0)
    z = np.zeros(a.size)
    lib.orc_tridiag_eigvec(a.size, _p(a), _p(b), lam, _p(z))
    return lam, z


def continued_fraction(alpha, beta, norm2: float, energy: float, omega: np.ndarray) -> np.ndarray:
    """correlator_continued_fraction (HubMatrix_GPU.cuh:820-835): g(w) for
    complex w; beta[0] unused, beta[i+1] couples i and i+1."""
    lib = load()
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    b = np.ascontiguousarray(beta, dtype=np.float64)
    w = np.ascontiguousarray(omega, dtype=np.complex128)
    wr, wi = np.ascontiguousarray(w.real), np.ascontiguousarray(w.imag)
    gr, gi = np.zeros(w.size), np.zeros(w.size)
    lib.orc_continued_fraction(a.size, _p(a), _p(b), norm2, energy, w.size, _p(wr), _p(wi), _p(gr), _p(gi))
    return gr + 1j * gi


# ---------------------------------------------------------------- numpy side --

def popcount(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64)
    c = np.zeros(v.shape, dtype=np.int64)
    while np.any(v):
        c += (v & np.uint64(1)).astype(np.int64)
        v = v >> np.uint64(1)
    return c


def spin_matrix(N: int, Q: int, terms: Sequence[tuple]):
    """Sparse one-spin matrix from the term semantics, independent of the
    ELL tables (used for Peierls terms, which the reference lacks).
    H: t (c+_i c_j + h.c.);  J: +t when row empty at i and full at j, else -t;
    N: v n_i;  P: t e^{+i phi} when the particle moved i -> j (row full at j),
    t e^{-i phi} otherwise.  Jordan-Wigner sign (-1)^(particles strictly
    between i and j) as in fermi_operator.h:26-40."""
    import scipy.sparse as sp
    states = np.array([n for n in range(1 << N) if bin(n).count("1") == Q], dtype=np.int64)
    address = {int(s): k for k, s in enumerate(states)}
    rows, cols, vals = [], [], []
    cplx = any(t[0] == "P" for t in terms)
    for kind, i, j, v, ph in [tuple(t) + (0.0,) * (5 - len(t)) for t in terms]:
        for a, n in enumerate(states):
            n = int(n)
            if kind == "N":
                if (n >> i) & 1:
                    rows.append(a); cols.append(a); vals.append(v)
                continue
            oi, oj = (n >> i) & 1, (n >> j) & 1
            if oi == oj:
                continue
            lo, hi = min(i, j), max(i, j)
            between = bin(n & (((1 << (hi - lo - 1)) - 1) << (lo + 1))).count("1") if hi - lo > 1 else 0
            sign = -1.0 if between & 1 else 1.0
            b = address[n ^ ((1 << i) | (1 << j))]
            if kind == "H":
                val = sign * v
            elif kind == "J":
                val = sign * v if (oi == 0 and oj == 1) else -sign * v
            else:
                phase = ph if oj == 1 else -ph
                val = sign * v * complex(math.cos(phase), math.sin(phase))
            rows.append(a); cols.append(b); vals.append(val)
    dt = np.complex128 if cplx else np.float64
    return sp.csr_matrix((np.array(vals, dtype=dt), (rows, cols)), shape=(len(states), len(states))), states


def hamiltonian(N: int, Qup: int, Qdn: int, up_terms, dn_terms, U: float, mask: int | None = None):
    """Sparse H = A_up (x) 1 + 1 (x) A_dn + U diag(popc(s_up & s_dn & mask)),
    up-index-major like the reference vectors."""
    import scipy.sparse as sp
    Au, su = spin_matrix(N, Qup, up_terms)
    Ad, sd = spin_matrix(N, Qdn, dn_terms)
    mask = mask_all(N) if mask is None else mask
    du = popcount((su[:, None] & sd[None, :]) & mask).ravel().astype(np.float64)
    H = sp.kron(Au, sp.identity(Ad.shape[0]), format="csr") + sp.kron(sp.identity(Au.shape[0]), Ad, format="csr")
    return (H + sp.diags(U * du)).tocsr()


def entanglement_entropy(psi: np.ndarray, N: int, Qup: int, Qdn: int, Asites: Sequence[int]):
    """Half-system entropy of psi (up-index-major).  Reshape as
    EEmatHubAB::Make_Write (MBL_test/include/entangle_entropy.h:22-44,
    177-197): row = idxUP_A*dimADN + idxDN_A, col = idxUP_B*dimBDN + idxDN_B,
    labels in order of first appearance.  Returns (S_vN, S_ref) with
    S_vN = -sum s^2 ln s^2 and S_ref = -sum s ln s (the reference's sum,
    MBL_test/src/Hubbard_EE_test.cu:80-83), s the singular values."""
    A = 0
    for s in Asites:
        A |= 1 << s
    B = ((1 << N) - 1) ^ A

    def labels(Q):
        states = [n for n in range(1 << N) if bin(n).count("1") == Q]
        la, lb = {}, {}
        ia, ib = [], []
        for n in states:
            a, b = n & A, n & B
            if a not in la:
                la[a] = len(la)
            if b not in lb:
                lb[b] = len(lb)
            ia.append(la[a]); ib.append(lb[b])
        return np.array(ia), np.array(ib), len(la), len(lb)

    ua, ub, nua, nub = labels(Qup)
    da, db, nda, ndb = labels(Qdn)
    M = np.zeros((nua * nda, nub * ndb), dtype=psi.dtype)
    P = psi.reshape(len(ua), len(da))
    rows = ua[:, None] * nda + da[None, :]
    cols = ub[:, None] * ndb + db[None, :]
    M[rows, cols] = P
    s = np.linalg.svd(M, compute_uv=False)
    s = s[s > 0]
    p = s * s
    p = p[p > 0]
    return float(-np.sum(p * np.log(p))), float(-np.sum(s * np.log(s)))


def ref_tables(N: int, Q: int, terms: Sequence[tuple]):
    """Run the reference's own H_TBq (oracle/_ref/ref_tables, built from the
    reference sources by `make -C oracle ref`).  Returns (state, address, Ax,
    Aj) or None when the dumper is not built."""
    if not REF_TABLES.exists():
        return None
    lines = [f"{N} {Q}"]
    for kind, i, j, v, *_ in terms:
        if kind == "N":
            lines.append(f"N {i} {v!r}")
        else:
            lines.append(f"{kind} {i} {j} {v!r}")
    lines.append("E")
    out = subprocess.run([str(REF_TABLES)], input="\n".join(lines).encode(), capture_output=True, check=True).stdout
    count, nslots = np.frombuffer(out[:8], dtype=np.int32)
    off = 8
    state = np.frombuffer(out[off:off + 4 * count], dtype=np.int32).astype(np.int64); off += 4 * count
    address = np.frombuffer(out[off:off + 4 * (1 << N)], dtype=np.int32).astype(np.int64); off += 4 * (1 << N)
    ax = np.frombuffer(out[off:off + 8 * count * nslots], dtype=np.float64).reshape(nslots, count); off += 8 * count * nslots
    aj = np.frombuffer(out[off:off + 4 * count * nslots], dtype=np.int32).astype(np.int64).reshape(nslots, count)
    return state, address, ax.copy(), aj


def num_threads() -> int:
    return int(load().orc_num_threads())


def sampled_rows(up: Tables, dn: Tables, U: float, idx: np.ndarray, fetch, mask: int | None = None):
    """Hubbard_mv_ (HubMatrix_GPU.cuh:114-161) restated for selected output
    elements only, for vectors too large for the host: y[i] for the flat
    indices i = u * dim_dn + d in idx, with x read through fetch(flat indices)
    -> float64 values.  Returns (y, scale) where scale[i] = sum of |terms|,
    the size the rounding of y[i] is measured against."""
    mask = mask_all(up.N) if mask is None else mask
    idx = np.asarray(idx, dtype=np.int64)
    nd = dn.count
    u, d = idx // nd, idx % nd
    axu, aju = up.Ax[:, u], up.Aj[:, u]          # (slots, n)
    axd, ajd = dn.Ax[:, d], dn.Aj[:, d]
    xu = fetch((aju * nd + d[None, :]).ravel()).reshape(axu.shape)
    xd = fetch((u[None, :] * nd + ajd).ravel()).reshape(axd.shape)
    x0 = fetch(idx)
    occ = np.array([bin(int(a) & int(b) & mask).count("1") for a, b in zip(up.state[u], dn.state[d])], dtype=np.float64)
    tu, td, t0 = axu * xu, axd * xd, U * occ * x0
    y = tu.sum(0) + td.sum(0) + t0
    scale = np.abs(tu).sum(0) + np.abs(td).sum(0) + np.abs(t0)
    return y, scale


def sxy_matvec(up: Tables, dn: Tables, x: np.ndarray) -> np.ndarray:
    """S_xy = (S+S- + S-S+)/2 on the product basis, restated from
    TotalSpin/include/HubMatrix_TotalSpin.cuh:20-66 (loop over site pairs
    i < j, vectorised over the basis): for a pair of singly occupied sites of
    opposite spin the exchanged state contributes -x (even number of
    particles strictly between i and j in the exchanged words) or +x; the
    diagonal is popcount(up ^ dn) / 2."""
    N = up.N
    su, sd = up.state.astype(np.uint64), dn.state.astype(np.uint64)
    nu, nd = su.size, sd.size
    U = np.repeat(su, nd)
    Dn = np.tile(sd, nu)
    xv = np.asarray(x).reshape(-1)
    one = np.uint64(1)

    def bit(w, i):
        return (w >> np.uint64(i)) & one

    def popc(w):
        c = np.zeros(w.shape, dtype=np.int64)
        for b in range(N):
            c += bit(w, b).astype(np.int64)
        return c

    y = 0.5 * popc(U ^ Dn) * xv
    for i in range(N):
        for j in range(i + 1, N):
            iup, idn, jup, jdn = bit(U, i), bit(Dn, i), bit(U, j), bit(Dn, j)
            sel = (iup != idn) & (iup == jdn) & (idn == jup)
            if not np.any(sel):
                continue
            ex = np.uint64((1 << i) | (1 << j))
            u2, d2 = U[sel] ^ ex, Dn[sel] ^ ex
            between = np.uint64(((1 << j) - 1) & ~((1 << (i + 1)) - 1))
            sgn = popc(u2 & between) + popc(d2 & between)
            k = np.searchsorted(su, u2) * nd + np.searchsorted(sd, d2)
            v = xv[k]
            y[np.nonzero(sel)[0]] += np.where(sgn % 2 == 0, -v, v)
    return y
