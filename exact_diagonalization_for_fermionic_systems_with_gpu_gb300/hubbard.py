"""Host-side mirror of the reference's operator surface over the C ABI.

Names and argument meaning follow the reference so that drivers read alike:

* ``H_TBq``      — one spin's basis and term list
                   (MBL_test/include/fermi_operator.h:42-242)
* ``Hubbard``    — the device operator: ``Hubbard_mv(x, y)`` on device
                   vectors (HubMatrix_GPU.cuh:30-182) and the Spectra concept
                   ``rows()/cols()/perform_op(x, y)`` on host arrays
                   (TotalSpin/include/HubMatrix_TotalSpin.cuh:181-322)
* ``Lanczos``    — ``random_vector`` / ``eigen`` / ``tridiagonal``
                   (HubMatrix_GPU.cuh:477-613)

All arithmetic runs in the compiled sm_103a library; numpy arrays and torch
tensors are only containers here.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from . import _capi
from ._capi import check

_KIND = {"H": _capi.ED_TERM_HOP, "J": _capi.ED_TERM_CURRENT, "N": _capi.ED_TERM_DENSITY, "P": _capi.ED_TERM_PEIERLS}


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def binom(n: int, k: int) -> int:
    return int(_capi.load().ed_binom(n, k))


def basis_unrank(n_sites: int, n_part: int, ranks) -> np.ndarray:
    r = np.ascontiguousarray(ranks, dtype=np.int64)
    out = np.empty(r.shape, dtype=np.uint64)
    check(_capi.load().ed_basis_unrank(n_sites, n_part, _ptr(r), r.size, _ptr(out)), "ed_basis_unrank")
    return out


def basis_rank(n_sites: int, n_part: int, words) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.empty(w.shape, dtype=np.int64)
    check(_capi.load().ed_basis_rank(n_sites, n_part, _ptr(w), w.size, _ptr(out)), "ed_basis_rank")
    return out


def random_vector(n: int, seed: int = 0) -> np.ndarray:
    """uniform(-1,1) start vector from Philox4x64-10 keyed by seed (not normalised)."""
    out = np.empty(int(n), dtype=np.float64)
    check(_capi.load().ed_random_vector(int(n), int(seed), _ptr(out)), "ed_random_vector")
    return out


def tridiag_lowest(alpha: Sequence[float], offdiag: Sequence[float]):
    """Lowest eigenpair of a symmetric tridiagonal matrix (host solver of the
    Lanczos T: Sturm bisection and inverse iteration)."""
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    o = np.ascontiguousarray(offdiag, dtype=np.float64)
    n = a.size
    e0 = np.zeros(1)
    z = np.zeros(n)
    check(_capi.load().ed_tridiag_lowest(n, _ptr(a), _ptr(o) if n > 1 else None, _ptr(e0), _ptr(z)),
          "ed_tridiag_lowest")
    return float(e0[0]), z


class H_TBq:
    """Basis and term list of one spin species (fermi_operator.h:42-242).

    ``Make_H / Make_J / Make_N`` record the same calls the reference makes;
    the tables are built inside the library when a ``Hubbard`` is created.
    """

    def __init__(self, N: int, Q: int):
        if not (1 <= N <= 62 and 0 <= Q <= N):
            raise ValueError("need 1 <= N <= 62 and 0 <= Q <= N")
        self.N, self.Q = int(N), int(Q)
        self.terms: List[tuple] = []

    @property
    def count(self) -> int:
        return binom(self.N, self.Q)

    @property
    def dim(self) -> int:
        return 1 << self.N

    @property
    def state(self) -> np.ndarray:
        return basis_unrank(self.N, self.Q, np.arange(self.count, dtype=np.int64))

    @property
    def address(self) -> np.ndarray:
        """address[word] = rank, -1 for words with the wrong popcount (N <= 26)."""
        if self.N > 26:
            raise ValueError("address table only for N <= 26")
        addr = np.full(1 << self.N, -1, dtype=np.int64)
        addr[self.state.astype(np.int64)] = np.arange(self.count, dtype=np.int64)
        return addr

    def Make_H(self, i: int, j: int, t: float) -> None:
        self.terms.append(("H", int(i), int(j), float(t), 0.0))

    def Make_J(self, i: int, j: int, t: float) -> None:
        self.terms.append(("J", int(i), int(j), float(t), 0.0))

    def Make_N(self, i: int, v: float) -> None:
        self.terms.append(("N", int(i), 0, float(v), 0.0))

    def Make_Peierls(self, i: int, j: int, t: float, phase: float) -> None:
        self.terms.append(("P", int(i), int(j), float(t), float(phase)))

    def extend(self, terms) -> "H_TBq":
        self.terms.extend(terms)
        return self

    def clear(self) -> None:
        self.terms = []

    def ctypes_terms(self):
        arr = (_capi.ed_term * max(len(self.terms), 1))()
        for k, (kind, i, j, v, ph) in enumerate(self.terms):
            arr[k].kind = _KIND[kind]
            arr[k].i, arr[k].j = i, j
            arr[k].value, arr[k].phase = v, ph
        return arr

    def ell(self):
        """The reference's own ELL tables (Ax, Aj) for this term list,
        slot-major with 10*Q+1 slots: arrays of shape (10*Q+1, count)."""
        ns = 10 * self.Q + 1
        ax = np.zeros(ns * self.count, dtype=np.float64)
        aj = np.zeros(ns * self.count, dtype=np.int64)
        t = self.ctypes_terms()
        check(_capi.load().ed_tables_ell(self.N, self.Q, t, len(self.terms), _ptr(ax), _ptr(aj), None),
              "ed_tables_ell")
        return ax.reshape(ns, self.count), aj.reshape(ns, self.count)


class Hubbard:
    """H = H_up (x) 1 + 1 (x) H_dn + U sum_i n_up n_dn on the device.

    ``dilution``: bit mask of the sites where U acts (the reference's
    dilution word, HubMatrix_GPU.cuh:72-95); None = all sites.
    ``complex_``: build a complex operator (needed for Peierls terms).
    """

    def __init__(self, HqUP: H_TBq, HqDN: H_TBq, U: float = 0.0, dilution: Optional[int] = None,
                 device: int = 0, complex_: Optional[bool] = None):
        if HqUP.N != HqDN.N:
            raise ValueError("both spins need the same number of sites")
        lib = _capi.load()
        if complex_ is None:
            complex_ = any(t[0] == "P" for t in HqUP.terms + HqDN.terms)
        self._up_terms = HqUP.ctypes_terms()
        self._dn_terms = HqDN.ctypes_terms()
        d = _capi.ed_model_desc()
        d.n_sites, d.n_up, d.n_dn = HqUP.N, HqUP.Q, HqDN.Q
        d.flags = _capi.ED_OP_COMPLEX if complex_ else _capi.ED_OP_REAL
        d.up_terms, d.n_up_terms = self._up_terms, len(HqUP.terms)
        d.dn_terms, d.n_dn_terms = self._dn_terms, len(HqDN.terms)
        d.U = float(U)
        d.interaction_mask = 0 if dilution is None else int(dilution)
        h = C.c_void_p()
        check(lib.ed_op_create(C.byref(h), C.byref(d), int(device)), "ed_op_create")
        self._h = h
        self._lib = lib
        self.U = float(U)
        self.N = HqUP.N
        self.device = int(device)
        self.dimUP = int(lib.ed_op_dim_up(h))
        self.dimDN = int(lib.ed_op_dim_dn(h))
        self.is_complex = bool(lib.ed_op_is_complex(h))
        self.matvec_kind = ("generic", "rows", "two_pass")[lib.ed_op_matvec_kind(h)]

    # -- Spectra concept (TotalSpin/include/HubMatrix_TotalSpin.cuh:279-311) --
    def rows(self) -> int:
        return int(self._lib.ed_op_rows(self._h))

    def cols(self) -> int:
        return int(self._lib.ed_op_cols(self._h))

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def perform_op(self, x: np.ndarray, y: np.ndarray) -> None:
        """y = H x on host arrays (synchronous, y overwritten)."""
        dt = np.complex128 if self.is_complex else np.float64
        if x.dtype != dt or y.dtype != dt or not x.flags.c_contiguous or not y.flags.c_contiguous:
            raise TypeError(f"perform_op needs C-contiguous {dt.__name__} arrays")
        if x.size != self.rows() or y.size != self.rows():
            raise ValueError("vector length must equal rows()")
        check(self._lib.ed_op_perform(self._h, _ptr(x), _ptr(y), _capi.ED_MEM_HOST, None), "ed_op_perform")

    def matvec(self, x: np.ndarray) -> np.ndarray:
        dt = np.complex128 if self.is_complex else np.float64
        x = np.ascontiguousarray(x, dtype=dt)
        y = np.empty_like(x)
        self.perform_op(x, y)
        return y

    # -- device vectors (HubMatrix_GPU.cuh:163-182) --------------------------
    def Hubbard_mv(self, x, y, stream=None) -> None:
        """y = H x on torch CUDA tensors (float64, or complex128 for complex
        operators); asynchronous on the given (default: current) stream."""
        import torch
        want = torch.complex128 if self.is_complex else torch.float64
        for t in (x, y):
            if not (t.is_cuda and t.dtype == want and t.is_contiguous() and t.numel() == self.rows()):
                raise TypeError(f"Hubbard_mv needs contiguous CUDA {want} tensors of length rows()")
        s = stream if stream is not None else torch.cuda.current_stream(x.device)
        check(self._lib.ed_op_perform(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                      _capi.ED_MEM_DEVICE, C.c_void_p(s.cuda_stream)), "ed_op_perform")

    def Write(self) -> np.ndarray:
        """The dense matrix (rows x rows, complex for complex operators)
        (Hubbard::Write, HubMatrix_GPU.cuh:224-240)."""
        n = self.rows()
        H = np.empty((n, 2 * n) if self.is_complex else (n, n))
        check(_capi.load().ed_op_write_dense(self.handle, _ptr(H), _capi.ED_MEM_HOST, None), "ed_op_write_dense")
        return H.view(np.complex128) if self.is_complex else H

    def autotune(self, steps: int = 30, apply: bool = True) -> dict:
        """ed_op_autotune: time the Lanczos step's kernel choices on this
        operator and (apply) keep the fastest.  Returns the timings and the
        result structure (for set_tuning on operators of the same shape)."""
        cfg = _capi.ed_tune_cfg(int(steps), 1 if apply else 0)
        res = _capi.ed_tune_result()
        check(_capi.load().ed_op_autotune(self.handle, C.byref(cfg), C.byref(res), None), "ed_op_autotune")
        return {"persistent": bool(res.persistent), "row_cost": res.row_cost, "us_per_step": res.us_per_step,
                "per_step_us": res.per_step_us, "persistent_us": list(res.persistent_us),
                "ctas_per_sm": res.ctas_per_sm, "one_cta_us": res.one_cta_us, "chunk": res.chunk,
                "chunk_us": list(res.chunk_us), "candidates": res.candidates, "result": res}

    def set_tuning(self, result) -> None:
        """ed_op_set_tuning: apply another operator's autotune result."""
        check(_capi.load().ed_op_set_tuning(self.handle, C.byref(result)), "ed_op_set_tuning")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.ed_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Lanczos:
    """Lanczos ground state (HubMatrix_GPU.cuh:477-613) on the device.

    ``mode='reference'`` reproduces the reference's stop test (checked every
    10 steps, maxN=1000); ``mode='fixed'`` runs exactly ``max_steps`` steps.
    After ``eigen`` the tridiagonal T is in ``a`` (alpha) and ``b`` (beta,
    b[0] = |f|) like the reference's host vectors.
    """

    def __init__(self, dimUP: int = 0, dimDN: int = 0):
        self.dimUP, self.dimDN = dimUP, dimDN
        self.a: List[float] = []
        self.b: List[float] = [0.0]
        self.result: Optional[_capi.ed_lanczos_result] = None

    def random_vector(self, n: int, seed: int = 0) -> np.ndarray:
        f = random_vector(n, seed)
        return f / np.linalg.norm(f)

    def clear(self) -> None:
        self.a, self.b = [], [0.0]

    def eigen(self, Hub: Hubbard, f: Optional[np.ndarray] = None, max_steps: int = 1000,
              mode: str = "reference", ritz: str = "stored", reorth: bool = False, seed: int = 0,
              evec_out=None):
        """Returns (eval, evec).  f: host start vector (None: Philox(seed))."""
        lib = _capi.load()
        cfg = _capi.ed_lanczos_cfg()
        cfg.max_steps = int(max_steps)
        cfg.mode = _capi.ED_LANCZOS_REFERENCE if mode == "reference" else _capi.ED_LANCZOS_FIXED
        cfg.reorth = 1 if reorth else 0
        cfg.ritz = {"none": _capi.ED_RITZ_NONE, "stored": _capi.ED_RITZ_STORED,
                    "recompute": _capi.ED_RITZ_RECOMPUTE}[ritz]
        cfg.seed = int(seed)
        n = Hub.rows()
        dt = np.complex128 if Hub.is_complex else np.float64
        start_ptr = None
        if f is not None:
            f = np.ascontiguousarray(f, dtype=dt)
            cfg.start = _capi.ED_START_USER
            start_ptr = _ptr(f)
        else:
            cfg.start = _capi.ED_START_RANDOM
        evec = None
        evec_ptr, evec_mem = None, _capi.ED_MEM_HOST
        if ritz != "none":
            if evec_out is not None:  # torch CUDA tensor
                evec = evec_out
                evec_ptr, evec_mem = C.c_void_p(evec_out.data_ptr()), _capi.ED_MEM_DEVICE
            else:
                evec = np.empty(n, dtype=dt)
                evec_ptr = _ptr(evec)
        alpha = np.zeros(max_steps, dtype=np.float64)
        beta = np.zeros(max_steps + 1, dtype=np.float64)
        res = _capi.ed_lanczos_result()
        check(lib.ed_lanczos_run(Hub.handle, C.byref(cfg), start_ptr, _capi.ED_MEM_HOST, evec_ptr, evec_mem,
                                 _ptr(alpha), _ptr(beta), C.byref(res), None), "ed_lanczos_run")
        self.result = res
        self.a = list(alpha[: res.steps])
        self.b = list(beta[: res.steps + 1])
        return res.e0, evec


def lanczos_multi(ops: Sequence[Hubbard], max_steps: int, starts=None, ritz: bool = True, evec_out=None,
                  seed: int = 0, results: Optional[list] = None):
    """ed_lanczos_batch over operators of any sectors, real or complex (up to
    16, one persistent launch).  starts: None (run b from Philox(seed + b)) or
    a float64 CUDA tensor holding the start vectors one after another (rows_b
    values each, 2 rows_b interleaved for complex operators).  evec_out: a
    float64 CUDA tensor of the same packed layout for the Ritz vectors (or
    None: numpy arrays are returned).  Returns (e0 [B], evecs as a list of
    per-run views (a copy for a complex run that starts at an odd offset),
    alpha [B, max_steps], beta [B, max_steps + 1])."""
    lib = _capi.load()
    B = len(ops)
    sizes = [op.rows() * (2 if op.is_complex else 1) for op in ops]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    cfg = _capi.ed_lanczos_cfg()
    cfg.max_steps = int(max_steps)
    cfg.mode = _capi.ED_LANCZOS_FIXED
    cfg.reorth = 0
    cfg.ritz = _capi.ED_RITZ_STORED if ritz else _capi.ED_RITZ_NONE
    cfg.seed = int(seed)
    handles = (C.c_void_p * B)(*[op.handle for op in ops])
    st_ptr, st_mem = None, _capi.ED_MEM_HOST
    if starts is not None:
        if isinstance(starts, np.ndarray):
            f = np.ascontiguousarray(starts, dtype=np.float64).reshape(-1)
            st_ptr = _ptr(f)
        else:
            st_ptr, st_mem = C.c_void_p(starts.data_ptr()), _capi.ED_MEM_DEVICE
        cfg.start = _capi.ED_START_USER
    else:
        cfg.start = _capi.ED_START_RANDOM
    evecs, ev_ptr, ev_mem = None, None, _capi.ED_MEM_HOST
    if ritz:
        if evec_out is not None:
            evecs, ev_ptr, ev_mem = evec_out, C.c_void_p(evec_out.data_ptr()), _capi.ED_MEM_DEVICE
        else:
            evecs = np.empty(int(offs[-1]))
            ev_ptr = _ptr(evecs)
    alpha = np.zeros((B, max_steps))
    beta = np.zeros((B, max_steps + 1))
    res = (_capi.ed_lanczos_result * B)()
    check(lib.ed_lanczos_batch(handles, B, C.byref(cfg), st_ptr, st_mem, ev_ptr, ev_mem, _ptr(alpha), _ptr(beta),
                               res, None), "ed_lanczos_batch")
    if results is not None:
        results.extend(res)
    views = None
    if ritz:
        views = []
        for b, op in enumerate(ops):
            v = evecs[int(offs[b]):int(offs[b + 1])]
            if op.is_complex:
                if isinstance(v, np.ndarray):
                    v = v.copy().view(np.complex128) if offs[b] % 2 else v.view(np.complex128)
                else:
                    import torch
                    # a complex view needs an even offset; after a real run of odd length, a copy
                    v = (v.clone() if offs[b] % 2 else v).view(torch.complex128)
            views.append(v)
    return np.array([r.e0 for r in res]), views, alpha, beta


def lanczos_batch(ops: Sequence[Hubbard], max_steps: int, seed: int = 0, starts: Optional[np.ndarray] = None,
                  ritz: bool = True, evec_out=None, results: Optional[list] = None):
    """ed_lanczos_batch: fixed-step Lanczos of up to 8 operators that share
    their hopping tables (one sector, disorder in the on-site terms) in one
    persistent launch.  Run b starts from Philox(seed + b) or starts[b]
    (a numpy array or a float64 CUDA tensor, (B, rows)).
    Returns (e0 [B], evecs, alpha [B, max_steps], beta [B, max_steps + 1]):
    evecs a (B, rows) numpy array, or evec_out (a (B, rows) float64 CUDA
    tensor) when given, or None without ritz.  A list passed as results
    receives the B ed_lanczos_result records (min_bits, launches, ...)."""
    lib = _capi.load()
    B = len(ops)
    n = ops[0].rows()
    cfg = _capi.ed_lanczos_cfg()
    cfg.max_steps = int(max_steps)
    cfg.mode = _capi.ED_LANCZOS_FIXED
    cfg.reorth = 0
    cfg.ritz = _capi.ED_RITZ_STORED if ritz else _capi.ED_RITZ_NONE
    cfg.seed = int(seed)
    handles = (C.c_void_p * B)(*[op.handle for op in ops])
    st_ptr, st_mem = None, _capi.ED_MEM_HOST
    if starts is not None and not isinstance(starts, np.ndarray):  # CUDA tensor (B, rows)
        cfg.start = _capi.ED_START_USER
        st_ptr, st_mem = C.c_void_p(starts.data_ptr()), _capi.ED_MEM_DEVICE
    elif starts is not None:
        f = np.ascontiguousarray(starts, dtype=np.float64).reshape(B, n)
        cfg.start = _capi.ED_START_USER
        st_ptr = _ptr(f)
    else:
        cfg.start = _capi.ED_START_RANDOM
    evecs, ev_ptr, ev_mem = None, None, _capi.ED_MEM_HOST
    if ritz:
        if evec_out is not None:
            evecs, ev_ptr, ev_mem = evec_out, C.c_void_p(evec_out.data_ptr()), _capi.ED_MEM_DEVICE
        else:
            evecs = np.empty((B, n))
            ev_ptr = _ptr(evecs)
    alpha = np.zeros((B, max_steps))
    beta = np.zeros((B, max_steps + 1))
    res = (_capi.ed_lanczos_result * B)()
    check(lib.ed_lanczos_batch(handles, B, C.byref(cfg), st_ptr, st_mem, ev_ptr, ev_mem, _ptr(alpha), _ptr(beta),
                               res, None), "ed_lanczos_batch")
    if results is not None:
        results.extend(res)
    return np.array([r.e0 for r in res]), evecs, alpha, beta

