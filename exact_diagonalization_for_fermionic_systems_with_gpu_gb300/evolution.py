"""Krylov time evolution psi(t) = exp(-i H t) psi0 (Krylov<C>,
MBL_test/include/HubMatrix_GPU.cuh:619-728) and the tridiagonal eigensolver
behind it (LAPACKf77::dsted as Krylov::Make_tridiagonal_eigen calls it)."""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _capi
from ._capi import check
from .hubbard import Hubbard, _ptr


def tridiag_eigen(alpha: Sequence[float], offdiag: Sequence[float], vectors: bool = True):
    """(evals ascending, Z with the unit eigenvectors as columns or None)."""
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    n = a.size
    b = np.ascontiguousarray(offdiag, dtype=np.float64)
    if b.size < max(n - 1, 0):
        raise ValueError("offdiag needs len(alpha) - 1 values")
    w = np.empty(n)
    z = np.empty((n, n)) if vectors else None  # column j at z[j] (row-major view of column-major)
    check(_capi.load().ed_tridiag_eigen(n, _ptr(a), _ptr(b) if n > 1 else None, _ptr(w),
                                        _ptr(z) if vectors else None), "ed_tridiag_eigen")
    return w, (z.T.copy() if vectors else None)


def tridiag_expm(alpha: Sequence[float], offdiag: Sequence[float], times: Sequence[float]) -> np.ndarray:
    """exp(-i T t) e_0 for every t: complex array (len(times), n)."""
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    n = a.size
    b = np.ascontiguousarray(offdiag, dtype=np.float64)
    t = np.ascontiguousarray(times, dtype=np.float64)
    out = np.empty((t.size, 2 * n))
    check(_capi.load().ed_tridiag_expm(n, _ptr(a), _ptr(b) if n > 1 else None, int(t.size), _ptr(t) if t.size else None,
                                       _ptr(out) if t.size else None), "ed_tridiag_expm")
    return out.view(np.complex128).reshape(t.size, n)


def krylov_evolve(H: Hubbard, psi0, times: Sequence[float], max_steps: int = 1000, tol: float = 1e-10,
                  reorth: bool = False, result: Optional[dict] = None, out=None):
    """exp(-i H t) psi0 for every t in times.  psi0: complex numpy array (host)
    or complex CUDA tensor (device); the result is (len(times), rows) of the
    same kind.  out, when given (that shape and kind), is added to and
    returned.  result, when given, receives steps / runs / norm / err_est /
    launches."""
    lib = _capi.load()
    cfg = _capi.ed_krylov_cfg(int(max_steps), 1 if reorth else 0, float(tol), 0 if out is None else 1, 0)
    res = _capi.ed_krylov_result()
    t = np.ascontiguousarray(times, dtype=np.float64)
    n = H.rows()
    if isinstance(psi0, np.ndarray):
        p0 = np.ascontiguousarray(psi0, dtype=np.complex128)
        if p0.size != n:
            raise ValueError(f"psi0 has {p0.size} values, the operator {n} rows")
        if out is None:
            out = np.empty((t.size, n), dtype=np.complex128)
        elif out.dtype != np.complex128 or out.shape != (t.size, n) or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous complex128 array of shape (len(times), rows)")
        check(lib.ed_krylov_evolve(H.handle, C.byref(cfg), _ptr(p0), _capi.ED_MEM_HOST, int(t.size),
                                   _ptr(t) if t.size else None, _ptr(out) if t.size else None, _capi.ED_MEM_HOST,
                                   C.byref(res), None), "ed_krylov_evolve")
    else:
        import torch
        p0 = psi0.to(torch.complex128).contiguous()
        if p0.numel() != n:
            raise ValueError(f"psi0 has {p0.numel()} values, the operator {n} rows")
        if out is None:
            out = torch.empty((t.size, n), dtype=torch.complex128, device=p0.device)
        elif out.dtype != torch.complex128 or tuple(out.shape) != (t.size, n) or not out.is_contiguous():
            raise ValueError("out must be a contiguous complex128 tensor of shape (len(times), rows)")
        check(lib.ed_krylov_evolve(H.handle, C.byref(cfg), C.c_void_p(p0.data_ptr()), _capi.ED_MEM_DEVICE,
                                   int(t.size), _ptr(t) if t.size else None,
                                   C.c_void_p(out.data_ptr()) if t.size else None, _capi.ED_MEM_DEVICE,
                                   C.byref(res), None), "ed_krylov_evolve")
    if result is not None:
        result.update(steps=res.steps, runs=res.runs, norm=res.norm, err_est=res.err_est, launches=res.launches)
    return out


class Krylov:
    """The reference's Krylov<double> driver surface (HubMatrix_GPU.cuh:619-728):
    Make_tridiagonal_eigen(Hub, phi0) fixes the start vector, and
    Krylov_time_evol(Hub, phi0, phi, dt) ADDS exp(-i H dt) phi0 into phi
    (phi: complex numpy array or CUDA tensor, updated in place)."""

    def __init__(self, dimUP: int = 0, dimDN: int = 0, max_steps: int = 1000, tol: float = 1e-10):
        self.dimUP, self.dimDN = dimUP, dimDN
        self.max_steps, self.tol = max_steps, tol
        self.steps = 0
        self.info: dict = {}

    def Make_tridiagonal_eigen(self, Hub: Hubbard, phi0) -> None:
        self.info = {}
        krylov_evolve(Hub, phi0, [], self.max_steps, self.tol, result=self.info)
        self.steps = self.info["steps"]

    def Krylov_time_evol(self, Hub: Hubbard, phi0, phi, dt: float) -> None:
        krylov_evolve(Hub, phi0, [dt], self.max_steps, self.tol, result=self.info, out=phi.reshape(1, -1))
        self.steps = self.info["steps"]

    def clear(self) -> None:
        self.steps = 0
        self.info = {}
