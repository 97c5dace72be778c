"""Several lowest eigenpairs (ed_eigs_lowest) behind the Spectra surface the
TotalSpinExcited drivers use (TotalSpinExcited_Lieb_randomHop.cu:133-143):

    eigs = SymEigsSolver(H, nev, 4 * (nev + 1))
    eigs.init()
    eigs.compute(SortRule.SmallestAlge, 1000, 1e-10, SortRule.SmallestAlge)
    if eigs.info() == CompInfo.Successful:
        eval, evec = eigs.eigenvalues(), eigs.eigenvectors()

Only the SmallestAlge selection exists (the one the drivers use)."""
from __future__ import annotations

import ctypes as C
import enum
from typing import Optional

import numpy as np

from . import _capi
from .hubbard import Hubbard, _ptr

ED_ERR_NOT_CONVERGED = 8


class SortRule(enum.Enum):
    SmallestAlge = "SmallestAlge"


class CompInfo(enum.Enum):
    Successful = 0
    NotComputed = 1
    NotConverging = 2
    NumericalIssue = 3


def eigs_lowest(H: Hubbard, nev: int, ncv: Optional[int] = None, tol: float = 1e-10, max_restarts: int = 1000,
                seed: int = 0, start: Optional[np.ndarray] = None, vectors: bool = True, result: Optional[dict] = None):
    """(evals ascending, evecs (nev, rows) or None, residual estimates).
    Raises on ED_ERR_NOT_CONVERGED unless result is given (then
    result['converged'] is False)."""
    lib = _capi.load()
    ncv = 4 * (nev + 1) if ncv is None else ncv
    cfg = _capi.ed_eigs_cfg(int(nev), int(ncv), int(max_restarts),
                            _capi.ED_START_USER if start is not None else _capi.ED_START_RANDOM, float(tol), int(seed))
    n = H.rows()
    f = None
    if start is not None:
        f = np.ascontiguousarray(start, dtype=np.float64)
        if f.size != n:
            raise ValueError(f"start has {f.size} values, the operator {n} rows")
    w = np.zeros(nev)
    r = np.zeros(nev)
    v = np.empty((nev, n)) if vectors else None
    res = _capi.ed_eigs_result()
    st = lib.ed_eigs_lowest(H.handle, C.byref(cfg), _ptr(f) if f is not None else None, _capi.ED_MEM_HOST, _ptr(w),
                            _ptr(v) if vectors else None, _capi.ED_MEM_HOST, _ptr(r), C.byref(res), None)
    if result is not None:
        result.update(nconv=res.nconv, restarts=res.restarts, n_matvec=res.n_matvec, launches=res.launches,
                      max_resid=res.max_resid, converged=(st == 0))
        if st not in (0, ED_ERR_NOT_CONVERGED):
            _capi.check(st, "ed_eigs_lowest")
    else:
        _capi.check(st, "ed_eigs_lowest")
    return w, v, r


class SymEigsSolver:
    """Spectra::SymEigsSolver<OpType>(op, nev, ncv) over a Hubbard operator."""

    def __init__(self, op: Hubbard, nev: int, ncv: int):
        if not 0 < nev < ncv:
            raise ValueError("need 0 < nev < ncv")
        self.op, self.nev, self.ncv = op, nev, ncv
        self._start: Optional[np.ndarray] = None
        self._info = CompInfo.NotComputed
        self._w = self._v = None
        self.stats: dict = {}

    def init(self, init_resid: Optional[np.ndarray] = None) -> None:
        self._start = None if init_resid is None else np.asarray(init_resid, dtype=np.float64)

    def compute(self, selection: SortRule = SortRule.SmallestAlge, maxit: int = 1000, tol: float = 1e-10,
                sorting: SortRule = SortRule.SmallestAlge) -> int:
        if selection != SortRule.SmallestAlge or sorting != SortRule.SmallestAlge:
            raise NotImplementedError("only SortRule.SmallestAlge")
        self.stats = {}
        self._w, self._v, _ = eigs_lowest(self.op, self.nev, self.ncv, tol, maxit, start=self._start,
                                          result=self.stats)
        self._info = CompInfo.Successful if self.stats["converged"] else CompInfo.NotConverging
        return int(self.stats["nconv"])

    def info(self) -> CompInfo:
        return self._info

    def eigenvalues(self) -> np.ndarray:
        return self._w

    def eigenvectors(self) -> np.ndarray:
        """rows x nev, column i the eigenvector of eigenvalues()[i] (Eigen's layout)."""
        return self._v.T

    def num_iterations(self) -> int:
        return int(self.stats.get("restarts", 0))

    def num_operations(self) -> int:
        return int(self.stats.get("n_matvec", 0))
