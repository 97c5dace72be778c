"""Observables of a ground state through the C ABI: expectation values,
site densities (Hellmann-Feynman derivatives), the Kubo Drude weight of the
reference (drude_v2_cal_Kagome_randomHop.cu:183-220), the second-order flux
response, and the half-system entanglement entropy.

Vectors may be numpy arrays (host) or torch CUDA tensors (device)."""
from __future__ import annotations

import ctypes as C
import math
from typing import Optional, Sequence

import numpy as np

from . import _capi
from ._capi import check
from .hubbard import Hubbard


def _mem(psi):
    """(pointer, mem flag, keepalive) for a numpy array or CUDA tensor."""
    if isinstance(psi, np.ndarray):
        arr = np.ascontiguousarray(psi)
        if arr.dtype == np.complex128:
            arr = arr.view(np.float64)
        return C.c_void_p(arr.ctypes.data), _capi.ED_MEM_HOST, arr
    return C.c_void_p(psi.data_ptr()), _capi.ED_MEM_DEVICE, psi


def _device(psi, op: Hubbard):
    import torch
    if isinstance(psi, np.ndarray):
        a = np.ascontiguousarray(psi, dtype=np.complex128 if op.is_complex else np.float64)
        t = torch.from_numpy(a.view(np.float64)).to(f"cuda:{op.device}")
        return t
    return psi.view(torch.float64) if psi.is_complex() else psi


def expect(op: Hubbard, psi) -> complex:
    """<psi|O|psi>."""
    p, mem, keep = _mem(psi)
    out = np.zeros(2)
    check(_capi.load().ed_op_expect(op.handle, p, mem, C.c_void_p(out.ctypes.data), None), "ed_op_expect")
    return complex(out[0], out[1]) if op.is_complex else float(out[0])


def site_densities(op: Hubbard, psi):
    """(<n_i,up>, <n_i,dn>, <n_i,up n_i,dn>) as three arrays of N values."""
    p, mem, keep = _mem(psi)
    nu, nd, dd = np.zeros(op.N), np.zeros(op.N), np.zeros(op.N)
    check(_capi.load().ed_site_densities(op.handle, p, mem, C.c_void_p(nu.ctypes.data), C.c_void_p(nd.ctypes.data),
                                         C.c_void_p(dd.ctypes.data), None), "ed_site_densities")
    return nu, nd, dd


def continued_fraction(alpha, beta, norm2: float, energy: float, omega) -> np.ndarray:
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    b = np.ascontiguousarray(beta, dtype=np.float64)
    w = np.ascontiguousarray(omega, dtype=np.complex128)
    g = np.zeros(w.size, dtype=np.complex128)
    check(_capi.load().ed_continued_fraction(a.size, C.c_void_p(a.ctypes.data), C.c_void_p(b.ctypes.data), norm2,
                                             energy, w.size, C.c_void_p(w.view(np.float64).ctypes.data),
                                             C.c_void_p(g.view(np.float64).ctypes.data)), "ed_continued_fraction")
    return g


# drude_v2_cal_Kagome_randomHop.cu:13-21
REFERENCE_KUBO = dict(lanczos_steps=200, n_omega=8000, omega_step=0.004, delta=0.01, omega_cutoff=0.01)


def drude_kubo(H: Hubbard, J: Hubbard, K: Hubbard, psi, e0: float, volume: float, want_sigma: bool = False,
               **kw):
    """drude_weight_Jx: returns (D, kinetic, vertex[, sigma])."""
    p = dict(REFERENCE_KUBO)
    p.update(kw)
    cfg = _capi.ed_kubo_cfg(lanczos_steps=p["lanczos_steps"], n_omega=p["n_omega"], omega_step=p["omega_step"],
                            delta=p["delta"], omega_cutoff=p["omega_cutoff"], volume=volume)
    res = _capi.ed_kubo_result()
    dpsi = _device(psi, H)
    sigma = np.zeros(p["n_omega"]) if want_sigma else None
    check(_capi.load().ed_drude_kubo(H.handle, J.handle, K.handle, C.c_void_p(dpsi.data_ptr()), e0, C.byref(cfg),
                                     C.byref(res), C.c_void_p(sigma.ctypes.data) if want_sigma else None, None),
          "ed_drude_kubo")
    out = (res.drude, res.kinetic, res.vertex)
    return out + (sigma,) if want_sigma else out


def response(H: Hubbard, dH: Hubbard, d2H: Optional[Hubbard], psi, e0: float, steps: int = 200):
    """(dE0/dtheta, d2E0/dtheta2) by Hellmann-Feynman and a linear-response
    Lanczos solve."""
    dpsi = _device(psi, H)
    first = C.c_double(0.0)
    second = C.c_double(0.0)
    check(_capi.load().ed_response(H.handle, dH.handle, d2H.handle if d2H is not None else None,
                                   C.c_void_p(dpsi.data_ptr()), e0, steps, C.byref(first),
                                   C.byref(second) if d2H is not None else None, None), "ed_response")
    return first.value, (second.value if d2H is not None else None)


def response_batch(Hs: Sequence[Hubbard], dHs: Sequence[Hubbard], d2Hs: Sequence[Hubbard], psis, e0s,
                   steps: int = 200):
    """ed_response_batch: (first [n], second [n]) for n operators whose
    normalised ground states psis (a float64 CUDA tensor) holds one after
    another; the n linear-response Lanczos runs share one launch."""
    n = len(Hs)
    arr = lambda ops: (C.c_void_p * n)(*[o.handle for o in ops])  # noqa: E731
    e0 = np.ascontiguousarray(e0s, dtype=np.float64)
    first = np.zeros(n)
    second = np.zeros(n)
    check(_capi.load().ed_response_batch(arr(Hs), arr(dHs), arr(d2Hs), n, C.c_void_p(psis.data_ptr()),
                                         C.c_void_p(e0.ctypes.data), steps, C.c_void_p(first.ctypes.data),
                                         C.c_void_p(second.ctypes.data), None), "ed_response_batch")
    return first, second


def response_subspace(H: Hubbard, dH: Hubbard, d2H: Hubbard, psis, e0: float, steps: int = 200):
    """ed_response_subspace: (D1, M), the g x g first- and second-order
    matrices over the ground subspace spanned by the g states psis (a (g,
    rows) CUDA tensor, complex for complex operators); see lowest_branch."""
    g = int(psis.shape[0])
    a = psis.contiguous()
    d1 = np.zeros(2 * g * g)
    d2 = np.zeros(2 * g * g)
    check(_capi.load().ed_response_subspace(H.handle, dH.handle, d2H.handle, C.c_void_p(a.data_ptr()), g, e0, steps,
                                            C.c_void_p(d1.ctypes.data), C.c_void_p(d2.ctypes.data), None),
          "ed_response_subspace")
    return d1.view(np.complex128).reshape(g, g), d2.view(np.complex128).reshape(g, g)


def lowest_branch(D1: np.ndarray, M: np.ndarray, tol: float = 1e-9):
    """(dE0/dtheta, d2E0/dtheta2) of the lowest branch of a degenerate level:
    the lowest eigenvalue of the first-order matrix D1 and, when D1 splits
    nothing (all its eigenvalues equal within tol), the lowest eigenvalue of
    the second-order matrix M; otherwise M's expectation value in D1's lowest
    eigenvector."""
    D1 = 0.5 * (D1 + D1.conj().T)
    M = 0.5 * (M + M.conj().T)
    w1, v1 = np.linalg.eigh(D1)
    if w1[-1] - w1[0] <= tol * max(1.0, abs(w1[0])):
        return float(w1[0]), float(np.linalg.eigvalsh(M)[0])
    c = v1[:, 0]
    return float(w1[0]), float(np.real(np.vdot(c, M @ c)))


def entanglement_entropy(op: Hubbard, psi, a_sites: Sequence[int]):
    """(S_vN, S_ref) for the sites in a_sites."""
    mask = 0
    for s in a_sites:
        mask |= 1 << int(s)
    p, mem, keep = _mem(psi)
    svn, sref = C.c_double(0.0), C.c_double(0.0)
    check(_capi.load().ed_entanglement_entropy(op.handle, p, mem, mask, C.byref(svn), C.byref(sref), None),
          "ed_entanglement_entropy")
    return svn.value, sref.value


def entanglement_entropy_batch(op: Hubbard, psis, a_sites: Sequence[int]):
    """(S_vN[n], S_ref[n]) of the n states psis[b] (a (n, rows) float64 CUDA
    tensor or numpy array) of op's sector, in one batched call."""
    mask = 0
    for s in a_sites:
        mask |= 1 << int(s)
    if isinstance(psis, np.ndarray):
        a = np.ascontiguousarray(psis, dtype=np.float64)
        n, ptr, mem = a.shape[0], C.c_void_p(a.ctypes.data), _capi.ED_MEM_HOST
    else:
        a = psis.contiguous()
        n, ptr, mem = a.shape[0], C.c_void_p(a.data_ptr()), _capi.ED_MEM_DEVICE
    if a.shape[1] != op.rows():
        raise ValueError("psis must be (n_states, rows)")
    svn, sref = np.zeros(n), np.zeros(n)
    check(_capi.load().ed_entanglement_entropy_batch(op.handle, int(n), ptr, mem, mask,
                                                     C.c_void_p(svn.ctypes.data), C.c_void_p(sref.ctypes.data), None),
          "ed_entanglement_entropy_batch")
    return svn, sref


def s2_apply(op: Hubbard, x):
    """y = S_xy x, S_xy = (S+S- + S-S+)/2 (TotalSpin::Hubbard::Hubbard_mv):
    a numpy array in gives a numpy array out, a CUDA tensor a CUDA tensor
    (on the current stream's device, synchronised)."""
    p, mem, keep = _mem(x)
    if mem == _capi.ED_MEM_HOST:
        y = np.empty(keep.size, dtype=np.float64)
        check(_capi.load().ed_s2_apply(op.handle, p, C.c_void_p(y.ctypes.data), mem, None), "ed_s2_apply")
        return y.view(np.complex128) if op.is_complex else y
    import torch
    y = torch.empty_like(x)
    check(_capi.load().ed_s2_apply(op.handle, p, C.c_void_p(y.data_ptr()), mem, None), "ed_s2_apply")
    torch.cuda.synchronize(y.device)
    return y


def s2_expect(op: Hubbard, psi):
    """(<S_xy>, S^2) of a normalised psi (S^2 = (N_up - N_dn)^2 / 4 + <S_xy>)."""
    p, mem, keep = _mem(psi)
    out = np.zeros(2)
    check(_capi.load().ed_s2_expect(op.handle, p, mem, C.c_void_p(out.ctypes.data), None), "ed_s2_expect")
    return float(out[0]), float(out[1])
