"""TEST INFRASTRUCTURE ONLY — the reference's own GPU matvec, launched from
its cubin (oracle/_ref/ref_mv.cubin, built by `make -C oracle ref` from
MBL_test/include/HubMatrix_GPU.cuh:114-161 unmodified).

RefHubbard mirrors the reference's `struct Hubbard` (HubMatrix_GPU.cuh:29-70):
the per-spin ELL tables (Ax double, Aj int, slot-major, 10*Q+1 slots, the
reference's own layout, here from the library's bit-exact H_TBq export), the
int state tables, the BPS choice (the smallest i dividing dim_dn with
dim_dn / i <= 1024) and the launch of Hubbard::Hubbard_mv (:163-182): grid
dim_up * BPS, block dim_dn / BPS, 12 bytes of shared memory per up slot.
The launch goes through the CUDA driver API (ctypes on libcuda) on a torch
stream, in torch's primary context.  Used by the GPU parity tests as a
second checker and to time the reference kernel on the same GPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "ref_mv.cubin"
ENTRY = b"_Z11Hubbard_mv_IdEvPKdPKiS1_S3_S3_S3_PT_S5_mmiidiii"  # Hubbard_mv_<double>


def available() -> bool:
    return CUBIN.exists()


_CU = None


def _driver():
    global _CU
    if _CU is None:
        cu = C.CDLL("libcuda.so.1")
        cu.cuCtxGetCurrent.argtypes = [C.POINTER(C.c_void_p)]
        cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        cu.cuModuleUnload.argtypes = [C.c_void_p]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        for f in (cu.cuCtxGetCurrent, cu.cuModuleLoad, cu.cuModuleGetFunction, cu.cuModuleUnload, cu.cuLaunchKernel):
            f.restype = C.c_int
        _CU = cu
    return _CU


def _ck(status: int, what: str) -> None:
    if status != 0:
        raise RuntimeError(f"{what} failed with CUDA driver error {status}")


def bps(dim_dn: int) -> int:
    """Blocks per sub-vector as the reference's constructor picks it
    (HubMatrix_GPU.cuh:53-61)."""
    for i in range(1, dim_dn):
        if dim_dn % i == 0 and dim_dn // i <= 1024:
            return i
    raise ValueError("the reference leaves BPS unset for this dim_dn")


class RefHubbard:
    """y = H x with the reference's kernel on torch float64 CUDA tensors."""

    def __init__(self, up, dn, U: float, dilution=None, device: int = 0):
        import torch
        if up.N != dn.N or up.N > 30:
            raise ValueError("both spins on the same N <= 30 sites (int state words)")
        self.dimUP, self.dimDN, self.N, self.U = up.count, dn.count, up.N, float(U)
        self.rows = self.dimUP * self.dimDN
        if self.rows >= 2 ** 31:
            raise ValueError("the reference kernel indexes with int")
        self.bps = bps(self.dimDN)
        self.threads = self.dimDN // self.bps
        axu, aju = up.ell()
        axd, ajd = dn.ell()
        self.ncu, self.ncd = axu.shape[0], axd.shape[0]
        if self.threads < self.ncu:
            raise ValueError("a block must have a thread per up slot")
        # every column the kernel dereferences must lie in its vector: the
        # up term reads Aj only where Ax != 0, the down term reads every slot
        if aju[axu != 0].size and not (0 <= aju[axu != 0].min() and aju[axu != 0].max() < self.dimUP):
            raise ValueError("up-table column out of range")
        if not (0 <= ajd.min() and ajd.max() < self.dimDN):
            raise ValueError("down-table column out of range")
        dev = torch.device("cuda", device)
        torch.zeros(1, device=dev)  # the primary context is current from here on
        self._t = {
            "AxUP": torch.from_numpy(np.ascontiguousarray(axu.ravel())).to(dev),
            "AjUP": torch.from_numpy(aju.ravel().astype(np.int32)).to(dev),
            "AxDN": torch.from_numpy(np.ascontiguousarray(axd.ravel())).to(dev),
            "AjDN": torch.from_numpy(ajd.ravel().astype(np.int32)).to(dev),
            "stateUP": torch.from_numpy(up.state.astype(np.int32)).to(dev),
            "stateDN": torch.from_numpy(dn.state.astype(np.int32)).to(dev),
        }
        torch.cuda.synchronize(dev)
        cu = _driver()
        ctx = C.c_void_p()
        _ck(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self._mod = C.c_void_p()
        _ck(cu.cuModuleLoad(C.byref(self._mod), str(CUBIN).encode()), "cuModuleLoad")
        self._fn = C.c_void_p()
        _ck(cu.cuModuleGetFunction(C.byref(self._fn), self._mod, ENTRY), "cuModuleGetFunction")
        # the dilution word of the second constructor (:72-95); all sites otherwise
        self.dilution = (1 << self.N) - 1 if dilution is None else int(dilution)
        self.launches = 0

    def __call__(self, x, y, stream=None) -> None:
        import torch
        for v in (x, y):
            if not (v.is_cuda and v.dtype == torch.float64 and v.is_contiguous() and v.numel() == self.rows):
                raise TypeError("needs contiguous float64 CUDA tensors of length rows")
        t = self._t
        args = [C.c_void_p(t["AxUP"].data_ptr()), C.c_void_p(t["AjUP"].data_ptr()),
                C.c_void_p(t["AxDN"].data_ptr()), C.c_void_p(t["AjDN"].data_ptr()),
                C.c_void_p(t["stateUP"].data_ptr()), C.c_void_p(t["stateDN"].data_ptr()),
                C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                C.c_uint64(self.dimUP), C.c_uint64(self.dimDN), C.c_int(self.ncu), C.c_int(self.ncd),
                C.c_double(self.U), C.c_int(self.dilution), C.c_int(self.N), C.c_int(self.bps)]
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        s = stream if stream is not None else torch.cuda.current_stream(x.device)
        shared = self.ncu * (8 + 4)
        _ck(_driver().cuLaunchKernel(self._fn, self.dimUP * self.bps, 1, 1, self.threads, 1, 1, shared,
                                     C.c_void_p(s.cuda_stream), params, None), "cuLaunchKernel")
        self.launches += 1

    def close(self) -> None:
        if getattr(self, "_mod", None) is not None and self._mod.value:
            _driver().cuModuleUnload(self._mod)
            self._mod = None
