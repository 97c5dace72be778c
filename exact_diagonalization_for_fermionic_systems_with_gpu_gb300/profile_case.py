"""Small, fixed workloads for profiling the kernels under ncu.

    python -m exact_diagonalization_for_fermionic_systems_with_gpu_gb300.profile_case \
        --case kagome12 --what lanczos --steps 20

--what lanczos : one fixed-step Lanczos solve, per-step kernels timed with events
--what fused   : one fixed-step Lanczos solve in the persistent kernel, phases
                 timed with device timestamps
--what solve   : the same solve without timing hooks (what bench.py runs)
--what perform : --steps operator applies through the FP64 C-ABI path
Cases: kagome12 (6+6, dim 853,776, L2-resident vectors), kagome12_flux
(complex, Peierls phases), chain12_66 / chain12_75 / chain12_84 (open L=12
chain, W=6 disorder, the three sectors of the MBL sweep), chain14 (7+7 open
chain with disorder, dim 11,778,624, vectors larger than L2), lieb18 (9+9,
dim 2.36e9, ~100 GB of device memory for a Lanczos run), lieb18_49 (4+9:
Lieb18's down rows under 3,060 up rows, dim 1.49e8, for profiling the
two-pass matvec on a small case).
"""
from __future__ import annotations

import argparse
import ctypes as C
import time

import numpy as np

from . import lattices as L
from .hubbard import H_TBq, Hubbard, random_vector
from . import _capi


def build_case(name: str):
    if name == "kagome12":
        t = L.kagome12()
        return Hubbard(H_TBq(12, 6).extend(t), H_TBq(12, 6).extend(t), 8.0)
    if name == "chain14":
        eps = random_vector(14, 100) * 6.0
        t = L.chain(14, periodic=False, eps=eps)
        return Hubbard(H_TBq(14, 7).extend(t), H_TBq(14, 7).extend(t), 1.0)
    if name == "lieb18":
        t = L.lieb18()
        return Hubbard(H_TBq(18, 9).extend(t), H_TBq(18, 9).extend(t), 4.0)
    if name == "lieb18_49":  # Lieb18's down rows (48,620 columns) under 3,060 up rows: 1.2 GB vectors
        t = L.lieb18()
        return Hubbard(H_TBq(18, 4).extend(t), H_TBq(18, 9).extend(t), 4.0)
    if name == "kagome12_flux":
        t = L.kagome12(flux=0.3)
        return Hubbard(H_TBq(12, 6).extend(t), H_TBq(12, 6).extend(t), 4.0)
    if name.startswith("chain12_"):  # chain12_66 / chain12_75 / chain12_84: open L=12, W=6, U=1
        qu, qd = int(name[-2]), int(name[-1])
        eps = random_vector(12, 100) * 6.0
        t = L.chain(12, periodic=False, eps=eps)
        return Hubbard(H_TBq(12, qu).extend(t), H_TBq(12, qd).extend(t), 1.0)
    raise SystemExit(f"unknown case {name}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="kagome12")
    ap.add_argument("--what", default="lanczos", choices=["lanczos", "fused", "solve", "perform"])
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--ritz", default="none", choices=["none", "stored"],
                    help="stored: keep the Krylov basis and form the Ritz vector, as the bench does")
    args = ap.parse_args()
    import torch
    op = build_case(args.case)
    lib = _capi.load()
    t0 = time.perf_counter()
    if args.what in ("lanczos", "fused", "solve"):
        ritz = _capi.ED_RITZ_STORED if args.ritz == "stored" else _capi.ED_RITZ_NONE
        cfg = _capi.ed_lanczos_cfg(max_steps=args.steps, mode=_capi.ED_LANCZOS_FIXED, reorth=0,
                                   ritz=ritz, start=_capi.ED_START_RANDOM,
                                   profile={"lanczos": 1, "fused": 2, "solve": 0}[args.what], seed=0)
        res = _capi.ed_lanczos_result()
        evec = np.empty(op.rows() * (2 if op.is_complex else 1)) if args.ritz == "stored" else None
        _capi.check(lib.ed_lanczos_run(op.handle, C.byref(cfg), None, 0,
                                       C.c_void_p(evec.ctypes.data) if args.ritz == "stored" else None, 0,
                                       None, None, C.byref(res), None), "ed_lanczos_run")
        n = max(res.n_matvec, 1)
        print(f"E0 {res.e0:.12f} steps {res.steps} matvec {res.matvec_ms / n * 1e3:.1f} us "
              f"axpy {res.axpy_ms / n * 1e3:.1f} us reduce {res.reduce_ms / n * 1e3:.1f} us "
              f"(barrier wait {res.barrier_ms / n * 1e3:.1f}, scalars {res.scalar_ms / n * 1e3:.1f}) "
              f"launches {res.launches}" + (f" persistent launch {res.fused_ms:.3f} ms, CTA finish spread: rows "
                                            f"{res.rows_spread_ms / n * 1e3:.1f} us axpy {res.axpy_spread_ms / n * 1e3:.1f} us"
                                            if res.fused_ms else ""))
    else:
        dt = torch.complex128 if op.is_complex else torch.float64
        x = torch.empty(op.rows(), dtype=torch.float64 if not op.is_complex else torch.float64,
                        device="cuda")
        n = op.rows() * (2 if op.is_complex else 1)
        x = torch.empty(n, dtype=torch.float64, device="cuda")
        _capi.check(lib.ed_random_vector_device(n, 1, C.c_void_p(x.data_ptr()), None), "random")
        x = x.view(dt) if op.is_complex else x
        y = torch.empty_like(x)
        op.Hubbard_mv(x, y)  # warm
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            op.Hubbard_mv(x, y)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / max(args.steps, 1)
        gbs = 16.0 * op.rows() * (2 if op.is_complex else 1) / (ms * 1e-3) / 1e9
        print(f"{args.steps} applies, {ms:.3f} ms each ({gbs:.0f} GB/s of 16 B x stored values), "
              f"|y| = {float(torch.linalg.vector_norm(y)):.6e}")
    print(f"wall {time.perf_counter() - t0:.2f} s")
    op.close()


if __name__ == "__main__":
    main()
