"""Small, fixed workloads for profiling the kernels under ncu.

    python -m exact_diagonalization_for_fermionic_systems_with_gpu_gb300.profile_case \
        --case kagome12 --what lanczos --steps 20

--what lanczos : one fixed-step Lanczos solve, per-step kernels timed with events
--what fused   : one fixed-step Lanczos solve in the persistent kernel, phases
                 timed with device timestamps
--what solve   : the same solve without timing hooks (what bench.py runs)
--what perform : --steps operator applies through the FP64 C-ABI path
--what adjoint : a --steps Lanczos solve with the Ritz vector regenerated in a
                 second pass, then dE0/dU and dE0/dt (the Lieb18 9+9 workload)
--what tune    : ed_op_autotune's timings and choice for the case's operator
                 (--steps per candidate) and, for sectors with a persistent plan,
                 the batch size sweeps.tune_batch picks (eight samples of the
                 case's shape); one JSON line
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


def case_spec(name: str):
    """(N, N_up, N_dn, up terms, down terms, U) of a named case."""
    if name == "kagome12":
        t = L.kagome12()
        return 12, 6, 6, t, t, 8.0
    if name == "chain14":
        eps = random_vector(14, 100) * 6.0
        t = L.chain(14, periodic=False, eps=eps)
        return 14, 7, 7, t, t, 1.0
    if name == "lieb18":
        t = L.lieb18()
        return 18, 9, 9, t, t, 4.0
    if name == "lieb18_49":  # Lieb18's down rows (48,620 columns) under 3,060 up rows: 1.2 GB vectors
        t = L.lieb18()
        return 18, 4, 9, t, t, 4.0
    if name == "kagome12_flux":
        t = L.kagome12(flux=0.3)
        return 12, 6, 6, t, t, 4.0
    if name.startswith("chain12_"):  # chain12_66 / chain12_75 / chain12_84: open L=12, W=6, U=1
        qu, qd = int(name[-2]), int(name[-1])
        eps = random_vector(12, 100) * 6.0
        t = L.chain(12, periodic=False, eps=eps)
        return 12, qu, qd, t, t, 1.0
    raise SystemExit(f"unknown case {name}")


def build_case(name: str):
    N, qu, qd, tu, td, U = case_spec(name)
    return Hubbard(H_TBq(N, qu).extend(tu), H_TBq(N, qd).extend(td), U)


def adjoint_run(name: str, op: Hubbard, steps: int) -> None:
    """The C5-style workload: a fixed-step Lanczos solve whose Ritz vector is
    regenerated by a second recurrence (three working vectors and u on the
    device, not the basis), then the adjoint derivatives
    dE0/dU = sum_i <n_i,up n_i,dn> and dE0/dt = <H_kin>/t (hopping terms
    -t with t = 1, so dE0/dt = <H_kin>), with E0 - <H_kin> - U dE0/dU as the
    Hellmann-Feynman consistency check.  Prints one JSON line."""
    import json
    import torch
    from . import observables as ob
    from .hubbard import Lanczos
    N, qu, qd, tu, td, U = case_spec(name)
    ev = torch.empty(op.rows(), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lz = Lanczos()
    e0, _ = lz.eigen(op, max_steps=steps, mode="fixed", ritz="recompute", seed=0, evec_out=ev)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    nu, nd, dd = ob.site_densities(op, ev)
    K = Hubbard(H_TBq(N, qu).extend(L.hopping_only(tu)), H_TBq(N, qd).extend(L.hopping_only(td)), 0.0)
    kin = ob.expect(K, ev)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    norm = float(torch.linalg.vector_norm(ev))
    K.close()
    print(json.dumps({"case": name, "dim": op.rows(), "lanczos_steps": steps, "ritz": "recompute",
                      "E0": e0, "dE0_dU": float(dd.sum()), "dE0_dt": kin,
                      "hf_check": e0 - kin - U * float(dd.sum()), "n_up": float(nu.sum()), "n_dn": float(nd.sum()),
                      "evec_norm": norm, "lanczos_s": round(t1 - t0, 3), "adjoint_s": round(t2 - t1, 3),
                      "matvec_kind": op.matvec_kind}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="kagome12")
    ap.add_argument("--what", default="lanczos", choices=["lanczos", "fused", "solve", "perform", "adjoint", "tune"])
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--ritz", default="none", choices=["none", "stored"],
                    help="stored: keep the Krylov basis and form the Ritz vector, as the bench does")
    args = ap.parse_args()
    import torch
    op = build_case(args.case)
    lib = _capi.load()
    t0 = time.perf_counter()
    if args.what == "adjoint":
        adjoint_run(args.case, op, args.steps)
    elif args.what == "tune":
        import json
        from . import sweeps
        info = op.autotune(steps=args.steps)
        info.pop("result")
        out = {"case": args.case, "dim": op.rows(), "matvec_kind": op.matvec_kind, "autotune": info}
        if op.matvec_kind != "two_pass":
            sample = [build_case(args.case) for _ in range(8)]
            if args.case.startswith("chain12_"):
                # eight disorder realisations of the sector (different on-site terms, same hops)
                qu, qd = int(args.case[-2]), int(args.case[-1])
                for o in sample:
                    o.close()
                sample = []
                for r in range(8):
                    eu, edn = sweeps.mbl_disorder(r, 12, 6.0)
                    sample.append(Hubbard(H_TBq(12, qu).extend(sweeps.mbl_chain_terms(eu)),
                                          H_TBq(12, qd).extend(sweeps.mbl_chain_terms(edn)), 1.0))
            out["batch_size"] = sweeps.tune_batch(sample)
            for o in sample:
                o.close()
        print(json.dumps(out))
    elif args.what in ("lanczos", "fused", "solve"):
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
