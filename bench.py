#!/usr/bin/env python3
"""Benchmark: Lanczos iterations/s of the Kagome 12-site cluster, 6+6, U=8
(dim 924^2 = 853,776), 300 fixed steps from a seeded uniform(-1,1) start
vector, E0 plus the ground-state Ritz vector — one "step" of this bench is
one such solve.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is whole-job Lanczos iterations/s
with the operator tables resident in HBM; `e2e` is the same metric through
the C ABI with the start vector coming from pinned host memory and the Ritz
vector going back to it inside the timed region.  With N > 1 (torchrun) every
rank solves its own replica (the path does not shard): scaling "weak".
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "kagome12_q66_U8_lanczos300_ritz"
N_SITES, Q_UP, Q_DN, U, STEPS, SEED = 12, 6, 6, 8.0, 300, 0
METRIC = "Lanczos iterations/s (Kagome12 6+6 U=8, 300 steps + Ritz vector)"
UNIT = "iters/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample budget")
    return p.parse_args()


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("ED_BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_op(ed, device):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    t = L.kagome12()
    return ed.Hubbard(ed.H_TBq(N_SITES, Q_UP).extend(t), ed.H_TBq(N_SITES, Q_DN).extend(t), U, device=device)


def cpu_baseline(budget_s: float, steps_hint: int | None = None):
    """The oracle (C port of the reference matvec + Lanczos, OpenMP over all
    host cores) on a bounded sample of the same solve."""
    import numpy as np
    from oracle import oracle as orc
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L
    t = orc.Tables(N_SITES, Q_UP, L.kagome12())
    f = np.empty(t.count * t.count)
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import hubbard
    f[:] = hubbard.random_vector(f.size, SEED)
    t0 = time.perf_counter()
    orc.lanczos(t, t, U, f, 3, mode="fixed", want_evec=False)
    per = (time.perf_counter() - t0) / 3
    n = steps_hint or max(3, min(STEPS, int(budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    orc.lanczos(t, t, U, f, n, mode="fixed", want_evec=False)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
            "sample": f"{n} Lanczos steps (matvec + recurrence, no Ritz pass) of the Kagome12 6+6 U=8 solve, "
                      f"oracle/hubbard_oracle.c with OpenMP, {dt:.2f} s"}


def run_reference(args, world, rank):
    """Reference arm: the reference's own algorithm on the host cores (the
    oracle port; the reference has no CPU matvec of its own and its sources do
    not travel to the GPU host), same metric and workload, bounded samples."""
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as orc
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import lattices as L, hubbard
    t = orc.Tables(N_SITES, Q_UP, L.kagome12())
    f = hubbard.random_vector(t.count * t.count, SEED)
    t0 = time.perf_counter()
    orc.lanczos(t, t, U, f, 2, mode="fixed", want_evec=False)
    per = (time.perf_counter() - t0) / 2
    n = max(2, min(STEPS, int(min(8.0, args.cpu_seconds) / max(per, 1e-6))))
    for _ in range(args.warmup):
        orc.lanczos(t, t, U, f, 2, mode="fixed", want_evec=False)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.lanczos(t, t, U, f, n, mode="fixed", want_evec=False)
        times.append(time.perf_counter() - t0)
    v = n * args.steps / sum(times)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "dim": t.count * t.count, "sample_steps_per_bench_step": n},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
                             "sample": f"{n} Lanczos steps per bench step, oracle/hubbard_oracle.c (OpenMP)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    import exact_diagonalization_for_fermionic_systems_with_gpu_gb300 as ed
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi, _build
    _build.build()
    lib = _capi.load()
    op = make_op(ed, local)
    D = op.rows()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    cfg = _capi.ed_lanczos_cfg(max_steps=STEPS, mode=_capi.ED_LANCZOS_FIXED, reorth=0, ritz=_capi.ED_RITZ_STORED,
                               start=_capi.ED_START_RANDOM, profile=0, seed=SEED)
    # same solve with CUDA events around the persistent Lanczos launch and
    # device timestamps of its phases (roofline)
    cfg_prof = _capi.ed_lanczos_cfg(max_steps=STEPS, mode=_capi.ED_LANCZOS_FIXED, reorth=0,
                                    ritz=_capi.ED_RITZ_STORED, start=_capi.ED_START_RANDOM, profile=2, seed=SEED)
    evec_dev = torch.empty(D, dtype=torch.float64, device="cuda")
    res = _capi.ed_lanczos_result()

    def solve_device(c=cfg):
        st = lib.ed_lanczos_run(op.handle, C.byref(c), None, 0, C.c_void_p(evec_dev.data_ptr()),
                                _capi.ED_MEM_DEVICE, None, None, C.byref(res), None)
        _capi.check(st, "ed_lanczos_run")
        return res.e0

    for _ in range(args.warmup):
        solve_device()
    torch.cuda.synchronize()

    e0s, ms, launches = [], [], 0
    mv_ms = ax_ms = rd_ms = fz_ms = 0.0
    nmv = 0
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between solves (not timed)
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            e0s.append(solve_device())
            ev1.record()
            torch.cuda.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            launches += res.launches
    torch.cuda.synchronize()
    barrier(world)
    ms_per_step = max_over_ranks(world, sum(ms) / len(ms))
    value = world * STEPS / (ms_per_step / 1000.0)
    # dominant kernel: CUDA events on the launching stream around the
    # persistent launch of additional solves (not part of `value`), and the
    # per-step split of its time from device timestamps
    n_prof = 3
    for _ in range(n_prof):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        solve_device(cfg_prof)
        mv_ms += res.matvec_ms
        ax_ms += res.axpy_ms
        rd_ms += res.reduce_ms
        fz_ms += res.fused_ms
        nmv += res.n_matvec

    # e2e: host start vector in, host Ritz vector out, through the C ABI
    f_host = torch.from_numpy(ed.random_vector(D, SEED)).pin_memory()
    evec_host = torch.empty(D, dtype=torch.float64).pin_memory()
    cfg_e2e = _capi.ed_lanczos_cfg(max_steps=STEPS, mode=_capi.ED_LANCZOS_FIXED, reorth=0, ritz=_capi.ED_RITZ_STORED,
                                   start=_capi.ED_START_USER, profile=0, seed=SEED)
    alpha = np.zeros(STEPS)
    beta = np.zeros(STEPS + 1)
    res2 = _capi.ed_lanczos_result()

    def solve_e2e():
        st = lib.ed_lanczos_run(op.handle, C.byref(cfg_e2e), C.c_void_p(f_host.data_ptr()), _capi.ED_MEM_HOST,
                                C.c_void_p(evec_host.data_ptr()), _capi.ED_MEM_HOST,
                                C.c_void_p(alpha.ctypes.data), C.c_void_p(beta.ctypes.data), C.byref(res2), None)
        _capi.check(st, "ed_lanczos_run(e2e)")

    for _ in range(max(1, args.warmup)):
        solve_e2e()
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solve_e2e()
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(world, sum(e2e_t) / len(e2e_t))
    e2e_value = world * STEPS / e2e_s

    # roofline of the dominant kernel, the persistent Lanczos launch (one per
    # solve, STEPS steps): algorithmic bytes per step are the matvec's read of
    # w_j and write of u (16 B x dim) plus the axpy's reads of u, w_j, w_{j-1}
    # and write of w_{j+1} (32 B x dim)
    fused_ms = fz_ms / n_prof
    alg_bytes = 48.0 * D * STEPS
    achieved = alg_bytes / (fused_ms * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    prof = ROOT / "profiles" / "lz_fused_kagome12_traffic.json"
    if prof.exists():
        try:
            traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch")
        except ValueError:
            traffic = None
    per_step = lambda t: t / max(nmv, 1) * 1000.0  # noqa: E731  (ms summed over steps -> us per step)

    if rank == 0:
        cpu = cpu_baseline(args.cpu_seconds) if world >= 1 else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "dim": D, "lanczos_steps_per_solve": STEPS, "U": U,
                       "lattice": "Kagome 12-site (reference KagomeLattice12 incl. -2 r^2 on-site)",
                       "start_vector": "Philox4x64-10 uniform(-1,1), seed 0", "ritz": "stored Krylov basis",
                       "l2": "256 MB write between solves (vectors themselves fit in L2)",
                       "parallelism": f"replicas x{world}", "E0": e0s[-1]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * D,
                    "d2h_bytes_per_step": 8 * D + 8 * (2 * STEPS + 1)},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_lz_fused<real, single class, gather schedule>",
                         "note": "one launch per solve; achieved = 48 B x dim x steps / mean CUDA-event duration of "
                                 "the launch; peak = measured HBM copy bandwidth (of measured); the vectors "
                                 "(6.8 MB each) are L2-resident, HBM sees the Krylov basis write-back",
                         "avg_launch_us": fused_ms * 1000.0,
                         "per_step_us": {"matvec_rows": per_step(mv_ms), "axpy": per_step(ax_ms),
                                         "reductions_barriers": per_step(rd_ms)}},
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    op.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
