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
N_SITES, Q_UP, Q_DN, U, SEED = 12, 6, 6, 8.0, 0
# Lanczos steps per solve; ED_BENCH_SOLVE_STEPS shrinks the solve (both arms
# and the config alike) for the CPU tests of the rank logic only
STEPS = int(os.environ.get("ED_BENCH_SOLVE_STEPS", "300"))
METRIC = "Lanczos iterations/s (Kagome12 6+6 U=8, 300 steps + Ritz vector)"
UNIT = "iters/s"
GOLDEN = ROOT / "tests" / "golden"


def workload_config(world: int) -> dict:
    """The workload both arms run (identical dicts, so the two lines compare)."""
    import math
    return {"workload": WORKLOAD, "dim": math.comb(N_SITES, Q_UP) * math.comb(N_SITES, Q_DN),
            "lanczos_steps_per_solve": STEPS, "U": U,
            "lattice": "Kagome 12-site (reference KagomeLattice12 incl. -2 r^2 on-site)",
            "start_vector": "Philox4x64-10 uniform(-1,1), seed 0",
            "outputs": "E0 and the normalised ground-state Ritz vector",
            "l2": "GPU arm: 256 MB device write between solves (one solve's vectors fit in L2)",
            "parallelism": f"replicas x{world}"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample budget")
    p.add_argument("--records", default="c5,sweep",
                   help="extra records after the headline: c5 (Lieb18 9+9 matvec GB/s), sweep (C3 + C4 "
                        "batched+adjoint vs plain); 'none' for the headline alone")
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


def _oracle_solve(orc, t, f, steps: int, ritz: bool = True):
    """One oracle solve: `steps` fixed Lanczos steps (Lanczos::eigen restated)
    and, with ritz, the reference's second recurrence for the Ritz vector."""
    return orc.lanczos(t, t, U, f, steps, mode="fixed", want_evec=ritz)


def cpu_baseline(budget_s: float):
    """The oracle (C port of the reference matvec + Lanczos, OpenMP over all
    host cores) on a bounded sample of the same solve: whole solves (300
    steps + the second-pass Ritz vector) until about budget_s."""
    from oracle import oracle as orc
    t = orc.Tables(N_SITES, Q_UP, orc.kagome12_terms())
    f = orc.philox_uniform(SEED, t.count * t.count)
    n, dt = 0, 0.0
    while n == 0 or (dt < budget_s and n < 8):
        t0 = time.perf_counter()
        _oracle_solve(orc, t, f, STEPS)
        dt += time.perf_counter() - t0
        n += 1
    return {"value": n * STEPS / dt, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
            "sample": f"{n} whole solves (300 Lanczos steps + second-pass Ritz vector) of the Kagome12 6+6 U=8 "
                      f"workload, oracle/hubbard_oracle.c with OpenMP, {dt:.2f} s"}


def run_reference(args, world, rank):
    """Reference arm: the reference's own algorithm for this path on the host
    cores (the oracle's C restatement of Hubbard_mv_ + Lanczos::eigen with its
    second-pass Ritz rebuild; the reference's matvec exists only as a GPU
    kernel and its sources do not travel to the GPU host).  Same workload,
    metric and config as the GPU arm; every timed step is one whole solve.
    Builds everything from the oracle (tables, lattice, start vector): the
    product package is not imported."""
    if rank != 0:
        return
    from oracle import oracle as orc
    t = orc.Tables(N_SITES, Q_UP, orc.kagome12_terms())
    f = orc.philox_uniform(SEED, t.count * t.count)
    for _ in range(args.warmup):
        _oracle_solve(orc, t, f, 10)  # warm-up: short solves (caches, thread pool)
    times, e0 = [], None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e0, _, _, _ = _oracle_solve(orc, t, f, STEPS)
        times.append(time.perf_counter() - t0)
    v = STEPS * args.steps / sum(times)
    sample = f"whole solves: {STEPS} Lanczos steps + second-pass Ritz vector, oracle/hubbard_oracle.c (OpenMP)"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(world), "impl": "reference",
            "result": {"E0": e0},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.num_threads(), "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _peak() -> float:
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def _profile_json(name: str):
    p = ROOT / "profiles" / name
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def c5_record(ed, lib, n_mv: int = 4) -> dict:
    """Lieb18 9+9 (dim 2.36e9, 18.9 GB per vector, far beyond L2): the
    Lanczos-path matvec timed with CUDA events on its stream (per-step
    kernels, profile 1), n_mv matvecs after a 2-step warm-up solve.
    Algorithmic bytes: 16 B x dim (read x, write u)."""
    import ctypes as C
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi, lattices as L
    t0 = time.perf_counter()
    t = L.lieb18()
    op = ed.Hubbard(ed.H_TBq(18, 9).extend(t), ed.H_TBq(18, 9).extend(t), 4.0)
    D = op.rows()
    build_s = time.perf_counter() - t0
    res = _capi.ed_lanczos_result()

    def run(n):
        cfg = _capi.ed_lanczos_cfg(max_steps=n, mode=_capi.ED_LANCZOS_FIXED, reorth=0, ritz=_capi.ED_RITZ_NONE,
                                   start=_capi.ED_START_RANDOM, profile=1, seed=SEED)
        _capi.check(lib.ed_lanczos_run(op.handle, C.byref(cfg), None, 0, None, 0, None, None, C.byref(res), None),
                    "ed_lanczos_run(lieb18)")

    run(2)
    run(n_mv)
    ms = res.matvec_ms / max(res.n_matvec, 1)
    axpy_ms = res.axpy_ms / max(res.n_matvec, 1)
    gbs = 16.0 * D / (ms * 1e-3) / 1e9
    peak = _peak()
    prof = _profile_json("lieb18_matvec_traffic.json")
    kind = op.matvec_kind
    op.close()
    # the gathers' own floor: every hop of every element loads one 8-byte
    # neighbour value into the SM (up and down terms), at most 128 B per
    # clock per SM through the L1/shared-memory path
    import numpy as np
    import torch
    ax, _ = ed.H_TBq(18, 9).extend(t).ell()
    nnz = int(np.count_nonzero(ax))
    dim = ed.binom(18, 9)
    gather_bytes = 8.0 * 2 * nnz * dim
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    try:
        clk = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["sm_max_mhz"]) * 1e6
    except (OSError, ValueError, KeyError):
        clk = 2.07e9
    floor_ms = gather_bytes / (sms * 128.0 * clk) * 1e3
    return {"workload": "lieb18_q99_U4_matvec", "dim": D, "matvecs": int(res.n_matvec), "matvec_kind": kind,
            "ms_per_matvec": ms, "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak,
            "bytes_per_matvec": 16.0 * D, "traffic_per_matvec": prof.get("dram_bytes_per_matvec"),
            "axpy_ms_per_step": axpy_ms, "min_bits": int(res.min_bits),
            "gather_bytes_per_matvec": gather_bytes, "load_path_floor_ms": floor_ms,
            "frac_of_load_path_floor": floor_ms / ms,
            "load_path_note": "2 x nnz(spin table) x dim 8-byte neighbour loads at 128 B/clk/SM (L1/shared path), "
                              "SM count and max SM clock of this GPU",
            "timing": "CUDA events on the launching stream around each matvec (both passes), vectors 18.9 GB "
                      "(no L2 flush needed)",
            "setup_s": round(time.perf_counter() - t0 - 0.0, 2), "build_s": round(build_s, 2)}


def _golden_sweep_e0() -> dict:
    table = {}
    try:
        fx = json.loads((GOLDEN / "flux_kagome12_q66_U4.json").read_text())
        for p in fx["points"]:
            table[round(p["phi"], 12)] = p["E0"]
        mb = json.loads((GOLDEN / "sweep_chain12_W6.json").read_text())
        for p in mb["points"]:
            table[(p["realisation"], tuple(p["sector"]))] = p["E0"]
    except (OSError, ValueError, KeyError):
        pass
    return table


def sweep_record() -> dict:
    """C3 (16 twists of Kagome12 6+6 U=4: E0, dE0/dPhi, d2E0/dPhi2) + C4 (64
    disorder realisations x 3 sectors of the L=12 chain: E0, entanglement,
    dE0/d eps_i), fixed Lanczos steps per instance (500 per twist, 300 per
    disorder sample), in three forms: tuned (batched + adjoint), plain
    per-instance, and plain per-instance with the tuned entanglement path.
    Host clock with device synchronisation."""
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import sweeps
    table = _golden_sweep_e0()
    out = {"workload": "C3 16 twists Kagome12 6+6 U=4 + C4 64 realisations x (6,6),(7,5),(8,4) L=12 U=1 W=6",
           "lanczos_steps": {"twist": sweeps.FLUX_STEPS, "disorder": 300},
           "response_steps": sweeps.FLUX_RESPONSE_STEPS, "forms": {}}
    worst, bits = float("nan"), 1 << 30
    for form in ("tuned", "plain_same_ee", "plain"):
        tot, parts = 0.0, {}
        for what, n in (("flux", 16), ("mbl", 64)):
            pts, tm = sweeps.run_form(what, n, form)
            tot += tm.total_s
            parts[what] = tm.summary()
            if form == "tuned":
                e = sweeps.attach_oracle(pts, table)
                worst = e if not worst >= e else worst
                bits = min(bits, min(p.min_bits for p in pts))
        out["forms"][form] = {"total_s": round(tot, 4), **{k: v["total_s"] for k, v in parts.items()}}
    t = out["forms"]["tuned"]["total_s"]
    out["speedup_vs_plain"] = round(out["forms"]["plain"]["total_s"] / t, 3)
    out["speedup_vs_plain_same_entropy"] = round(out["forms"]["plain_same_ee"]["total_s"] / t, 3)
    out["batch_sizes"] = sweeps.batch_choices()
    out["err_vs_oracle_max"] = worst
    out["err_vs_oracle_instances"] = len(table)
    out["min_bits"] = bits
    return out


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
    peak = _peak()
    traffic = _profile_json("lz_fused_kagome12_traffic.json").get("dram_bytes_per_launch")
    min_bits = int(res.min_bits)
    per_step = lambda t: t / max(nmv, 1) * 1000.0  # noqa: E731  (ms summed over steps -> us per step)

    records = [r for r in args.records.split(",") if r and r != "none"]
    extra = {}
    if "c5" in records:
        extra["c5_matvec"] = c5_record(ed, lib)
    if "sweep" in records:
        extra["sweep"] = sweep_record()
    try:
        e0_oracle = json.loads((GOLDEN / "energies.json").read_text())["kagome12_q66_U8"]["E0"]
    except (OSError, ValueError, KeyError):
        e0_oracle = None

    if rank == 0:
        cpu = cpu_baseline(args.cpu_seconds) if world >= 1 else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": workload_config(world),
            "result": {"E0": e0s[-1],
                       "err_vs_oracle": abs(e0s[-1] - e0_oracle) if e0_oracle is not None else None,
                       "oracle": "scipy eigsh (tol 1e-13) of the oracle's Kronecker-sum Hamiltonian, "
                                 "tests/golden/energies.json kagome12_q66_U8",
                       "min_bits": min_bits,
                       "arithmetic": "int64 fixed point, one exponent per vector, exact integer sums, one "
                                     "rounding per element; FP64 scalars and boundary vectors",
                       "ritz": "stored Krylov basis"},
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
            **extra,
        }
        print(json.dumps(line), flush=True)
    op.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
