"""Multi-GPU is replicas only: every rank solves its own instance and the
bench reports the maximum time over ranks.  The rank logic runs here as two
gloo processes on the CPU (no GPU involved)."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_max_over_ranks_and_barrier_gloo():
    port = free_port()
    code = ("import sys; sys.path.insert(0, %r); import bench; "
            "w, r, l = bench.dist_setup(2); bench.barrier(w); "
            "print('MAX', bench.max_over_ranks(w, 1.5 + r)); "
            "import torch.distributed as d; d.destroy_process_group()") % str(ROOT)
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), ED_BENCH_BACKEND="gloo")
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
        assert "MAX 2.5" in o


def test_reference_arm_two_ranks_rank0_prints_once():
    """bench.py --impl reference under torchrun (world size 2, gloo): rank 0
    alone runs the host-core reference sample and prints one JSON line; the
    other rank exits 0 without work."""
    port = free_port()
    env = dict(os.environ, ED_BENCH_BACKEND="gloo", ED_BENCH_SOLVE_STEPS="10")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.3"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["config"]["lanczos_steps_per_solve"] == 10
