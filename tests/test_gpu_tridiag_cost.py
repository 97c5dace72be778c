"""Where the Lanczos tridiagonal eigensolve runs: on this GPU FP64 issues at
1/64 of the FP32 rate, so the host's Sturm bisection run by one device
thread (tests/cpp/tridiag_device_cost.cu) reproduces the host's eigenvalue
bit for bit but takes tens of times longer than the host cores; the test
checks the bit-identity and that the device is the slower place, and prints
the timings."""
import shutil
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_device_bisection_reproduces_host_and_costs_more(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    csrc = ROOT / "exact_diagonalization_for_fermionic_systems_with_gpu_gb300" / "csrc"
    exe = tmp_path / "tridiag_device_cost"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I", str(csrc),
                    str(ROOT / "tests/cpp/tridiag_device_cost.cu"), str(csrc / "ed_tridiag.cpp"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = [l.split() for l in out.stdout.splitlines() if l.startswith("n=300 thread1")]
    assert rows
    dev_us, host_us = float(rows[0][3]), float(rows[0][6])
    assert dev_us > 5 * host_us
