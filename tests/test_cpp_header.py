"""The header-only C++ surface (include/ed_hubbard.hpp) compiles against the
C ABI, links the library, and (on a GPU) reproduces the golden E0."""
import shutil
import subprocess

import pytest

from conftest import ROOT


def build_example(tmp_path, edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _capi
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    libdir = _capi.lib_path().parent
    exe = tmp_path / "chain8_lanczos"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests/cpp/chain8_lanczos.cpp"),
                    "-o", str(exe), f"-L{libdir}", "-ledgb300", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def test_cpp_header_builds_and_runs_host_part(tmp_path, edlib):
    exe = build_example(tmp_path, edlib)
    out = subprocess.run([str(exe), "--basis-only"], capture_output=True, text=True, check=True).stdout
    assert "count 70 first 15 last 240" in out


@pytest.mark.gpu
def test_cpp_header_lanczos_on_gpu(tmp_path, edlib, golden_energies):
    exe = build_example(tmp_path, edlib)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    e0 = float(out.split("E0 ")[1].split()[0])
    g = golden_energies["chain8_pbc_q44_U4"]["E0"]
    assert abs(e0 - g) < 1e-10 * abs(g)
    eig = out.split("EIGS ")[1].split()
    assert int(eig[0]) == 3 and abs(float(eig[1]) - g) < 1e-10 * abs(g)
    assert abs(float(eig[2]) - golden_energies["chain8_pbc_q44_U4"]["E1"]) < 1e-9
    ee = out.split("EE ")[1].split()
    assert abs(float(ee[0]) - golden_energies["chain8_pbc_q44_U4"]["EE_vN_A0123"]) < 1e-8
    assert ee[2] == "1" and int(ee[3]) in (0, 1, 2)
    kry = out.split("KRYLOV ")[1].split()
    assert abs(float(kry[3]) - 1.0) < 1e-12
    bat = out.split("BATCH ")[1].split()
    assert bat[2] == "1" and abs(float(bat[0]) - g) < 1e-9 * abs(g)


def test_gather_schedule_host_check(tmp_path):
    """The down-term gather schedule (host code, no GPU): every table entry
    scheduled exactly once, no bank pair used twice by one half warp in one
    step, step counts covering the entries; and the persistent kernel's unit
    queue covering every (row, column) exactly once."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    csrc = ROOT / "exact_diagonalization_for_fermionic_systems_with_gpu_gb300/csrc"
    exe = tmp_path / "gather_schedule_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(csrc), str(ROOT / "tests/cpp/gather_schedule_check.cpp"),
                    str(csrc / "ed_tables.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.strip().splitlines()
    assert len(lines) == 6 and all(l.endswith(" ok") for l in lines)
    assert lines[-1] == "unit queue ok"
