"""In-tree build of the C-ABI library ``_lib/libedgb300.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel (one -gencode, no
cmake), then linked into one shared library with the CUDA runtime.  The
library exports exactly the functions declared in ``include/ed_hubbard.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
BUILD = PKG / "_build"
LIBNAME = "libedgb300.so"

SOURCES = ["ed_tables.cpp", "ed_matvec.cu", "ed_matvec_tma.cu", "ed_matvec_striped.cu", "ed_lanczos.cu", "ed_lanczos_fused.cu", "ed_tridiag.cpp", "ed_capi.cu",
           "ed_observables.cu", "ed_noalloc.cu", "ed_krylov.cu", "ed_eigs.cu", "ed_ee_bidiag.cu", "ed_dense.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include")]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _compile(src: str) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *NVCC_FLAGS, "-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    lib = lib_path()
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "ed_hubbard.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False) -> Path:
    """Compile and link the library if any source is newer than it."""
    if not force and not _stale():
        return lib_path()
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    LIBDIR.mkdir(parents=True, exist_ok=True)
    tmp = LIBDIR / (LIBNAME + ".tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lcusolver", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


def build_oracle() -> Path:
    """Build the CPU checker (oracle/_build/liboracle.so) and, when the
    reference checkout is present, the reference table dumper."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    # the recipe knows where the reference checkout lies (REF_ROOT, or the
    # environment's ED_REFERENCE_ROOT) and skips the reference targets when it
    # is absent
    cmd = ["make", "-s", "-C", str(ROOT / "oracle"), "ref-if-present"]
    if os.environ.get("ED_REFERENCE_ROOT"):
        cmd.append(f"REF_ROOT={os.environ['ED_REFERENCE_ROOT']}")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference table dumper build failed:\n{r.stdout}\n{r.stderr}")
    return ROOT / "oracle" / "_build" / "liboracle.so"


if __name__ == "__main__":
    print(build(force=True))
    print(build_oracle())
