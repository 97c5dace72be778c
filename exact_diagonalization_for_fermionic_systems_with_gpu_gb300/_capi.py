"""ctypes binding of the C ABI declared in include/ed_hubbard.h.

Loading fails loudly when the compiled library is absent: there is no CPU
fallback behind this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB = None

ED_OK = 0
ED_ERR_ARG, ED_ERR_CUDA, ED_ERR_ALLOC, ED_ERR_TABLE, ED_ERR_RANGE = 1, 2, 3, 4, 5
ED_ERR_NONFINITE, ED_ERR_BREAKDOWN, ED_ERR_NOT_CONVERGED, ED_ERR_TIMEOUT, ED_ERR_NOT_BUILT = 6, 7, 8, 9, 10
STATUS_NAMES = {
    0: "ED_OK", 1: "ED_ERR_ARG", 2: "ED_ERR_CUDA", 3: "ED_ERR_ALLOC", 4: "ED_ERR_TABLE",
    5: "ED_ERR_RANGE", 6: "ED_ERR_NONFINITE", 7: "ED_ERR_BREAKDOWN", 8: "ED_ERR_NOT_CONVERGED",
    9: "ED_ERR_TIMEOUT", 10: "ED_ERR_NOT_BUILT",
}

ED_TERM_HOP, ED_TERM_CURRENT, ED_TERM_DENSITY, ED_TERM_PEIERLS = 0, 1, 2, 3
ED_OP_REAL, ED_OP_COMPLEX = 0, 1
ED_MV_GENERIC, ED_MV_ROWS, ED_MV_TWO_PASS = 0, 1, 2
ED_MEM_HOST, ED_MEM_DEVICE = 0, 1
ED_LANCZOS_REFERENCE, ED_LANCZOS_FIXED = 0, 1
ED_RITZ_NONE, ED_RITZ_STORED, ED_RITZ_RECOMPUTE = 0, 1, 2
ED_START_RANDOM, ED_START_USER = 0, 1


class EdError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({status})")
        self.status = status


class ed_term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("i", C.c_int32), ("j", C.c_int32), ("pad_", C.c_int32),
                ("value", C.c_double), ("phase", C.c_double)]


class ed_model_desc(C.Structure):
    _fields_ = [("n_sites", C.c_int32), ("n_up", C.c_int32), ("n_dn", C.c_int32), ("flags", C.c_int32),
                ("up_terms", C.POINTER(ed_term)), ("n_up_terms", C.c_int32), ("pad0_", C.c_int32),
                ("dn_terms", C.POINTER(ed_term)), ("n_dn_terms", C.c_int32), ("pad1_", C.c_int32),
                ("U", C.c_double), ("interaction_mask", C.c_uint64)]


class ed_lanczos_cfg(C.Structure):
    _fields_ = [("max_steps", C.c_int32), ("mode", C.c_int32), ("reorth", C.c_int32), ("ritz", C.c_int32),
                ("start", C.c_int32), ("profile", C.c_int32), ("seed", C.c_uint64)]


class ed_lanczos_result(C.Structure):
    _fields_ = [("e0", C.c_double), ("steps", C.c_int32), ("converged", C.c_int32), ("status", C.c_int32),
                ("min_bits", C.c_int32), ("residual", C.c_double), ("launches", C.c_int64),
                ("matvec_ms", C.c_double), ("axpy_ms", C.c_double), ("n_matvec", C.c_int32), ("pad_", C.c_int32),
                ("reduce_ms", C.c_double), ("barrier_ms", C.c_double), ("scalar_ms", C.c_double),
                ("fused_ms", C.c_double), ("rows_spread_ms", C.c_double), ("axpy_spread_ms", C.c_double)]


class ed_kubo_cfg(C.Structure):
    _fields_ = [("lanczos_steps", C.c_int32), ("n_omega", C.c_int32), ("omega_step", C.c_double),
                ("delta", C.c_double), ("omega_cutoff", C.c_double), ("volume", C.c_double)]


class ed_kubo_result(C.Structure):
    _fields_ = [("drude", C.c_double), ("kinetic", C.c_double), ("vertex", C.c_double)]


class ed_tune_cfg(C.Structure):
    _fields_ = [("steps", C.c_int32), ("apply", C.c_int32)]


class ed_tune_result(C.Structure):
    _fields_ = [("persistent", C.c_int32), ("candidates", C.c_int32), ("row_cost", C.c_double),
                ("us_per_step", C.c_double), ("per_step_us", C.c_double), ("persistent_us", C.c_double * 3),
                ("ctas_per_sm", C.c_int32), ("chunk", C.c_int32), ("one_cta_us", C.c_double),
                ("chunk_us", C.c_double * 2)]


class ed_eigs_cfg(C.Structure):
    _fields_ = [("nev", C.c_int32), ("ncv", C.c_int32), ("max_restarts", C.c_int32), ("start", C.c_int32),
                ("tol", C.c_double), ("seed", C.c_uint64)]


class ed_eigs_result(C.Structure):
    _fields_ = [("nconv", C.c_int32), ("restarts", C.c_int32), ("n_matvec", C.c_int64), ("launches", C.c_int64),
                ("max_resid", C.c_double)]


class ed_krylov_cfg(C.Structure):
    _fields_ = [("max_steps", C.c_int32), ("reorth", C.c_int32), ("tol", C.c_double), ("accumulate", C.c_int32),
                ("pad_", C.c_int32)]


class ed_krylov_result(C.Structure):
    _fields_ = [("steps", C.c_int32), ("runs", C.c_int32), ("norm", C.c_double), ("err_est", C.c_double),
                ("launches", C.c_int64)]


# name -> (restype, argtypes); the list is also the export check used by the tests
SIGNATURES = {
    "ed_status_string": (C.c_char_p, [C.c_int]),
    "ed_version": (C.c_int, []),
    "ed_binom": (C.c_int64, [C.c_int, C.c_int]),
    "ed_basis_unrank": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p]),
    "ed_basis_rank": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p]),
    "ed_basis_unrank_device": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "ed_basis_rank_device": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "ed_tables_ell": (C.c_int, [C.c_int, C.c_int, C.POINTER(ed_term), C.c_int, C.c_void_p, C.c_void_p,
                                C.c_void_p]),
    "ed_op_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(ed_model_desc), C.c_int]),
    "ed_op_destroy": (C.c_int, [C.c_void_p]),
    "ed_op_rows": (C.c_int64, [C.c_void_p]),
    "ed_op_cols": (C.c_int64, [C.c_void_p]),
    "ed_op_dim_up": (C.c_int64, [C.c_void_p]),
    "ed_op_dim_dn": (C.c_int64, [C.c_void_p]),
    "ed_op_is_complex": (C.c_int, [C.c_void_p]),
    "ed_op_matvec_kind": (C.c_int, [C.c_void_p]),
    "ed_op_perform": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "ed_op_perform_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_lanczos_run": (C.c_int, [C.c_void_p, C.POINTER(ed_lanczos_cfg), C.c_void_p, C.c_int, C.c_void_p,
                                 C.c_int, C.c_void_p, C.c_void_p, C.POINTER(ed_lanczos_result), C.c_void_p]),
    "ed_lanczos_batch": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(ed_lanczos_cfg), C.c_void_p, C.c_int, C.c_void_p,
                                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_op_autotune": (C.c_int, [C.c_void_p, C.POINTER(ed_tune_cfg), C.POINTER(ed_tune_result), C.c_void_p]),
    "ed_op_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(ed_tune_result)]),
    "ed_op_write_dense": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "ed_random_vector": (C.c_int, [C.c_int64, C.c_uint64, C.c_void_p]),
    "ed_random_vector_device": (C.c_int, [C.c_int64, C.c_uint64, C.c_void_p, C.c_void_p]),
    "ed_tridiag_lowest": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_vec_dot": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ed_vec_zdot": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ed_op_expect": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ed_s2_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "ed_s2_expect": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ed_site_densities": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "ed_continued_fraction": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int,
                                        C.c_void_p, C.c_void_p]),
    "ed_drude_kubo": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                C.POINTER(ed_kubo_cfg), C.POINTER(ed_kubo_result), C.c_void_p, C.c_void_p]),
    "ed_response": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                              C.c_void_p, C.c_void_p]),
    "ed_response_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_response_subspace": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_entanglement_entropy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_uint64, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    "ed_entanglement_entropy_batch": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_uint64, C.c_void_p,
                                                C.c_void_p, C.c_void_p]),
    "ed_tridiag_eigen": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_bidiag_singular_values": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_tridiag_expm": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ed_eigs_lowest": (C.c_int, [C.c_void_p, C.POINTER(ed_eigs_cfg), C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                 C.c_int, C.c_void_p, C.POINTER(ed_eigs_result), C.c_void_p]),
    "ed_dense_sym_eigen": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ed_krylov_evolve": (C.c_int, [C.c_void_p, C.POINTER(ed_krylov_cfg), C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_int, C.POINTER(ed_krylov_result), C.c_void_p]),
}


def lib_path() -> Path:
    return Path(__file__).resolve().parent / "_lib" / "libedgb300.so"


def load(build_if_missing: bool = False):
    """Load the C-ABI library (building it first when asked)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not p.exists():
        if not build_if_missing:
            raise ImportError(f"{p} is missing; build it with exact_diagonalization_for_fermionic_systems_with_gpu_gb300"
                              "._build.build() (nvcc, sm_103a)")
        from . import _build
        _build.build()
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int, where: str) -> None:
    if status != ED_OK:
        raise EdError(status, where)
