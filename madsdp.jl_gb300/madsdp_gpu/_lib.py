"""ctypes binding of libmadsdp_gpu.so (include/madsdp_gpu.h).

The structs below mirror the C declarations field by field.  Loading fails
loudly when the library has not been built: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libmadsdp_gpu.so")

i32, i64, f64 = C.c_int32, C.c_int64, C.c_double
P = C.POINTER


class Components(C.Structure):
    _fields_ = [
        ("algorithm", i32), ("direction", i32), ("step", i32), ("centering", i32),
        ("initial_point", i32), ("schur", i32), ("precision", i32), ("centering_max_iter", i32),
        ("tau", f64), ("shrink", f64), ("boundary", f64), ("sigma_exponent", f64),
        ("initial_ratio", f64), ("ratio", f64), ("scale", f64), ("initial_shift", f64),
        ("max_shift", f64), ("dc_beta", f64), ("dc_delta", f64), ("dc_A", f64),
    ]


class Options(C.Structure):
    _fields_ = [
        ("tol", f64), ("max_iter", i32), ("max_schur_reg", i32), ("max_wall_time", f64),
        ("mu_min", f64), ("regularize_schur", f64), ("datasparsity", i32), ("mixed_refine", i32),
        ("switch_tol", f64),
    ]


class ProblemDesc(C.Structure):
    _fields_ = [
        ("nblocks", i32), ("m", i32), ("ns", i32), ("pad0", i32),
        ("sides", P(i32)), ("C", P(P(f64))), ("A_nnz", P(i64)),
        ("A_con", P(P(i32))), ("A_row", P(P(i32))), ("A_col", P(P(i32))), ("A_val", P(P(f64))),
        ("b", P(f64)), ("d_lin", P(f64)), ("C_lin", P(f64)),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("status", i32), ("iter", i32), ("iter_fp32", i32), ("iter_fp64", i32),
        ("pobj", f64), ("dobj", f64), ("inf_pr", f64), ("inf_du", f64), ("gap", f64),
        ("mu", f64), ("sigma", f64), ("alpha", f64), ("beta", f64), ("solve_ns", f64),
        ("n_newton", i32), ("n_predictor", i32),
    ]


class IterRecord(C.Structure):
    _fields_ = [(k, f64) for k in ("iter", "pobj", "dobj", "inf_pr", "inf_du", "gap", "mu", "alpha", "beta", "phase")]


# (name, restype, argtypes) for every symbol declared in include/madsdp_gpu.h
SIGNATURES = [
    ("msdp_default_components", None, [P(Components)]),
    ("msdp_default_options", None, [P(Options)]),
    ("msdp_context_create", i32, [C.c_int, P(C.c_void_p)]),
    ("msdp_context_destroy", i32, [C.c_void_p]),
    ("msdp_last_error", C.c_char_p, [C.c_void_p]),
    ("msdp_context_stream", C.c_void_p, [C.c_void_p]),
    ("msdp_device_count", i32, []),
    ("msdp_batch_create", i32, [C.c_void_p, P(ProblemDesc), i32, P(Components), P(Options), P(C.c_void_p)]),
    ("msdp_batch_destroy", i32, [C.c_void_p]),
    ("msdp_batch_device_bytes", i64, [C.c_void_p]),
    ("msdp_batch_set_initial_point", i32, [C.c_void_p, i32, P(P(f64)), P(f64), P(f64)]),
    ("msdp_batch_set_iterate", i32, [C.c_void_p, i32, P(P(f64)), P(P(f64)), P(f64), P(f64), P(f64)]),
    ("msdp_batch_initialize", i32, [C.c_void_p]),
    ("msdp_batch_launch_solve", i32, [C.c_void_p]),
    ("msdp_batch_launch_initialize", i32, [C.c_void_p]),
    ("msdp_batch_upload_bytes", i64, [C.c_void_p]),
    ("msdp_batch_iterate", i32, [C.c_void_p, i32]),
    ("msdp_batch_solve", i32, [C.c_void_p]),
    ("msdp_batch_synchronize", i32, [C.c_void_p]),
    ("msdp_batch_get_stats", i32, [C.c_void_p, i32, P(Stats)]),
    ("msdp_batch_get_all_stats", i32, [C.c_void_p, P(Stats)]),
    ("msdp_batch_get_solution", i32, [C.c_void_p, i32, P(P(f64)), P(f64), P(f64), P(f64)]),
    ("msdp_batch_solution_size", i64, [C.c_void_p]),
    ("msdp_batch_get_all_solutions", i32, [C.c_void_p, P(f64)]),
    ("msdp_batch_get_trajectory", i32, [C.c_void_p, i32, P(IterRecord), i32, P(i32)]),
    ("msdp_batch_update_residuals", i32, [C.c_void_p]),
    ("msdp_batch_prepare", i32, [C.c_void_p, P(i32)]),
    ("msdp_batch_solve_directions", i32, [C.c_void_p, f64, i32]),
    ("msdp_batch_correction", i32, [C.c_void_p]),
    ("msdp_batch_get_directions", i32, [C.c_void_p, i32, P(P(f64)), P(P(f64)), P(f64), P(f64), P(f64)]),
    ("msdp_batch_get_residuals", i32, [C.c_void_p, i32, P(f64), P(P(f64)), P(f64)]),
    ("msdp_batch_get_block_matrix", i32, [C.c_void_p, i32, i32, i32, P(f64)]),
    ("msdp_batch_launch_count", i64, [C.c_void_p]),
    ("msdp_batch_get_profile", i32, [C.c_void_p, i32, P(f64), i32]),
    ("msdp_profile_field_name", C.c_char_p, [i32]),
    ("msdp_server_create", i32, [C.c_void_p, P(Components), P(Options), i64, i32, P(C.c_void_p)]),
    ("msdp_server_destroy", i32, [C.c_void_p]),
    ("msdp_server_submit", i32, [C.c_void_p, P(ProblemDesc), P(i64)]),
    ("msdp_server_step", i32, [C.c_void_p, i32, P(i32), P(i32)]),
    ("msdp_server_step_budget", i32, [C.c_void_p, i32, f64, P(i32), P(i32)]),
    ("msdp_server_counts", i32, [C.c_void_p, P(i32), P(i32), P(i64)]),
    ("msdp_server_result", i32, [C.c_void_p, i64, P(Stats), P(P(f64)), P(f64), P(f64), P(f64), P(f64)]),
    ("msdp_server_finished", i32, [C.c_void_p, P(i64), i32, P(i32)]),
    ("msdp_server_launch_count", i64, [C.c_void_p]),
    ("msdp_solve_static", i32, [P(ProblemDesc), P(Components), P(Options), C.c_void_p, P(P(f64)), P(f64),
                                P(f64), P(f64), P(Stats)]),
    ("msdp_solver_create", i32, [C.c_void_p, P(ProblemDesc), P(Components), P(Options), P(C.c_void_p)]),
    ("msdp_solver_destroy", i32, [C.c_void_p]),
    ("msdp_solver_set_initial_point", i32, [C.c_void_p, P(P(f64)), P(f64), P(f64)]),
    ("msdp_solver_solve", i32, [C.c_void_p]),
    ("msdp_solver_get_stats", i32, [C.c_void_p, P(Stats)]),
    ("msdp_solver_get_solution", i32, [C.c_void_p, P(P(f64)), P(f64), P(f64), P(f64)]),
    ("msdp_solver_get_trajectory", i32, [C.c_void_p, P(IterRecord), i32, P(i32)]),
    ("msdp_solver_device_bytes", i64, [C.c_void_p]),
    ("msdp_solver_get_profile", i32, [C.c_void_p, P(f64), i32]),
    ("msdp_solver_profile_field_name", C.c_char_p, [i32]),
    ("msdp_solver_get_counters", i32, [C.c_void_p, P(i64), i32]),
    ("msdp_solver_counter_name", C.c_char_p, [i32]),
    ("msdp_solver_launch_count", i64, [C.c_void_p]),
    ("msdp_solver_last_error", C.c_char_p, [C.c_void_p]),
    ("msdp_solver_set_iterate", i32, [C.c_void_p, P(P(f64)), P(P(f64)), P(f64), P(f64), P(f64)]),
    ("msdp_solver_prepare", i32, [C.c_void_p, P(i32)]),
    ("msdp_solver_schur_assemble", i32, [C.c_void_p, i32, P(f64)]),
    ("msdp_solver_get_block_matrix", i32, [C.c_void_p, i32, i32, P(f64)]),
    ("msdp_solver_step_eig", i32, [C.c_void_p, i32, P(f64), P(f64), P(f64)]),
    ("msdp_schur_create", i32, [C.c_void_p, i32, i32, P(C.c_void_p)]),
    ("msdp_schur_destroy", i32, [C.c_void_p]),
    ("msdp_schur_factorize", i32, [C.c_void_p, P(f64), P(i32)]),
    ("msdp_schur_solve", i32, [C.c_void_p, P(f64)]),
    ("msdp_schur_fp64_active", i32, [C.c_void_p]),
    ("msdp_dense_cholesky", i32, [i32, i32, C.c_void_p, i64, P(i32), C.c_void_p]),
    ("msdp_tc_gemm", i32, [i32, i32, i32, i64, i64, i64, f64, C.c_void_p, i64, C.c_void_p, i64, f64, C.c_void_p, i64,
                           i32, C.c_void_p]),
]

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the library once; raise if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"libmadsdp_gpu.so not found at {path}; build it with "
            "`python madsdp.jl_gb300/build.py` (the GPU path has no CPU fallback)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


ERRORS = {0: "OK", -1: "INVALID_ARGUMENT", -2: "CUDA", -3: "OUT_OF_MEMORY", -4: "UNSUPPORTED", -5: "INITIAL_POINT",
          -6: "TOO_LARGE"}
