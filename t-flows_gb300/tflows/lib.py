"""ctypes binding of libtfs_gb300.so (declarations in include/tfs_solver.h)
and of the host-only generator libtfs_synth.so (include/tfs_synth.h).  Both
are built in-tree by ``tflows.build``; a missing library raises instead of
falling back to anything else."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

TFS_OK = 0
TFS_ERR_ARG, TFS_ERR_MATRIX, TFS_ERR_CUDA, TFS_ERR_NONFINITE = 1, 2, 3, 4
TFS_ERR_TOPOLOGY, TFS_ERR_TIMEOUT, TFS_ERR_BUDGET = 5, 6, 7
TFS_CG, TFS_BICG, TFS_CGS = 0, 1, 2
TFS_PREC_NONE, TFS_PREC_DIAG, TFS_PREC_DIC = 0, 1, 2
TFS_FP64, TFS_MIXED = 0, 1
TFS_SYNTH_POISSON, TFS_SYNTH_CONVDIFF = 0, 1
# options of a handle (tfs_set_option)
(TFS_OPT_LAUNCH, TFS_OPT_LAYOUT, TFS_OPT_BICG, TFS_OPT_SELL_UNIFORM, TFS_OPT_SPMV, TFS_OPT_SPMV_GRID,
 TFS_OPT_LEVEL_TPB, TFS_OPT_TAIL_PF, TFS_OPT_FUSE_L0, TFS_OPT_PDL, TFS_OPT_PDL_VEC, TFS_OPT_FWD_PRE,
 TFS_OPT_BWD_PRE, TFS_OPT_DIC_BLOCK, TFS_OPT_L2_WINDOW) = range(1, 16)

_PKG = Path(__file__).resolve().parent
# TFS_LIBRARY selects another build of the library (same ABI).
lib_path = Path(os.environ["TFS_LIBRARY"]) if os.environ.get("TFS_LIBRARY") else _PKG / "lib" / "libtfs_gb300.so"
synth_path = _PKG / "lib" / "libtfs_synth.so"

i32, i64, u64, dbl = C.c_int32, C.c_int64, C.c_uint64, C.c_double
P_i32, P_dbl, P_void = C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_void_p


class tfs_tuning(C.Structure):
    _fields_ = [("level_tpb", C.c_int32), ("spmv_chunks", C.c_int32),
                ("prec_ms", C.c_double * 4), ("spmv_ms", C.c_double * 2),
                ("spmv_kernel", C.c_int32), ("pad", C.c_int32), ("spmv_pipe_ms", C.c_double * 2)]


class tfs_stats(C.Structure):
    _fields_ = [("iterations", i32), ("true_residuals", i32), ("n_levels", i32), ("status", i32),
                ("solve_ms", dbl), ("spmv_ns_total", dbl), ("spmv_launches", i64),
                ("sweep_ns_total", dbl), ("sweep_launches", i64), ("kernel_launches", i64),
                ("device_bytes", i64), ("spmv_kernel", i32), ("sell_width", i32),
                ("dic_kernel", i32), ("pad", i32)]


class tfs_result(C.Structure):
    _fields_ = [("ticket", i64), ("niter", i32), ("status", i32), ("ini_res", dbl), ("fin_res", dbl),
                ("queued_ms", dbl), ("run_ms", dbl), ("latency_ms", dbl),
                ("device_begin_ns", i64), ("device_end_ns", i64)]


class tfs_server_stats(C.Structure):
    _fields_ = [(k, i64) for k in ("submitted", "completed", "refused", "evictions", "registrations",
                                   "resident_bytes", "resident_systems", "running", "queued",
                                   "peak_running")]


class TfsError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: status {status} ({status_string(status)}) {detail}".rstrip())


# (name, restype, argtypes) of every exported symbol of the C ABI.
SIGNATURES = {
    "tfs_topology_register": (C.c_int, [i32, i32, P_i32, P_i32, P_i32, C.POINTER(P_void)]),
    "tfs_release": (C.c_int, [P_void]),
    "tfs_set_precision": (C.c_int, [P_void, C.c_int]),
    "tfs_set_default_precision": (C.c_int, [C.c_int]),
    "tfs_set_option": (C.c_int, [P_void, C.c_int, C.c_int]),
    "tfs_get_option": (C.c_int, [P_void, C.c_int, C.POINTER(C.c_int)]),
    "tfs_diag_dic_timeout": (C.c_int, [P_void, C.c_longlong]),
    "tfs_solve": (C.c_int, [C.c_int, P_void, i32, i32, P_i32, P_i32, P_i32, P_dbl, P_dbl, P_dbl,
                            i32, P_i32, dbl, P_dbl, P_dbl]),
    "tfs_cg": (C.c_int, [i32, i32, P_i32, P_i32, P_i32, P_dbl, P_dbl, P_dbl, i32, P_i32, dbl, P_dbl, P_dbl]),
    "tfs_bicg": (C.c_int, [i32, i32, P_i32, P_i32, P_i32, P_dbl, P_dbl, P_dbl, i32, P_i32, dbl, P_dbl, P_dbl]),
    "tfs_cgs": (C.c_int, [i32, i32, P_i32, P_i32, P_i32, P_dbl, P_dbl, P_dbl, i32, P_i32, dbl, P_dbl, P_dbl]),
    "tfs_solve_device": (C.c_int, [C.c_int, P_void, P_void, P_void, P_void, i32, P_i32, dbl, P_dbl, P_dbl]),
    "tfs_spmv": (C.c_int, [P_void, P_dbl, P_dbl, P_dbl]),
    "tfs_residual": (C.c_int, [P_void, P_dbl, P_dbl, P_dbl]),
    "tfs_prec_form": (C.c_int, [P_void, P_dbl, i32, P_dbl]),
    "tfs_prec_solve": (C.c_int, [P_void, P_dbl, i32, P_dbl, P_dbl]),
    "tfs_get_stats": (C.c_int, [P_void, C.POINTER(tfs_stats)]),
    "tfs_get_levels": (C.c_int, [P_void, P_i32]),
    "tfs_time_spmv": (C.c_int, [P_void, P_dbl, C.c_int, C.c_int, P_dbl]),
    "tfs_time_prec": (C.c_int, [P_void, P_dbl, C.c_int, C.c_int, P_dbl]),
    "tfs_profile_prec": (C.c_int, [P_void, P_dbl, C.c_int, C.c_int, P_dbl, P_dbl, P_i32, P_i32]),
    "tfs_autotune": (C.c_int, [P_void, P_dbl, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "tfs_faces_register": (C.c_int, [P_void, C.c_int32, P_i32, P_i32]),
    "tfs_assemble_faces_device": (C.c_int, [P_void, P_void, P_void, P_void, P_void, P_void, P_void]),
    "tfs_status_string": (C.c_char_p, [C.c_int]),
    "tfs_last_error": (C.c_char_p, []),
    "tfs_batch_create": (C.c_int, [C.c_int, C.POINTER(P_void), C.POINTER(P_void)]),
    "tfs_batch_release": (C.c_int, [P_void]),
    "tfs_batch_configure": (C.c_int, [P_void, C.c_int, C.c_int]),
    "tfs_batch_solve_device": (C.c_int, [P_void, C.c_int, C.c_int, C.c_int, C.POINTER(P_void),
                                         C.POINTER(P_void), C.POINTER(P_void), P_i32, P_dbl, P_i32,
                                         P_dbl, P_dbl, P_i32]),
    "tfs_batch_solve": (C.c_int, [P_void, C.c_int, C.c_int, C.c_int, C.POINTER(P_void),
                                  C.POINTER(P_void), C.POINTER(P_void), P_i32, P_dbl, P_i32, P_dbl,
                                  P_dbl, P_i32]),
    "tfs_batch_last_ms": (C.c_int, [P_void, P_dbl]),
    "tfs_batch_copy": (C.c_int, [P_void, C.c_int, C.POINTER(P_void), C.POINTER(P_void),
                                 C.POINTER(C.c_size_t)]),
    "tfs_server_create": (C.c_int, [C.c_int, i64, C.c_int, C.POINTER(P_void)]),
    "tfs_server_destroy": (C.c_int, [P_void]),
    "tfs_server_add_system": (C.c_int, [P_void, i32, i32, P_i32, P_i32, P_i32, C.POINTER(i64)]),
    "tfs_server_submit": (C.c_int, [P_void, i64, C.c_int, C.c_int, C.c_int, P_void, P_void, P_void,
                                    P_void, C.c_int, i32, dbl, C.POINTER(i64)]),
    "tfs_server_submit_host": (C.c_int, [P_void, i64, C.c_int, C.c_int, C.c_int, P_void, P_void, P_void,
                                         C.c_int, i32, dbl, C.POINTER(i64)]),
    "tfs_server_wait": (C.c_int, [P_void, i64, dbl, C.POINTER(tfs_result)]),
    "tfs_server_get_stats": (C.c_int, [P_void, C.POINTER(tfs_server_stats)]),
    "tfs_residual_norm_noalloc": (C.c_int, [i32, P_void, P_void, P_void, P_void, P_void, P_void, P_void]),
    "tfs_use_device": (C.c_int, [C.c_int]),
    "tfs_device_alloc": (C.c_int, [C.c_size_t, C.POINTER(P_void)]),
    "tfs_device_free": (C.c_int, [P_void]),
    "tfs_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P_void)]),
    "tfs_host_free": (C.c_int, [P_void]),
    "tfs_copy": (C.c_int, [P_void, P_void, P_void, C.c_size_t]),
    "tfs_memcpy": (C.c_int, [P_void, P_void, C.c_size_t]),
    "tfs_topology_build_device": (C.c_int, [C.c_int32, C.c_int32, P_void, P_void, P_void, P_void, P_void,
                                            P_void, P_i32]),
    "tfs_sync": (C.c_int, [P_void]),
    "tfs_timer_start": (C.c_int, [P_void]),
    "tfs_timer_stop": (C.c_int, [P_void, P_dbl]),
    "tfs_topology_count": (i32, [i32, i32, P_i32]),
    "tfs_topology_build": (C.c_int, [i32, i32, P_i32, P_i32, P_i32, P_i32, P_i32, P_i32]),
}

# Symbols of libtfs_synth.so (include/tfs_synth.h).
SYNTH_SIGNATURES = {
    "tfs_synth_create": (C.c_int, [C.c_int, i32, i32, i32, dbl, u64, C.c_int, C.POINTER(P_void)]),
    "tfs_synth_dims": (C.c_int, [P_void, P_i32, P_i32, P_i32]),
    "tfs_synth_export": (C.c_int, [P_void, P_i32, P_i32, P_i32, P_i32, P_dbl, P_dbl]),
    "tfs_synth_free": (None, [P_void]),
    "tfs_synth_loguniform": (i64, [i64, i64, u64, u64]),
    "tfs_synth_uniform": (dbl, [u64, u64, u64]),
}

_lib = None
_synth = None


def load_synth_library() -> C.CDLL:
    """Load libtfs_synth.so (the seeded synthetic systems; host code only)."""
    global _synth
    if _synth is not None:
        return _synth
    if not synth_path.exists():
        raise FileNotFoundError(f"{synth_path} is missing: build it with `python -m tflows.build` "
                                "(or __graft_entry__.build())")
    lib = C.CDLL(str(synth_path))
    for name, (res, args) in SYNTH_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _synth = lib
    return lib


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libtfs_gb300.so and declare its signatures (raises if absent)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else lib_path
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with `python -m tflows.build` "
                                "(or __graft_entry__.build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load_library().tfs_status_string(status).decode()
    except Exception:  # library not loadable: plain number
        return str(status)


def last_error() -> str:
    return load_library().tfs_last_error().decode(errors="replace")


def check(status: int, where: str) -> None:
    if status != TFS_OK:
        raise TfsError(status, where, last_error())
