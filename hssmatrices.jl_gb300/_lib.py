"""ctypes binding of the C ABI in ``include/hssgpu.h`` (``lib/libhssgpu.so``).

Loading fails loudly if the library has not been built: there is no CPU path.
Status codes map to Python exceptions the way the reference's Julia errors do
(``DimensionMismatch``/``ArgumentError`` -> ValueError, ``SingularException``
-> numpy.linalg.LinAlgError).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

HSS_OK = 0
HSS_ERR_BAD_DIMS = 1
HSS_ERR_OOM = 2
HSS_ERR_SINGULAR = 3
HSS_ERR_NO_CONVERGENCE = 4
HSS_ERR_TIMEOUT = 5
HSS_ERR_CUDA = 6
HSS_ERR_INVALID = 7

TRACE = {"mv_leaf": 0, "mv_up": 1, "mv_down": 2, "mv_final": 3, "factor_leaf": 4, "factor_merge": 5,
         "solve_up": 6, "solve_down": 7, "mv_dx": 8}

HSS_PREC_FP64 = 0
HSS_PREC_FP32 = 1

# hss_set_option switches
HSS_OPT_GENERIC_FACTOR = 1
HSS_OPT_RESIDUAL_FP64 = 2
HSS_OPT_LEVEL_PRODUCT = 3
HSS_OPT_GRAPHS = 4
HSS_OPT_SAMPLE_DF = 5
HSS_OPT_FLAT_PRODUCT = 6
HSS_OPT_POLL_LIMIT = 7
HSS_OPT_FAIL_ALLOC = 8
HSS_OPT_TENSOR_RESIDUAL = 9

NODE_FIELDS = 16
CLUSTER_FIELDS = 6
INFO_FIELDS = 13

# every symbol include/hssgpu.h declares
EXPORTS = [
    "hss_create", "hss_create_batch", "hss_inspect", "hss_destroy", "hss_size", "hss_ntrees", "hss_node_info",
    "hss_ulv_cols", "hss_matmul", "hss_matmul_host", "hss_matmul_batch", "hss_ulvfactor",
    "hss_factor_destroy", "hss_ulvsolve", "hss_ulvsolve_host", "hss_ulvsolve_batch",
    "hss_ulvfactsolve_host", "hss_factor_bytes", "hss_autotune", "hss_autotune_info", "hss_last_error", "hss_version", "hss_ulvrefactor",
    "hss_trace_begin", "hss_trace_end", "hss_trace_times", "hss_launch_counter", "hss_set_option", "hss_matmul_noalloc",
    "hss_batcher_create", "hss_batcher_destroy", "hss_batcher_factor", "hss_batcher_solve",
    "hss_sample", "hss_sumsq", "hss_rc_create", "hss_rc_destroy", "hss_rc_size", "hss_rc_compress",
    "hss_rc_ranks", "hss_rc_sample", "hss_export_size", "hss_export", "hss_getindex", "hss_full", "hss_hssmul", "hss_recompress", "hss_orthonormalize",
    "hss_device_bytes", "hss_transpose", "hss_matmul_t", "hss_ldiv", "hss_rdiv", "hss_ulvfactsolve",
]


class HssError(RuntimeError):
    """Error returned by the CUDA library."""

    def __init__(self, code, msg):
        super().__init__(f"[hss status {code}] {msg}")
        self.code = code


class NoConvergence(HssError):
    pass


class HssTimeout(HssError, TimeoutError):
    """A bounded device-side wait ran out (HSS_ERR_TIMEOUT); the plan stays usable."""


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("residual", C.c_double)]


_lib = None

P = C.c_void_p
I64 = C.c_int64
I32 = C.c_int32
D = C.c_double
PI64 = C.POINTER(C.c_int64)
PD = C.POINTER(C.c_double)


def _declare(lib):
    sig = {
        "hss_create": (C.c_int, [I64, PI64, PD, I64, C.POINTER(P)]),
        "hss_create_batch": (C.c_int, [I32, PI64, C.POINTER(PI64), C.POINTER(PD), PI64, C.POINTER(P)]),
        "hss_inspect": (C.c_int, [I64, PI64, I64, PI64]),
        "hss_destroy": (C.c_int, [P]),
        "hss_size": (C.c_int, [P, I32, PI64, PI64]),
        "hss_ntrees": (C.c_int, [P, C.POINTER(I32)]),
        "hss_node_info": (C.c_int, [P, I64, PI64]),
        "hss_ulv_cols": (C.c_int, [P, I64, PI64, I64, PI64]),
        "hss_matmul": (C.c_int, [P, P, I64, I64, P, I64, D, D, P]),
        "hss_matmul_host": (C.c_int, [P, PD, I64, I64, PD, I64, D, D]),
        "hss_matmul_noalloc": (C.c_int, [P, P, I64, I64, P, I64, D, D, P]),
        "hss_matmul_batch": (C.c_int, [P, C.POINTER(P), PI64, PI64, C.POINTER(P), PI64, D, D, P]),
        "hss_ulvfactor": (C.c_int, [P, I32, C.POINTER(P), P]),
        "hss_factor_destroy": (C.c_int, [P]),
        "hss_ulvsolve": (C.c_int, [P, P, I64, I64, P, I64, D, I32, C.POINTER(SolveStats), P]),
        "hss_ulvsolve_host": (C.c_int, [P, PD, I64, I64, PD, I64, D, I32, C.POINTER(SolveStats)]),
        "hss_ulvfactsolve": (C.c_int, [P, P, I64, I64, P, I64, D, I32, C.POINTER(SolveStats), P]),
        "hss_ulvsolve_batch": (C.c_int, [P, C.POINTER(P), PI64, PI64, C.POINTER(P), PI64, D, I32,
                                         C.POINTER(SolveStats), P]),
        "hss_ulvfactsolve_host": (C.c_int, [P, I32, PD, I64, I64, PD, I64, D, I32, C.POINTER(SolveStats)]),
        "hss_factor_bytes": (C.c_int, [P, PI64]),
        "hss_device_bytes": (C.c_int, [P, P, PI64]),
        "hss_transpose": (C.c_int, [P, C.POINTER(P), P]),
        "hss_matmul_t": (C.c_int, [P, P, I64, I64, P, I64, D, D, P]),
        "hss_ldiv": (C.c_int, [P, P, D, D, C.POINTER(P), P]),
        "hss_rdiv": (C.c_int, [P, P, D, D, C.POINTER(P), P]),
        "hss_autotune": (C.c_int, [P, I64, P]),
        "hss_autotune_info": (C.c_int, [P, C.POINTER(C.c_int32), C.c_char_p, C.POINTER(C.c_int32), C.c_char_p,
                                        C.POINTER(C.c_int32)]),
        "hss_ulvrefactor": (C.c_int, [P, P]),
        "hss_trace_begin": (C.c_int, [I32]),
        "hss_trace_end": (C.c_int, [C.POINTER(D), PI64]),
        "hss_trace_times": (C.c_int, [C.POINTER(D), I64, PI64]),
        "hss_launch_counter": (C.c_int64, []),
        "hss_set_option": (C.c_int, [I32, I64]),
        "hss_batcher_create": (C.c_int, [C.POINTER(P)]),
        "hss_batcher_destroy": (C.c_int, [P]),
        "hss_batcher_factor": (C.c_int, [P, I32, C.POINTER(P), I32, C.POINTER(P), P]),
        "hss_batcher_solve": (C.c_int, [P, I32, C.POINTER(P), C.POINTER(P), PI64, PI64, C.POINTER(P), PI64, D, I32,
                                        C.POINTER(SolveStats), P]),
        "hss_sample": (C.c_int, [P, I64, I64, I64, I32, P, I64, I64, P, I64, D, D, P]),
        "hss_sumsq": (C.c_int, [P, I64, I64, I64, PD, P]),
        "hss_rc_create": (C.c_int, [I64, PI64, C.POINTER(P)]),
        "hss_rc_destroy": (C.c_int, [P]),
        "hss_rc_size": (C.c_int, [P, PI64, PI64]),
        "hss_rc_compress": (C.c_int, [P, P, I64, P, I64, P, I64, P, I64, P, I64, I64, D, D, C.POINTER(P), P]),
        "hss_rc_ranks": (C.c_int, [P, C.POINTER(I32)]),
        "hss_rc_sample": (C.c_int, [P, P, I64, I32, P, I64, I64, P, I64, P]),
        "hss_getindex": (C.c_int, [P, P, I64, P, I64, P, I64, P]),
        "hss_full": (C.c_int, [P, P, I64, P]),
        "hss_hssmul": (C.c_int, [P, P, C.POINTER(C.c_void_p), P]),
        "hss_recompress": (C.c_int, [P, D, D, C.POINTER(C.c_void_p), P]),
        "hss_orthonormalize": (C.c_int, [P, C.POINTER(C.c_void_p), P]),
        "hss_export_size": (C.c_int, [P, PI64, PI64]),
        "hss_export": (C.c_int, [P, PI64, PD]),
        "hss_last_error": (C.c_char_p, []),
        "hss_version": (C.c_int32, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load ``libhssgpu.so`` (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path) or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise ImportError(f"libhssgpu.so is not built ({path}); call __graft_entry__.build()")
        _build.build()
    lib = C.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


def check(rc):
    if rc == HSS_OK:
        return
    msg = _lib.hss_last_error().decode(errors="replace")
    if rc == HSS_ERR_BAD_DIMS or rc == HSS_ERR_INVALID:
        raise ValueError(msg)
    if rc == HSS_ERR_SINGULAR:
        raise np.linalg.LinAlgError(msg)
    if rc == HSS_ERR_NO_CONVERGENCE:
        raise NoConvergence(rc, msg)
    if rc == HSS_ERR_OOM:
        raise MemoryError(msg)
    if rc == HSS_ERR_TIMEOUT:
        raise HssTimeout(rc, msg)
    raise HssError(rc, msg)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(PD)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(PI64)
