"""ctypes binding of the native library (include/siml_gb300.h).

The library is built in-tree by ``siml_gb300.build``; if it is missing this
module raises instead of falling back to any other implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libsiml_gb300.so")

SIML_OK = 0
SIML_ERR_INVALID = 1
SIML_ERR_STATE = 2
SIML_ERR_CUDA = 3
SIML_ERR_NOMEM = 4
SIML_ERR_TIMEOUT = 5
SIML_ERR_UNSUPPORTED = 6
SIML_ERR_RANGE = 7

SIML_HOST = 0
SIML_DEVICE = 1
SIML_HOST_QUEUED = 2   # siml_rows: pinned, mapped host memory written directly, call queued

SIML_TUNE_ROWS_WINDOW = 1
SIML_TUNE_ROWS_ENTRIES = 2
SIML_TUNE_ROW_STRIDE = 3
SIML_TUNE_SORT_WINDOW = 4
SIML_TUNE_ROWS_LAYOUT = 5
SIML_ROWS_PADDED = 0
SIML_ROWS_BALANCED = 1
SIML_ROWS_SCHEDULED = 2
SIML_TUNE_SCHED_GROUPS = 6
SIML_TUNE_SCHED_ROWS = 7
SIML_TUNE_RARE_FIXUP = 8
SIML_ENTRIES_AUTO = 0
SIML_ENTRIES_U16 = 1
SIML_ENTRIES_U32 = 2
SIML_ENTRIES_OFFSETS = 3

SYNTH_UNIFORM_20_90 = 0
SYNTH_LOGNORMAL_45 = 1
SYNTH_BIMODAL_35_110 = 2
SYNTH_CHEM_45 = 3


class SimlError(RuntimeError):
    """A native call failed (CUDA error, allocation failure, timeout)."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int
_F32 = ctypes.c_float
_U64 = ctypes.c_uint64

_SIGNATURES = {
    "siml_version": (ctypes.c_char_p, []),
    "siml_last_error": (ctypes.c_char_p, []),
    "siml_create": (_I32, [_I32, ctypes.POINTER(_P)]),
    "siml_destroy": (_I32, [_P]),
    "siml_set_stream": (_I32, [_P, _P]),
    "siml_sync": (_I32, [_P]),
    "siml_query_done": (_I32, [_P, ctypes.POINTER(_I32)]),
    "siml_set_ref": (_I32, [_P, _P, _P, _P, _P, _I64, _I64, _I64, _I32]),
    "siml_set_query": (_I32, [_P, _P, _P, _P, _P, _I64, _I64, _I64, _I32]),
    "siml_write_ref_rows": (_I32, [_P, _I64, _P, _P, _P, _P, _I64, _I64, _I64]),
    "siml_set_sizes": (_I32, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "siml_rows": (_I32, [_P, _I64, _I64, _P, _I64, _I32]),
    "siml_row_single": (_I32, [_P, _I64, _P, _I32]),
    "siml_neighbors": (_I32, [_P, _I64, _I64, _F32, _F32, _I64, _P, _P, _P, _I32]),
    "siml_hist101": (_I32, [_P, _I64, _I64, _P, _I64, _I32]),
    "siml_topk": (_I32, [_P, _I64, _I64, _I64, _P, _P, _I32]),
    "siml_async_status": (_I32, [_P]),
    "siml_eval_pairs": (_I32, [_P, ctypes.POINTER(ctypes.c_uint64), _I32]),
    "siml_hist_global": (_I32, [_P, _I64, _I64, _P, _I32]),
    "siml_topk_noalloc": (_I32, [_P, _I64, _I64, _I64, _P, _P]),
    "siml_neighbors_range": (_I32, [_P, _I64, _I64, _I64, _I64, _F32, _F32, _I64, _P, _P, _P, _I32]),
    "siml_batch_create": (_I32, [_P, _I64, _P, _F32, _F32, _I64, _I64, _P]),
    "siml_batch_create_shaped": (_I32, [_P, _I64, _P, _F32, _F32, _I64, _I64, _I64, _I64, _P]),
    "siml_batch_shape": (_I32, [_P, _P]),
    "siml_batch_info": (_I32, [_P, _P, _P, _P, _P, _P]),
    "siml_batch_run": (_I32, [_P, _P, _P, _P, _P]),
    "siml_batch_destroy": (_I32, [_P]),
    "siml_compile_width": (_I64, [_P, _P, _I64]),
    "siml_compile_smiles": (_I32, [_P, _P, _I64, _P, _P, _P, _P, _I64]),
    "siml_compile_stage": (_I64, [_P, _P, _I64, _P, _P, _P, _P]),
    "siml_compile_scatter": (_I32, [_P, _I64, _P, _P, _P, _P, _P, _I64]),
    "siml_row_histogram101": (_I32, [_P, _P, _I64, _I64, _I64, _P, _I32]),
    "siml_row_histogram101_f64": (_I32, [_P, _P, _I64, _I64, _I64, _P, _I32]),
    "siml_synth_lengths": (_I32, [_U64, _I32, _I64, _I64, _P]),
    "siml_synth_smiles": (_I32, [_U64, _I32, _I64, _I64, _P, _I64, _P]),
    "siml_db_stats": (_I32, [_P, _P]),
    "siml_set_tuning": (_I32, [_P, _I32, _I64]),
    "siml_get_tuning": (_I32, [_P, _I32, ctypes.POINTER(_I64)]),
    "siml_launch_count": (_I64, [_P]),
    "siml_debug_set_row_vid": (_I32, [_P, _I64, _I64, ctypes.c_uint32]),
    "siml_mem_info": (_I32, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "siml_rows_info": (_I32, [_P, ctypes.POINTER(ctypes.c_int64)]),
    "siml_rows_vocab": (_I32, [_P, ctypes.POINTER(ctypes.c_int64)]),
    "siml_vocab_stats": (_I32, [_P, _P]),
    "siml_compile_width_gpu": (_I64, [_P, _P, _P, _I64]),
    "siml_compile_smiles_gpu": (_I32, [_P, _P, _P, _I64, _P, _P, _P, _P, _I64]),
    "siml_compile_stage_gpu": (_I64, [_P, _P, _P, _I64, _P, _P, _P, _P]),
    "siml_debug_fail_alloc": (_I32, [_I64]),
    "siml_debug_async_status": (_I32, [ctypes.c_int]),
    "siml_compile_scatter_gpu": (_I32, [_P, _P, _I64, _P, _P, _P, _P, _P, _I64]),
    "siml_last_kernel_ms": (ctypes.c_double, [_P]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Loads the native library (once) and declares every entry point."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "siml_gb300 native library not found at %s; build it with "
                "`python -m siml_gb300.build`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    msg = lib().siml_last_error()
    return msg.decode("utf-8", "replace") if msg else ""


def check(rc: int, what: str = "") -> None:
    """Maps a native status to the exception the reference raises for it."""
    if rc == SIML_OK:
        return
    msg = last_error() or ("%s failed with status %d" % (what, rc))
    if rc in (SIML_ERR_INVALID, SIML_ERR_UNSUPPORTED):
        raise ValueError(msg)
    if rc in (SIML_ERR_RANGE, SIML_ERR_STATE):
        raise RuntimeError(msg)
    raise SimlError(rc, msg)


# CUDA's handle for the legacy default stream (cudaStreamLegacy).  A NULL
# stream given to siml_set_stream selects the engine's own stream instead.
CUDA_STREAM_LEGACY = 1


def stream_arg(stream) -> ctypes.c_void_p:
    """siml_set_stream argument for a torch stream.  Torch's default stream has
    handle 0, which is the legacy default stream: it is passed as
    cudaStreamLegacy, so the engine's work is ordered with torch's."""
    h = int(stream.cuda_stream)
    return ctypes.c_void_p(h if h != 0 else CUDA_STREAM_LEGACY)


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
