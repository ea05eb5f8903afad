"""ctypes binding of liblshg.so (include/lshg.h).

The library is built in-tree by lshongpu_gb300.build (or __graft_entry__.build()).
There is no fallback: if the shared library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

c_int, c_int64, c_float, c_double, c_void_p, c_char_p, c_size_t = (
    C.c_int, C.c_int64, C.c_float, C.c_double, C.c_void_p, C.c_char_p, C.c_size_t)


class Point(C.Structure):
    """struct Point {int ID; float distance;} (LinearScan/point.h:3-7)."""
    _fields_ = [("ID", C.c_int32), ("distance", c_float)]


class ResultStruct(C.Structure):
    """struct Result (LinearScan/resultDTO.h:5-32) with a caller-owned results buffer."""
    _fields_ = [
        ("results", C.POINTER(Point)),
        ("preprocess_ms", c_int64),
        ("construction_ms", c_int64),
        ("scan_ms", c_int64),
        ("recall", c_float),
        ("avg_distance", c_float),
        ("preprocess_us", c_double),
        ("construction_us", c_double),
        ("scan_us", c_double),
    ]


class Options(C.Structure):
    _fields_ = [
        ("thread_queue_size", c_int),
        ("candidates", c_int),
        ("cp_hashes", c_int),
        ("cp_rounds", c_int),
        ("stream", c_void_p),
        ("fp64_recheck", c_int),
        ("sketch_scan", c_int),
    ]


class IndexParams(C.Structure):
    _fields_ = [
        ("implementation", c_int),
        ("distanceFunc", c_int),
        ("sketchDim", c_int),
        ("d", c_int),
        ("framework", c_int),
        ("keysImplementation", c_int),
        ("bucketKeyBits", c_int),
        ("tables", c_int),
        ("runWithSketchedData", c_int),
        ("opt", Options),
    ]


class ServerParams(C.Structure):
    _fields_ = [
        ("max_batch", c_int),
        ("max_queue", c_int),
        ("streams", c_int),
        ("use_graphs", c_int),
        ("hbm_reserve_mb", c_int64),
        ("batch_window_us", c_int),
    ]


P = c_void_p
_SIGS = {
    "lshg_version": (c_char_p, []),
    "lshg_last_error": (c_char_p, []),
    "lshg_calculate_k": (c_int, [c_int]),
    "lshg_launch_count": (c_int64, []),
    "lshg_profile_enable": (c_int, [c_int]),
    "lshg_profile_report": (c_int, [C.c_char_p, c_int]),
    "lshg_options_default": (None, [C.POINTER(Options)]),
    "lshg_linear_scans": (c_int, [c_int, c_int, c_int, c_int, c_int, P, P, c_int, c_int, C.POINTER(ResultStruct)]),
    "lshg_linear_scans_ex": (c_int, [c_int, c_int, c_int, c_int, c_int, P, P, c_int, c_int, C.POINTER(Options),
                                     C.POINTER(ResultStruct)]),
    "lshg_lsh": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, P, P, c_int, c_int, c_int, c_int, c_int,
                         C.POINTER(ResultStruct)]),
    "lshg_lsh_ex": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, P, P, c_int, c_int, c_int, c_int, c_int,
                            C.POINTER(Options), C.POINTER(ResultStruct)]),
    "lshg_random_normals": (c_int, [c_int64, c_double, P]),
    "lshg_random_plus_minus": (c_int, [c_int64, P]),
    "lshg_random_bools": (c_int, [c_int64, P]),
    "lshg_index_build": (c_int, [C.POINTER(IndexParams), P, c_int64, c_int, C.POINTER(c_void_p)]),
    "lshg_index_query": (c_int, [P, P, c_int, c_int, P, c_int, P]),
    "lshg_index_free": (c_int, [P]),
    "lshg_index_query_noalloc": (c_int, [P, P, c_int, c_int, P, P]),
    "lshg_index_query_async": (c_int, [P, P, c_int, c_int, P, c_int, P]),
    "lshg_index_sync": (c_int, [P, P]),
    "lshg_index_export": (c_int, [P, c_int, P, C.POINTER(c_size_t)]),
    "lshg_index_sketch_queries": (c_int, [P, P, c_int, P, P]),
    "lshg_index_save": (c_int, [P, c_char_p]),
    "lshg_index_load": (c_int, [c_char_p, C.POINTER(c_void_p)]),
    "lshg_merge_topk": (c_int, [P, c_int, c_int, c_int, c_int, P]),
    "lshg_validate": (c_int, [P, c_int, P, c_int, c_int, c_int, C.POINTER(c_float), C.POINTER(c_float)]),
    "lshg_parse_file": (c_int, [c_char_p, C.POINTER(c_int), C.POINTER(c_int), C.POINTER(C.POINTER(c_float))]),
    "lshg_write_file": (c_int, [c_char_p, P, c_int, c_int]),
    "lshg_free": (None, [P]),
    "lshg_read_truth": (c_int, [c_char_p, C.POINTER(c_int), C.POINTER(c_int), C.POINTER(C.POINTER(Point))]),
    "lshg_server_params_default": (None, [C.POINTER(ServerParams)]),
    "lshg_server_create": (c_int, [C.POINTER(ServerParams), C.POINTER(c_void_p)]),
    "lshg_server_add_index": (c_int, [P, c_int, P]),
    "lshg_server_submit": (c_int, [P, c_int, P, c_int, c_int, C.POINTER(c_int64)]),
    "lshg_server_wait": (c_int, [P, c_int64, P, c_int64, C.POINTER(c_double)]),
    "lshg_server_stats": (c_int, [P, C.POINTER(c_int64), C.POINTER(c_int64), C.POINTER(c_int64), C.POINTER(c_int64)]),
    "lshg_server_destroy": (c_int, [P]),
}

# Public symbol list (everything include/lshg.h declares).
SYMBOLS = sorted(_SIGS)

_LIB = None


class LshgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"lshg status {status}: {message}")
        self.status = status


def lib_path() -> str:
    """The in-tree build, or the library named by LSHG_LIBRARY (an alternate build)."""
    return os.environ.get("LSHG_LIBRARY") or _build.lib_path()


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: build the engine first (python -m lshongpu_gb300.build or __graft_entry__.build())")
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int) -> None:
    if status != 0:
        raise LshgError(status, lib().lshg_last_error().decode(errors="replace"))
