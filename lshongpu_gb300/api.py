"""Python mirror of the reference launch surface, over the C ABI (include/lshg.h).

    linear_scans(implementation, k, d, N_query, N_data, data, queries, sketchDim,
                 distanceFunc)                          -- LinearScan/kernel.cu:27
    LSH(implementation, keysImplementation, k, d, N_query, N_data, data, queries,
        sketchDim, distanceFunc, bucketKeyBits, tables, runWithSketchedData)
                                                        -- LinearScan/kernel.cu:91
    calculate_k(k)                                      -- launchHelper.cuh:21-25

Each returns a Result mirroring struct Result (resultDTO.h:5-32): `results` is an
N_query x k array of Point (ID, distance) in ascending distance.  Errors raise
LshgError instead of exiting the process (cudaHelpers.cuh:8-15).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import (IndexParams, LshgError, Options, Point, ResultStruct, ServerParams, check, lib)

POINT_DTYPE = np.dtype([("ID", np.int32), ("distance", np.float32)])

# implementation codes (kernel.cu:25) and the engine's tensor-core scan
IMPL_EXACT = 2
IMPL_SIMHASH = 3
IMPL_WMH = 4
IMPL_WMH_ONEBIT = 5
IMPL_JL = 6
IMPL_TC = 8
IMPL_TC_FP8 = 9
IMPL_CWS = 10  # consistent weighted sampling (no reference counterpart)
# keysImplementation codes (kernel.cu:65-85)
KEYS_SIMHASH = 3
KEYS_WMH = 4
KEYS_WMH_ONEBIT = 5
KEYS_CROSSPOLY = 7
KEYS_CWS = 10  # consistent weighted sampling (no reference counterpart)
# sketch_scan option: how Hamming / one-bit Jaccard sketch scans run
SKETCH_SCAN_AUTO, SKETCH_SCAN_POPCOUNT, SKETCH_SCAN_TENSOR = 0, 1, 2
# distance functions (distanceFunctions.cuh:54-71)
ANGULAR, JACCARD, EUCLIDEAN = 1, 2, 3


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def calculate_k(k: int) -> int:
    return int(lib().lshg_calculate_k(int(k)))


def launch_count() -> int:
    """Kernel launches issued by the library in this process."""
    return int(lib().lshg_launch_count())


def profile_enable(on: bool = True) -> None:
    check(lib().lshg_profile_enable(int(on)))


def profile_report() -> dict[str, tuple[int, float]]:
    """{kernel: (launches, total_ms)} since the last report (CUDA events on the launching stream)."""
    buf = C.create_string_buffer(1 << 16)  # one call: reporting drains the records
    lib().lshg_profile_report(buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out


@dataclass
class Result:
    results: np.ndarray  # (N_query, k) POINT_DTYPE
    preprocessTime: int = 0
    constructionTime: int = 0
    scanTime: int = 0
    recall: float = 0.0
    avgDistance: float = 0.0
    preprocess_us: float = 0.0
    construction_us: float = 0.0
    scan_us: float = 0.0

    @property
    def ids(self) -> np.ndarray:
        return self.results["ID"]

    @property
    def distances(self) -> np.ndarray:
        return self.results["distance"]


def make_options(thread_queue_size: int = 128, candidates: int = 0, cp_hashes: int = 1, cp_rounds: int = 3,
                 stream: int | None = None, fp64_recheck: int = -1, sketch_scan: int = 0) -> Options:
    o = Options()
    lib().lshg_options_default(C.byref(o))
    o.thread_queue_size = thread_queue_size
    o.candidates = candidates
    o.cp_hashes = cp_hashes
    o.cp_rounds = cp_rounds
    o.stream = stream
    o.fp64_recheck = fp64_recheck
    o.sketch_scan = sketch_scan
    return o


def _result(out: np.ndarray, r: ResultStruct) -> Result:
    return Result(out, r.preprocess_ms, r.construction_ms, r.scan_ms, r.recall, r.avg_distance, r.preprocess_us,
                  r.construction_us, r.scan_us)


def linear_scans(implementation: int, k: int, d: int, N_query: int, N_data: int, data, queries, sketchDim: int,
                 distanceFunc: int, options: Options | None = None) -> Result:
    data, queries = _f32(data), _f32(queries)
    assert data.size >= N_data * d and queries.size >= N_query * d
    out = np.zeros((N_query, k), dtype=POINT_DTYPE)
    r = ResultStruct()
    r.results = out.ctypes.data_as(C.POINTER(Point))
    L = lib()
    if options is None:
        st = L.lshg_linear_scans(implementation, k, d, N_query, N_data, _ptr(data), _ptr(queries), sketchDim,
                                 distanceFunc, C.byref(r))
    else:
        st = L.lshg_linear_scans_ex(implementation, k, d, N_query, N_data, _ptr(data), _ptr(queries), sketchDim,
                                    distanceFunc, C.byref(options), C.byref(r))
    check(st)
    return _result(out, r)


def LSH(implementation: int, keysImplementation: int, k: int, d: int, N_query: int, N_data: int, data, queries,
        sketchDim: int, distanceFunc: int, bucketKeyBits: int, tables: int, runWithSketchedData: bool,
        options: Options | None = None) -> Result:
    data, queries = _f32(data), _f32(queries)
    out = np.zeros((N_query, k), dtype=POINT_DTYPE)
    r = ResultStruct()
    r.results = out.ctypes.data_as(C.POINTER(Point))
    L = lib()
    if options is None:
        st = L.lshg_lsh(implementation, keysImplementation, k, d, N_query, N_data, _ptr(data), _ptr(queries),
                        sketchDim, distanceFunc, bucketKeyBits, tables, int(bool(runWithSketchedData)), C.byref(r))
    else:
        st = L.lshg_lsh_ex(implementation, keysImplementation, k, d, N_query, N_data, _ptr(data), _ptr(queries),
                           sketchDim, distanceFunc, bucketKeyBits, tables, int(bool(runWithSketchedData)),
                           C.byref(options), C.byref(r))
    check(st)
    return _result(out, r)


lsh = LSH


# ---- host random generators --------------------------------------------------------

def random_normals(count: int, stddev: float = 1.0) -> np.ndarray:
    out = np.empty(count, dtype=np.float32)
    check(lib().lshg_random_normals(count, stddev, _ptr(out)))
    return out


def random_plus_minus(count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.int32)
    check(lib().lshg_random_plus_minus(count, _ptr(out)))
    return out


def random_bools(count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.uint8)
    check(lib().lshg_random_bools(count, _ptr(out)))
    return out


# ---- resident index ----------------------------------------------------------------

EXPORT_DATA, EXPORT_SKETCHES, EXPORT_KEYS, EXPORT_OFFSETS, EXPORT_BUCKETS = 0, 1, 2, 3, 4
EXPORT_QUERY_COUNTERS, EXPORT_CWS_CODES = 5, 6


class Index:
    """Resident index: build once, query many times (the serving form of runLsh)."""

    def __init__(self, data=None, *, implementation: int = IMPL_EXACT, distanceFunc: int = ANGULAR,
                 sketchDim: int = 0, framework: int = 0, keysImplementation: int = 0, bucketKeyBits: int = 0,
                 tables: int = 0, runWithSketchedData: bool = False, options: Options | None = None,
                 device_ptr: int | None = None, n: int | None = None, d: int | None = None, _handle=None):
        self.params = IndexParams()
        self._h = C.c_void_p(_handle) if _handle else C.c_void_p()
        if _handle:
            return
        if device_ptr is None:
            data = _f32(data)
            n, d = data.shape
        p = self.params
        p.implementation, p.distanceFunc, p.sketchDim, p.d = implementation, distanceFunc, sketchDim, d
        p.framework, p.keysImplementation, p.bucketKeyBits, p.tables = framework, keysImplementation, bucketKeyBits, tables
        p.runWithSketchedData = int(bool(runWithSketchedData))
        p.opt = options if options is not None else make_options()
        src = device_ptr if device_ptr is not None else _ptr(data)
        check(lib().lshg_index_build(C.byref(p), src, n, 1 if device_ptr is not None else 0, C.byref(self._h)))
        self.n, self.d = n, d

    def query(self, queries, k: int) -> np.ndarray:
        q = _f32(queries)
        nq = q.shape[0]
        out = np.zeros((nq, k), dtype=POINT_DTYPE)
        check(lib().lshg_index_query(self._h, _ptr(q), nq, k, _ptr(out), 0, None))
        return out

    def query_device(self, q_ptr: int, nq: int, k: int, out_ptr: int, stream: int | None = None) -> None:
        """Queries and results already in device memory (float [nq][d], Point [nq][k])."""
        check(lib().lshg_index_query(self._h, q_ptr, nq, k, out_ptr, 1, stream))

    def query_device_async(self, q_ptr: int, nq: int, k: int, out_ptr: int, stream: int | None = None) -> None:
        """Enqueue a batch (device buffers) without waiting; see `sync`."""
        check(lib().lshg_index_query_async(self._h, q_ptr, nq, k, out_ptr, 1, stream))

    def query_host_async(self, q_ptr: int, nq: int, k: int, out_ptr: int, stream: int | None = None) -> None:
        """Enqueue a batch on host (page-locked) buffers -- upload, query, download --
        without waiting; the buffers must stay valid until `sync`."""
        check(lib().lshg_index_query_async(self._h, q_ptr, nq, k, out_ptr, 0, stream))

    def sync(self, stream: int | None = None) -> None:
        """Wait for enqueued batches and raise the first device error kept since the last report."""
        check(lib().lshg_index_sync(self._h, stream))

    def export(self, what: int) -> bytes:
        nb = C.c_size_t(0)
        check(lib().lshg_index_export(self._h, what, None, C.byref(nb)))
        buf = (C.c_char * max(1, nb.value))()
        check(lib().lshg_index_export(self._h, what, buf, C.byref(nb)))
        return bytes(buf[: nb.value])

    def query_counters(self) -> tuple[int, int]:
        """(LSH bucket entries walked, distinct LSH candidates scored), cumulative since
        the build or load; read after the queries' streams have been synchronised."""
        v = np.frombuffer(self.export(5), dtype=np.uint64)
        return int(v[0]), int(v[1])

    def sketch_queries(self, queries, sketch_dtype, sketch_width: int, tables: int = 0):
        q = _f32(queries)
        nq = q.shape[0]
        sk = np.zeros((nq, sketch_width), dtype=sketch_dtype) if sketch_width else None
        keys = np.zeros((nq, tables), dtype=np.uint16) if tables else None
        check(lib().lshg_index_sketch_queries(self._h, _ptr(q), nq, _ptr(sk) if sk is not None else None,
                                              _ptr(keys) if keys is not None else None))
        return sk, keys

    def save(self, path: str) -> None:
        check(lib().lshg_index_save(self._h, path.encode()))

    @classmethod
    def load(cls, path: str) -> "Index":
        h = C.c_void_p()
        check(lib().lshg_index_load(path.encode(), C.byref(h)))
        return cls(_handle=h.value)

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            check(lib().lshg_index_free(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- sharding / validation / text format ---------------------------------------------

def merge_topk(lists: np.ndarray, k: int) -> np.ndarray:
    """lists: (shards, N_query, k_in) POINT_DTYPE with global IDs -> (N_query, k)."""
    lists = np.ascontiguousarray(lists, dtype=POINT_DTYPE)
    shards, nq, kin = lists.shape
    out = np.zeros((nq, k), dtype=POINT_DTYPE)
    check(lib().lshg_merge_topk(_ptr(lists), shards, nq, kin, k, _ptr(out)))
    return out


def validate(truth: np.ndarray, results: np.ndarray, reportK: int) -> tuple[float, float]:
    """runValidation (validation.cpp:200-208): (recall@reportK, distance ratio)."""
    truth = np.ascontiguousarray(truth, dtype=POINT_DTYPE)
    results = np.ascontiguousarray(results, dtype=POINT_DTYPE)
    rec, ratio = C.c_float(), C.c_float()
    check(lib().lshg_validate(_ptr(truth), truth.shape[1], _ptr(results), results.shape[0], results.shape[1],
                              reportK, C.byref(rec), C.byref(ratio)))
    return rec.value, ratio.value


def parse_file(path: str) -> np.ndarray:
    """parseFile (gloveparser.cu:9-86): reference text format -> (n, d) float32."""
    n, d = C.c_int(), C.c_int()
    ptr = C.POINTER(C.c_float)()
    check(lib().lshg_parse_file(path.encode(), C.byref(n), C.byref(d), C.byref(ptr)))
    try:
        arr = np.ctypeslib.as_array(ptr, shape=(n.value * d.value,)).copy() if n.value * d.value else np.zeros(0, np.float32)
    finally:
        lib().lshg_free(ptr)
    return arr.reshape(n.value, d.value)


def read_truth(path: str) -> np.ndarray:
    """GoldStandard truth file -> (n, k) POINT_DTYPE (validation.cpp:62-107)."""
    n, k = C.c_int(), C.c_int()
    ptr = C.POINTER(Point)()
    check(lib().lshg_read_truth(path.encode(), C.byref(n), C.byref(k), C.byref(ptr)))
    try:
        raw = C.string_at(ptr, n.value * k.value * 8) if n.value * k.value else b""
    finally:
        lib().lshg_free(ptr)
    return np.frombuffer(raw, dtype=POINT_DTYPE).reshape(n.value, k.value).copy()


def write_truth(path: str, truth: np.ndarray) -> None:
    """Write (n, k) points in the GoldStandard truth format (goldstandard.cpp:123-134)."""
    with open(path, "w") as f:
        f.write(f"{truth.shape[0]}\n{truth.shape[1]}\n")
        for q, row in enumerate(truth):
            f.write(f"{q}:\n")
            for p in row:
                f.write(f"{int(p['ID'])} {float(p['distance']):.9g}\n")


def write_file(path: str, x) -> None:
    x = _f32(x)
    check(lib().lshg_write_file(path.encode(), _ptr(x), x.shape[0], x.shape[1]))


# ---- serving -------------------------------------------------------------------------

class Server:
    """Continuous-batching request loop over resident indexes (lshg_server_*)."""

    def __init__(self, max_batch: int = 4096, max_queue: int = 65536, streams: int = 2, use_graphs: bool = True,
                 hbm_reserve_mb: int = 1024, batch_window_us: int = 200):
        p = ServerParams()
        lib().lshg_server_params_default(C.byref(p))
        p.max_batch, p.max_queue, p.streams, p.use_graphs = max_batch, max_queue, streams, int(use_graphs)
        p.hbm_reserve_mb, p.batch_window_us = hbm_reserve_mb, batch_window_us
        self._h = C.c_void_p()
        check(lib().lshg_server_create(C.byref(p), C.byref(self._h)))
        self._k = {}
        self._indexes = {}

    def add_index(self, index_id: int, index: Index) -> None:
        check(lib().lshg_server_add_index(self._h, index_id, index.handle))
        self._indexes[index_id] = index

    def submit(self, index_id: int, queries, k: int) -> int:
        q = _f32(queries)
        t = C.c_int64()
        check(lib().lshg_server_submit(self._h, index_id, _ptr(q), q.shape[0], k, C.byref(t)))
        self._k[t.value] = (q.shape[0], k)
        return t.value

    def wait(self, ticket: int, timeout_us: int = 60_000_000) -> tuple[np.ndarray, float]:
        nq, k = self._k[ticket]
        out = np.zeros((nq, k), dtype=POINT_DTYPE)
        lat = C.c_double()
        check(lib().lshg_server_wait(self._h, ticket, _ptr(out), timeout_us, C.byref(lat)))
        del self._k[ticket]
        return out, lat.value

    def stats(self) -> dict:
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().lshg_server_stats(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"completed": a.value, "launches": b.value, "graph_replays": c.value, "rejected": d.value}

    def close(self) -> None:
        if self._h:
            check(lib().lshg_server_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = [
    "POINT_DTYPE", "Result", "LshgError", "calculate_k", "linear_scans", "LSH", "lsh", "random_normals",
    "random_plus_minus", "random_bools", "Index", "merge_topk", "validate", "parse_file", "write_file", "Server",
    "make_options", "launch_count", "profile_enable", "profile_report", "IMPL_EXACT", "IMPL_SIMHASH", "IMPL_WMH",
    "IMPL_WMH_ONEBIT", "IMPL_JL", "IMPL_TC", "IMPL_TC_FP8", "IMPL_CWS", "KEYS_SIMHASH", "KEYS_WMH", "KEYS_WMH_ONEBIT", "KEYS_CROSSPOLY", "KEYS_CWS",
    "SKETCH_SCAN_AUTO", "SKETCH_SCAN_POPCOUNT", "SKETCH_SCAN_TENSOR",
    "ANGULAR", "JACCARD", "EUCLIDEAN", "EXPORT_DATA", "EXPORT_SKETCHES", "EXPORT_KEYS", "EXPORT_OFFSETS",
    "EXPORT_BUCKETS", "EXPORT_QUERY_COUNTERS", "EXPORT_CWS_CODES", "POINT_DTYPE", "read_truth", "write_truth",
]
