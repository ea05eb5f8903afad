"""ctypes binding of the CPU oracle (oracle.c, gold_port.cpp) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module,
as the checker.  The engine (lshongpu_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIB = None
P = C.c_void_p
i64 = C.c_int64
i32 = C.c_int

_SIGS = {
    "or_random_normals": (None, [i64, C.c_double, P]),
    "or_random_plus_minus": (None, [i64, P]),
    "or_random_bools": (None, [i64, P]),
    "or_normalize": (None, [P, i64, i32]),
    "or_row_norms": (None, [P, i64, i32, P]),
    "or_jaccard_shift": (None, [P, i64, P, i64, i32]),
    "or_exact_topk": (None, [P, i64, P, i64, i32, i32, i32, P, P]),
    "or_fp64_topk": (None, [P, i64, P, i64, i32, i32, P, P]),
    "or_fp64_topk_mt": (None, [P, i64, P, i64, i32, i32, i32, P, P]),
    "or_simhash": (None, [P, i64, i32, P, i32, i32, P]),
    "or_jl": (None, [P, i64, i32, P, i32, P]),
    "or_crosspoly": (None, [P, i64, i32, i32, i32, i32, i32, P, P]),
    "or_wmh_bounds": (i32, [P, i64, P, i64, i32, P, P, i32]),
    "or_wmh_sketch": (i64, [P, i64, i32, P, P, i32, P, i32, i32, i32, i32, i32, P, i32, P, P]),
    "or_cws_tables": (None, [i32, i32, P]),
    "or_cws_tables_seeded": (None, [i32, i32, i32, P]),
    "or_cws_keys": (None, [P, i64, i32, i32, i32, P]),
    "or_cws_logf": (C.c_float, [C.c_float]),
    "or_cws_sketch": (None, [P, i64, i32, i32, P, P]),
    "or_sketch_scan": (None, [P, i64, P, i64, i32, i32, P, P, i32, i32, i32, i32, P, P, P]),
    "or_lsh_build": (None, [P, i64, i32, i32, P, P]),
    "or_lsh_query": (None, [P, i64, P, i64, i32, P, i32, i32, P, P, i32, i32, P, P, i32, i32, i32, i32, P, P]),
    "or_goldstandard": (C.c_double, [P, i64, P, i64, i32, i32, i32, P, P]),
}


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = _build.lib_path()
        if not os.path.exists(path):
            _build.build_oracle()
        L = C.CDLL(path)
        for n, (r, a) in _SIGS.items():
            f = getattr(L, n)
            f.restype, f.argtypes = r, a
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def random_normals(count, stddev=1.0):
    out = np.empty(count, np.float32)
    lib().or_random_normals(count, stddev, _p(out))
    return out


def random_plus_minus(count):
    out = np.empty(count, np.int32)
    lib().or_random_plus_minus(count, _p(out))
    return out


def random_bools(count):
    out = np.empty(count, np.uint8)
    lib().or_random_bools(count, _p(out))
    return out


def normalize(x):
    x = _f32(x).copy()
    lib().or_normalize(_p(x), x.shape[0], x.shape[1])
    return x


def row_norms(x):
    x = _f32(x)
    out = np.empty(x.shape[0], np.float32)
    lib().or_row_norms(_p(x), x.shape[0], x.shape[1], _p(out))
    return out


def jaccard_shift(x, q):
    x, q = _f32(x).copy(), _f32(q).copy()
    lib().or_jaccard_shift(_p(x), x.shape[0], _p(q), q.shape[0], x.shape[1])
    return x, q


def exact_topk(x, q, k, dist=1):
    x, q = _f32(x), _f32(q)
    ids = np.empty((q.shape[0], k), np.int32)
    ds = np.empty((q.shape[0], k), np.float32)
    lib().or_exact_topk(_p(x), x.shape[0], _p(q), q.shape[0], x.shape[1], dist, k, _p(ids), _p(ds))
    return ids, ds


def fp64_topk(x, q, k, threads=1):
    x, q = _f32(x), _f32(q)
    ids = np.empty((q.shape[0], k), np.int32)
    ds = np.empty((q.shape[0], k), np.float64)
    if threads > 1:
        lib().or_fp64_topk_mt(_p(x), x.shape[0], _p(q), q.shape[0], x.shape[1], k, threads, _p(ids), _p(ds))
    else:
        lib().or_fp64_topk(_p(x), x.shape[0], _p(q), q.shape[0], x.shape[1], k, _p(ids), _p(ds))
    return ids, ds


def simhash(x, planes, words, bits):
    x, planes = _f32(x), _f32(planes)
    out = np.empty((x.shape[0], words), np.uint32)
    lib().or_simhash(_p(x), x.shape[0], x.shape[1], _p(planes), words, bits, _p(out))
    return out


def jl(x, R, sdim):
    x, R = _f32(x), _f32(R)
    out = np.empty((x.shape[0], sdim), np.float32)
    lib().or_jl(_p(x), x.shape[0], x.shape[1], _p(R), sdim, _p(out))
    return out


def crosspoly(x, P_, tables, hashes, rounds, diag):
    x = _f32(x)
    diag = np.ascontiguousarray(diag, np.int32)
    out = np.empty((x.shape[0], tables), np.uint16)
    lib().or_crosspoly(_p(x), x.shape[0], x.shape[1], P_, tables, hashes, rounds, _p(diag), _p(out))
    return out


def wmh_bounds(x, q):
    x, q = _f32(x), _f32(q)
    d = x.shape[1]
    start = np.empty(d, np.int32)
    cap = 1 << 20
    mp = np.empty(cap, np.int32)
    M = lib().or_wmh_bounds(_p(x), x.shape[0], _p(q), q.shape[0], d, _p(start), _p(mp), cap)
    return start, mp[:M].copy(), M


def wmh_sketch(x, start, mp, M, u, H, T, onebit, words, hashBits, bitmap):
    """u: (H, T) float32 uniforms.  Returns (sketch, n_over_T)."""
    x = _f32(x)
    u = _f32(u)
    bitmap = np.ascontiguousarray(bitmap, np.uint8)
    n = x.shape[0]
    out8 = np.zeros((n, H), np.uint8)
    out32 = np.zeros((n, max(words, 1)), np.uint32)
    over = lib().or_wmh_sketch(_p(x), n, x.shape[1], _p(np.ascontiguousarray(start, np.int32)),
                               _p(np.ascontiguousarray(mp, np.int32)), M, _p(u), H, T, int(onebit), words, hashBits,
                               _p(bitmap), len(bitmap), _p(out8), _p(out32))
    return (out32 if onebit else out8), int(over)


def cws_tables(d, S):
    """Consistent weighted sampling draw table [d][S][4]: r, 1/r, ln c, beta."""
    out = np.empty((d, S, 4), np.float32)
    lib().or_cws_tables(d, S, _p(out))
    return out


def cws_key_tables(d, S):
    """Draw table of CWS LSH keys (keysImplementation 10), [d][S][4]."""
    out = np.empty((d, S, 4), np.float32)
    lib().or_cws_tables_seeded(d, S, 1, _p(out))
    return out


def cws_keys(x, L, K, bits):
    """CWS LSH keys [n][L] u16 of preprocessed rows x: L * K samples hashed K a table."""
    x = _f32(x)
    smp = cws_sketch(x, L * K, cws_key_tables(x.shape[1], L * K))
    out = np.empty((x.shape[0], L), np.uint16)
    lib().or_cws_keys(_p(smp), x.shape[0], L, K, bits, _p(out))
    return out


def cws_logf(x):
    return np.float32(lib().or_cws_logf(C.c_float(float(x))))


def cws_sketch(x, S, tab=None):
    """(index, t) samples [n][S][2] int32 of nonnegative rows x (after preprocessing)."""
    x = _f32(x)
    n, d = x.shape
    tab = cws_tables(d, S) if tab is None else np.ascontiguousarray(tab, np.float32)
    out = np.empty((n, S, 2), np.int32)
    lib().or_cws_sketch(_p(x), n, d, S, _p(tab), _p(out))
    return out


def sketch_scan(x, q, kind, xs, qs, width, C_, dist, k, want_cand=False):
    x, q = _f32(x), _f32(q)
    nq = q.shape[0]
    ids = np.empty((nq, k), np.int32)
    ds = np.empty((nq, k), np.float32)
    cand = np.empty((nq, C_), np.uint64) if want_cand else None
    xs, qs = np.ascontiguousarray(xs), np.ascontiguousarray(qs)
    lib().or_sketch_scan(_p(x), x.shape[0], _p(q), nq, x.shape[1], kind, _p(xs), _p(qs), width, C_, dist, k,
                         _p(cand), _p(ids), _p(ds))
    return (ids, ds, cand) if want_cand else (ids, ds)


def lsh_build(keys, tables, S):
    keys = np.ascontiguousarray(keys, np.uint16)
    n = keys.shape[0]
    off = np.empty(tables * S, np.int32)
    b = np.empty(tables * n, np.int32)
    lib().or_lsh_build(_p(keys), n, tables, S, _p(off), _p(b))
    return off, b


def lsh_query(x, q, qkeys, tables, S, off, buckets, sketched, kind, xs, qs, width, C_, dist, k):
    x, q = _f32(x), _f32(q)
    nq = q.shape[0]
    ids = np.empty((nq, k), np.int32)
    ds = np.empty((nq, k), np.float32)
    qkeys = np.ascontiguousarray(qkeys, np.uint16)
    xs = None if xs is None else np.ascontiguousarray(xs)
    qs = None if qs is None else np.ascontiguousarray(qs)
    lib().or_lsh_query(_p(x), x.shape[0], _p(q), nq, x.shape[1], _p(qkeys), tables, S, _p(off), _p(buckets),
                       int(sketched), kind, _p(xs), _p(qs), width, C_, dist, k, _p(ids), _p(ds))
    return ids, ds


def goldstandard(x, q, k, threads=1):
    """Port of GoldStandard computeGoldStandard: returns (ids, -cos, seconds)."""
    x, q = _f32(x), _f32(q)
    ids = np.empty((q.shape[0], k), np.int32)
    ds = np.empty((q.shape[0], k), np.float32)
    t = lib().or_goldstandard(_p(x), x.shape[0], _p(q), q.shape[0], x.shape[1], k, threads, _p(ids), _p(ds))
    return ids, ds, t


# ---- the reference's own GPU kernels (oracle/ref_harness.cpp + oracle/_ref cubins) -----

REF_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")
_RH = None


def reference_gpu_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_kernels.txt"))


def ref_gpu():
    """Load the harness and the reference cubins (GPU machine only)."""
    global _RH
    if _RH is None:
        path = _build.harness_path()
        if not os.path.exists(path):
            _build.build_harness()
        L = C.CDLL(path)
        L.rh_error.restype = C.c_char_p
        for n in ("rh_init", "rh_knn", "rh_simhash", "rh_jl", "rh_crosspoly", "rh_wmh"):
            getattr(L, n).restype = C.c_int
        L.rh_init.argtypes = [C.c_char_p]
        L.rh_knn.argtypes = [P, i32, P, i32, i32, i32, i32, P, P, P]
        L.rh_simhash.argtypes = [P, i32, i32, i32, P, i32, P]
        L.rh_jl.argtypes = [P, i32, i32, i32, P, i32, P]
        L.rh_crosspoly.argtypes = [P, i32, i32, i32, i32, i32, P, P]
        L.rh_wmh.argtypes = [P, i32, i32, i32, P, P, i32, i32, i32, i32, i32, P, i32, P]
        if L.rh_init(REF_DIR.encode()) != 0:
            raise RuntimeError("reference harness: " + L.rh_error().decode())
        _RH = L
    return _RH


def _rh_check(st):
    if st != 0:
        raise RuntimeError("reference harness: " + ref_gpu().rh_error().decode())


def ref_knn(x, q, k, func=1):
    """The reference's exact scan kernel (impl 2) -> (ids, dists, kernel ms)."""
    x, q = _f32(x), _f32(q)
    ids = np.empty((q.shape[0], k), np.int32)
    ds = np.empty((q.shape[0], k), np.float32)
    ms = C.c_float()
    _rh_check(ref_gpu().rh_knn(_p(x), x.shape[0], _p(q), q.shape[0], x.shape[1], k, func, _p(ids), _p(ds),
                               C.byref(ms)))
    return ids, ds, ms.value


def ref_simhash(x, planes, words, launch_q=64):
    x, planes = _f32(x), _f32(planes)
    out = np.empty((x.shape[0], words), np.uint32)
    _rh_check(ref_gpu().rh_simhash(_p(x), x.shape[0], launch_q, x.shape[1], _p(planes), words, _p(out)))
    return out


def ref_jl(x, R, sdim, launch_q=64):
    x, R = _f32(x), _f32(R)
    out = np.empty((x.shape[0], sdim), np.float32)
    _rh_check(ref_gpu().rh_jl(_p(x), x.shape[0], launch_q, x.shape[1], _p(R), sdim, _p(out)))
    return out


def ref_crosspoly(x, P_, tables, diag, launch_q=64):
    x = _f32(x)
    diag = np.ascontiguousarray(diag, np.int32)
    out = np.empty((x.shape[0], tables), np.uint16)
    _rh_check(ref_gpu().rh_crosspoly(_p(x), x.shape[0], launch_q, x.shape[1], P_, tables, _p(diag), _p(out)))
    return out


def ref_wmh(x, start, mp, M, H, onebit, words, hashBits, bitmap, launch_q=64):
    x = _f32(x)
    start = np.ascontiguousarray(start, np.int32)
    mp = np.ascontiguousarray(mp, np.int32)
    bitmap = np.ascontiguousarray(bitmap, np.uint8)
    out = np.empty((x.shape[0], words), np.uint32) if onebit else np.empty((x.shape[0], H), np.uint8)
    _rh_check(ref_gpu().rh_wmh(_p(x), x.shape[0], launch_q, x.shape[1], _p(start), _p(mp), M, H, int(onebit), words,
                               hashBits, _p(bitmap), len(bitmap), _p(out)))
    return out
