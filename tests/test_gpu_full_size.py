"""Parity at the measurement workloads' full sizes, through properties that do not need
the CPU oracle to scan the whole batch.

* headline (1.2M x 100 clustered unit vectors, 10,000 queries, tensor-core scan with the
  FP64 re-check): every returned id distinct and in range, every distance within the FP32
  error bound of its FP64 value, rows ordered up to inversions inside that bound, and
  recall@32 against the FP64 oracle on a sample of queries;
* 1024-bit SimHash (1.2M, C = 1,024, tensor-core sketch scan), byte weighted MinHash and
  consistent weighted sampling (500k sparse Gamma rows, 256 samples, C = 4,096): the
  results of a few queries of a full batch equal the oracle's scan of the index's own
  sketches (exact top-C by sketch distance, then the exact re-rank), and for CWS a sample
  of base rows' (index, t) pairs equals the oracle's sampler;
* cross-polytope LSH (1M x 128, L = 32, K = 2): queries of a full batch equal the oracle's
  bucket walk over the index's own keys and bucket tables.
"""
import os

import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100


def fp64_angular(x, q, ids):
    qq = q.astype(np.float64)
    rows = x[ids].astype(np.float64)
    dot = np.einsum("qd,qkd->qk", qq, rows)
    return 1.0 - dot / (np.linalg.norm(qq, axis=1)[:, None] * np.linalg.norm(rows, axis=2))


def test_headline_full_size(engine, orc):
    n, nq, k = 1_200_000, 10_000, 32
    x = datasets.clustered(n, D, 100)
    q = datasets.clustered(nq, D, 101)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1,
                       options=engine.make_options(candidates=64))
    res = idx.query(q, k)
    ids, ds = res["ID"], res["distance"].astype(np.float64)
    assert ((ids >= 0) & (ids < n)).all()
    assert all(len(set(r.tolist())) == k for r in ids)
    band = 2 * (2 * D + 7) * 2.0 ** -24
    d64 = fp64_angular(x, q, ids)
    assert np.abs(ds - d64).max() <= band / 2
    inv = ds[:, 1:] < ds[:, :-1]  # FP32 inversions only between FP64-reordered near-ties
    assert (ds[:, :-1] - ds[:, 1:])[inv].max(initial=0.0) <= band
    sub = 24
    tids, _ = orc.fp64_topk(x, q[:sub], k, threads=max(1, os.cpu_count() or 1))
    rec = np.mean([len(set(a.tolist()) & set(b.tolist())) / k for a, b in zip(ids[:sub], tids)])
    assert rec >= 0.99


def test_simhash_1024_full_size(engine, orc):
    n, nq, words, C = 1_200_000, 2048, 32, 1024
    x = datasets.clustered(n, D, 100)
    q = datasets.clustered(nq, D, 101)
    idx = engine.Index(x, implementation=3, sketchDim=words, options=engine.make_options(candidates=C))
    res = idx.query(q, 32)  # a batch on the tensor-core sketch scan
    skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint32).reshape(n, words)
    pick = np.array([0, 777, 2047])
    skq, _ = idx.sketch_queries(q[pick], np.uint32, words)
    ids, ds = orc.sketch_scan(x, q[pick], 3, skx, skq, words, C, 1, 32)
    assert np.array_equal(res["ID"][pick], ids)
    assert np.array_equal(res["distance"][pick], ds)


@pytest.mark.parametrize("impl", [4, 10])
def test_weighted_minhash_full_size(engine, orc, impl):
    n, nq, S, C = 500_000, 256, 256, 4096
    x = datasets.sparse_gamma(n, D, 100)
    q = datasets.sparse_gamma(nq, D, 101)
    idx = engine.Index(x, implementation=impl, distanceFunc=2, sketchDim=S)
    res = idx.query(q, 32)  # the threshold filter at full size
    xp = np.frombuffer(idx.export(engine.EXPORT_DATA), np.float32).reshape(n, D)
    pick = np.array([0, 129, 255])
    qp = orc.normalize(q[pick])
    if impl == 4:
        skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint8).reshape(n, S)
        skq, _ = idx.sketch_queries(q[pick], np.uint8, S)
    else:
        skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.int32).reshape(n, S, 2)
        skq, _ = idx.sketch_queries(q[pick], np.int32, 2 * S)
        skq = skq.reshape(len(pick), S, 2)
        rows = np.random.default_rng(5).choice(n, 2000, replace=False)
        tab = orc.cws_tables(D, S)
        assert np.array_equal(skx[rows], orc.cws_sketch(xp[rows], S, tab))
        assert np.array_equal(skq, orc.cws_sketch(qp, S, tab))
    ids, ds = orc.sketch_scan(xp, qp, impl, skx, skq, S, C, 2, 32)
    assert np.array_equal(res["ID"][pick], ids)
    assert np.array_equal(res["distance"][pick], ds)


def test_crosspoly_lsh_full_size(engine, orc):
    """Configuration 4a (1M x 128 with 28 zero dimensions, L = 32 tables of K = 2
    cross-polytope hashes): for queries of a full batch, the results equal the oracle's
    bucket walk over the index's own keys and bucket tables."""
    n, nq, L, bits = 1_000_000, 1024, 32, 16
    x = datasets.clustered(n, D, 100, pad_to=128)
    q = datasets.clustered(nq, D, 101, pad_to=128)
    idx = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7, bucketKeyBits=bits,
                       tables=L, options=engine.make_options(cp_hashes=2))
    res = idx.query(q, 32)
    S = 1 << bits
    off = np.frombuffer(idx.export(engine.EXPORT_OFFSETS), np.int32)
    bk = np.frombuffer(idx.export(engine.EXPORT_BUCKETS), np.int32)
    xp = np.frombuffer(idx.export(engine.EXPORT_DATA), np.float32).reshape(n, 128)  # normalised for the keys
    pick = np.array([0, 500, 1023])
    _, qk = idx.sketch_queries(q[pick], np.uint32, 0, L)
    ids, ds = orc.lsh_query(xp, orc.normalize(q[pick]), qk, L, S, off, bk, 0, 0, None, None, 0, 32, 1, 32)
    assert np.array_equal(res["ID"][pick], ids)
    assert np.array_equal(res["distance"][pick], ds)
