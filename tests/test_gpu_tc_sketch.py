"""GPU parity of the tensor-core sketch scan (tc_hamming.cu): Hamming and one-bit Jaccard
scans of SimHash / one-bit weighted-MinHash sketches as +-1 E4M3 GEMMs.

The scan must select exactly the candidates of the XOR/popcount scan -- the top-C by
(sketch distance, lower id) -- so after the FP32 re-rank the ids and distances are
compared bit-exactly with the CPU oracle.  Cases cover every selection regime: a small
base where every point survives, sampled prepasses (64- and 8-point group maxima), rows
of 1, 2, 3 and 8 chunks of 128 bits, C from 32 to 4096, a partial second query tile, and
bases of duplicated points whose ties overflow the candidate arrays (those queries are
rescanned by the popcount scan on the device).
"""
import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100
TENSOR, POPCOUNT = 2, 1


def data(n, nq, seed=5, count=20):
    return datasets.clustered(n, D, seed, count=count), datasets.clustered(nq, D, seed + 1, count=count)


def simhash_oracle(engine, orc, x, q, words, C, k=32):
    planes = engine.random_normals(D * 32 * words)
    return orc.sketch_scan(x, q, 3, orc.simhash(x, planes, words, 32), orc.simhash(q, planes, words, 32), words, C, 1,
                           k)


@pytest.mark.parametrize("C,n,words,nq", [
    (32, 3000, 4, 130),       # small base: every point survives; 1 chunk
    (128, 6000, 8, 130),      # 2 chunks
    (1024, 12000, 32, 130),   # 8 chunks, block select
    (4096, 12000, 10, 70),    # 3 chunks (last one half padding), C = 4096
    (128, 120000, 8, 130),    # prepass every 8th tile, 64-point maxima
    (1024, 120000, 32, 130),  # prepass, 8-point maxima (C too large for 64-point groups)
])
def test_tc_simhash_matches_oracle(engine, orc, C, n, words, nq):
    x, q = data(n, nq, count=40)
    opt = engine.make_options(candidates=C, sketch_scan=TENSOR)
    r = engine.linear_scans(3, 32, D, nq, n, x, q, words, 1, options=opt)
    ids, ds = simhash_oracle(engine, orc, x, q, words, C)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


@pytest.mark.parametrize("C,n", [(256, 4000), (256, 140000)])
def test_tc_onebit_minhash_matches_oracle(engine, orc, C, n):
    """One-bit weighted MinHash (8 words = 256 one-bit samples): the resident index's
    sketches, scanned on the tensor cores, against the oracle's scan of the same sketches
    and its generalized-Jaccard re-rank of the preprocessed rows."""
    W, nq = 8, 100
    x = datasets.sparse_gamma(n, D, 31)
    q = datasets.sparse_gamma(nq, D, 32)
    idx = engine.Index(x, implementation=5, distanceFunc=2, sketchDim=W,
                       options=engine.make_options(candidates=C, sketch_scan=TENSOR))
    xp = np.frombuffer(idx.export(engine.EXPORT_DATA), np.float32).reshape(n, D)
    skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint32).reshape(n, W)
    skq, _ = idx.sketch_queries(q, np.uint32, W)
    qp = orc.normalize(q)  # nonnegative data: the recorded shift is zero
    res = idx.query(q, 32)
    ids, ds = orc.sketch_scan(xp, qp, 5, skx, skq, W, C, 2, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)


@pytest.mark.parametrize("C", [128, 1024])
def test_tc_simhash_tie_overflow_rescanned(engine, orc, C):
    """20,000 copies of one point among 60,000: queries near it tie with all copies at the
    same Hamming distance, more than their candidate arrays hold, and are rescanned by the
    popcount scan; the other queries take the tensor-core path.  All equal the oracle."""
    words = 8
    base, q = data(40000, 96, seed=41, count=30)
    dup = np.repeat(base[:1], 20000, axis=0)
    x = np.ascontiguousarray(np.concatenate([base, dup]))
    q = np.ascontiguousarray(np.concatenate([np.repeat(base[:1], 32, axis=0) + 1e-3 * q[:32], q[32:]]))
    nq, n = q.shape[0], x.shape[0]
    opt = engine.make_options(candidates=C, sketch_scan=TENSOR)
    r = engine.linear_scans(3, 32, D, nq, n, x, q, words, 1, options=opt)
    ids, ds = simhash_oracle(engine, orc, x, q, words, C)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


def test_tc_and_popcount_paths_agree_by_default(engine):
    """The default (auto) choice sends a 200-query batch to the tensor cores and a 20-query
    batch to the popcount scan; both equal the popcount scan forced on the same queries."""
    x, q = data(50000, 200, seed=51, count=40)
    auto = engine.Index(x, implementation=3, sketchDim=32, options=engine.make_options(candidates=1024))
    pop = engine.Index(x, implementation=3, sketchDim=32,
                       options=engine.make_options(candidates=1024, sketch_scan=POPCOUNT))
    for qq in (q, q[:20]):
        assert np.array_equal(auto.query(qq, 32), pop.query(qq, 32))


@pytest.mark.parametrize("C,n,S", [(256, 4000, 64), (4096, 60000, 256), (1024, 150000, 200)])
def test_byte_minhash_filter_scan_matches_oracle(engine, orc, C, n, S):
    """Byte weighted MinHash (implementation 4) through the threshold-filter scan: samples
    bit-sliced, a histogram prepass on every S-th tile, survivors with at least tau equal
    samples, the integer select; against the oracle's scan of the same sketches and its
    generalized-Jaccard re-rank.  200 samples leave a partly padded group of 32."""
    nq = 100
    x = datasets.sparse_gamma(n, D, 33)
    q = datasets.sparse_gamma(nq, D, 34)
    idx = engine.Index(x, implementation=4, distanceFunc=2, sketchDim=S,
                       options=engine.make_options(candidates=C, sketch_scan=TENSOR))
    xp = np.frombuffer(idx.export(engine.EXPORT_DATA), np.float32).reshape(n, D)
    skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint8).reshape(n, S)
    skq, _ = idx.sketch_queries(q, np.uint8, S)
    res = idx.query(q, 32)
    ids, ds = orc.sketch_scan(xp, orc.normalize(q), 4, skx, skq, S, C, 2, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)


def test_byte_minhash_filter_ties_rescanned(engine, orc):
    """A third of the base is one duplicated row: queries equal to it tie with every copy
    at the top match count, overflow the candidate arrays and are rescanned; all equal the
    oracle."""
    n, nq, S, C = 45000, 80, 64, 512
    x = datasets.sparse_gamma(n, D, 35)
    x[::3] = x[0]
    q = datasets.sparse_gamma(nq, D, 36)
    q[:20] = x[0]
    idx = engine.Index(x, implementation=4, distanceFunc=2, sketchDim=S,
                       options=engine.make_options(candidates=C, sketch_scan=TENSOR))
    xp = np.frombuffer(idx.export(engine.EXPORT_DATA), np.float32).reshape(n, D)
    skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint8).reshape(n, S)
    skq, _ = idx.sketch_queries(q, np.uint8, S)
    res = idx.query(q, 32)
    ids, ds = orc.sketch_scan(xp, orc.normalize(q), 4, skx, skq, S, C, 2, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)
