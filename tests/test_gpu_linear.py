"""GPU parity of the linear scans (implementations 2, 3, 4, 5, 6) against the CPU oracle.

Integer outputs (sketch words, bytes, ids) are compared bit-exactly; distances are
compared bit-exactly where the reference's arithmetic is restated exactly (angular,
generalized Jaccard, Hamming/Jaccard sketch distances, JL projections) and with a
stated tolerance for the Euclidean distance (the reference squares through pow()).
"""
import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100


def data(n, nq, seed=5, d=D):
    return datasets.clustered(n, d, seed, count=20), datasets.clustered(nq, d, seed + 1, count=20)


# ---- implementation 2: exact scan -----------------------------------------------------

@pytest.mark.parametrize("n,nq,k", [(1000, 7, 32), (5003, 64, 64), (2049, 33, 100), (300, 1, 1024)])
def test_exact_angular_bit_exact(engine, orc, n, nq, k):
    x, q = data(n, nq)
    kk = engine.calculate_k(k)
    r = engine.linear_scans(2, kk, D, nq, n, x, q, 0, 1)
    ids, ds = orc.exact_topk(x, q, kk, dist=1)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


@pytest.mark.parametrize("d,n", [(300, 3000), (64, 20000)])
def test_exact_angular_dims(engine, orc, d, n):
    """d = 300 does not fit two point tiles in shared memory and runs the single-buffered
    scan; d = 64 with 157 tiles exercises the double-buffered pipeline over many tiles."""
    nq = 40
    x, q = data(n, nq, seed=17, d=d)
    r = engine.linear_scans(2, 32, d, nq, n, x, q, 0, 1)
    ids, ds = orc.exact_topk(x, q, 32, dist=1)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


def test_exact_ties_lower_index_and_short_base(engine, orc):
    x, q = data(40, 5)
    x = np.concatenate([x, x[:10]])  # exact duplicates: equal distances, lower id first
    r = engine.linear_scans(2, 64, D, 5, 50, x, q, 0, 1)
    ids, ds = orc.exact_topk(x, q, 64, dist=1)
    assert np.array_equal(r.ids, ids) and np.array_equal(r.distances, ds)
    assert (r.ids[:, 50:] == -1).all() and (r.distances[:, 50:] == 2147483648.0).all()


def test_exact_jaccard_bit_exact(engine, orc):
    x = datasets.sparse_gamma(3000, D, 3)
    q = datasets.sparse_gamma(17, D, 4)
    r = engine.linear_scans(2, 32, D, 17, 3000, x, q, 0, 2)
    xs, qs = orc.jaccard_shift(x, q)
    xs, qs = orc.normalize(xs), orc.normalize(qs)
    ids, ds = orc.exact_topk(xs, qs, 32, dist=2)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


def test_exact_euclidean_tolerance(engine, orc):
    from conftest import ids_equal_up_to_ties

    x, q = data(2000, 9)
    r = engine.linear_scans(2, 32, D, 9, 2000, x, q, 0, 3)
    ids, ds = orc.exact_topk(x, q, 32, dist=3)
    assert np.allclose(r.distances, ds, rtol=1e-6, atol=1e-6)  # tolerance: 1e-6 relative
    assert ids_equal_up_to_ties(r.ids, r.distances, ids, ds, 2e-6) == 0


def test_exact_index_repeatable(engine):
    x, q = data(4000, 50)
    idx = engine.Index(x, implementation=2, distanceFunc=1)
    a = idx.query(q, 32)
    b = idx.query(q, 32)
    assert np.array_equal(a, b)
    r = engine.linear_scans(2, 32, D, 50, 4000, x, q, 0, 1)
    assert np.array_equal(a, r.results)


def test_invalid_implementation_raises(engine):
    x, q = data(100, 2)
    with pytest.raises(engine.LshgError) as e:
        engine.linear_scans(7, 32, D, 2, 100, x, q, 0, 1)
    assert e.value.status == 1


# ---- implementation 3: SimHash --------------------------------------------------------

@pytest.mark.parametrize("words", [4, 8, 32])
def test_simhash_sketch_bits(engine, orc, words):
    x, q = data(1500, 11)
    idx = engine.Index(x, implementation=3, sketchDim=words)
    sk = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint32).reshape(1500, words)
    planes = engine.random_normals(D * 32 * words)
    assert np.array_equal(sk, orc.simhash(x, planes, words, 32))
    qs, _ = idx.sketch_queries(q, np.uint32, words)
    assert np.array_equal(qs, orc.simhash(q, planes, words, 32))


def test_simhash_tensor_core_projection_large(engine, orc):
    """30,000 points x 1,024 planes: the tensor-core projection (split-BF16 GEMM, then the
    reference's FMA chain for the signs inside the GEMM's error band) equals the oracle's
    sign bits exactly, for the base (export) and for a query batch."""
    words, n, nq = 32, 30000, 2000
    x, q = data(n, nq, seed=91)
    idx = engine.Index(x, implementation=3, sketchDim=words)
    planes = engine.random_normals(D * 32 * words)
    sk = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint32).reshape(n, words)
    assert np.array_equal(sk, orc.simhash(x, planes, words, 32))
    qs, _ = idx.sketch_queries(q, np.uint32, words)
    assert np.array_equal(qs, orc.simhash(q, planes, words, 32))


def test_simhash_projection_band_overflow(engine, orc):
    """Zero rows put every sign of theirs inside the band (0 >= 0 is a 1 bit): the recheck
    lists overflow and the SIMT projection redoes the batch; bits still equal the oracle's."""
    words, n = 8, 12000
    x, _ = data(n, 1, seed=93)
    x[::2] = 0.0
    idx = engine.Index(x, implementation=3, sketchDim=words)
    planes = engine.random_normals(D * 32 * words)
    sk = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint32).reshape(n, words)
    assert np.array_equal(sk, orc.simhash(x, planes, words, 32))
    assert np.all(sk[::2] == 0xFFFFFFFF)


# C picks the scan's layout: 32, 8 or 2 queries a CTA with append buffers checked every
# 1, 2 or 4 tiles; 32 words (1024 bits) runs the width-specialised kernel, 8 the generic one
@pytest.mark.parametrize("C,n,words", [(128, 6000, 8), (256, 6000, 8), (1024, 6000, 8), (1024, 40000, 8),
                                       (4096, 6000, 8), (128, 6000, 32), (1024, 20000, 32), (4096, 6000, 32)])
def test_simhash_scan_rerank(engine, orc, C, n, words):
    nq = 21
    x, q = data(n, nq)
    opt = engine.make_options(candidates=C)
    r = engine.linear_scans(3, 32, D, nq, n, x, q, words, 1, options=opt)
    planes = engine.random_normals(D * 32 * words)
    ids, ds = orc.sketch_scan(x, q, 3, orc.simhash(x, planes, words, 32), orc.simhash(q, planes, words, 32), words,
                              C, 1, 32)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


# ---- implementation 6: JL -------------------------------------------------------------

def test_jl_sketch_and_scan(engine, orc):
    n, nq, S = 3000, 13, 16
    x, q = data(n, nq)
    xs, qs = orc.normalize(x), orc.normalize(q)
    R = engine.random_normals(S * D, 1.0 / S)
    idx = engine.Index(x, implementation=6, sketchDim=S)
    sk = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.float32).reshape(n, S)
    assert np.array_equal(sk, orc.jl(xs, R, S))
    opt = engine.make_options(candidates=256)
    r = engine.linear_scans(6, 32, D, nq, n, x, q, S, 3, options=opt)
    ids, ds = orc.sketch_scan(xs, qs, 6, orc.jl(xs, R, S), orc.jl(qs, R, S), S, 256, 1, 32)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


# ---- implementations 4 / 5: weighted MinHash -------------------------------------------

def wmh_oracle(orc, x, q, H, uniforms, onebit, words=0):
    xs, qs = orc.jaccard_shift(x, q)
    xs, qs = orc.normalize(xs), orc.normalize(qs)
    start, mp, M = orc.wmh_bounds(xs, qs)
    T = 4096
    u = uniforms(H, T)
    bm = orc.random_bools(255)
    skx, ox = orc.wmh_sketch(xs, start, mp, M, u, H, T, onebit, words, 32, bm)
    skq, oq = orc.wmh_sketch(qs, start, mp, M, u, H, T, onebit, words, 32, bm)
    assert ox == 0 and oq == 0
    return xs, qs, skx, skq


@pytest.mark.parametrize("S", [64, 256])  # 256 samples: the width-specialised scan
def test_wmh_byte_sketch_and_scan(engine, orc, uniforms, S):
    n, nq = 2000, 9
    x = datasets.sparse_gamma(n, D, 7)
    q = datasets.sparse_gamma(nq, D, 8)
    xs, qs, skx, skq = wmh_oracle(orc, x, q, S, uniforms, 0)
    idx = engine.Index(x, implementation=4, sketchDim=S)  # statistics from the base only
    xs2, _, skx2, _ = wmh_oracle(orc, x, x[:0], S, uniforms, 0)
    assert np.array_equal(np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.uint8).reshape(n, S), skx2)
    opt = engine.make_options(candidates=256)
    r = engine.linear_scans(4, 32, D, nq, n, x, q, S, 2, options=opt)
    ids, ds = orc.sketch_scan(xs, qs, 4, skx, skq, S, 256, 2, 32)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


@pytest.mark.parametrize("W", [4, 8])  # 8 words: the width-specialised scan
def test_wmh_onebit_sketch_and_scan(engine, orc, uniforms, W):
    n, nq = 2000, 9
    x = datasets.sparse_gamma(n, D, 9)
    q = datasets.sparse_gamma(nq, D, 10)
    xs, qs, skx, skq = wmh_oracle(orc, x, q, W * 32, uniforms, 1, W)
    opt = engine.make_options(candidates=256)
    r = engine.linear_scans(5, 32, D, nq, n, x, q, W, 2, options=opt)
    ids, ds = orc.sketch_scan(xs, qs, 5, skx, skq, W, 256, 2, 32)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)
