"""GPU parity of the (K,L) LSH framework (lshFramework.cuh) against the CPU oracle:
keys bit-exact, bucket tables identical (ids sorted within buckets), query results
bit-exact (distinct candidates, top-k by (distance, id))."""
import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100
WALK_LIST_CAP = 6144  # distinct ids a query the bucket walk lists (kSplitCap in csrc/lsh.cu)


def data(n, nq, seed=21):
    return datasets.clustered(n, D, seed, count=12), datasets.clustered(nq, D, seed + 1, count=12)


def lsh_index_arrays(engine, idx, n, tables, S):
    keys = np.frombuffer(idx.export(engine.EXPORT_KEYS), np.uint16).reshape(n, tables)
    off = np.frombuffer(idx.export(engine.EXPORT_OFFSETS), np.int32)
    bk = np.frombuffer(idx.export(engine.EXPORT_BUCKETS), np.int32)
    return keys, off, bk


@pytest.mark.parametrize("hashes,bits", [(1, 8), (2, 16)])
def test_crosspoly_keys_buckets_query(engine, orc, hashes, bits):
    n, nq, L, P = 4000, 16, 8, 128
    x, q = data(n, nq)
    S = 1 << bits
    opt = engine.make_options(cp_hashes=hashes)
    idx = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7, bucketKeyBits=bits,
                       tables=L, options=opt)
    xn, qn = orc.normalize(x), orc.normalize(q)
    diag = engine.random_plus_minus(P * L * 3 * hashes)
    okeys = orc.crosspoly(xn, P, L, hashes, 3, diag)
    keys, off, bk = lsh_index_arrays(engine, idx, n, L, S)
    assert np.array_equal(keys, okeys)
    ooff, obk = orc.lsh_build(okeys, L, S)
    assert np.array_equal(off, ooff)
    assert np.array_equal(bk, obk)
    _, qk = idx.sketch_queries(q, np.uint32, 0, L)
    oqk = orc.crosspoly(qn, P, L, hashes, 3, diag)
    assert np.array_equal(qk, oqk)
    res = idx.query(q, 32)
    ids, ds = orc.lsh_query(xn, qn, oqk, L, S, ooff, obk, 0, 0, None, None, 0, 32, 1, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)


@pytest.mark.parametrize("d", [5, 16, 30, 64, 99, 200, 513])
def test_crosspoly_keys_every_lane_layout(engine, orc, d):
    """Base and query keys bit-identical to the oracle for every lane layout of the key
    kernel: P < 32 (a unit in one lane: P = 8, 16), P = 32 (one lane, four-float chunks),
    units spread over 2 .. 32 lanes (P = 64 .. 1024), 16-byte loads (d % 4 == 0) and
    scalar loads, one and two rotations a key."""
    P = 1 << (d - 1).bit_length()
    n, nq, L = 1500, 16, 4
    x = datasets.clustered(n, d, 71, count=12)
    q = datasets.clustered(nq, d, 72, count=12)
    xn, qn = orc.normalize(x), orc.normalize(q)
    for hashes in (1, 2):
        if (2 * P) ** hashes > 65536:
            continue
        bits = max(8, ((2 * P) ** hashes - 1).bit_length())
        idx = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7,
                           bucketKeyBits=bits, tables=L, options=engine.make_options(cp_hashes=hashes))
        diag = engine.random_plus_minus(P * L * 3 * hashes)
        keys, _, _ = lsh_index_arrays(engine, idx, n, L, 1 << bits)
        assert np.array_equal(keys, orc.crosspoly(xn, P, L, hashes, 3, diag)), (d, hashes)
        _, qk = idx.sketch_queries(q, np.uint32, 0, L)
        assert np.array_equal(qk, orc.crosspoly(qn, P, L, hashes, 3, diag)), (d, hashes)


def walked_and_distinct(qkeys, off, bk, tables, S, n):
    """Bucket entries each query walks and its distinct candidates, from the oracle's tables."""
    ent, dis = [], []
    for row in qkeys:
        parts = []
        for t in range(tables):
            key = int(row[t])
            st = off[t * S + key]
            en = off[t * S + key + 1] if key + 1 < S else t * n + n
            parts.append(bk[st:en])
        a = np.concatenate(parts)
        ent.append(a.size)
        dis.append(np.unique(a).size)
    return np.array(ent), np.array(dis)


@pytest.mark.parametrize("d,P", [(100, 128), (37, 64)])
def test_crosspoly_many_candidates_and_counters(engine, orc, d, P):
    """~20k distinct candidates a query (many scoring batches per query) and 640 queries,
    more than the query kernel's resident CTAs, so CTAs answer further queries after
    clearing their dedupe bitmaps.  d = 37 takes the direct row path, d = 100 the rows
    staged by bulk copies.  The kernel's counters must equal the entries walked and the
    distinct candidates computed from the oracle's tables."""
    n, nq, L, bits = 40000, 640, 12, 8
    x = datasets.clustered(n, d, 61, count=2)
    q = datasets.clustered(nq, d, 62, count=2)
    S = 1 << bits
    idx = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7, bucketKeyBits=bits,
                       tables=L, options=engine.make_options(cp_hashes=1))
    xn, qn = orc.normalize(x), orc.normalize(q)
    diag = engine.random_plus_minus(P * L * 3)
    okeys = orc.crosspoly(xn, P, L, 1, 3, diag)
    oqk = orc.crosspoly(qn, P, L, 1, 3, diag)
    ooff, obk = orc.lsh_build(okeys, L, S)
    ent, dis = walked_and_distinct(oqk, ooff, obk, L, S, n)
    assert dis.min() > WALK_LIST_CAP  # the case this test is for
    assert idx.query_counters() == (0, 0)
    res = idx.query(q, 32)
    ids, ds = orc.lsh_query(xn, qn, oqk, L, S, ooff, obk, 0, 0, None, None, 0, 32, 1, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)
    assert idx.query_counters() == (int(ent.sum()), int(dis.sum()))


def test_crosspoly_mixed_list_sizes_one_batch(engine, orc):
    """One batch where 25 queries (24 in a 30,000-point cluster, one of the small-cluster
    ones) have more distinct candidates than the bucket walk lists and go through the fused
    kernel, and 39 (among 2,000 small clusters) have a few hundred to a few thousand and are
    scored from their lists; both parts must equal the oracle and the counters the oracle's
    totals."""
    d, P, L, bits, n = D, 128, 12, 8, 40000
    x = np.concatenate([datasets.clustered(30000, d, 71, count=1, center_seed=55),
                        datasets.clustered(10000, d, 72, count=2000, center_seed=56)])
    q = np.concatenate([datasets.clustered(24, d, 73, count=1, center_seed=55),
                        datasets.clustered(40, d, 74, count=2000, center_seed=56)])
    S = 1 << bits
    idx = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7, bucketKeyBits=bits,
                       tables=L, options=engine.make_options(cp_hashes=1))
    xn, qn = orc.normalize(x), orc.normalize(q)
    diag = engine.random_plus_minus(P * L * 3)
    oqk = orc.crosspoly(qn, P, L, 1, 3, diag)
    ooff, obk = orc.lsh_build(orc.crosspoly(xn, P, L, 1, 3, diag), L, S)
    ent, dis = walked_and_distinct(oqk, ooff, obk, L, S, n)
    assert (dis > WALK_LIST_CAP).sum() == 25 and (dis <= WALK_LIST_CAP).sum() == 39  # the case this test is for
    res = idx.query(q, 32)
    ids, ds = orc.lsh_query(xn, qn, oqk, L, S, ooff, obk, 0, 0, None, None, 0, 32, 1, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)
    assert idx.query_counters() == (int(ent.sum()), int(dis.sum()))


def test_simhash_keys_sketched_query(engine, orc):
    n, nq, L, bits, W = 3000, 12, 6, 10, 8
    x, q = data(n, nq, seed=31)
    r = engine.LSH(3, 3, 32, D, nq, n, x, q, W, 1, bits, L, True, options=engine.make_options(candidates=512))
    kp = engine.random_normals(L * D * bits)
    okeys = (orc.simhash(x, kp, L, bits) & 0xFFFF).astype(np.uint16)
    oqk = (orc.simhash(q, kp, L, bits) & 0xFFFF).astype(np.uint16)
    S = 1 << bits
    ooff, obk = orc.lsh_build(okeys, L, S)
    sp = engine.random_normals(W * D * 32)
    xs, qs = orc.simhash(x, sp, W, 32), orc.simhash(q, sp, W, 32)
    ids, ds = orc.lsh_query(x, q, oqk, L, S, ooff, obk, 1, 3, xs, qs, W, 512, 1, 32)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)


def test_lsh_exact_reference_entry_point(engine, orc):
    n, nq, L, bits = 2500, 10, 4, 12
    x, q = data(n, nq, seed=41)
    r = engine.LSH(2, 3, 64, D, nq, n, x, q, 0, 1, bits, L, False)
    kp = engine.random_normals(L * D * bits)
    okeys = (orc.simhash(x, kp, L, bits) & 0xFFFF).astype(np.uint16)
    oqk = (orc.simhash(q, kp, L, bits) & 0xFFFF).astype(np.uint16)
    ooff, obk = orc.lsh_build(okeys, L, 1 << bits)
    ids, ds = orc.lsh_query(x, q, oqk, L, 1 << bits, ooff, obk, 0, 0, None, None, 0, 64, 1, 64)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)
    # fewer than k distinct candidates leave empty entries
    assert ((r.ids == -1) == (ids == -1)).all()


def test_lsh_bad_key_range_rejected(engine):
    x, q = data(100, 2)
    with pytest.raises(engine.LshgError):
        engine.LSH(2, 7, 32, D, 2, 100, x, q, 0, 1, 6, 4, False)  # 2P = 256 keys > 2^6 buckets


# ---- weighted-MinHash bucket keys (keysImplementation 4 and 5) ---------------------------

def wmh_keys_oracle(orc, xs, start, mp, M, u, H, onebit, tables, bits, bm):
    """Keys of shifted, normalised rows: byte samples (one per table, u8 widened to u16)
    or `bits` one-bit samples packed into a word per table (lshFramework.cuh:47-53 ->
    weightedMinHash.cuh:432-466)."""
    sk, over = orc.wmh_sketch(xs, start, mp, M, u, H, u.shape[1], onebit, tables, bits, bm)
    assert over == 0
    return (sk & 0xFFFF).astype(np.uint16) if onebit else sk.astype(np.uint16)


def shift_by_base(x, q):
    """The recorded min shift replayed on queries: |min floor| over the base only."""
    mn = np.minimum(0, np.floor(x).min(axis=0)).astype(np.int32)
    return (np.asarray(q, np.float32) + np.abs(mn).astype(np.float32)).astype(np.float32)


@pytest.mark.parametrize("onebit,bits,dist", [(0, 8, 2), (0, 10, 1), (1, 6, 1), (1, 12, 2)])
def test_wmh_keys_buckets_query(engine, orc, uniforms, onebit, bits, dist):
    """Weighted-MinHash keys: byte samples (keysImplementation 4) and one-bit samples
    (5) at two bucketKeyBits each.  Index (statistics from the base): base and query keys
    bit-exact, bucket offsets and contents equal to the oracle's, query results equal.
    Reference entry point LSH() (statistics over base and queries, as runLsh computes
    them): results equal to the oracle's."""
    n, nq, L = 3000, 12, 6
    x = datasets.sparse_gamma(n, D, 91 + bits)
    q = datasets.sparse_gamma(nq, D, 191 + bits)
    keys_impl = 5 if onebit else 4
    H = L * bits if onebit else L
    S = 1 << bits
    u = uniforms(H, 4096)
    bm = orc.random_bools(255)

    # resident index: shift and normalise with the base's statistics, replayed on queries
    idx = engine.Index(x, implementation=2, distanceFunc=dist, framework=1, keysImplementation=keys_impl,
                       bucketKeyBits=bits, tables=L)
    xs, _ = orc.jaccard_shift(x, x[:0])
    xs = orc.normalize(xs)
    qs = orc.normalize(shift_by_base(x, q))
    start, mp, M = orc.wmh_bounds(xs, xs[:0])
    okeys = wmh_keys_oracle(orc, xs, start, mp, M, u, H, onebit, L, bits, bm)
    if not onebit:
        assert okeys.max() < S
    keys, off, bk = lsh_index_arrays(engine, idx, n, L, S)
    assert np.array_equal(keys, okeys)
    ooff, obk = orc.lsh_build(okeys, L, S)
    assert np.array_equal(off, ooff)
    assert np.array_equal(bk, obk)
    oqk = wmh_keys_oracle(orc, qs, start, mp, M, u, H, onebit, L, bits, bm)
    _, qk = idx.sketch_queries(q, np.uint32, 0, L)
    assert np.array_equal(qk, oqk)
    res = idx.query(q, 32)
    ids, ds = orc.lsh_query(xs, qs, oqk, L, S, ooff, obk, 0, 0, None, None, 0, 32, dist, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)
    assert (ids[:, 0] >= 0).all()  # every query finds candidates in its buckets

    # reference entry point: statistics over base and queries
    r = engine.LSH(2, keys_impl, 32, D, nq, n, x, q, 0, dist, bits, L, False)
    xs2, qs2 = orc.jaccard_shift(x, q)
    xs2, qs2 = orc.normalize(xs2), orc.normalize(qs2)
    start2, mp2, M2 = orc.wmh_bounds(xs2, qs2)
    ok2 = wmh_keys_oracle(orc, xs2, start2, mp2, M2, u, H, onebit, L, bits, bm)
    oq2 = wmh_keys_oracle(orc, qs2, start2, mp2, M2, u, H, onebit, L, bits, bm)
    off2, bk2 = orc.lsh_build(ok2, L, S)
    ids2, ds2 = orc.lsh_query(xs2, qs2, oq2, L, S, off2, bk2, 0, 0, None, None, 0, 32, dist, 32)
    assert np.array_equal(r.ids, ids2)
    assert np.array_equal(r.distances, ds2)


def test_wmh_byte_keys_need_256_buckets(engine):
    x = datasets.sparse_gamma(200, D, 5)
    with pytest.raises(engine.LshgError):
        engine.Index(x, implementation=2, distanceFunc=2, framework=1, keysImplementation=4, bucketKeyBits=7, tables=4)


@pytest.mark.parametrize("K,bits,dist", [(1, 10, 2), (2, 12, 2), (3, 8, 1)])
def test_cws_keys_buckets_query(engine, orc, K, bits, dist):
    """Consistent-weighted-sampling keys (keysImplementation 10; K samples a table hashed
    into bucketKeyBits bits): base and query keys bit-exact against the oracle, bucket
    offsets and contents equal, query results equal -- through the resident index and
    the reference-shaped LSH() entry point; a save/load round trip answers alike."""
    import os
    import tempfile

    n, nq, L = 4000, 16, 8
    x = datasets.sparse_gamma(n, D, 301 + bits)
    q = datasets.sparse_gamma(nq, D, 401 + bits)
    S = 1 << bits
    opt = engine.make_options(cp_hashes=K)
    idx = engine.Index(x, implementation=2, distanceFunc=dist, framework=1, keysImplementation=10,
                       bucketKeyBits=bits, tables=L, options=opt)
    xs = orc.normalize(x)  # nonnegative data: the recorded shift is zero
    qs = orc.normalize(q)
    okeys = orc.cws_keys(xs, L, K, bits)
    keys, off, bk = lsh_index_arrays(engine, idx, n, L, S)
    assert np.array_equal(keys, okeys)
    ooff, obk = orc.lsh_build(okeys, L, S)
    assert np.array_equal(off, ooff)
    assert np.array_equal(bk, obk)
    oqk = orc.cws_keys(qs, L, K, bits)
    _, qk = idx.sketch_queries(q, np.uint32, 0, L)
    assert np.array_equal(qk, oqk)
    res = idx.query(q, 32)
    ids, ds = orc.lsh_query(xs, qs, oqk, L, S, ooff, obk, 0, 0, None, None, 0, 32, dist, 32)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)
    assert (ids[:, 0] >= 0).all()

    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "cws_keys.lshg")
        idx.save(path)
        assert np.array_equal(engine.Index.load(path).query(q, 32), res)

    r = engine.LSH(2, 10, 32, D, nq, n, x, q, 0, dist, bits, L, False, options=opt)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)
