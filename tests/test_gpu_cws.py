"""GPU parity of consistent weighted sampling (implementation 10, csrc/cws.cu).

The samples are a deterministic function of the draw table and the preprocessed rows, so
the index's (index, t) pairs -- base and queries -- are compared bit for bit with the
oracle's restatement; the scan must select exactly the oracle's top-C by
(1 - matches / S, id), so after the generalized-Jaccard re-rank ids and distances are
compared exactly.  Cases cover the three scan forms: the threshold filter over 16-plane
codes, 8-plane codes and per-position dictionary ranks (batches of 64 queries and
more), the direct scan over the pairs
(small batches, listed queries, and bases whose codes need more than 16 bits), and ties
that overflow the filter's candidate arrays.
"""
import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

CWS = 10


def build(engine, x, S, C):
    return engine.Index(x, implementation=CWS, distanceFunc=2, sketchDim=S,
                        options=engine.make_options(candidates=C))


def exported(engine, idx, n, d, S):
    xp = np.frombuffer(idx.export(engine.EXPORT_DATA), np.float32).reshape(n, d)
    skx = np.frombuffer(idx.export(engine.EXPORT_SKETCHES), np.int32).reshape(n, S, 2)
    plan = np.frombuffer(idx.export(engine.EXPORT_CWS_CODES), np.int32)
    return xp, skx, plan


def check_against_oracle(engine, orc, idx, x, q, S, C, k=32):
    n, d = x.shape
    xp, skx, plan = exported(engine, idx, n, d, S)
    skq, _ = idx.sketch_queries(q, np.int32, 2 * S)
    skq = skq.reshape(q.shape[0], S, 2)
    qp = orc.normalize(q)  # nonnegative data: the recorded shift is zero
    tab = orc.cws_tables(d, S)
    assert np.array_equal(skx, orc.cws_sketch(xp, S, tab))
    assert np.array_equal(skq, orc.cws_sketch(qp, S, tab))
    res = idx.query(q, k)
    ids, ds = orc.sketch_scan(xp, qp, CWS, skx, skq, S, C, 2, k)
    assert np.array_equal(res["ID"], ids)
    assert np.array_equal(res["distance"], ds)
    return plan


@pytest.mark.parametrize("C,n,S,nq", [
    (256, 4000, 64, 100),      # filter: every 16th tile in the prepass, one pass of two groups
    (4096, 60000, 256, 70),    # filter: C = 4096, 8 groups, a partial second query block
    (1024, 150000, 96, 130),   # filter: 3 groups (two passes, the second with one group)
    (1024, 20000, 128, 20),    # direct: a batch below 64 queries, the base split over the grid
])
def test_cws_matches_oracle(engine, orc, C, n, S, nq):
    x = datasets.sparse_gamma(n, 100, 41)
    q = datasets.sparse_gamma(nq, 100, 42)
    idx = build(engine, x, S, C)
    plan = check_against_oracle(engine, orc, idx, x, q, S, C)
    # d = 100: 7 index bits and a few bits of t, at most ~150 distinct codes a position --
    # dictionary ranks, compared as bytes
    assert plan[4] == 8 and plan[5] == 1


def test_cws_sixteen_plane_codes(engine, orc):
    """Log-normal weights over 500 dimensions: 15-bit codes with more than 255 distinct
    codes at some position, so the 16-bit codes are sliced into 16 planes."""
    rng = np.random.default_rng(5)
    d = 500
    x = (np.exp(rng.normal(0, 1.5, (40000, d))) * (rng.random((40000, d)) < 0.5)).astype(np.float32)
    q = (np.exp(rng.normal(0, 1.5, (80, d))) * (rng.random((80, d)) < 0.5)).astype(np.float32)
    idx = build(engine, x, 64, 256)
    plan = check_against_oracle(engine, orc, idx, x, q, 64, 256)
    assert plan[4] == 16 and plan[5] == 0


def test_cws_eight_plane_codes(engine, orc):
    """d = 3 and weights within a factor of two: codes of at most 8 bits, one byte plane a bit."""
    rng = np.random.default_rng(7)
    x = (0.5 + 0.5 * rng.random((9000, 3))).astype(np.float32)
    q = (0.5 + 0.5 * rng.random((80, 3))).astype(np.float32)
    idx = build(engine, x, 64, 256)
    plan = check_against_oracle(engine, orc, idx, x, q, 64, 256)
    assert plan[4] == 8 and plan[5] == 0


def test_cws_wide_codes_scan_directly(engine, orc):
    """Log-normal weights over 1,200 dimensions spread t so that the codes need 17 bits:
    every batch takes the direct scan over the (index, t) pairs."""
    rng = np.random.default_rng(8)
    d = 1200
    x = (np.exp(rng.normal(0, 3, (1500, d))) * (rng.random((1500, d)) < 0.3)).astype(np.float32)
    q = (np.exp(rng.normal(0, 3, (70, d))) * (rng.random((70, d)) < 0.3)).astype(np.float32)
    idx = build(engine, x, 64, 256)
    plan = check_against_oracle(engine, orc, idx, x, q, 64, 256)
    assert plan[4] == 0


def test_cws_ties_rescanned(engine, orc):
    """A third of the base is one duplicated row: queries equal to it tie with every copy
    at all S samples, overflow the filter's candidate arrays and are rescanned directly."""
    n, nq, S, C = 45000, 80, 64, 512
    x = datasets.sparse_gamma(n, 100, 43)
    x[::3] = x[0]
    q = datasets.sparse_gamma(nq, 100, 44)
    q[:20] = x[0]
    idx = build(engine, x, S, C)
    check_against_oracle(engine, orc, idx, x, q, S, C)


def test_cws_query_samples_outside_the_base_range(engine, orc):
    """A base of near-copies of four rows keeps t in a narrow range; log-normal queries
    draw some samples below it.  Those samples get a code no base sample has and never
    match (and the near-copies tie, overflow the filter's arrays and are rescanned)."""
    rng = np.random.default_rng(9)
    d, S, C = 8, 128, 256
    proto = (0.5 + 0.5 * rng.random((4, d))).astype(np.float32)
    x = np.abs(proto[rng.integers(0, 4, 12000)] * (1 + 1e-3 * rng.standard_normal((12000, d)))).astype(np.float32)
    q = np.exp(rng.normal(0, 2, (70, d))).astype(np.float32)
    idx = build(engine, x, S, C)
    plan = check_against_oracle(engine, orc, idx, x, q, S, C)
    skq, _ = idx.sketch_queries(q, np.int32, 2 * S)
    assert (skq.reshape(70, S, 2)[:, :, 1] < plan[0]).any()


def test_cws_persistence(engine, orc, tmp_path):
    x = datasets.sparse_gamma(20000, 100, 45)
    q = datasets.sparse_gamma(90, 100, 46)
    idx = build(engine, x, 128, 1024)
    before = idx.query(q, 32)
    path = str(tmp_path / "cws.lshg")
    idx.save(path)
    loaded = engine.Index.load(path)
    assert np.array_equal(loaded.query(q, 32), before)
    assert np.array_equal(np.frombuffer(loaded.export(engine.EXPORT_CWS_CODES), np.int32),
                          np.frombuffer(idx.export(engine.EXPORT_CWS_CODES), np.int32))
    check_against_oracle(engine, orc, loaded, x, q, 128, 1024)


def test_cws_linear_scans_entry_point(engine, orc):
    """The reference-shaped call (linearScans with implementation 10): the base and the
    queries are preprocessed together, as in the reference's weighted MinHash."""
    x = datasets.sparse_gamma(8000, 100, 47)
    q = datasets.sparse_gamma(64, 100, 48)
    r = engine.linear_scans(CWS, 32, 100, 64, 8000, x, q, 64, 2, options=engine.make_options(candidates=512))
    xp = orc.normalize(x)
    qp = orc.normalize(q)
    tab = orc.cws_tables(100, 64)
    ids, ds = orc.sketch_scan(xp, qp, CWS, orc.cws_sketch(xp, 64, tab), orc.cws_sketch(qp, 64, tab), 64, 512, 2, 32)
    assert np.array_equal(r.ids, ids)
    assert np.array_equal(r.distances, ds)
