"""GPU checks of the tensor-core exact scan (implementation 8): BF16 tcgen05 GEMM with
fused top-candidate selection, then exact FP32 re-rank.

Tolerance stated: recall@k >= 0.99 against the exact FP32 scan (the oracle), and every
returned distance equals the oracle's FP32 distance for that id bit for bit (the
re-rank uses the reference's arithmetic).
"""
import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100


def recall(a, b):
    return float(np.mean([len(set(x.tolist()) & set(y.tolist())) / len(y) for x, y in zip(a, b)]))


def fp64_band(d):
    """Twice the FP32 error bound of an angular distance in d dimensions: entries closer
    than this are ordered by their FP64 distances (the default FP64 re-check), so their
    FP32 values may be out of order by at most this much."""
    return 2 * (2 * d + 7) * 2.0 ** -24


def assert_order(row, strict, d=D):
    """Ascending (distance, id); with the FP64 re-check an FP32 inversion is allowed only
    between entries within fp64_band(d) of each other."""
    keys = [(float(v), int(i)) for i, v in zip(row["ID"], row["distance"]) if i >= 0]
    for (da, ia), (db, ib) in zip(keys, keys[1:]):
        if (db, ib) < (da, ia):
            assert not strict and da - db <= fp64_band(d), ((da, ia), (db, ib))


@pytest.mark.parametrize("n,nq,k", [(1000, 200, 32), (50, 7, 32), (20000, 300, 32), (6000, 129, 100)])
def test_tc_scan_recall_and_exact_distances(engine, orc, n, nq, k):
    x = datasets.clustered(n, D, 61, count=40)
    q = datasets.clustered(nq, D, 62, count=40)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    res = idx.query(q, k)
    kk = min(k, n)
    ids, ds = orc.exact_topk(x, q, k, dist=1)
    assert recall(res["ID"][:, :kk], ids[:, :kk]) >= 0.99
    # returned distances are the exact FP32 distances of the returned ids
    lookup = [dict(zip(i.tolist(), d.tolist())) for i, d in zip(ids, ds)]
    checked = 0
    for qi in range(nq):
        for rid, rd in zip(res["ID"][qi], res["distance"][qi]):
            if rid in lookup[qi]:
                assert np.float32(rd) == np.float32(lookup[qi][rid])
                checked += 1
    assert checked >= 0.99 * nq * kk
    # ascending, ties by lower id (FP64 order within the FP32 error bound)
    for row in res:
        assert_order(row, strict=False)
    # without the FP64 re-check: strictly the FP32 order
    plain = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1,
                         options=engine.make_options(fp64_recheck=0)).query(q, k)
    for row in plain:
        assert_order(row, strict=True)


def test_tc_reference_entry_point_matches_index(engine):
    x = datasets.clustered(3000, D, 71, count=30)
    q = datasets.clustered(64, D, 72, count=30)
    r = engine.linear_scans(engine.IMPL_TC, 32, D, 64, 3000, x, q, 0, 1)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    assert np.array_equal(r.results, idx.query(q, 32))


def test_tc_rejects_unsupported(engine):
    x = datasets.clustered(300, D, 3, count=5)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    with pytest.raises(engine.LshgError):
        idx.query(x[:4], 256)
    with pytest.raises(engine.LshgError):
        engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=2)


def _query_both_paths(idx, q, k):
    """The filter path and the per-row list kernel (forced for every query) on the same
    inputs."""
    import os

    a = idx.query(q, k)
    os.environ["LSHG_TC_FORCE_FALLBACK"] = "1"
    try:
        b = idx.query(q, k)
    finally:
        del os.environ["LSHG_TC_FORCE_FALLBACK"]
    return a, b


# n chosen to exercise every prepass regime: no prepass (keep every point), 8-column
# group maxima, 64-column maxima of every tile, and of every second tile
@pytest.mark.parametrize("n,nq,k", [(1500, 64, 32), (6000, 129, 32), (20000, 200, 32), (140000, 256, 32),
                                    (40000, 130, 100)])
def test_tc_filter_path_equals_list_kernel(engine, orc, n, nq, k):
    x = datasets.clustered(n, D, 81, count=60)
    q = datasets.clustered(nq, D, 82, count=60)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    a, b = _query_both_paths(idx, q, k)
    # both select the exact top-CT by tensor-core score, so the outputs are identical
    assert np.array_equal(a["ID"], b["ID"])
    assert np.array_equal(a["distance"], b["distance"])
    sub = min(nq, 40)
    ids, _ = orc.exact_topk(x, q[:sub], k, dist=1)
    assert recall(a["ID"][:sub], ids) >= 0.99


def test_tc_overflow_duplicates(engine, orc):
    """5,000 copies of one point: a query at that point has 5,000 tied survivors, more than
    its candidate array holds, and goes through the on-device list-kernel fallback; the
    other queries of the same batch stay on the filter path."""
    n = 20000
    x = datasets.clustered(n, D, 91, count=40)
    x[1000:6000] = x[777]
    q = datasets.clustered(48, D, 92, count=40)
    q[5] = x[777]
    q[17] = x[777] * 3.0   # same direction
    q[30] = x[777] + 0.001 * q[30]
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    res = idx.query(q, 32)
    ids, ds = orc.exact_topk(x, q, 32, dist=1)
    for i in (5, 17):
        # ties broken by the lower id: the point itself, then the first copies
        assert res["ID"][i].tolist() == ids[i].tolist()
        assert np.array_equal(res["distance"][i], ds[i])
    assert recall(res["ID"], ids) >= 0.99
    a, b = _query_both_paths(idx, q, 32)
    assert np.array_equal(a["ID"], b["ID"]) and np.array_equal(a["distance"], b["distance"])


@pytest.mark.parametrize("n,nq,k,d", [(3000, 1, 1, 100), (3000, 5, 64, 37), (9000, 130, 65, 128), (20, 9, 32, 100),
                                      (70000, 200, 10, 64)])
def test_tc_edge_shapes(engine, orc, n, nq, k, d):
    """Odd and full-width dimensions (7 or 8 MMA K steps, or 3 for d = 37), a single
    query, k at the 64 / 128 candidate switch, a base smaller than k (missing results are
    (-1, 2^31) as in the reference) and a batch that is not a multiple of 128 rows."""
    x = datasets.clustered(n, d, 131, count=20)
    q = datasets.clustered(nq, d, 132, count=20)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    res = idx.query(q, k)
    kk = min(k, n)
    ids, ds = orc.exact_topk(x, q, kk, dist=1)
    assert recall(res["ID"][:, :kk], ids) >= 0.99
    if n < k:
        assert np.all(res["ID"][:, n:] == -1)
        assert np.all(res["distance"][:, n:] == np.float32(2.0 ** 31))
    a, b = _query_both_paths(idx, q, k)
    assert np.array_equal(a["ID"], b["ID"]) and np.array_equal(a["distance"], b["distance"])


# ---- E4M3 (FP8) tensor-core scores (implementation 9) ------------------------------------
# Tolerance stated: recall@k >= 0.99 against the exact FP32 scan (E4M3 keeps 3 mantissa
# bits, so more near-equal neighbours trade places at the candidate boundary than with
# BF16; 128 candidates are re-ranked a query at every k), and every returned distance
# equals the oracle's FP32 distance for that id bit for bit (the re-rank is the same FP32
# code).


@pytest.mark.parametrize("n,nq,k,d", [(1000, 200, 32, 100), (20000, 300, 32, 100), (6000, 129, 100, 100),
                                      (70000, 200, 10, 64), (3000, 5, 64, 37), (9000, 130, 32, 128)])
def test_tc_fp8_recall_and_exact_distances(engine, orc, n, nq, k, d):
    x = datasets.clustered(n, d, 161, count=40)
    q = datasets.clustered(nq, d, 162, count=40)
    idx = engine.Index(x, implementation=engine.IMPL_TC_FP8, distanceFunc=1)
    res = idx.query(q, k)
    kk = min(k, n)
    ids, ds = orc.exact_topk(x, q, kk, dist=1)
    rec = recall(res["ID"][:, :kk], ids)
    assert rec >= 0.99, f"E4M3 recall@{kk} = {rec:.4f}"
    lookup = [dict(zip(i.tolist(), dd.tolist())) for i, dd in zip(ids, ds)]
    for qi in range(nq):
        for rid, rd in zip(res["ID"][qi], res["distance"][qi]):
            if rid in lookup[qi]:
                assert np.float32(rd) == np.float32(lookup[qi][rid])
    for row in res:
        assert_order(row, strict=False, d=d)


def test_tc_fp8_overflow_and_persistence(engine, orc, tmp_path):
    """Tied duplicates send a query through the (BF16) list-kernel fallback while the rest
    of the batch stays on the E4M3 filter; a saved and reloaded E4M3 index answers the same."""
    n = 20000
    x = datasets.clustered(n, D, 171, count=40)
    x[1000:6000] = x[777]
    q = datasets.clustered(48, D, 172, count=40)
    q[5] = x[777]
    idx = engine.Index(x, implementation=engine.IMPL_TC_FP8, distanceFunc=1)
    res = idx.query(q, 32)
    ids, ds = orc.exact_topk(x, q, 32, dist=1)
    assert res["ID"][5].tolist() == ids[5].tolist()
    assert np.array_equal(res["distance"][5], ds[5])
    assert recall(res["ID"], ids) >= 0.99
    p = str(tmp_path / "fp8.idx")
    idx.save(p)
    again = engine.Index.load(p).query(q, 32)
    assert np.array_equal(again, res)


def near_tie_set(nq=16, close=24, ties=20, background=20000, seed=7):
    """Per query: `close` points well inside its top-k, then `ties` copies of one point at
    cosine distance ~0.2 whose coordinates differ by single-ulp nudges, so their exact
    distances differ by ~1e-9 -- below FP32 resolution at 0.2 (ulp 1.5e-8) -- and the
    k-th boundary falls among them; plus random background points far away."""
    g = np.random.default_rng(seed)
    q = g.standard_normal((nq, D))
    q /= np.linalg.norm(q, axis=1, keepdims=True)

    def toward(qv, cos):
        r = g.standard_normal(D)
        r -= r.dot(qv) * qv
        r /= np.linalg.norm(r)
        return cos * qv + np.sqrt(1 - cos * cos) * r

    rows = [g.standard_normal((background, D))]
    for qv in q:
        rows.append(np.array([toward(qv, 0.995 - 0.001 * c) for c in range(close)]))
        p0 = toward(qv, 0.8).astype(np.float32)
        tie = np.repeat(p0[None], ties, axis=0)
        for t in range(ties):
            for j in g.choice(D, 6, replace=False):
                tie[t, j] = np.nextafter(tie[t, j], np.float32(np.inf if g.random() < 0.5 else -np.inf))
        rows.append(tie)
    x = np.concatenate(rows).astype(np.float32)
    x = x[g.permutation(len(x))]
    return np.ascontiguousarray(x), q.astype(np.float32)


@pytest.mark.parametrize("impl", [8, 9])
def test_fp64_boundary_recheck_orders_near_ties(engine, orc, impl):
    """With the FP64 boundary re-check (default for implementations 8 and 9) the top-k ids
    and their order equal the FP64 oracle's on a set built so that FP32 and FP64 orders
    differ at the k-th place; without it (fp64_recheck = 0) they differ on most queries.
    Returned distances are the FP32 distances of the reference's formula, within the
    FP32 error bound (2d + 7) * 2^-24 of the FP64 distance."""
    k = 32
    x, q = near_tie_set()
    ids64, d64 = orc.fp64_topk(x, q, k)
    on = engine.Index(x, implementation=impl, distanceFunc=1).query(q, k)
    off = engine.Index(x, implementation=impl, distanceFunc=1,
                       options=engine.make_options(fp64_recheck=0)).query(q, k)
    assert np.array_equal(on["ID"], ids64)
    assert (~np.all(off["ID"] == ids64, axis=1)).sum() >= len(q) // 2  # the case this test is for
    ids32, ds32 = orc.exact_topk(x, q, 64, dist=1)
    bound = (2 * D + 7) * 2.0 ** -24
    for qi in range(len(q)):
        exact = dict(zip(ids32[qi].tolist(), ds32[qi].tolist()))
        for pid, dist, dd in zip(on["ID"][qi].tolist(), on["distance"][qi].tolist(), d64[qi]):
            assert np.float32(dist) == np.float32(exact[pid])
            assert abs(dist - dd) <= bound
