"""CPU checks of the consistent-weighted-sampling oracle (oracle.c, or_cws_*).

CWS has no reference counterpart, so the oracle is pinned to the mathematics it
restates: its logarithm against math.log, its draw table against the Gamma(2, 1) and
uniform laws, and its samples against the defining property of the sampler -- two
vectors' samples agree with probability equal to their generalized Jaccard similarity
sum(min) / sum(max), without bias, with the binomial spread of S independent samples.
"""
import math

import numpy as np
import pytest

from lshongpu_gb300 import datasets


def test_logf_accuracy(orc):
    rng = np.random.default_rng(0)
    xs = np.concatenate([
        rng.random(2000).astype(np.float32) * 10,
        np.float32(10.0) ** rng.uniform(-44, 38, 2000).astype(np.float32),   # subnormals to 1e38
        np.float32(2.0) ** np.arange(-149, 128, dtype=np.float32),            # powers of two
        np.nextafter(np.float32(2.0) ** np.arange(-120, 120, dtype=np.float32), np.float32(0)),
    ])
    xs = xs[(xs > 0) & np.isfinite(xs)]
    for x in xs:
        v, t = float(orc.cws_logf(x)), math.log(float(x))
        # 2 ulp of the result, or 2^-24 absolute near x = 1 where ln x is tiny
        assert abs(v - t) <= max(2.5e-7 * abs(t), 1.2e-7), (x, v, t)


def test_table_laws(orc):
    tab = orc.cws_tables(100, 256)
    r, inv, lnc, beta = tab[..., 0], tab[..., 1], tab[..., 2], tab[..., 3]
    assert np.all(r > 0) and np.all((beta >= 0) & (beta <= 1))
    assert np.array_equal(inv, (np.float32(1) / r).astype(np.float32))
    assert abs(r.mean() - 2.0) < 0.05 and abs(r.var() - 2.0) < 0.15     # Gamma(2, 1)
    assert abs(np.exp(lnc.astype(np.float64)).mean() - 2.0) < 0.05
    assert abs(beta.mean() - 0.5) < 0.01
    # a draw depends on (sample, dimension) only, not on the table's shape
    assert np.array_equal(orc.cws_tables(40, 64), tab[:40, :64])


def test_samples_estimate_generalized_jaccard(orc):
    S = 4096
    x = datasets.sparse_gamma(120, 100, 37)
    x = x / np.linalg.norm(x, axis=1, keepdims=True)
    sk = orc.cws_sketch(x.astype(np.float32), S)
    rng = np.random.default_rng(1)
    pairs = rng.integers(0, 120, (600, 2))
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    est = np.array([np.mean(np.all(sk[a] == sk[b], axis=1)) for a, b in pairs])
    J = np.array([np.minimum(x[a], x[b]).sum() / np.maximum(x[a], x[b]).sum() for a, b in pairs])
    sd = np.sqrt(J * (1 - J) / S)
    assert abs((est - J).mean()) < 0.002
    assert np.sqrt(((est - J) ** 2).mean()) < 1.3 * np.sqrt((sd ** 2).mean())


def test_samples_consistent(orc):
    """Equal vectors give equal samples; a vector with no positive entry gets (d, 0)."""
    x = datasets.sparse_gamma(4, 50, 5)
    x = (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32)
    x = np.concatenate([x, x[:1], np.zeros((1, 50), np.float32)])
    sk = orc.cws_sketch(x, 64)
    assert np.array_equal(sk[0], sk[4])
    assert np.all(sk[5, :, 0] == 50) and np.all(sk[5, :, 1] == 0)
    assert np.all((sk[:4, :, 0] >= 0) & (sk[:4, :, 0] < 50))
    for i in range(4):  # every sample picks a positive dimension
        assert np.all(x[i, sk[i, :, 0]] > 0)


@pytest.mark.parametrize("C", [32, 64])
def test_scan_orders_by_matches_then_id(orc, C):
    """The oracle's CWS scan keeps the top-C by (1 - matches / S, id): checked against a
    direct numpy restatement on a small case."""
    x = datasets.sparse_gamma(300, 20, 11)
    q = datasets.sparse_gamma(5, 20, 12)
    xn, qn = orc.normalize(x), orc.normalize(q)
    S = 32
    tab = orc.cws_tables(20, S)
    sx, sq = orc.cws_sketch(xn, S, tab), orc.cws_sketch(qn, S, tab)
    _, _, cand = orc.sketch_scan(xn, qn, 10, sx, sq, S, C, 2, 8, want_cand=True)
    for i in range(5):
        m = np.all(sx == sq[i][None], axis=2).sum(axis=1)
        dist = (np.float32(1) - (m.astype(np.float32) / np.float32(S))).astype(np.float32)
        order = np.lexsort((np.arange(300), dist))[:C]
        assert np.array_equal((cand[i] & 0xFFFFFFFF).astype(np.int64), order)
