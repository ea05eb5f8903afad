"""Serving loop and persistence on the GPU: every request's result is the same alone
and in the mix (continuous batching across streams, CUDA-graph replays), admission
refuses what cannot fit, and a saved index answers like the original."""
import os
import tempfile

import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100


@pytest.fixture(scope="module")
def indexes(engine):
    x = datasets.clustered(20000, D, 51, count=50)
    exact = engine.Index(x, implementation=2, distanceFunc=1)
    sim = engine.Index(x, implementation=3, sketchDim=16, options=engine.make_options(candidates=256))
    cp = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7, bucketKeyBits=16,
                      tables=8, options=engine.make_options(cp_hashes=2))
    tc = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    return x, {0: exact, 1: sim, 2: cp, 3: tc}


def test_same_alone_and_in_the_mix(engine, indexes):
    x, idx = indexes
    rng = np.random.default_rng(3)
    srv = engine.Server(max_batch=1024, streams=2, use_graphs=True)
    for i, ix in idx.items():
        srv.add_index(i, ix)
    reqs = []
    for t in range(60):
        which = int(rng.integers(0, len(idx)))
        nq = int(np.exp(rng.uniform(0, np.log(300))))
        k = int(rng.choice([10, 32, 100]))
        q = datasets.clustered(nq, D, 1000 + t, count=50)
        reqs.append((which, q, k, srv.submit(which, q, k)))
    lat = []
    for which, q, k, tk in reqs:
        out, l = srv.wait(tk)
        alone = idx[which].query(q, k)
        assert np.array_equal(out, alone), f"request on index {which} differs in the mix"
        lat.append(l)
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["launches"] <= len(reqs)
    assert st["graph_replays"] >= 1
    assert min(lat) > 0
    srv.close()


@pytest.mark.parametrize("which", [0, 2, 3])
def test_batching_window_coalesces_requests(engine, indexes, which):
    """A burst of 40 requests (k from {10, 32, 100}) submitted within the 50 ms batching
    window is answered in at most one launch a candidate class (exact scan and LSH: one;
    tensor-core scan: k <= 32 and k > 32, its FP64 re-check ordering the near-ties at every
    k of the launch) -- far fewer launches than requests -- and every request still equals
    its own query alone."""
    x, idx = indexes
    rng = np.random.default_rng(7)
    srv = engine.Server(max_batch=4096, streams=2, use_graphs=True, batch_window_us=50_000)
    srv.add_index(which, idx[which])
    reqs = []
    for t in range(40):
        nq = int(rng.integers(1, 40))
        k = int(rng.choice([10, 32, 100]))
        q = datasets.clustered(nq, D, 2000 + t, count=50)
        reqs.append((q, k))
    tickets = [srv.submit(which, q, k) for q, k in reqs]
    for (q, k), tk in zip(reqs, tickets):
        out, _ = srv.wait(tk)
        assert np.array_equal(out, idx[which].query(q, k))
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["launches"] <= (2 if which == 3 else 1) + 2  # a burst split by the window at most once more
    assert st["launches"] < len(reqs) // 4
    srv.close()


def test_tensor_core_launch_with_several_k(engine, indexes):
    """Requests of k = 10, 20, 32 and 5 on the tensor-core index coalesced into one launch
    (the FP64 re-check then orders the near-ties at each of those places in turn): every
    request equals its own query alone."""
    x, idx = indexes
    srv = engine.Server(max_batch=4096, streams=1, use_graphs=True, batch_window_us=50_000)
    srv.add_index(3, idx[3])
    reqs = [(datasets.clustered(64, D, 3000 + t, count=50), k) for t, k in enumerate((10, 20, 32, 5, 32, 10))]
    tickets = [srv.submit(3, q, k) for q, k in reqs]
    for (q, k), tk in zip(reqs, tickets):
        out, _ = srv.wait(tk)
        assert np.array_equal(out, idx[3].query(q, k)), k
    assert srv.stats()["launches"] <= 3
    srv.close()


def test_admission_by_free_hbm(engine, indexes):
    _, idx = indexes
    srv = engine.Server(hbm_reserve_mb=1 << 30)  # more than any GPU has: everything refused
    srv.add_index(0, idx[0])
    q = datasets.clustered(4, D, 9, count=50)
    with pytest.raises(engine.LshgError) as e:
        srv.submit(0, q, 32)
    assert e.value.status == 7
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_persistence_roundtrip(engine, indexes):
    x, idx = indexes
    q = datasets.clustered(40, D, 77, count=50)
    with tempfile.TemporaryDirectory() as td:
        for i, ix in idx.items():
            p = os.path.join(td, f"ix{i}.lshg")
            ix.save(p)
            re = engine.Index.load(p)
            assert np.array_equal(re.query(q, 32), ix.query(q, 32))
            with open(p, "r+b") as f:  # corrupt one byte: the checksum catches it
                f.seek(100)
                b = f.read(1)
                f.seek(100)
                f.write(bytes([b[0] ^ 0xFF]))
            with pytest.raises(engine.LshgError):
                engine.Index.load(p)


def _with_checksum(buf: bytearray) -> bytearray:
    """Recompute the file's trailing FNV-1a 64 checksum after an edit."""
    h = 1469598103934665603
    for c in bytes(buf[:-8]):
        h = ((h ^ c) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    buf[-8:] = h.to_bytes(8, "little")
    return buf


def test_load_rejects_inconsistent_files(engine):
    """A file whose checksum is valid but whose scalars disagree with its buffers (or
    that names an unknown implementation) is refused with LSHG_ERR_IO before any of it
    reaches the GPU; a truncated file is refused too; the intact file still loads."""
    import ctypes as C

    from lshongpu_gb300._lib import IndexParams

    x = datasets.clustered(300, 16, 5, count=10)
    q = datasets.clustered(8, 16, 6, count=10)
    ix = engine.Index(x, implementation=2, distanceFunc=1)
    off_params, off_n = 8, 8 + C.sizeof(IndexParams)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "ix.lshg")
        ix.save(p)
        good = bytearray(open(p, "rb").read())

        def n_plus_one(b):
            b[off_n:off_n + 8] = (301).to_bytes(8, "little")

        def unknown_impl(b):
            b[off_params:off_params + 4] = (7).to_bytes(4, "little")

        for edit in (n_plus_one, unknown_impl):
            b = bytearray(good)
            edit(b)
            with open(p, "wb") as f:
                f.write(_with_checksum(b))
            with pytest.raises(engine.LshgError) as e:
                engine.Index.load(p)
            assert e.value.status == 9
            assert "inconsistent" in str(e.value)
        with open(p, "wb") as f:
            f.write(good[: len(good) // 2])
        with pytest.raises(engine.LshgError) as e:
            engine.Index.load(p)
        assert e.value.status == 9
        with open(p, "wb") as f:
            f.write(good)
        assert np.array_equal(engine.Index.load(p).query(q, 32), ix.query(q, 32))


def test_cws_index_same_alone_and_in_the_mix(engine):
    """A consistent-weighted-sampling index (64 candidates, so k = 100 needs 128) behind the
    serving loop: requests of every k are coalesced only where the candidate count is the
    same, and each result equals the request alone."""
    x = datasets.sparse_gamma(20000, D, 71)
    cws = engine.Index(x, implementation=engine.IMPL_CWS, distanceFunc=2, sketchDim=64,
                       options=engine.make_options(candidates=64))
    rng = np.random.default_rng(11)
    srv = engine.Server(max_batch=1024, streams=2, use_graphs=True, batch_window_us=20_000)
    srv.add_index(0, cws)
    reqs = []
    for t in range(30):
        nq = int(np.exp(rng.uniform(0, np.log(200))))
        k = int(rng.choice([10, 32, 100]))
        q = datasets.sparse_gamma(nq, D, 3000 + t)
        reqs.append((q, k, srv.submit(0, q, k)))
    for q, k, tk in reqs:
        out, _ = srv.wait(tk)
        assert np.array_equal(out, cws.query(q, k))
    assert srv.stats()["completed"] == len(reqs)
    srv.close()
