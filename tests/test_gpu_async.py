"""The stream-ordered query entry point (lshg_index_query_async + lshg_index_sync): the
same results as the synchronous query, several batches in flight on one stream, and
device-side errors kept until the next synchronisation reports them."""
import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100


@pytest.mark.parametrize("impl", ["tc", "exact"])
def test_async_batches_match_sync_query(engine, impl):
    import torch

    x = datasets.clustered(30000, D, 141, count=40)
    qs = [datasets.clustered(257, D, 142 + i, count=40) for i in range(3)]
    code = engine.IMPL_TC if impl == "tc" else engine.IMPL_EXACT
    idx = engine.Index(x, implementation=code, distanceFunc=1)
    refs = [idx.query(q, 32) for q in qs]
    stream = torch.cuda.Stream()
    dqs = [torch.from_numpy(q).cuda() for q in qs]
    outs = [torch.full((q.shape[0], 32, 2), -7, dtype=torch.int32, device="cuda") for q in qs]
    torch.cuda.synchronize()
    for dq, out in zip(dqs, outs):  # three batches in flight, no host wait in between
        idx.query_device_async(dq.data_ptr(), dq.shape[0], 32, out.data_ptr(), stream=stream.cuda_stream)
    idx.sync(stream.cuda_stream)
    for dq, q, out, ref in zip(dqs, qs, outs, refs):
        got = out.cpu().numpy()
        assert np.array_equal(got[:, :, 0], ref["ID"])
        assert np.array_equal(got[:, :, 1].view(np.float32), ref["distance"])
        assert np.array_equal(dq.cpu().numpy(), q)  # the caller's queries are untouched


@pytest.mark.parametrize("impl", ["tc", "lsh"])
def test_async_host_buffers_two_streams(engine, impl):
    """Host (page-locked) buffers: upload, query and download enqueued per batch on two
    streams at once; every batch equals the synchronous query."""
    import torch

    x = datasets.clustered(30000, D, 143, count=40)
    qs = [datasets.clustered(300 + 17 * i, D, 144 + i, count=40) for i in range(4)]
    if impl == "tc":
        idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    else:
        idx = engine.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7, bucketKeyBits=16,
                           tables=8, options=engine.make_options(cp_hashes=2))
    refs = [idx.query(q, 16) for q in qs]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    hqs = [torch.from_numpy(q).pin_memory() for q in qs]
    outs = [torch.full((q.shape[0], 16, 2), -7, dtype=torch.int32).pin_memory() for q in qs]
    torch.cuda.synchronize()
    for i, (hq, out) in enumerate(zip(hqs, outs)):
        idx.query_host_async(hq.data_ptr(), hq.shape[0], 16, out.data_ptr(), stream=streams[i & 1].cuda_stream)
    for st in streams:
        idx.sync(st.cuda_stream)
    for hq, q, out, ref in zip(hqs, qs, outs, refs):
        got = out.numpy()
        assert np.array_equal(got[:, :, 0], ref["ID"])
        assert np.array_equal(got[:, :, 1].view(np.float32), ref["distance"])
        assert np.array_equal(hq.numpy(), q)


def test_async_device_error_reported_at_sync(engine):
    """A zero query row makes the weighted-MinHash sampler hit its draw limit on the
    device; the asynchronous call returns at once and the next sync reports it."""
    import torch

    x = datasets.sparse_gamma(2000, D, 151)
    q = datasets.sparse_gamma(8, D, 152)
    q[3] = 0.0
    idx = engine.Index(x, implementation=4, distanceFunc=2, sketchDim=64)
    dq = torch.from_numpy(q).cuda()
    out = torch.empty((8, 32, 2), dtype=torch.int32, device="cuda")
    idx.query_device_async(dq.data_ptr(), 8, 32, out.data_ptr())
    with pytest.raises(engine.LshgError) as e:
        idx.sync()
    assert e.value.status == 6  # LSHG_ERR_SAMPLER_LIMIT
    idx.sync()  # the error was reported once; the index stays usable
    assert idx.query(q[:3], 32).shape == (3, 32)


def test_device_error_reported_on_its_own_stream(engine):
    """Two streams with batches in flight on one index: only the stream whose batch holds
    a zero query row (the weighted-MinHash sampler hits its draw limit) reports
    LSHG_ERR_SAMPLER_LIMIT at its sync; the other stream's sync is clean and its results
    equal the synchronous query's."""
    import torch

    x = datasets.sparse_gamma(2000, D, 153)
    good = datasets.sparse_gamma(8, D, 154)
    bad = good.copy()
    bad[5] = 0.0
    idx = engine.Index(x, implementation=4, distanceFunc=2, sketchDim=64)
    ref = idx.query(good, 32)
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    dbad, dgood = torch.from_numpy(bad).cuda(), torch.from_numpy(good).cuda()
    oa = torch.empty((8, 32, 2), dtype=torch.int32, device="cuda")
    ob = torch.full((8, 32, 2), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    idx.query_device_async(dbad.data_ptr(), 8, 32, oa.data_ptr(), stream=sa.cuda_stream)
    idx.query_device_async(dgood.data_ptr(), 8, 32, ob.data_ptr(), stream=sb.cuda_stream)
    idx.sync(sb.cuda_stream)  # clean: stream A's error is not reported here
    with pytest.raises(engine.LshgError) as e:
        idx.sync(sa.cuda_stream)
    assert e.value.status == 6  # LSHG_ERR_SAMPLER_LIMIT
    idx.sync(sa.cuda_stream)  # reported once
    got = ob.cpu().numpy()
    assert np.array_equal(got[:, :, 0], ref["ID"])
    assert np.array_equal(got[:, :, 1].view(np.float32), ref["distance"])


def test_row_copy_wait_gives_up_with_timeout_status(engine, monkeypatch):
    """The re-rank's first row-copy wait is made to run out (test hook: it waits on a
    barrier nothing arrives on, for 1 ms): the kernel raises LSHG_ERR_TIMEOUT on the
    stream's error word, reads the rows directly instead, waits for its copy in flight
    before it exits, and the results equal the staged read's.  The index stays usable."""
    import torch

    x = datasets.clustered(20000, D, 161, count=40)
    q = datasets.clustered(200, D, 162, count=40)
    idx = engine.Index(x, implementation=engine.IMPL_TC, distanceFunc=1)
    ref = idx.query(q, 32)
    dq = torch.from_numpy(q).cuda()
    out = torch.full((200, 32, 2), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    monkeypatch.setenv("LSHG_TEST_ROW_WAIT_STALL", "1")
    idx.query_device_async(dq.data_ptr(), 200, 32, out.data_ptr())
    with pytest.raises(engine.LshgError) as e:
        idx.sync()
    assert e.value.status == 8  # LSHG_ERR_TIMEOUT
    monkeypatch.delenv("LSHG_TEST_ROW_WAIT_STALL")
    got = out.cpu().numpy()
    assert np.array_equal(got[:, :, 0], ref["ID"])
    assert np.array_equal(got[:, :, 1].view(np.float32), ref["distance"])
    idx.sync()  # reported once
    assert np.array_equal(idx.query(q, 32), ref)
