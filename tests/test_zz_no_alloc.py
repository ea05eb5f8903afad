"""The allocation-free query entry point (lshg_index_query_noalloc) against the regular
one (lshg_index_query on device buffers).

It exists for callers that cannot allocate device memory while answering queries; its
temporaries live in one fixed 32 MiB device array.  Results must be identical to the
allocating path's (same kernels, bit-exact), on two calls in a row (the second call
reuses the array with the first call's leftovers in it).  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from lshongpu_gb300 import datasets

pytestmark = pytest.mark.gpu

D = 100


def test_noalloc_matches_allocating_entry_point(engine):
    import torch

    x = datasets.clustered(20000, D, 81, count=40)
    q1 = datasets.clustered(300, D, 82, count=40)
    q2 = datasets.clustered(300, D, 83, count=40)
    q3 = datasets.clustered(200, D, 84, count=40)
    q4 = datasets.clustered(48, D, 85, count=40)
    idx = engine.Index(x, implementation=engine.IMPL_EXACT, distanceFunc=engine.ANGULAR)
    lib = engine.lib()
    # k <= 128 runs the register-blocked scan; k = 256 and 1024 the general scan with
    # block top-C queues and a merge of the per-split lists
    for q, k in ((q1, 32), (q2, 100), (q3, 256), (q4, 1024)):
        dq = torch.from_numpy(q).cuda()
        ref = torch.empty((q.shape[0], k, 2), dtype=torch.int32, device="cuda")
        idx.query_device(dq.data_ptr(), q.shape[0], k, ref.data_ptr())
        torch.cuda.synchronize()
        for _ in range(2):  # two calls in a row on the shared array
            out = torch.full((q.shape[0], k, 2), -7, dtype=torch.int32, device="cuda")
            st = lib.lshg_index_query_noalloc(idx.handle, dq.data_ptr(), q.shape[0], k, out.data_ptr(), None)
            assert st == 0, lib.lshg_last_error()
            torch.cuda.synchronize()
            assert torch.equal(out, ref)


def test_noalloc_rejects_oversized_batches_and_other_indexes(engine):
    import torch

    x = datasets.clustered(5000, D, 84, count=20)
    idx = engine.Index(x, implementation=engine.IMPL_EXACT, distanceFunc=engine.ANGULAR)
    lib = engine.lib()
    nq, k = 20000, 1024  # needs far more than the fixed array holds
    dq = torch.zeros((nq, D), dtype=torch.float32, device="cuda")
    out = torch.empty((nq, k, 2), dtype=torch.int32, device="cuda")
    assert lib.lshg_index_query_noalloc(idx.handle, dq.data_ptr(), nq, k, out.data_ptr(), None) == 1
    assert b"temporaries" in lib.lshg_last_error()
    sim = engine.Index(x, implementation=engine.IMPL_SIMHASH, sketchDim=8)
    assert lib.lshg_index_query_noalloc(sim.handle, dq.data_ptr(), 4, 32, out.data_ptr(), None) == 5
