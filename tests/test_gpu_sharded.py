"""The base split into shards -- one engine index each -- answered per shard and merged
(shard ids made global, lshg_merge_topk by (distance, id)) equals one index over the
whole base: bit-exactly for the exact scan, and at recall@32 >= 0.99 with exact FP32
distances for the tensor-core scan.  Two processes, one shard each, exchanging their
lists over a gloo process group (host-side only; no kernel waits on another) give the
same answer.  This is the engine's multi-GPU path, run here on one GPU."""
import os
import socket
import tempfile

import numpy as np
import pytest

from lshongpu_gb300 import datasets, sharded

pytestmark = pytest.mark.gpu

D = 100


def shard_answer(engine, x, q, k, shards, impl):
    parts = []
    for r in range(shards):
        lo, hi = sharded.shard_bounds(len(x), shards, r)
        ix = engine.Index(x[lo:hi], implementation=impl, distanceFunc=1)
        parts.append(sharded.globalize(ix.query(q, k), lo))
    return engine.merge_topk(np.stack(parts), k)


@pytest.mark.parametrize("shards", [2, 3])
def test_split_exact_index_merges_to_single_answer(engine, shards):
    x = datasets.clustered(30001, D, 171, count=40)
    q = datasets.clustered(100, D, 172, count=40)
    single = engine.Index(x, implementation=engine.IMPL_EXACT, distanceFunc=1).query(q, 32)
    assert np.array_equal(shard_answer(engine, x, q, 32, shards, engine.IMPL_EXACT), single)


def test_split_tensor_core_index_merges(engine, orc):
    x = datasets.clustered(40000, D, 173, count=40)
    q = datasets.clustered(200, D, 174, count=40)
    merged = shard_answer(engine, x, q, 32, 2, engine.IMPL_TC)
    ids, ds = orc.exact_topk(x, q, 32, dist=1)
    rec = np.mean([len(set(a.tolist()) & set(b.tolist())) / 32 for a, b in zip(merged["ID"], ids)])
    assert rec >= 0.99
    lookup = [dict(zip(i.tolist(), d.tolist())) for i, d in zip(ids, ds)]
    for row, ref in zip(merged, lookup):
        for pid, dist in zip(row["ID"].tolist(), row["distance"].tolist()):
            if pid in ref:
                assert np.float32(dist) == np.float32(ref[pid])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, x, q, k, out_path):
    import torch.distributed as dist

    import lshongpu_gb300 as L

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    lo, hi = sharded.shard_bounds(len(x), world, rank)
    ix = L.Index(x[lo:hi], implementation=L.IMPL_EXACT, distanceFunc=1)
    merged = sharded.merge_across_ranks(ix.query(q, k), lo, k)
    if rank == 0:
        np.save(out_path, merged)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gloo_with_engine_indexes(engine):
    import torch.multiprocessing as mp

    x = datasets.clustered(20001, D, 175, count=30)
    q = datasets.clustered(64, D, 176, count=30)
    single = engine.Index(x, implementation=engine.IMPL_EXACT, distanceFunc=1).query(q, 32)
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "merged.npy")
        mp.start_processes(_rank, args=(2, _free_port(), x, q, 32, out), nprocs=2, join=True, start_method="spawn")
        merged = np.load(out)
    assert np.array_equal(merged, single)
