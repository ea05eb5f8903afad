"""Sharded k-NN across ranks: each rank owns a contiguous slice of the base (its own
resident Index on its GPU), answers the query batch locally, and one all-gather of the
per-rank top-k lists followed by lshg_merge_topk gives the global answer.

The reference is single-GPU (device 0 only, cudaHelpers.cu:16-18); this is the engine's
scale-out path.  It works with any torch.distributed backend (NCCL on GPUs, gloo for the
CPU tests); the exchange is the only collective on the data path.
"""
from __future__ import annotations

import numpy as np

from .api import POINT_DTYPE, merge_topk


def shard_bounds(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous, balanced slice [lo, hi) of n base points owned by `rank`."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def globalize(local: np.ndarray, id_offset: int) -> np.ndarray:
    """Local result ids -> global ids (empty entries stay -1)."""
    out = np.array(local, dtype=POINT_DTYPE, copy=True)
    ids = out["ID"]
    ids[ids >= 0] += id_offset
    return out


def merge_across_ranks(local: np.ndarray, id_offset: int, k: int, group=None) -> np.ndarray:
    """All-gather every rank's (N_query, k_local) top-k and merge into the global top-k."""
    import torch
    import torch.distributed as dist

    g = globalize(local, id_offset)
    world = dist.get_world_size(group)
    raw = torch.from_numpy(g.view(np.int32).copy())
    backend = dist.get_backend(group)
    if backend == "nccl":
        raw = raw.cuda()
    parts = [torch.empty_like(raw) for _ in range(world)]
    dist.all_gather(parts, raw, group=group)
    stacked = np.stack([p.cpu().numpy() for p in parts]).view(POINT_DTYPE)
    stacked = stacked.reshape(world, local.shape[0], local.shape[1])
    return merge_topk(stacked, k)
