"""Partition-range sharding of a batched step across ranks.

The batched engine sends a binding row to partition top_bits(fmix32(join
key)); binding partition p only meets relation partition p, and every count
is a sum over partitions.  So N ranks can each evaluate a contiguous range of
partitions of the same step (QFG_OPT_SHARD_INDEX / QFG_OPT_SHARD_COUNT) and
one element-wise int64 sum of the 4 * n counters gives the full counts.  That
sum is the only exchange; nothing on the data path crosses ranks.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from . import _capi as C


def fmix32(x) -> np.ndarray:
    """MurmurHash3's 32-bit finalizer on uint32 (as the engine computes it)."""
    h = np.asarray(x).astype(np.int64).astype(np.uint32)
    with np.errstate(over="ignore"):
        h ^= h >> np.uint32(16)
        h *= np.uint32(0x85EBCA6B)
        h ^= h >> np.uint32(13)
        h *= np.uint32(0xC2B2AE35)
        h ^= h >> np.uint32(16)
    return h


def shard_range(bits: int, shard: int, count: int):
    """Partitions [lo, hi) owned by `shard` of `count` at `bits` partition bits."""
    return (shard << bits) // count, ((shard + 1) << bits) // count


def shard_mask(keys, bits: int, shard: int, count: int) -> np.ndarray:
    """Which binding rows (by join-key value) fall in the shard."""
    lo, hi = shard_range(bits, shard, count)
    p = fmix32(keys) >> np.uint32(32 - bits)
    return (p >= lo) & (p < hi)


def evaluate_sharded(engine, bindings, literals: Sequence, group=None,
                     device: Optional[str] = None) -> np.ndarray:
    """Evaluates this rank's shard of the step and sums the counts over the
    process group (torch.distributed).  Every rank holds the same binding set
    and relations; the result on every rank is the full [n, 4] counts."""
    import torch
    import torch.distributed as dist
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    engine.set_option(C.QFG_OPT_SHARD_COUNT, world)
    engine.set_option(C.QFG_OPT_SHARD_INDEX, rank)
    try:
        counts = engine.evaluate_step(bindings, literals)
    finally:
        engine.set_option(C.QFG_OPT_SHARD_INDEX, 0)
        engine.set_option(C.QFG_OPT_SHARD_COUNT, 1)
    t = torch.from_numpy(counts)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
