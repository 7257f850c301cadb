"""Row sharding of one fact table over ranks (one process per GPU).

The path shards by fact rows with no data-path exchange: rank r owns rows
[shard_range(total, world, r)) of the global table, runs the whole query on
its slice, and the per-rank group rows are summed by key afterwards -- the
host-side equivalent of concatenating the reference's per-bulk reduced runs
(core/pipeline.cu:360-472), which are summed per key here because the
partial sums of a key from different shards belong to one group.
"""
from __future__ import annotations

import numpy as np


def shard_range(total: int, world: int, rank: int) -> tuple[int, int]:
    """Rows [begin, end) of `rank` when `total` rows are split into `world`
    contiguous shards whose sizes differ by at most one row."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(total, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def merge_partial_groups(parts: list[tuple[np.ndarray, np.ndarray]]):
    """Sums per-shard (keys [g, k] int32, sums [g, m] int64) results by key;
    rows come back sorted by key, as one shard's result is."""
    parts = [(np.asarray(k, np.int32), np.asarray(s, np.int64)) for k, s in parts]
    parts = [(k, s) for k, s in parts if len(s)]
    if not parts:
        return np.zeros((0, 0), np.int32), np.zeros((0, 0), np.int64)
    keys = np.concatenate([k for k, _ in parts])
    sums = np.concatenate([s for _, s in parts])
    if keys.shape[1] == 0:  # scalar aggregate: one row
        return keys[:1], sums.sum(axis=0, keepdims=True, dtype=np.int64)
    uniq, inv = np.unique(keys, axis=0, return_inverse=True)
    out = np.zeros((len(uniq), sums.shape[1]), np.int64)
    np.add.at(out, inv.reshape(-1), sums)
    return uniq.astype(np.int32), out


def gather_and_merge(local: tuple[np.ndarray, np.ndarray], group=None):
    """All ranks contribute their shard's result; every rank gets the merged
    result (torch.distributed object all-gather: one small exchange after the
    scan, outside any timed region)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(local[0]), np.asarray(local[1])), group=group)
    return merge_partial_groups(parts)
