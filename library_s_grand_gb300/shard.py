"""Shot sharding across ranks (one process per GPU).

Shots are independent, so a batch splits into contiguous shot ranges, one per
rank; every rank decodes its range on its own GPU with the codes resident there,
and the per-shot results are gathered where they are wanted.  The decode itself
needs no collective: the gather is the only exchange, and it moves 72-byte result
records, never syndromes.
"""
from __future__ import annotations

import numpy as np


def shard_range(num_shots: int, rank: int, world: int):
    """Contiguous [lo, hi) of the shots rank `rank` decodes; sizes differ by <= 1."""
    base, extra = divmod(num_shots, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def record_slice(rec_lens, shot_code, lo, hi):
    """Offsets [a, b) of shots lo..hi-1 in a concatenated record array."""
    if shot_code is None:
        return lo * rec_lens[0], hi * rec_lens[0]
    lens = np.asarray(rec_lens, dtype=np.int64)[np.asarray(shot_code)]
    starts = np.concatenate([[0], np.cumsum(lens)])
    return int(starts[lo]), int(starts[hi])


def decode_sharded(decode, records, rec_lens, num_shots, shot_code=None, group=None, dst=0):
    """Decode this rank's shard with decode(records_slice, shot_code_slice) ->
    structured result array, and gather all shards on rank `dst` in shot order
    (other ranks get None).  `group`: a torch.distributed process group (None:
    the default group)."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    lo, hi = shard_range(num_shots, rank, world)
    a, b = record_slice(rec_lens, shot_code, lo, hi)
    sc = None if shot_code is None else np.asarray(shot_code)[lo:hi]
    res = decode(np.asarray(records).ravel()[a:b], sc)
    parts = [None] * world if rank == dst else None
    dist.gather_object(res, parts, dst=dst, group=group)
    if rank != dst:
        return None
    return np.concatenate([p for p in parts if len(p)]) if parts else res
