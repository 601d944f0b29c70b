"""Batch sharding across GPUs (one process per GPU): signals are independent, so a batch is split into
contiguous ranges of signals balanced by cumulative bytes, every rank builds its own plans (plans and
twiddle tables are replicated, never exchanged) and no collective touches the data path."""
import numpy as np


def shard_ranges(signal_bytes, world):
    """Contiguous [start, stop) signal ranges, one per rank, balanced by cumulative bytes: rank r takes the
    signals whose first byte falls in [r * total / world, (r + 1) * total / world).  Every rank's share is
    within one signal of total / world."""
    sizes = np.asarray(signal_bytes, dtype=np.int64)
    if world < 1:
        raise ValueError("world size must be at least 1")
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]) if len(sizes) else np.zeros(0, np.int64)
    total = int(sizes.sum())
    bounds = [int(np.searchsorted(starts, (total * r + world - 1) // world, side="left")) for r in range(world)]
    bounds.append(len(sizes))
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def shard_of(signal_bytes, world, rank):
    """This rank's [start, stop) range (see shard_ranges)."""
    return shard_ranges(signal_bytes, world)[rank]


def uniform_shard(batch, world, rank):
    """[start, stop) of `batch` equal signals for this rank."""
    return shard_of([1] * batch, world, rank)
