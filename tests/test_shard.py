"""Batch sharding across ranks (no GPU): the ranges cover every signal once, balance bytes within one signal,
and a two-rank gloo run that transforms each rank's shard and gathers the results reproduces the unsharded
batch."""
import os
import socket

import numpy as np
import pytest

from kfr_gb300.shard import shard_ranges, uniform_shard
from kfr_gb300.workloads import uneven_lengths


def test_ranges_cover_and_balance():
    lengths = uneven_lengths(2000, seed=5)
    sizes = [16 * n for n in lengths]
    for world in (1, 2, 3, 4, 8):
        r = shard_ranges(sizes, world)
        assert r[0][0] == 0 and r[-1][1] == len(sizes)
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        shares = [sum(sizes[a:b]) for a, b in r]
        assert max(shares) - min(shares) <= 2 * max(sizes)
    assert [uniform_shard(10, 4, k) for k in range(4)] == [(0, 3), (3, 5), (5, 8), (8, 10)]
    assert shard_ranges([], 2) == [(0, 0), (0, 0)]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    from oracle.oracle import Oracle

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    lengths = uneven_lengths(120, hi=2048, seed=9)
    offs = np.concatenate([[0], np.cumsum(lengths)])
    rng = np.random.default_rng(1)
    x = rng.standard_normal(offs[-1]) + 1j * rng.standard_normal(offs[-1])
    a, b = shard_ranges([16 * n for n in lengths], world)[rank]
    orc = Oracle("orc")
    mine = {i: orc.dft(x[offs[i]:offs[i + 1]].reshape(1, -1))[0] for i in range(a, b)}
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        full = {}
        for g in gathered:
            assert not (set(g) & set(full))
            full.update(g)
        ok = sorted(full) == list(range(len(lengths)))
        for i in range(len(lengths)):
            ref = orc.dft(x[offs[i]:offs[i + 1]].reshape(1, -1))[0]
            ok = ok and np.allclose(full[i], ref)
        q.put(ok)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharded_batch():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=5) is True
