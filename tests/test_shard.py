"""p-range sharding across ranks (CPU, gloo, world size 2): each rank sieves
its own window with the oracle, the windows tile the range exactly, and the
merged factor list equals the single-rank result."""
import os
import socket

import numpy as np
import pytest


def test_shard_windows_tile_the_range():
    import rsieve.shard as sh

    for p0, p1, world in [(3, 1000, 2), (10**9, 10**9 + 12345, 3), (10**13, 10**13 + 10**11 - 1, 8), (5, 5, 4)]:
        wins = [sh.shard_range(p0, p1, r, world) for r in range(world)]
        assert wins[0][0] == p0 and wins[-1][1] == p1
        for (a, b), (c, d) in zip(wins, wins[1:]):
            assert c == b + 1
        for a, b in wins[:-1]:
            if a <= b:
                assert (b + 1) % 2 == 0 or b + 1 == p1 + 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for p in (os.path.join(root, "cuda-riesel-sieve_gb300"), os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    import torch.distributed as dist

    import oracle
    import rsieve.shard as sh
    import rsieve.synth as S

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b, s, ks, nl = S.plain_job(3)
    job = oracle.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl])
    a, z = sh.shard_range(10**6, 10**6 + 400000, rank, world)
    f, _ = job.sieve(a, z, datless=True, threads=2)
    parts = [None] * world
    dist.all_gather_object(parts, [tuple(map(int, x)) for x in f])
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        q.put(parts)


def test_two_rank_shards_match_single_rank():
    pytest.importorskip("torch.distributed")
    import multiprocessing as mp

    import oracle
    import rsieve.shard as sh
    import rsieve.synth as S

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    dt = [("p", "<u8"), ("k", "<u4"), ("n", "<u4")]
    merged = sh.merge([np.array(x, dtype=dt) for x in parts])
    b, s, ks, nl = S.plain_job(3)
    job = oracle.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl])
    whole, _ = job.sieve(10**6, 10**6 + 400000, datless=True)
    assert len(whole) > 0
    assert [tuple(map(int, x)) for x in merged] == [tuple(map(int, x)) for x in whole]
