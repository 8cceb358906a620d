"""The N > 1 path on CPU: world_size-2 gloo process groups (no GPU).

Scenes are sharded across ranks without overlap, every scene is owned by exactly one
rank, and the timing reduction takes the slowest rank's time and the sum of the units.
"""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, queue):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import torch.distributed as dist
    import ethersph_gb300  # noqa: F401
    from ethersph_gb300 import distributed, scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        reqs = scenes.poisson_stream(rate=10.0, count=25, seed=3)
        mine = distributed.shard(reqs, rank, world)
        names = [r.seed for r in mine]
        units = float(sum(r.nsteps for r in mine))
        ms = 10.0 * (rank + 1)  # rank 1 is "slower"
        dist.barrier()
        t, u, rate = distributed.aggregate(ms, units)
        queue.put((rank, names, units, t, u, rate))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharding_and_timing():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    (_, n0, u0, t0, s0, r0), (_, n1, u1, t1, s1, r1) = out
    assert not set(n0) & set(n1)
    assert len(n0) + len(n1) == 25
    assert t0 == t1 == 20.0                        # slowest rank
    assert s0 == s1 == u0 + u1                     # all ranks' work
    assert r0 == pytest.approx((u0 + u1) / 0.020)


def test_shard_rejects_bad_rank():
    import ethersph_gb300  # noqa: F401
    from ethersph_gb300 import distributed
    assert distributed.shard(list(range(5)), 1, 2) == [1, 3]
    with pytest.raises(ValueError):
        distributed.shard([1], 2, 2)
