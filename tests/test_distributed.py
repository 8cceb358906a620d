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


def _stream_scenes():
    # a small mixed stream the oracle steps in seconds: 2D dam breaks of different sizes,
    # a thermal cavity, a periodic channel, a 3D dam break
    from ethersph_gb300 import scenes
    return [scenes.dam_break_2d(dx=0.1), scenes.dam_break_2d(dx=0.08, water_w=0.6, water_h=1.2, box_w=2.4, box_h=1.8),
            scenes.natural_convection_2d(n=16), scenes.poiseuille_periodic_2d(n_across=8),
            scenes.dam_break_3d(dx=0.1, tank=(0.8, 0.4, 0.6), column=(0.3, 0.3, 0.4)),
            scenes.dam_break_2d(dx=0.12)]


def _step_scene(scene, steps=35):
    import oracle
    fluid, walls = oracle.scene_arrays(scene)
    return oracle.run(scene.params(), fluid, walls, 1, steps, mode=oracle.GATHER, threads=1)


def _stepping_worker(rank, world, port, queue):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root), str(root / "oracle")]
    import torch.distributed as dist
    import ethersph_gb300  # noqa: F401
    from ethersph_gb300 import distributed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        every = _stream_scenes()
        mine = distributed.shard(list(range(len(every))), rank, world)
        results = {k: _step_scene(every[k]) for k in mine}   # this rank's scenes only
        units = float(sum(len(r["rho"]) * 35 for r in results.values()))
        gathered = [None] * world
        dist.all_gather_object(gathered, results)
        _, total, _ = distributed.aggregate(1.0, units)
        if rank == 0:
            queue.put((gathered, total))
    finally:
        dist.destroy_process_group()


def test_two_ranks_step_their_shards_like_one_rank():
    # scene sharding is the whole multi-GPU design: two ranks stepping their shards of a
    # stream (here through the CPU restatement) give the same results, bit for bit, as one
    # rank stepping every scene, and the units add up over the ranks
    import sys
    from pathlib import Path
    import multiprocessing as mp
    import numpy as np
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_stepping_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered, total = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    merged = {}
    for part in gathered:
        assert not set(part) & set(merged)
        merged.update(part)
    every = _stream_scenes()
    assert sorted(merged) == list(range(len(every)))
    single = {k: _step_scene(s) for k, s in enumerate(every)}
    for k in single:
        for f in single[k]:
            assert np.array_equal(merged[k][f], single[k][f]), (k, f)
    assert total == float(sum(len(r["rho"]) * 35 for r in single.values()))
