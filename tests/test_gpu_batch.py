"""Batched scenes and the serving loop on the GPU.

* a scene stepped inside a batch gives bitwise the same state as the same scene on a
  single-scene handle (its particles keep their relative (cell, id) order and every
  neighbour sum its order), in both forms;
* a scene's result is bitwise the same alone and in a mix with other scenes added and
  retired around it (the serving guarantee);
* a scene stops at its step budget (frozen, state kept) while others go on;
* capacities are enforced, retired scenes free their memory.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scenes_mod():
    from ethersph_gb300 import scenes
    return scenes


def batch_mod():
    from ethersph_gb300 import batch
    return batch


def single(pkg, scene, nsteps, precision, shape=None):
    with pkg.Simulation(scene.params(precision=precision), scene.n_fluid, scene.n_wall) as sim:
        for w in scene.walls:
            sim.upload_walls(w)
        sim.upload_fluid(scene.fluid)
        if shape:
            sim.set_launch_shape(*shape)
        sim.step(1, nsteps)
        return sim.download()


def make_batch(scene, precision, particles=200_000, cells=400_000, walls=60_000, slots=16):
    B = batch_mod().Batch
    return B(scene.params(precision=precision), particles, cells, walls, slots)


def equal(a, b):
    return all(np.array_equal(a[k], b[k]) for k in a)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_scene_equals_single_handle(pkg, precision):
    sc = scenes_mod()
    a = sc.dam_break_2d(dx=0.03)
    b = sc.dam_break_2d(dx=0.02, water_w=0.6, water_h=1.2, box_w=2.4, box_h=1.8)
    shape = (1, 1, 1, 128)
    ref_a = single(pkg, a, 40, precision, shape)
    ref_b = single(pkg, b, 40, precision, shape)
    with make_batch(a, precision) as bt:
        bt.set_launch_shape(*shape)
        ia = bt.add_scene(a, 1, 40)
        ib = bt.add_scene(b, 1, 40)
        bt.step(40)
        bt.synchronize()
        got_a, got_b = bt.download(ia), bt.download(ib)
    assert equal(got_a, ref_a) and equal(got_b, ref_b)


def test_alone_and_in_a_mix_are_identical(pkg):
    sc = scenes_mod()
    rng = np.random.default_rng(3)
    target = sc.random_dam_break_2d(rng, dx=0.02, total_step=60)
    others = [sc.random_dam_break_2d(rng, dx=0.02, total_step=60) for _ in range(4)]
    poise = sc.random_poiseuille_2d(rng, total_step=60)
    shape = (1, 1, 1, 128)
    with make_batch(target, 1) as bt:
        bt.set_launch_shape(*shape)
        t = bt.add_scene(target, 1, 60)
        bt.step(60)
        bt.synchronize()
        alone = bt.download(t)
    with make_batch(target, 1) as bt:
        bt.set_launch_shape(*shape)
        o0 = bt.add_scene(others[0], 1, 60)
        o1 = bt.add_scene(others[1], 1, 25)
        bt.step(10)
        t = bt.add_scene(target, 1, 60)        # arrives while others run
        p = bt.add_scene(poise, 1, 60)         # a periodic channel in the same launches
        bt.step(20)
        bt.retire(o0)                          # leaves mid-run
        o2 = bt.add_scene(others[2], 1, 60)
        bt.step(40)
        bt.synchronize()
        mixed = bt.download(t)
        assert bt.info(t)["finished"] and bt.info(o1)["finished"]
        assert not bt.info(o2)["finished"]
        _ = p
    assert equal(alone, mixed)


def test_budget_freezes_scene(pkg):
    sc = scenes_mod()
    a = sc.dam_break_2d(dx=0.03)
    b = sc.dam_break_2d(dx=0.025)
    ref = single(pkg, a, 7, 0)
    with make_batch(a, 0) as bt:
        ia = bt.add_scene(a, 1, 7)
        ib = bt.add_scene(b, 1, 20)
        bt.step(20)
        bt.synchronize()
        got = bt.download(ia)
        info = bt.info(ia)
        assert info["finished"] and info["steps_done"] == 7
        assert bt.info(ib)["steps_done"] == 20
    assert equal(got, ref)


def test_capacity_and_retire(pkg):
    from ethersph_gb300 import _abi
    sc = scenes_mod()
    a = sc.dam_break_2d(dx=0.03)
    with make_batch(a, 1, particles=a.n_fluid * 2 + 10, cells=200_000, walls=10_000, slots=4) as bt:
        ids = [bt.add_scene(a, 1, 10), bt.add_scene(a, 1, 10)]
        assert not bt.fits(a)
        with pytest.raises(_abi.SphError) as e:
            bt.add_scene(a, 1, 10)
        assert e.value.code == 3  # SPH_ERR_OOM
        free0 = bt.free()
        bt.retire(ids[0])
        assert bt.free()["particles"] == free0["particles"] + a.n_fluid
        assert bt.fits(a)
        k = bt.add_scene(a, 1, 10)
        bt.step(10)
        bt.synchronize()
        assert bt.info(k)["finished"] and bt.info(ids[1])["finished"]


def test_check_deletes_per_scene(pkg, orc):
    sc = scenes_mod()
    a = sc.dam_break_2d(dx=0.04)
    a.check = pkg.AABBCheck(hi=(4.0, 1.0))
    ref = single(pkg, a, 12, 0)
    assert len(ref["rho"]) < a.n_fluid
    b = sc.dam_break_2d(dx=0.03)
    with make_batch(a, 0) as bt:
        ib = bt.add_scene(b, 1, 12)
        ia = bt.add_scene(a, 1, 12)
        bt.step(12)
        bt.synchronize()
        assert equal(bt.download(ia), ref)
        assert bt.info(ib)["n_fluid"] == b.n_fluid


def test_serving_loop_runs_a_poisson_stream(pkg):
    from ethersph_gb300 import scenes, serve
    reqs = scenes.poisson_stream(rate=200.0, count=12, seed=1, steps=(50, 150))
    srv = serve.Server(budget_bytes=2e9, precision=1, keep_results=True)
    try:
        rep = srv.run(reqs)
    finally:
        srv.close()
    s = rep.summary()
    assert s["requests"] == len(reqs)
    assert s["latency_p99_s"] >= s["latency_p50_s"] > 0
    for c in rep.completed:
        assert np.all(np.isfinite(c.result["x"]))
    # every result equals the same request run alone (bit for bit: a scene's sums only
    # see its own particles and constants, whatever else shares the batch)
    assert len(rep.completed) == len(reqs)
    for c in rep.completed:
        scene = c.request.build()
        alone = serve_alone(pkg, scene, c.request.nsteps)
        assert equal(alone, c.result), c.request


def serve_alone(pkg, scene, nsteps):
    from ethersph_gb300 import batch, serve
    cells = batch.footprint(scene, 1)[1]
    with batch.Batch(scene.params(precision=1), scene.n_fluid + 10, cells + 16, scene.n_wall + 10, 2) as bt:
        bt.set_launch_shape(*serve.DEFAULT_LAUNCH_SHAPE)  # the server's shape
        sid = bt.add_scene(scene, 1, nsteps)
        steps = 0
        while steps < nsteps:  # the server steps whole bundles of 10; frozen scenes stay put
            bt.step(10)
            steps += 10
        bt.synchronize()
        return bt.download(sid)
