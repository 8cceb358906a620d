"""The benchmark's workloads at their full sizes, on the GPU, checked through what does not
depend on size:

* the plain FP64 step against the oracle over the first steps (the oracle finishes a few
  steps of these scenes in seconds on the host cores);
* the neighbour pairs against the oracle's count, and exact mass;
* the FP32-compensated form, at the launch shape the autotuner picks on the scene (the
  neighbour list on these scenes), against the FP64 form within the form's bar;
* scenes of the 512-scene batch equal to the same scenes run alone, bit for bit.

Sizes: the 256 x 256 natural-convection cavity (65,536 fluid + 3,108 walls), the 3D dam
break at dx = 0.005 (3,456,000 fluid + 1,678,380 walls), 512 seeded dam breaks at
dx = 0.01 (8.75 M fluid).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if len(b) else 0.0


def scenes_mod():
    from ethersph_gb300 import scenes
    return scenes


def gpu(pkg, s, steps, precision, tune=False):
    with pkg.Simulation(s.params(precision=precision), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        shape = sim.autotune(2) if tune else None
        pairs = sim.count_pairs()
        if steps:
            sim.step(1, steps)
        out = sim.download()
        out["mass_total"] = sim.stats().total_mass
        return out, pairs, shape


def oracle(orc, s, steps):
    fluid, walls = orc.scene_arrays(s)
    return orc.run(s.params(), fluid, walls, 1, steps, mode=orc.GATHER, threads=0)


@pytest.fixture(scope="module")
def cavity():
    return scenes_mod().natural_convection_2d(n=256)


def test_cavity_256_fp64_matches_oracle(pkg, orc, cavity):
    got, _, _ = gpu(pkg, cavity, 3, 0)
    ref = oracle(orc, cavity, 3)
    for k in ("x", "v", "rho", "p", "c", "t"):
        assert rel(got[k], ref[k]) <= 1e-12, (k, rel(got[k], ref[k]))


def test_cavity_256_pairs_and_mass(pkg, orc, cavity):
    got, pairs, _ = gpu(pkg, cavity, 0, 0)
    fluid, walls = orc.scene_arrays(cavity)
    assert pairs == orc.neighbour_counts(cavity.params(), fluid["x"], walls["x"])
    assert got["mass_total"] == pytest.approx(float(np.sum(cavity.fluid.mass_)), rel=1e-15)


def test_cavity_256_fp32c_autotuned_follows_fp64(pkg, cavity):
    a, _, _ = gpu(pkg, cavity, 300, 0)
    b, _, shape = gpu(pkg, cavity, 300, 1, tune=True)
    print("autotuned shape", shape)
    for k in ("rho", "v", "t"):
        assert rel(b[k], a[k]) <= 1e-4, (k, rel(b[k], a[k]))
    assert np.array_equal(a["mass"], b["mass"])


def test_dam_break_3d_full_size(pkg, orc):
    s = scenes_mod().dam_break_3d(dx=0.005)
    assert s.n_fluid == 3_456_000
    got, pairs, _ = gpu(pkg, s, 1, 0)
    ref = oracle(orc, s, 1)
    for k in ("x", "v", "rho", "p", "c"):
        assert rel(got[k], ref[k]) <= 1e-12, (k, rel(got[k], ref[k]))
    fluid, walls = orc.scene_arrays(s)
    assert pairs == orc.neighbour_counts(s.params(), fluid["x"], walls["x"])
    a, _, _ = gpu(pkg, s, 20, 0)
    b, _, shape = gpu(pkg, s, 20, 1, tune=True)
    print("autotuned shape", shape)
    for k in ("rho", "v"):
        assert rel(b[k], a[k]) <= 1e-4, (k, rel(b[k], a[k]))
    assert b["mass_total"] == a["mass_total"]


def test_batched_512_scenes_equal_alone(pkg):
    from ethersph_gb300 import batch
    scenes = scenes_mod().batched_dam_breaks(512, seed=0)
    nf = sum(s.n_fluid for s in scenes)
    assert nf > 8_000_000
    nw = sum(s.n_wall for s in scenes)
    nc = sum(batch.footprint(s, 1)[1] for s in scenes)
    picks = [0, 200, 511]
    with batch.Batch(scenes[0].params(precision=1), nf + 1024, nc + 1024, nw + 1024, 512) as bt:
        ids = [bt.add_scene(s, 1, 10) for s in scenes]
        shape = bt.autotune(2)
        bt.step(10)
        bt.synchronize()
        got = {q: bt.download(ids[q]) for q in picks}
    for q in picks:
        s = scenes[q]
        with pkg.Simulation(s.params(precision=1), s.n_fluid, s.n_wall) as sim:
            for w in s.walls:
                sim.upload_walls(w)
            sim.upload_fluid(s.fluid)
            sim.set_launch_shape(*shape)
            sim.step(1, 10)
            alone = sim.download()
        for k in alone:
            assert np.array_equal(got[q][k], alone[k]), (q, k)
