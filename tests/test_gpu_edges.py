"""Edge cases of the step on the GPU: empty and single-particle scenes, a fluid the
check removes entirely, coincident particles, a grid too large to build, and a scene
without walls; each against the oracle where it has a state to compare."""
import dataclasses
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes():
    from ethersph_gb300 import scenes
    return scenes


def _subset(s, idx):
    f = s.fluid
    g = type(f)(len(idx), f.x_vec_.shape[1])
    for name in f._vector_fields + f._scalar_fields:
        getattr(g, name)[:] = getattr(f, name)[idx]
    return dataclasses.replace(s, fluid=g)


def _gpu(pkg, s, steps, precision=0):
    with pkg.Simulation(s.params(precision=precision), max(s.n_fluid, 1), s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        if steps:
            sim.step(1, steps)
        return sim.download(), sim.stats()


def _oracle(orc, s, steps):
    fluid, walls = orc.scene_arrays(s)
    return orc.run(s.params(), fluid, walls, 1, steps, mode=orc.GATHER, threads=4)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if len(b) else 0.0


@pytest.mark.parametrize("precision", [0, 1])
def test_empty_fluid_steps(pkg, precision):
    s = _subset(_scenes().dam_break_2d(dx=0.05), np.arange(0))
    got, st = _gpu(pkg, s, 40, precision)
    assert len(got["rho"]) == 0 and st.n_fluid == 0 and st.total_mass == 0.0


def test_single_particle_falls_freely(pkg, orc):
    # one particle far from every wall: no pair terms, v = g t and x from the
    # reference's update (UpdateVelocity.jl, UpdatePosition.jl), as the oracle has it
    s = _scenes().dam_break_2d(dx=0.05)
    x = s.fluid.x_vec_
    top = np.flatnonzero(x[:, 1] == x[:, 1].max())
    k = int(top[np.argmin(np.abs(x[top, 0] - 0.5))])  # top row, middle: no wall within r_cut
    one = _subset(s, np.array([k]))
    got, _ = _gpu(pkg, one, 30)
    ref = _oracle(orc, one, 30)
    for key in ("x", "v", "rho"):
        assert _rel(got[key], ref[key]) <= 1e-15, key
    assert got["v"][0, 1] == pytest.approx(-9.81 * 30 * s.td.dt_, rel=1e-12)


def test_check_removes_every_particle(pkg):
    s = _scenes().dam_break_2d(dx=0.05)
    s = dataclasses.replace(s, check=dataclasses.replace(s.check, hi=(-1.0, -1.0)))
    got, st = _gpu(pkg, s, 12)  # the check of step 5 deletes all; steps 6..12 run empty
    assert len(got["rho"]) == 0 and st.n_fluid == 0


def test_coincident_particles_stay_finite(pkg, orc):
    # two particles at one position: r = 0, the NaN guard of Neighbour.jl:78-84 zeroes grad W
    s = _scenes().dam_break_2d(dx=0.05)
    idx = np.arange(s.n_fluid)
    idx = np.concatenate([idx, idx[:1]])
    twin = _subset(s, idx)
    got, _ = _gpu(pkg, twin, 10)
    ref = _oracle(orc, twin, 10)
    assert np.all(np.isfinite(got["v"])) and np.all(np.isfinite(got["rho"]))
    for key in ("x", "v", "rho"):
        assert _rel(got[key], ref[key]) <= 1e-11, key


def test_scene_without_walls(pkg, orc):
    s = _scenes().dam_break_2d(dx=0.05)
    s = dataclasses.replace(s, walls=[type(s.walls[0])(0, 2)], check=None)
    got, _ = _gpu(pkg, s, 25)
    ref = _oracle(orc, s, 25)
    for key in ("x", "v", "rho"):
        assert _rel(got[key], ref[key]) <= 1e-10, key


def test_grid_too_large_is_refused(pkg):
    from ethersph_gb300 import _abi
    s = _scenes().dam_break_2d(dx=0.05)
    s = dataclasses.replace(s, domain_lo=(-1e3, -1e3), domain_hi=(1e3, 1e3))  # ~1e12 cells
    with pytest.raises(_abi.SphError) as e:
        pkg.Simulation(s.params(), s.n_fluid, s.n_wall)
    assert e.value.code in (1, 5)
    assert math.isfinite(s.kernel.influence_radius_)
