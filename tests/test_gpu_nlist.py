"""Neighbour list of the FP32-compensated form (momentum lanes SPH_LANES_LIST + t).

The continuity gather records each particle's neighbours within r_cut in its walk order
and the momentum gather reads that list instead of walking the cells again.  With one
lane per particle the list visits the same pairs in the same order as the cell walk; the
two kernels differ only where the compiler fuses a*b+c differently in the two inlined
copies of the pair terms, so the states agree to rounding (bitwise on most scenes), in
every solve variant; a particle whose list does not fit walks the cells; the other lane
counts reorder the compensated sums and stay within the FP32 form's tolerance.  The
stencil pruning of the walks (same code, a runtime switch) is bitwise neutral.
"""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIST = 16  # SPH_LANES_LIST (_abi.LANES_LIST)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if len(b) else 0.0


def scenes_mod():
    from ethersph_gb300 import scenes
    return scenes


def run(pkg, s, steps, shape, precision=1):
    with pkg.Simulation(s.params(precision=precision), s.n_fluid + 4000, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        if "rules" in s.meta:
            sim.upload_buffers(s.meta["rules"], s.meta["inlet"], s.meta["outlet"])
        if shape:
            sim.set_launch_shape(*shape)
        sim.step(1, steps)
        out = sim.download()
        out["id"] = sim.download_ids()
        return out


def make(name):
    sc = scenes_mod()
    return {"cavity": lambda: sc.natural_convection_2d(n=48),              # thermal terms
            "dam_break": lambda: sc.dam_break_2d(dx=0.03),                 # fluid + compulsive walls
            "lid": lambda: sc.lid_driven_cavity_2d(n=40),                  # wall pressure
            "periodic": lambda: sc.poiseuille_periodic_2d(n_across=16),    # rows that wrap
            "inlet_outlet": lambda: sc.poiseuille_inlet_outlet_2d(n_across=10, total_step=200),  # buffers
            "dam_break_3d": lambda: sc.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4), column=(0.2, 0.2, 0.3)),
            }[name]()


def same_pairs(a, b, tol=1e-6):
    # the same particles (ids), the same state to rounding
    assert np.array_equal(a["id"], b["id"])
    for k in ("x", "v", "rho", "p", "c"):
        assert rel(a[k], b[k]) <= tol, (k, rel(a[k], b[k]))
    assert np.array_equal(a["mass"], b["mass"])


@pytest.mark.parametrize("name", ["cavity", "dam_break", "lid", "periodic", "inlet_outlet", "dam_break_3d"])
def test_one_lane_list_follows_one_lane_walk(pkg, name):
    s = make(name)
    walk = run(pkg, s, 80, (1, 1, 1, 128))
    lst = run(pkg, s, 80, (1, LIST + 1, 1, 128))
    same_pairs(lst, walk)


@pytest.mark.parametrize("code", [LIST - 1, LIST + 1, LIST + 2, LIST + 4])
def test_list_lanes_follow_fp64(pkg, code):
    s = scenes_mod().natural_convection_2d(n=48)
    ref = run(pkg, s, 120, None, precision=0)
    got = run(pkg, s, 120, (-1 if code == LIST - 1 else 1, code, 1, 64))
    for k in ("rho", "v", "x", "t"):
        assert rel(got[k], ref[k]) <= 1e-4, (k, rel(got[k], ref[k]))


@pytest.mark.parametrize("name", ["cavity", "dam_break", "lid", "periodic", "inlet_outlet", "dam_break_3d"])
@pytest.mark.parametrize("code", [LIST - 1, LIST + 1, LIST + 2])
def test_two_lane_list_writer_reads_like_the_one_lane_list(pkg, name, code):
    # continuity on two lanes records each particle's list from both ends (lane 0 from the
    # first entry up, lane 1 from the last down); momentum reads the two segments as one
    # list: after one step density and position equal the one-lane list's to FP32
    # summation-order noise, in every solve variant (the first step's velocity is not
    # compared there: from rest it is a near-zero residual of large pressure terms, which
    # any change of summation order moves), and over a developed flow (200 steps; the
    # thermal cavity, which starts at rest, 1,000) the state stays within the form's bar
    # of the FP64 step
    s = make(name)
    one = run(pkg, s, 1, (1, code, 1, 64))
    two = run(pkg, s, 1, (2, code, 1, 64))
    assert np.array_equal(two["id"], one["id"])
    for k in ("rho", "x"):
        assert rel(two[k], one[k]) <= 1e-6, (name, code, k, rel(two[k], one[k]))
    steps = 1000 if name == "cavity" else 200
    ref = run(pkg, s, steps, None, precision=0)
    got = run(pkg, s, steps, (2, code, 1, 64))
    assert np.array_equal(got["id"], ref["id"])
    for k in ("rho", "v", "x"):
        assert rel(got[k], ref[k]) <= 1e-4, (name, code, k, rel(got[k], ref[k]))
    assert np.array_equal(got["mass"], ref["mass"])


def test_two_lane_lists_that_do_not_fit_walk_the_cells(pkg):
    # as below, with the two-lane writer: the two segments together overflow the row
    s = scenes_mod().dam_break_2d(dx=0.03)
    f = s.fluid
    f.gap_[:] = 2.0 * f.gap_
    s = dataclasses.replace(s, fluid=f)
    walk = run(pkg, s, 30, (2, 1, 1, 128))
    lst = run(pkg, s, 30, (2, LIST + 1, 1, 128))
    same_pairs(lst, walk)


def test_lists_that_do_not_fit_walk_the_cells(pkg):
    # the list depth follows the uploaded spacing: claiming twice the real spacing sizes
    # it for about a quarter of the real neighbours, so nearly every particle's list
    # overflows and momentum walks the cells for it; the state follows the walk's
    s = scenes_mod().dam_break_2d(dx=0.03)
    f = s.fluid
    f.gap_[:] = 2.0 * f.gap_
    s = dataclasses.replace(s, fluid=f)
    walk = run(pkg, s, 30, (1, 1, 1, 128))
    lst = run(pkg, s, 30, (1, LIST + 1, 1, 128))
    same_pairs(lst, walk)


def test_batch_with_list_equals_single_handles(pkg):
    from ethersph_gb300 import batch
    sc = scenes_mod()
    a = sc.dam_break_2d(dx=0.03)
    b = sc.dam_break_2d(dx=0.02, water_w=0.6, water_h=1.2, box_w=2.4, box_h=1.8)
    shape = (1, LIST + 1, 1, 128)
    ref_a, ref_b = run(pkg, a, 40, shape), run(pkg, b, 40, shape)
    with batch.Batch(a.params(precision=1), 200_000, 400_000, 60_000, 16) as bt:
        bt.set_launch_shape(*shape)
        ia = bt.add_scene(a, 1, 40)
        bt.step(10)
        ib = bt.add_scene(b, 1, 40)  # the list grows with the live particles
        bt.step(40)
        bt.synchronize()
        got_a, got_b = bt.download(ia), bt.download(ib)
    for k in got_a:
        assert np.array_equal(got_a[k], ref_a[k]), k
        assert np.array_equal(got_b[k], ref_b[k]), k


def test_list_shapes_are_checked(pkg):
    from ethersph_gb300 import _abi
    s = scenes_mod().dam_break_2d(dx=0.05)
    with pkg.Simulation(s.params(precision=1), s.n_fluid, s.n_wall) as sim:
        for bad in ((4, LIST + 1, 1, 128), (8, LIST + 2, 1, 128), (1, LIST + 3, 1, 128), (1, LIST + 8, 1, 128),
                    (1, LIST - 1, 1, 512)):
            with pytest.raises(_abi.SphError) as e:
                sim.set_launch_shape(*bad)
            assert e.value.code == 1, bad  # SPH_ERR_ARG
        sim.set_launch_shape(-1, LIST + 4, 2, 256)


def test_autotune_may_pick_the_list(pkg):
    s = scenes_mod().natural_convection_2d(n=64)
    with pkg.Simulation(s.params(precision=1), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        sim.step(1, 5)
        before = sim.download()
        shape = sim.autotune(2)
        after = sim.download()
        sim.step(6, 20)
    assert shape[1] in (-1, 1, 2, 4, 8, LIST - 1, LIST + 1, LIST + 2, LIST + 4)
    if shape[1] >= LIST - 1:
        assert shape[0] in (-1, 1)
    for k in before:
        assert np.array_equal(before[k], after[k]), k


def test_solve_with_autotune_follows_fp64(pkg):
    # solve(...; precision=FP32-compensated, autotune=True): the launch shape is picked
    # on the uploaded scene (cell walk or list) and the result stays within the form's bar
    sc = scenes_mod()
    a = sc.natural_convection_2d(n=64, total_step=200)
    b = sc.natural_convection_2d(n=64, total_step=200)
    pkg.solve(a.fluid, *a.walls, a.kernel, a.model, a.td, domain_lo=a.domain_lo, domain_hi=a.domain_hi)
    pkg.solve(b.fluid, *b.walls, b.kernel, b.model, b.td, domain_lo=b.domain_lo, domain_hi=b.domain_hi,
              precision=1, autotune=True)
    for k in ("rho_", "v_vec_", "x_vec_", "t_"):
        assert rel(getattr(b.fluid, k), getattr(a.fluid, k)) <= 1e-4, k


def run_pruning(pkg, s, steps, shape, on):
    with pkg.Simulation(s.params(precision=1), s.n_fluid + 4000, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        if "rules" in s.meta:
            sim.upload_buffers(s.meta["rules"], s.meta["inlet"], s.meta["outlet"])
        sim.set_stencil_pruning(on)
        sim.set_launch_shape(*shape)
        sim.step(1, steps)
        out = sim.download()
        out["id"] = sim.download_ids()
        return out


def clamped(name):
    # a domain that ends inside the fluid: particles above it sit in the grid's top cells
    # with their true positions (clamped keys), where the stencil pruning must keep them
    sc = scenes_mod()
    if name == "clamped_2d":
        s = sc.dam_break_2d(dx=0.03)
        return dataclasses.replace(s, domain_hi=(s.domain_hi[0], 1.2), check=None)
    s = sc.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4), column=(0.2, 0.2, 0.3))
    hi = list(s.domain_hi)
    hi[1] = 0.15
    return dataclasses.replace(s, domain_hi=tuple(hi), check=None)


@pytest.mark.parametrize("name", ["cavity", "dam_break", "lid", "periodic", "inlet_outlet", "dam_break_3d",
                                  "clamped_2d", "clamped_3d"])
def test_stencil_pruning_skips_only_rejected_candidates(pkg, name):
    # with one lane per particle the pruned walk visits the accepted neighbours in the same
    # order as the full stencil: the states are bitwise equal (cell walk, pipelined walk,
    # and the list the continuity walk records)
    s = clamped(name) if name.startswith("clamped") else make(name)
    for shape in ((1, 1, 1, 128), (-1, -1, -1, 128), (1, LIST + 1, 1, 128)):
        full = run_pruning(pkg, s, 40, shape, False)
        pruned = run_pruning(pkg, s, 40, shape, True)
        for k in full:
            assert np.array_equal(pruned[k], full[k]), (name, shape, k)
