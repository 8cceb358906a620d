"""GPU parity: the CUDA library (through its C ABI) against the CPU restatement.

The plain FP64 path sums each particle's neighbours in the same order as the
restatement's gather mode and uses the same IEEE operation sequence, so results
agree to the last few ulps (cos/exp are the only library functions that may round
differently).  Tolerances (L-inf, relative to each field's magnitude):
  1 step:    1e-13      100 steps: 1e-10
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_1 = 1e-13
TOL_100 = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def run_gpu(pkg, scene, first, nsteps, precision=0, sub=0):
    prm = scene.params(precision=precision, cell_subdivision=sub)
    with pkg.Simulation(prm, scene.n_fluid, scene.n_wall) as sim:
        for w in scene.walls:
            sim.upload_walls(w)
        sim.upload_fluid(scene.fluid)
        if nsteps:
            sim.step(first, nsteps)
        return sim.download()


def run_oracle(orc, scene, first, nsteps, threads=8, sub=0):
    fluid, walls = orc.scene_arrays(scene)
    return orc.run(scene.params(cell_subdivision=sub), fluid, walls, first, nsteps, mode=orc.GATHER,
                   threads=threads)


def compare(got, ref, tol, keys=("x", "v", "rho", "p", "c")):
    assert len(got["rho"]) == len(ref["rho"])
    errs = {k: rel(got[k], ref[k]) for k in keys if k in ref and k in got}
    bad = {k: e for k, e in errs.items() if not e <= tol}
    assert not bad, f"errors above {tol}: {bad}"
    return errs


def scenes_mod():
    from ethersph_gb300 import scenes
    return scenes


def test_upload_download_roundtrip(pkg):
    s = scenes_mod().dam_break_2d(dx=0.05)
    got = run_gpu(pkg, s, 1, 0)
    assert np.array_equal(got["x"], s.fluid.x_vec_)
    assert np.array_equal(got["v"], s.fluid.v_vec_)
    assert np.array_equal(got["rho"], s.fluid.rho_)
    assert np.array_equal(got["mass"], s.fluid.mass_)


def test_dam_break_one_step(pkg, orc):
    s = scenes_mod().dam_break_2d(dx=0.02)  # 5,000 fluid + 1,518 walls
    compare(run_gpu(pkg, s, 1, 1), run_oracle(orc, s, 1, 1), TOL_1)


@pytest.mark.parametrize("sub", [1, 2, 3])
def test_dam_break_100_steps(pkg, orc, sub):
    s = scenes_mod().dam_break_2d(dx=0.02)
    errs = compare(run_gpu(pkg, s, 1, 100, sub=sub), run_oracle(orc, s, 1, 100, sub=sub), TOL_100)
    print(f"dam break 100 steps (cell subdivision {sub}):", errs)


def test_3d_subdivisions_agree(pkg, orc):
    # the cell size changes only the neighbour order: the grids agree to rounding
    s = scenes_mod().dam_break_3d(dx=0.04, tank=(0.8, 0.4, 0.4), column=(0.24, 0.2, 0.4))
    a = run_gpu(pkg, s, 1, 20, sub=1)
    for sub in (2, 3):
        b = run_gpu(pkg, s, 1, 20, sub=sub)
        compare(a, b, 1e-11)
        compare(b, run_oracle(orc, s, 1, 20, sub=sub), 1e-11)


def test_thermal_cavity_100_steps(pkg, orc):
    s = scenes_mod().natural_convection_2d(n=64)
    errs = compare(run_gpu(pkg, s, 1, 100), run_oracle(orc, s, 1, 100), TOL_100,
                   keys=("x", "v", "rho", "p", "c", "t"))
    print("thermal cavity 100 steps:", errs)


@pytest.mark.parametrize("kernel", ["CubicSpline", "Gaussian", "WendlandC2", "WendlandC4"])
def test_every_kernel_2d(pkg, orc, kernel):
    s = scenes_mod().dam_break_2d(dx=0.04, kernel=kernel, gamma=7)
    compare(run_gpu(pkg, s, 1, 31), run_oracle(orc, s, 1, 31), 1e-11)


@pytest.mark.parametrize("kernel", ["CubicSpline", "WendlandC4"])
def test_dam_break_3d(pkg, orc, kernel):
    s = scenes_mod().dam_break_3d(dx=0.04, tank=(0.8, 0.4, 0.4), column=(0.24, 0.2, 0.4), kernel=kernel)
    compare(run_gpu(pkg, s, 1, 31), run_oracle(orc, s, 1, 31), 1e-11)


def test_thermostatic_only_solve(pkg, orc):
    sc = scenes_mod()
    s = sc.natural_convection_2d(n=32)
    s.walls = [s.walls[1]]  # thermostatic walls only: FluidThermostaticWallSolve
    s.solve = 1
    compare(run_gpu(pkg, s, 1, 31), run_oracle(orc, s, 1, 31), 1e-11, keys=("x", "v", "rho", "t"))


def test_velocity_wall_cavity(pkg, orc):
    s = scenes_mod().lid_driven_cavity_2d(n=40)
    errs = compare(run_gpu(pkg, s, 1, 60), run_oracle(orc, s, 1, 60), 1e-11)
    print("lid-driven cavity 60 steps:", errs)


def test_periodic_poiseuille(pkg, orc):
    s = scenes_mod().poiseuille_periodic_2d(n_across=20)
    got = run_gpu(pkg, s, 1, 60)
    ref = run_oracle(orc, s, 1, 60)
    compare(got, ref, 1e-11)
    L = s.meta["L"]
    assert got["x"][:, 0].min() >= 0.0 and got["x"][:, 0].max() < L


def test_check_deletes_like_the_reference(pkg, orc):
    s = scenes_mod().dam_break_2d(dx=0.04)
    s.check = pkg.AABBCheck(hi=(4.0, 1.0))  # removes the upper half of the column at step 5
    got = run_gpu(pkg, s, 1, 12)
    ref = run_oracle(orc, s, 1, 12)
    assert len(got["rho"]) < s.n_fluid
    compare(got, ref, 1e-12)


def test_deterministic_bitwise(pkg):
    s = scenes_mod().dam_break_2d(dx=0.02)
    a = run_gpu(pkg, s, 1, 40)
    b = run_gpu(pkg, s, 1, 40)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_split_runs_equal_one_run(pkg):
    # checkpoint/resume: 20 steps, download, re-upload, 20 more == 40 steps
    s = scenes_mod().dam_break_2d(dx=0.02)
    full = run_gpu(pkg, s, 1, 40)
    prm = s.params()
    with pkg.Simulation(prm, s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        sim.step(1, 20)
        mid = sim.download()
    s2 = scenes_mod().dam_break_2d(dx=0.02)
    f = s2.fluid
    f.x_vec_[:], f.v_vec_[:], f.rho_[:], f.p_[:], f.c_[:] = mid["x"], mid["v"], mid["rho"], mid["p"], mid["c"]
    resumed = run_gpu(pkg, s2, 21, 20)
    for k in ("x", "v", "rho", "p", "c"):
        assert np.array_equal(full[k], resumed[k]), k


def test_pair_counts_match_oracle(pkg, orc):
    s = scenes_mod().dam_break_2d(dx=0.02)
    prm = s.params()
    with pkg.Simulation(prm, s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        got = sim.count_pairs()
    assert got == orc.neighbour_counts(prm, s.fluid.x_vec_, s.walls[0].x_vec_)


def test_stats_mass_exact(pkg):
    s = scenes_mod().natural_convection_2d(n=64)
    with pkg.Simulation(s.params(), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        m0 = sim.stats().total_mass
        sim.step(1, 50)
        st = sim.stats()
    # masses never change; the FP64 sum follows the cell-sorted order (last-bit effects)
    assert st.total_mass == pytest.approx(m0, rel=1e-14)
    assert st.n_fluid == s.n_fluid
    assert st.steps_done == 50


def test_time_stages_leave_state_unchanged(pkg):
    s = scenes_mod().dam_break_2d(dx=0.02)
    with pkg.Simulation(s.params(), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        sim.step(1, 5)
        before = sim.download()
        ms = sim.time_stages(3)
        after = sim.download()
        sim.step(6, 5)
        cont = sim.download()
    assert all(v > 0 for v in ms.values())
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    ref = run_gpu(pkg, s, 1, 10)
    for k in ref:
        assert np.array_equal(ref[k], cont[k]), k


def test_errors_are_reported(pkg):
    from ethersph_gb300 import _abi
    s = scenes_mod().dam_break_2d(dx=0.05)
    with pkg.Simulation(s.params(), s.n_fluid, s.n_wall) as sim:
        with pytest.raises(_abi.SphError) as e:
            sim.step(1, 1)
        assert e.value.code == 7  # SPH_ERR_STATE
        f = s.fluid
        f.rho_[3] = np.nan
        sim.upload_fluid(f)
        with pytest.raises(_abi.SphError) as e:
            sim.step(1, 2)
        assert e.value.code == 4  # SPH_ERR_NAN
    with pkg.Simulation(s.params(precision=1), s.n_fluid, s.n_wall) as sim:
        for bad_shape in ((3, 1, 1, 128), (1, 1, 1, 48), (1, 1, 1, 2048), (1, -1, 1, 512)):
            with pytest.raises(_abi.SphError) as e:
                sim.set_launch_shape(*bad_shape)
            assert e.value.code == 1  # SPH_ERR_ARG
        sim.set_launch_shape(1, -1, 1, 256)
    with pytest.raises(_abi.SphError):
        pkg.Simulation(s.params(), 10, 0).upload_fluid(s.fluid)  # capacity overflow
    bad = s.params()
    bad.dim = 5
    with pytest.raises(_abi.SphError):
        pkg.Simulation(bad, 10, 10)


def test_solve_entry_point(pkg, orc):
    # solve(fluid, walls, kernel, model, td; check) — the reference call shape
    sc = scenes_mod()
    s = sc.dam_break_2d(dx=0.04, total_step=20)
    ref = run_oracle(orc, s, 1, 20)
    pkg.solve(s.fluid, s.walls[0], s.kernel, s.model, s.td, check=s.check, domain_lo=s.domain_lo,
              domain_hi=s.domain_hi)
    got = dict(x=s.fluid.x_vec_, v=s.fluid.v_vec_, rho=s.fluid.rho_)
    compare(got, ref, 1e-12, keys=("x", "v", "rho"))


def _slanted(p):
    # a check closure that is not a box (a slanted plane): the wedge right of it leaves
    return p.x_vec_[0] < 0.99 - 0.02 * p.x_vec_[1]


def test_solve_runs_a_check_closure_at_every_check_step(pkg, orc):
    # check(p) runs on the host at every check step (check_interval 5 < output_interval
    # 100), as FluidWallSolve.jl:73-81 runs it; the oracle is stepped the same way: to each
    # check step with the device box off, then the closure deletes with deleteat! order
    import dataclasses
    sc = scenes_mod()
    s = dataclasses.replace(sc.dam_break_2d(dx=0.04, total_step=60), check=None)
    assert s.td.check_interval_ == 5 and s.td.output_interval_ > s.td.check_interval_
    fluid, walls = orc.scene_arrays(s)
    prm = s.params()
    step, dropped = 1, 0
    while step <= 60:
        nxt = min(60, (step // 5 + 1) * 5 if step % 5 else step)
        fluid = orc.run(prm, fluid, walls, step, nxt - step + 1, mode=orc.GATHER, threads=8)
        step = nxt + 1
        if nxt % 5 == 0:
            keep = fluid["x"][:, 0] < 0.99 - 0.02 * fluid["x"][:, 1]
            dropped += int(np.count_nonzero(~keep))
            fluid = {k: np.ascontiguousarray(a[keep]) for k, a in fluid.items()}
    assert dropped > 0
    pkg.solve(s.fluid, s.walls[0], s.kernel, s.model, s.td, check=_slanted, domain_lo=s.domain_lo,
              domain_hi=s.domain_hi)
    got = dict(x=s.fluid.x_vec_, v=s.fluid.v_vec_, rho=s.fluid.rho_, p=s.fluid.p_)
    assert len(got["rho"]) == len(fluid["rho"])
    compare(got, fluid, 1e-12, keys=("x", "v", "rho", "p"))


def test_download_ids_name_the_survivors(pkg, orc):
    s = scenes_mod().dam_break_2d(dx=0.04)
    s.check = pkg.AABBCheck(hi=(4.0, 1.0))
    with pkg.Simulation(s.params(), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        sim.step(1, 12)
        ids = sim.download_ids()
        got = sim.download()
    assert len(ids) == len(got["rho"]) < s.n_fluid
    assert np.all(np.diff(ids) > 0)
    assert np.array_equal(got["mass"], s.fluid.mass_[ids])
