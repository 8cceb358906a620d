"""Physical validation on the GPU (both forms).

* Plane Poiseuille flow, periodic in x: the velocity profile against the transient
  analytic series (the series of PoiseuilleFlow2D.jl:28-35).  With the channel width
  taken between the walls' effective no-slip planes (half a spacing outside the outer
  fluid rows, H + dx) the L2 error is about 2%; against the nominal H about 12%.
* A settled column in a closed tank stays put (no particle escapes, small motion).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(pkg, scene, nsteps, precision):
    with pkg.Simulation(scene.params(precision=precision), scene.n_fluid, scene.n_wall) as sim:
        for w in scene.walls:
            sim.upload_walls(w)
        sim.upload_fluid(scene.fluid)
        sim.step(1, nsteps)
        return sim.download()


@pytest.mark.parametrize("precision", [0, 1])
def test_poiseuille_matches_the_analytic_profile(pkg, precision):
    from ethersph_gb300 import scenes
    s = scenes.poiseuille_periodic_2d(n_across=20, reynolds=0.5)
    m = s.meta
    steps = 3000
    r = run(pkg, s, steps, precision)
    t = steps * s.td.dt_
    y, ux = r["x"][:, 1], r["v"][:, 0]
    eff = scenes.poiseuille_ux_theory(y + m["dx"] / 2, t, m["H"] + m["dx"], m["nu"], m["f"])
    nom = scenes.poiseuille_ux_theory(y, t, m["H"], m["nu"], m["f"])
    err_eff = np.linalg.norm(ux - eff) / np.linalg.norm(eff)
    err_nom = np.linalg.norm(ux - nom) / np.linalg.norm(nom)
    print(f"poiseuille precision={precision}: L2 effective {err_eff:.4f}, nominal {err_nom:.4f}")
    assert err_eff < 0.04 and err_nom < 0.15
    assert np.abs(r["v"][:, 1]).max() < 1e-3 * m["umax"]  # no cross-channel flow
    assert len(r["rho"]) == s.n_fluid


def test_settled_column_stays_put(pkg):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_2d(dx=0.04, water_w=2.0, water_h=1.0, box_w=2.0, box_h=2.0)
    s.check = None
    a = run(pkg, s, 500, 0)
    b = run(pkg, s, 500, 1)
    for r in (a, b):
        assert len(r["rho"]) == s.n_fluid
        assert np.abs(r["x"] - s.fluid.x_vec_).max() < 1.0 * 0.04
        assert np.abs(r["v"]).max() < 0.3 * math.sqrt(2 * 9.81 * 1.0)
    assert np.max(np.abs(a["v"] - b["v"])) / np.max(np.abs(a["v"])) < 1e-4


def test_solve_writes_vtp_at_output_steps(pkg, tmp_path):
    from ethersph_gb300 import scenes, vtp
    s = scenes.dam_break_2d(dx=0.05, total_step=250)
    io = vtp.VTPIO(3, "collapse_dry_", ".vtp", str(tmp_path), [":rho_", ":p_", ":c_"],
                   ["Density", "Pressure", "SoundSpeed"])
    pkg.solve(s.fluid, s.walls[0], s.kernel, s.model, s.td, check=s.check, vtp_io=io,
              domain_lo=s.domain_lo, domain_hi=s.domain_hi)
    files = sorted(p.name for p in tmp_path.iterdir())
    assert files == ["collapse_dry_000.vtp", "collapse_dry_001.vtp", "collapse_dry_002.vtp"]
    last = vtp.read_vtp_arrays(str(tmp_path / "collapse_dry_002.vtp"))
    # step 200's fluid (deletions only shrink it) followed by the walls
    assert int(np.sum(last["Type"] == 1)) >= len(s.fluid)
    assert int(np.sum(last["Type"] == 2)) == s.n_wall
    assert last["Step"][0] == 2 and np.all(np.isfinite(last["Density"][last["Type"] == 1]))


def test_3d_dam_break_conserves_mass(pkg):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_3d(dx=0.03, tank=(0.9, 0.3, 0.6), column=(0.3, 0.3, 0.45))
    with pkg.Simulation(s.params(precision=1), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        m0 = sim.stats().total_mass
        sim.step(1, 400)
        st = sim.stats()
        masses = sim.download()["mass"]
    assert st.n_fluid == s.n_fluid
    # every particle keeps its mass exactly; the FP64 sum is taken in the current
    # (cell-sorted) order, so it may differ from the initial sum in the last bit
    assert np.array_equal(np.sort(masses), np.sort(s.fluid.mass_))
    assert st.total_mass == pytest.approx(m0, rel=1e-14)
    assert st.kinetic_energy > 0.0 and np.isfinite(st.max_speed)
