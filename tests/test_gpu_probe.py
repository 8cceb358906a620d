"""SPH interpolation at points on the device (sph_probe) against the oracle's
kernelValueInterpolation restatement, and as a validation tool (the Poiseuille profile
across the channel, probed on a line as the reference's post-processing does).

Bar: the oracle sums the same terms in upload order, the device in cell order, so the
two agree to FP64 rounding (relative 1e-12 of the field's magnitude).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(pkg, s, precision, steps):
    sim = pkg.Simulation(s.params(precision=precision), s.n_fluid, s.n_wall)
    for w in s.walls:
        sim.upload_walls(w)
    sim.upload_fluid(s.fluid)
    if steps:
        sim.step(1, steps)
    return sim


def _oracle_probe(orc, s, sim, pts, names):
    d = sim.download()
    fields = []
    for nm in names:
        fields.append({"Density": d["rho"], "Pressure": d["p"], "SoundSpeed": d["c"], "Mass": d["mass"],
                       "Temperature": d.get("t"), "VelocityX": d["v"][:, 0], "VelocityY": d["v"][:, 1],
                       "VelocityZ": d["v"][:, -1]}[nm])
    p = sim.params
    period = (p.domain_hi[0] - p.domain_lo[0]) if p.periodic_x else 0.0
    return orc.probe(p.kernel, p.dim, p.influence_radius, pts, d["x"], d["mass"], d["rho"], fields,
                     periodic_x=bool(p.periodic_x), period=period)


def _close(a, b, tol=1e-12):
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    scale = np.maximum(np.max(np.abs(b[fin]), axis=None), 1e-300)
    assert np.max(np.abs(a[fin] - b[fin])) / scale < tol


@pytest.mark.parametrize("precision", [0, 1])
def test_probe_matches_oracle_thermal_cavity(pkg, orc, precision):
    from ethersph_gb300 import scenes
    s = scenes.natural_convection_2d(n=48)
    names = ["Density", "VelocityX", "VelocityY", "Temperature", "Pressure", "Mass"]
    rng = np.random.default_rng(1)
    pts = np.concatenate([rng.uniform(-0.05, 1.05, (400, 2)), [[5.0, 5.0]]])  # last: far outside
    with _sim(pkg, s, precision, 60) as sim:
        got = sim.probe(pts, names)
        ref = _oracle_probe(orc, s, sim, pts, names)
    for k in range(len(names)):
        _close(got[k], ref[k])
    assert np.all(np.isnan(got[:, -1]))  # none_value: no particle in range


def test_probe_matches_oracle_3d_and_none_value(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4), column=(0.2, 0.2, 0.3))
    names = ["Density", "VelocityZ", "SoundSpeed"]
    rng = np.random.default_rng(2)
    pts = rng.uniform(-0.1, 0.7, (300, 3))
    with _sim(pkg, s, 1, 40) as sim:
        got = sim.probe(pts, names, none_value=-1.0)
        ref = _oracle_probe(orc, s, sim, pts, names)
    ref[np.isnan(ref)] = -1.0
    for k in range(len(names)):
        _close(got[k], ref[k])
    assert np.any(got[0] == -1.0) and np.any(got[0] > 0)


def test_probe_validates_poiseuille_profile(pkg, orc):
    # the reference checks its channel flow against the analytic series by interpolating
    # VelocityX on a line across the channel (PoiseuilleFlow2D.jl:28-35 + VTPToDataFrame)
    from ethersph_gb300 import kernelValueInterpolation, scenes
    s = scenes.poiseuille_periodic_2d(n_across=20, reynolds=0.5)
    m = s.meta
    steps = 3000
    with _sim(pkg, s, 1, steps) as sim:
        L = m["L"]
        ys = np.linspace(0.1 * m["H"], 0.9 * m["H"], 17)
        line = np.stack([np.full_like(ys, 0.37 * L), ys], axis=1)
        ux = kernelValueInterpolation(line, sim, "VelocityX")
        ref = _oracle_probe(orc, s, sim, line, ["VelocityX"])[0]
        # the same line through the periodic seam gives the same profile
        seam = sim.probe(np.stack([np.full_like(ys, 1e-9), ys], axis=1), ["vx"])[0]
    _close(ux, ref)
    t = steps * s.td.dt_
    eff = scenes.poiseuille_ux_theory(ys + m["dx"] / 2, t, m["H"] + m["dx"], m["nu"], m["f"])
    assert np.linalg.norm(ux - eff) / np.linalg.norm(eff) < 0.04
    assert np.linalg.norm(seam - ux) / np.linalg.norm(ux) < 0.02


def test_probe_errors(pkg):
    from ethersph_gb300 import _abi, scenes
    s = scenes.dam_break_2d(dx=0.1)
    with _sim(pkg, s, 0, 0) as sim:
        for bad in (["vz"], ["t_"]):
            with pytest.raises(_abi.SphError) as e:
                sim.probe([[0.5, 0.5]], bad)
            assert e.value.code == 1
        with pytest.raises(_abi.SphError):
            sim.probe([[0.5, 0.5]], [])
        assert sim.probe(np.zeros((0, 2)), ["rho_"]).shape == (1, 0)
        d = sim.probe([[0.5, 0.5]], ["rho_", "mass_"])
        assert math.isfinite(d[0, 0]) and d[1, 0] > 0
