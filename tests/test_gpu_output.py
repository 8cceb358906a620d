"""Staged VTP output (sph_output_*) against the host-side writer.

`solve` with staged output takes device snapshots at output steps and writes the files
on a library thread while the next steps run; without it every output step downloads
the state and the Python writer (the same layout as writeVTP) writes the file.  Both
must give byte-identical files (WallTime fixed) and the same final state, including
after deletions, for every wall kind and both arithmetic forms.
"""
import dataclasses
import filecmp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WALL_TIME = "2026/12/03__10:20:30.30"


def _scene(name):
    from ethersph_gb300 import scenes
    if name == "dam_break":
        s = scenes.dam_break_2d(dx=0.05, total_step=240)
    elif name == "cavity":
        s = scenes.natural_convection_2d(n=32, total_step=120)
    elif name == "lid":
        s = scenes.lid_driven_cavity_2d(n=24, total_step=90)
    else:
        s = scenes.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4), column=(0.2, 0.2, 0.3), total_step=60)
    return s


FIELDS = {
    "dam_break": (["rho_", "p_", "c_"], ["Density", "Pressure", "SoundSpeed"]),
    "cavity": ([":rho_", ":p_", ":c_", ":t_", ":kappa_", ":cp_", ":mass_", ":gap_"],
               ["Density", "Pressure", "SoundSpeed", "Temperature", "Kappa", "Cp", "Mass", "Gap"]),
    "lid": (["rho_", "gap_", "t_"], ["Density", "Gap", "Temperature"]),
    "dam_break_3d": (["rho_", "p_", "c_"], ["Density", "Pressure", "SoundSpeed"]),
}


def _solve(pkg, name, outdir, staged, precision, interval):
    from ethersph_gb300 import vtp
    s = _scene(name)
    td = dataclasses.replace(s.td, output_interval_=interval)
    syms, names = FIELDS[name]
    io = vtp.VTPIO(4, name + "_", ".vtp", str(outdir), syms, names)
    fluid = pkg.solve(s.fluid, *s.walls, s.kernel, s.model, td, check=s.check, vtp_io=io, precision=precision,
                      domain_lo=s.domain_lo, domain_hi=s.domain_hi, periodic_x=s.periodic_x,
                      staged_output=staged, wall_time=WALL_TIME)
    return fluid


@pytest.mark.parametrize("name,precision,interval", [("dam_break", 0, 40), ("dam_break", 1, 7), ("cavity", 1, 30),
                                                     ("cavity", 0, 60), ("lid", 0, 15), ("dam_break_3d", 1, 20)])
def test_staged_files_equal_host_writer(pkg, tmp_path, name, precision, interval):
    a_dir, b_dir = tmp_path / "staged", tmp_path / "host"
    fa = _solve(pkg, name, a_dir, True, precision, interval)
    fb = _solve(pkg, name, b_dir, False, precision, interval)
    files = sorted(os.listdir(b_dir))
    assert sorted(os.listdir(a_dir)) == files
    assert len(files) >= 3
    for f in files:
        assert filecmp.cmp(a_dir / f, b_dir / f, shallow=False), f
    for k in ("x_vec_", "v_vec_", "rho_", "p_", "c_", "mass_"):
        assert np.array_equal(getattr(fa, k), getattr(fb, k)), k


def test_staged_output_after_deletions_matches_download(pkg, tmp_path):
    # dam break whose check deletes particles: the last file holds exactly the
    # downloaded survivors, in upload order, followed by the walls
    from ethersph_gb300 import scenes, vtp
    s = scenes.dam_break_2d(dx=0.05, total_step=200)
    # remove everything above 1.2 m at the first check step
    s = dataclasses.replace(s, check=dataclasses.replace(s.check, hi=(s.check.hi[0], 1.2)))
    n0 = s.n_fluid
    with pkg.Simulation(s.params(), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        io = vtp.VTPIO(2, "d_", ".vtp", str(tmp_path), ["rho_", "mass_"], ["Density", "Mass"])
        sim.output_open(io, WALL_TIME)
        sim.step(1, 200)
        sim.output_write(5, 0.125)
        sim.output_flush()
        got = sim.download()
        ids = sim.download_ids()
    assert len(ids) < n0
    a = vtp.read_vtp_arrays(str(tmp_path / "d_05.vtp"))
    nf = len(ids)
    assert np.array_equal(a["Points"][:nf, :2], got["x"]) and np.array_equal(a["Density"][:nf], got["rho"])
    assert np.array_equal(a["Mass"][:nf], s.fluid.mass_[ids])
    assert np.all(a["Type"][:nf] == 1) and np.all(a["Type"][nf:] == 2) and len(a["Type"]) == nf + s.n_wall
    assert a["Step"][0] == 5 and a["Time"][0] == 0.125 and a["WallTime"] == WALL_TIME


def test_output_errors(pkg, tmp_path):
    from ethersph_gb300 import scenes, vtp
    s = scenes.dam_break_2d(dx=0.1)
    with pkg.Simulation(s.params(), s.n_fluid, s.n_wall) as sim:
        for w in s.walls:
            sim.upload_walls(w)
        sim.upload_fluid(s.fluid)
        with pytest.raises(RuntimeError, match="SPH_ERR_STATE"):
            sim.output_write(0, 0.0)
        with pytest.raises(RuntimeError, match="SPH_ERR_ARG"):
            sim.output_open(vtp.VTPIO(1, "a", ".vtp", str(tmp_path), ["drho_"], ["X"]))
        blocker = tmp_path / "not_a_dir"
        blocker.write_text("x")
        with pytest.raises(RuntimeError, match="SPH_ERR_IO"):
            sim.output_open(vtp.VTPIO(1, "a", ".vtp", str(blocker), ["rho_"], ["Density"]))
        # a directory removed after opening: the write fails on the library thread and
        # the error comes back from the flush
        d = tmp_path / "gone"
        sim.output_open(vtp.VTPIO(1, "a", ".vtp", str(d), ["rho_"], ["Density"]))
        os.rmdir(d)
        sim.output_write(1, 0.0)
        with pytest.raises(RuntimeError, match="SPH_ERR_IO"):
            sim.output_flush()
        sim.output_flush()  # the error is reported once
