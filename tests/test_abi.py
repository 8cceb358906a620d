"""C ABI checks that need no GPU: the library loads, exports every entry point the
public header declares, and the ctypes structs match the C layout."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(sph_\w+)\s*\(", text, flags=re.M))
    return names


def test_header_declares_the_entry_points():
    names = declared_symbols()
    for required in ("sph_create", "sph_upload_fluid", "sph_upload_walls", "sph_step", "sph_download_fluid",
                     "sph_stats", "sph_last_error", "sph_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(pkg):
    from ethersph_gb300 import _abi
    lib = _abi.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert set(declared_symbols()) == set(_abi.SIGNATURES)
    assert lib.sph_version() == _abi.ABI_VERSION


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc needed to read the C layout")
def test_struct_layout_matches_c(tmp_path, pkg):
    from ethersph_gb300 import _abi
    fields = [f for f, _ in _abi.SphParams._fields_]
    sfields = [f for f, _ in _abi.SphStats._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{ROOT}/include/ethersph_gpu.h"',
           "int main(void) {", 'printf("%zu\\n", sizeof(SphParams));', 'printf("%zu\\n", sizeof(SphStats));']
    src += [f'printf("%zu\\n", offsetof(SphParams, {f}));' for f in fields]
    src += [f'printf("%zu\\n", offsetof(SphStats, {f}));' for f in sfields]
    src += ["return 0; }"]
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(c)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == C.sizeof(_abi.SphParams)
    assert out[1] == C.sizeof(_abi.SphStats)
    offs = out[2:]
    assert offs[: len(fields)] == [getattr(_abi.SphParams, f).offset for f in fields]
    assert offs[len(fields):] == [getattr(_abi.SphStats, f).offset for f in sfields]


def test_create_without_device_fails_cleanly(pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ethersph_gb300 import _abi, scenes
    s = scenes.dam_break_2d(dx=0.05)
    with pytest.raises(_abi.SphError) as e:
        pkg.Simulation(s.params(), s.n_fluid, s.n_wall)
    assert e.value.code == 8  # SPH_ERR_NO_DEVICE


def test_params_from_scene(pkg):
    from ethersph_gb300 import scenes
    s = scenes.natural_convection_2d(n=32)
    p = s.params()
    assert p.dim == 2 and p.kernel == 2 and p.solve == 2 and p.thermal == 1
    assert p.h == s.kernel.h_ and p.sigma == s.kernel.sigma_
    assert p.density_reinitialized_interval == 30
    assert p.check_enabled == 0


def test_vtp_writer_roundtrip(tmp_path, pkg):
    from ethersph_gb300 import scenes, vtp
    s = scenes.natural_convection_2d(n=16)
    io = vtp.VTPIO(4, "cavity_", ".vtp", str(tmp_path), [":rho_", ":p_", ":c_", ":t_"],
                   ["Density", "Pressure", "SoundSpeed", "Temperature"])
    path = io.write(3, 0.25, s.fluid, s.walls)
    assert path.endswith("cavity_0003.vtp")
    a = vtp.read_vtp_arrays(path)
    n = s.n_fluid + s.n_wall
    assert a["Points"].shape == (n, 3)
    assert np.array_equal(a["Points"][: s.n_fluid, :2], s.fluid.x_vec_)
    assert np.all(a["Type"][: s.n_fluid] == 1) and set(a["Type"][s.n_fluid:]) == {2, 3}
    assert np.array_equal(a["Temperature"][: s.n_fluid], s.fluid.t_)
    # walls have no density field and no velocity: NaN, as writeVTP writes them
    assert np.all(np.isnan(a["Density"][s.n_fluid:])) and np.all(np.isnan(a["Velocity"][s.n_fluid:]))
    assert a["Step"][0] == 3 and a["Time"][0] == 0.25
