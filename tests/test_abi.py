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


def test_python_constants_match_the_header():
    from ethersph_gb300 import _abi
    text = "".join(h.read_text() for h in HEADERS)
    defines = dict(re.findall(r"^#define\s+(SPH_\w+)\s+(-?\d+)\s*$", text, flags=re.M))
    assert int(defines["SPH_LANES_LIST"]) == _abi.LANES_LIST
    assert int(defines["SPH_NUM_STAGES"]) == _abi.NUM_STAGES


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
    assert a["WallTime"].count("__") == 1 and len(a["WallTime"]) == len("yyyy/mm/dd__HH:MM:SS.SS")


def test_vtp_layout_is_well_formed_xml(tmp_path, pkg):
    # the header parses as XML, every offset points at a UInt64 size header whose
    # payload ends where the next one starts, and the block ends the file
    import xml.etree.ElementTree as ET
    from ethersph_gb300 import scenes, vtp
    s = scenes.lid_driven_cavity_2d(n=12)
    io = vtp.VTPIO(2, "lid_", ".vtp", str(tmp_path), ["rho_", "gap_", "t_"], ["Density", "Gap", "T<&>"])
    path = io.write(7, 1.5, s.fluid, s.walls, wall_time="2026/01/02__03:04:05.05")
    raw = open(path, "rb").read()
    mark = raw.index(b'<AppendedData encoding="raw">')
    base = raw.index(b"_", mark) + 1
    root = ET.fromstring(raw[:mark] + b"</VTKFile>")
    arrays = root.iter("DataArray")
    offs = sorted(int(a.get("offset")) for a in arrays)
    pos = 0
    for o in offs:
        assert o == pos
        size = int(np.frombuffer(raw, dtype=np.uint64, count=1, offset=base + o)[0])
        pos = o + 8 + size
    assert raw[base + pos:] == b"\n  </AppendedData>\n</VTKFile>\n"
    a = vtp.read_vtp_arrays(path)
    nf, n = s.n_fluid, s.n_fluid + s.n_wall
    assert a["WallTime"] == "2026/01/02__03:04:05.05"
    # static-velocity walls carry their velocity; no group has t_ here; gap_ everywhere
    assert np.array_equal(a["Velocity"][nf:], s.walls[0].v_vec_)
    assert np.all(np.isnan(a["T<&>"])) and np.all(np.isfinite(a["Gap"]))
    assert np.array_equal(a["connectivity"], np.arange(n)) and np.array_equal(a["offsets"], np.arange(1, n + 1))


def test_vtp_rejects_non_scalar_fields(tmp_path, pkg):
    from ethersph_gb300 import scenes, vtp
    s = scenes.dam_break_2d(dx=0.1)
    for bad in ("x_vec_", ":drho_", "sum_kernel_weight_"):
        io = vtp.VTPIO(1, "d_", ".vtp", str(tmp_path), [bad], ["X"])
        with pytest.raises(ValueError):
            io.write(0, 0.0, s.fluid, s.walls)


def test_scene_footprint_matches_the_host_model(pkg):
    # the admission arithmetic of batch.footprint (Python) and sph_scene_footprint (the
    # library's own grid builder) agree; no device is needed
    import ctypes as C
    from ethersph_gb300 import _abi, batch, scenes
    lib = _abi.load_library()
    cases = [scenes.dam_break_2d(dx=0.05), scenes.natural_convection_2d(n=40),
             scenes.poiseuille_periodic_2d(n_across=16), scenes.lid_driven_cavity_2d(n=20),
             scenes.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4), column=(0.2, 0.2, 0.3))]
    for s in cases:
        for prec in (0, 1):
            out = (C.c_int64 * 3)()
            _abi.check(lib, None, lib.sph_scene_footprint(C.byref(s.params(precision=prec)), s.n_fluid, s.n_wall,
                                                          out))
            assert tuple(out) == batch.footprint(s, prec), (s.name, prec)
    bad = cases[0].params()
    bad.dim = 4
    assert lib.sph_scene_footprint(C.byref(bad), 1, 1, (C.c_int64 * 3)()) == 1


def test_julia_binding_names_declared_entry_points_and_fields():
    # the Julia binding is not run here (no Julia); check it against the header: every
    # symbol it ccalls is declared, and its SphParams mirror has the C fields in order
    jl = (ROOT / "ethersphcpu.jl_gb300" / "julia" / "EtherSPHGPU.jl").read_text()
    called = set(re.findall(r"ccall\(\(:(sph_\w+), libsph\)", jl))
    assert called and called <= declared_symbols(), called - declared_symbols()
    assert {"sph_output_open", "sph_output_write", "sph_probe", "sph_batch_add_scene",
            "sph_scene_footprint"} <= called
    hdr = (ROOT / "include" / "ethersph_gpu.h").read_text()
    for name in ("SphParams", "SphStats", "SphBufferRules"):  # mirrors: the C fields in order
        m = re.search(r"struct %s\n(.*?)\nend" % name, jl, flags=re.S)
        assert m, name
        jl_fields = re.findall(r"^\s*(\w+)::", m.group(1), flags=re.M)
        c_body = re.search(r"typedef struct %s \{(.*?)\}\s*%s;" % (name, name), hdr, flags=re.S).group(1)
        c_body = re.sub(r"/\*.*?\*/", "", c_body, flags=re.S)
        c_fields = re.findall(r"\b(\w+)(?:\[\d\])?\s*;", c_body)
        assert jl_fields == c_fields, name


def _c_prototypes():
    """name -> (return type, [parameter types]) of every entry point of the header."""
    hdr = (ROOT / "include" / "ethersph_gpu.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"([A-Za-z_][\w \*]*?)\s*\b(sph_\w+)\s*\(([^)]*)\)\s*;", hdr):
        ps = []
        for prm in params.split(","):
            prm = " ".join(prm.split())
            if prm in ("", "void"):
                continue
            ps.append(re.sub(r"\s*\b\w+$", "", prm))  # drop the parameter name
        protos[name] = (" ".join(ret.split()), ps)
    return protos


def _julia_types_for(ctype):
    c = ctype.replace("const", "").replace(" ", "")
    base = {"int32_t": {"Int32"}, "int64_t": {"Int64"}, "double": {"Float64"}, "char*": {"Cstring"},
            "char**": {"Ptr{Cstring}"}, "void*": {"Ptr{Cvoid}"}, "void**": {"Ref{Ptr{Cvoid}}", "Ptr{Ptr{Cvoid}}"},
            "SphHandle*": {"Ptr{Cvoid}"},
            "SphHandle**": {"Ref{Ptr{Cvoid}}", "Ptr{Ptr{Cvoid}}"}}
    if c in base:
        return base[c]
    m = re.fullmatch(r"(\w+)\*", c)
    jl = {"double": "Float64", "int64_t": "Int64", "int32_t": "Int32"}.get(m.group(1), m.group(1)) if m else None
    assert jl, ctype
    return {f"Ptr{{{jl}}}", f"Ref{{{jl}}}"}


def test_julia_ccall_types_match_the_header_prototypes():
    # every ccall of the Julia binding passes the argument and return types the header
    # declares (arity, widths, pointer element types), so the binding cannot drift from
    # the C ABI unnoticed while no Julia is available to run it
    jl = (ROOT / "ethersphcpu.jl_gb300" / "julia" / "EtherSPHGPU.jl").read_text()
    protos = _c_prototypes()
    calls = re.findall(r"ccall\(\(:(sph_\w+), libsph\),\s*(\w+),\s*\(([^()]*)\)", jl, flags=re.S)
    assert len(calls) >= 20
    for name, ret, types in calls:
        c_ret, c_params = protos[name]
        jl_types = [" ".join(x.split()) for x in types.split(",") if x.strip()]
        assert len(jl_types) == len(c_params), (name, jl_types, c_params)
        assert ret in _julia_types_for(c_ret), (name, ret, c_ret)
        for k, (a, c) in enumerate(zip(jl_types, c_params)):
            assert a in _julia_types_for(c), (name, k, a, c)
