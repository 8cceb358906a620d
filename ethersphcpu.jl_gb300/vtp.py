"""VTP (VTK XML PolyData) output of particle groups, as writeVTP writes it.

Mirrors src/DataIO/VTPIO.jl:8-98: one file per output step named
dir_path/file_name<step padded to step_digit><file_suffix>, holding every particle group
as vertices with
  field data  Step (Int64), Time (Float64), WallTime ("yyyy/mm/dd__HH:MM:SS.SS",
              DataIO.jl:10; Julia's Dates prints the second for both "SS")
  point data  Velocity (NaN for particles without velocity: fixed walls),
              Type (1 for the first group, 2 for the second, ...),
              one Float64 array per (field_symbol, field_name) (NaN for groups without it).
Every array sits in the appended raw block with a UInt64 size header and an "offset"
attribute, the layout src/DataIO/VTPToDataFrame.jl:40-62 reads back.  The library's
own writer (sph_output_*, used by `solve`) writes the same bytes; this one serves the
host-side path and the tests.
"""
from __future__ import annotations

import datetime
import os
import re
from xml.sax.saxutils import unescape

import numpy as np

# fields of the reference's particle types that are not a scalar state (vectors and
# atomic accumulators): getParticleFields! cannot put them in a Float64 column
REJECTED = frozenset({"x_vec_", "v_vec_", "normal_vec_", "dv_vec_", "drho_", "sum_kernel_weight_",
                      "sum_weighted_scalar_", "sum_weighted_vector_", "dt_"})


def wall_time_now() -> str:
    d = datetime.datetime.now()
    return d.strftime("%Y/%m/%d__%H:%M:%S.") + f"{d.second:02d}"


def _esc(s: str) -> str:
    return s.replace("&", "&amp;").replace("<", "&lt;").replace(">", "&gt;").replace('"', "&quot;")


def _fd(t: str, name: str) -> str:
    return (f'      <DataArray type="{t}" Name="{name}" NumberOfComponents="1" NumberOfTuples="1" '
            f'format="appended" offset="')


def _pd(t: str, name: str, comps: int) -> str:
    return f'        <DataArray type="{t}" Name="{_esc(name)}" NumberOfComponents="{comps}" format="appended" offset="'


def write_vtp_file(path: str, step: int, t: float, points: np.ndarray, velocity: np.ndarray, types: np.ndarray,
                   columns: list, wall_time: str) -> None:
    """Write one file: points (n, 3), velocity (n, dim), types (n,) int64, columns
    [(name, (n,) float64)]."""
    n = len(types)
    dim = velocity.shape[1]
    close = '"/>\n'
    wt = wall_time.encode() + b"\0"
    arrs = [
        ('<?xml version="1.0"?>\n'
         '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
         "  <PolyData>\n    <FieldData>\n" + _fd("Int64", "Step"), close, np.int64(step).tobytes()),
        (_fd("Float64", "Time"), close, np.float64(t).tobytes()),
        (_fd("String", "WallTime"), close, wt),
        (f'    </FieldData>\n    <Piece NumberOfPoints="{n}" NumberOfVerts="{n}" NumberOfLines="0" '
         'NumberOfStrips="0" NumberOfPolys="0">\n      <PointData>\n' + _pd("Float64", "Velocity", dim), close,
         np.ascontiguousarray(velocity, dtype=np.float64).tobytes()),
        (_pd("Int64", "Type", 1), close, np.ascontiguousarray(types, dtype=np.int64).tobytes()),
    ]
    for name, col in columns:
        arrs.append((_pd("Float64", name, 1), close, np.ascontiguousarray(col, dtype=np.float64).tobytes()))
    arrs += [
        ("      </PointData>\n      <Points>\n" + _pd("Float64", "Points", 3), close + "      </Points>\n",
         np.ascontiguousarray(points, dtype=np.float64).tobytes()),
        ("      <Verts>\n" + _pd("Int64", "connectivity", 1), close, np.arange(n, dtype=np.int64).tobytes()),
        (_pd("Int64", "offsets", 1),
         close + '      </Verts>\n    </Piece>\n  </PolyData>\n  <AppendedData encoding="raw">\n_',
         np.arange(1, n + 1, dtype=np.int64).tobytes()),
    ]
    head, off = [], 0
    for h, tail, data in arrs:
        head.append(f"{h}{off}{tail}")
        off += 8 + len(data)
    with open(path, "wb") as f:
        f.write("".join(head).encode())
        for _, _, data in arrs:
            f.write(np.uint64(len(data)).tobytes())
            f.write(data)
        f.write(b"\n  </AppendedData>\n</VTKFile>\n")


class VTPIO:
    """VTPIO(step_digit, file_name, file_suffix, dir_path, field_symbols, field_names)
    (VTPIO.jl:8-15)."""

    def __init__(self, step_digit, file_name, file_suffix, dir_path, field_symbols, field_names):
        self.step_digit_ = int(step_digit)
        self.file_name_ = file_name
        self.file_suffix_ = file_suffix
        self.dir_path_ = dir_path
        self.field_symbols_ = [str(s).lstrip(":") for s in field_symbols]
        self.field_names_ = list(field_names)

    def file_at(self, step: int) -> str:  # vtpFileNameAtStep (VTPIO.jl:17-19)
        return os.path.join(self.dir_path_, f"{self.file_name_}{str(step).zfill(self.step_digit_)}{self.file_suffix_}")

    def assure_dir(self) -> None:  # assureDirPathExist (DataIO.jl:35-40)
        os.makedirs(self.dir_path_, exist_ok=True)

    def write(self, step: int, t: float, fluid, walls=(), wall_time: str | None = None) -> str:
        """writeVTP(step, t, vtp_io, [fluid, walls...]) (VTPIO.jl:41-98)."""
        self.assure_dir()
        for sym in self.field_symbols_:
            if sym in REJECTED:
                raise ValueError(f"field {sym} is not a scalar particle state")
        groups = [fluid] + list(walls)
        dim = fluid.x_vec_.shape[1]
        n = sum(len(g) for g in groups)
        pts = np.zeros((n, 3))
        vel = np.full((n, dim), np.nan)
        typ = np.zeros(n, dtype=np.int64)
        fields = np.full((len(self.field_symbols_), n), np.nan)
        o = 0
        for gi, g in enumerate(groups):
            m = len(g)
            pts[o:o + m, :dim] = g.x_vec_
            typ[o:o + m] = gi + 1
            if "v_vec_" in g._vector_fields:
                vel[o:o + m] = g.v_vec_
            for k, sym in enumerate(self.field_symbols_):
                if sym in g._scalar_fields:
                    fields[k, o:o + m] = getattr(g, sym)
            o += m
        path = self.file_at(step)
        write_vtp_file(path, step, t, pts, vel, typ, list(zip(self.field_names_, fields)),
                       wall_time if wall_time is not None else wall_time_now())
        return path


def read_vtp_arrays(path: str) -> dict:
    """Decode every array of a file in the appended raw layout (for tests and tools):
    name -> ndarray ((n, comps) for vectors); WallTime -> str."""
    raw = open(path, "rb").read()
    mark = raw.index(b'<AppendedData encoding="raw">')
    base = raw.index(b"_", mark) + 1
    head = raw[:mark].decode()
    out = {}
    types = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "Int32": np.int32}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)" NumberOfComponents="(\d+)"[^>]*?offset="(\d+)"/>',
                         head):
        t, nc, off = m.group(1), int(m.group(3)), int(m.group(4))
        name = unescape(m.group(2), {"&quot;": '"'})
        size = int(np.frombuffer(raw, dtype=np.uint64, count=1, offset=base + off)[0])
        data = raw[base + off + 8: base + off + 8 + size]
        if t == "String":
            out[name] = data.rstrip(b"\0").decode()
            continue
        a = np.frombuffer(data, dtype=types[t])
        out[name] = a.reshape(-1, nc) if nc > 1 else a
    return out
