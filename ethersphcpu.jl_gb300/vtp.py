"""VTP (VTK XML PolyData) output of particle groups, as writeVTP writes it.

Mirrors src/DataIO/VTPIO.jl:8-98: one file per output step named
dir_path/file_name<step padded to step_digit><file_suffix>, holding every particle group
as vertices with
  field data  Step (integer), Time (float), WallTime (yyyy/mm/dd__HH:MM:SS.SS)
  point data  Velocity (NaN for particles without velocity: fixed walls),
              Type (1 for the first group, 2 for the second, ...),
              one array per (field_symbol, field_name) (NaN for groups without it).
Arrays are written inline as base64 binary (VTK "binary" format, UInt64 size header).
"""
from __future__ import annotations

import base64
import datetime
import os

import numpy as np

_VTK_TYPES = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32", np.dtype(np.int64): "Int64",
              np.dtype(np.int32): "Int32"}


def _b64(a: np.ndarray) -> str:
    raw = np.ascontiguousarray(a).tobytes()
    return base64.b64encode(np.uint64(len(raw)).tobytes() + raw).decode("ascii")


def _array(name: str, a: np.ndarray, ncomp: int = 1) -> str:
    t = _VTK_TYPES[a.dtype]
    return (f'<DataArray type="{t}" Name="{name}" NumberOfComponents="{ncomp}" format="binary">'
            f"{_b64(a)}</DataArray>\n")


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

    def write(self, step: int, t: float, fluid, walls=()) -> str:
        """writeVTP(step, t, vtp_io, [fluid, walls...]) (VTPIO.jl:41-98)."""
        self.assure_dir()
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
            if hasattr(g, "v_vec_"):
                vel[o:o + m] = g.v_vec_
            for k, sym in enumerate(self.field_symbols_):
                if hasattr(g, sym):
                    fields[k, o:o + m] = getattr(g, sym)
            o += m
        wall = datetime.datetime.now().strftime("%Y/%m/%d__%H:%M:%S.%f")[:-4]
        conn = np.arange(n, dtype=np.int64)
        offs = np.arange(1, n + 1, dtype=np.int64)
        body = ['<?xml version="1.0"?>\n',
                '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
                "<PolyData>\n<FieldData>\n",
                _array("Step", np.array([step], dtype=np.int64)),
                _array("Time", np.array([t], dtype=np.float64)),
                f'<DataArray type="String" Name="WallTime" NumberOfTuples="1" format="ascii">'
                f'{" ".join(str(b) for b in wall.encode())} 0</DataArray>\n',
                "</FieldData>\n",
                f'<Piece NumberOfPoints="{n}" NumberOfVerts="{n}" NumberOfLines="0" NumberOfStrips="0" '
                'NumberOfPolys="0">\n<PointData>\n',
                _array("Velocity", vel, dim),
                _array("Type", typ)]
        for k, name in enumerate(self.field_names_):
            body.append(_array(name, fields[k]))
        body += ["</PointData>\n<Points>\n", _array("Points", pts, 3), "</Points>\n<Verts>\n",
                 _array("connectivity", conn), _array("offsets", offs), "</Verts>\n</Piece>\n</PolyData>\n",
                 "</VTKFile>\n"]
        path = self.file_at(step)
        with open(path, "w") as f:
            f.write("".join(body))
        return path


def read_vtp_arrays(path: str) -> dict:
    """Decode the binary arrays of a file written by VTPIO.write (for tests and tools)."""
    import re
    text = open(path).read()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="(\w+)" NumberOfComponents="(\d+)" format="binary">'
                         r"([^<]*)</DataArray>", text):
        t, name, nc, data = m.group(1), m.group(2), int(m.group(3)), m.group(4)
        raw = base64.b64decode(data)
        dt = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "Int32": np.int32}[t]
        a = np.frombuffer(raw[8:], dtype=dt)
        out[name] = a.reshape(-1, nc) if nc > 1 else a
    return out
