"""ctypes view of the C ABI declared in include/ethersph_gpu.h.

The shared library is built in-tree (``lib/libethersph_gpu.so``, see build.py).  There
is no CPU fallback: loading fails loudly when the library is missing or built for
another ABI version.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libethersph_gpu.so"
ABI_VERSION = 1

SPH_OK = 0
ERRORS = {
    1: "SPH_ERR_ARG", 2: "SPH_ERR_CUDA", 3: "SPH_ERR_OOM", 4: "SPH_ERR_NAN",
    5: "SPH_ERR_GRID_OVERFLOW", 6: "SPH_ERR_TIMEOUT", 7: "SPH_ERR_STATE", 8: "SPH_ERR_NO_DEVICE",
    9: "SPH_ERR_IO",
}
# probe field codes (SPH_PROBE_*), by particle field symbol and by VTP column name
PROBE_FIELDS = {"rho_": 0, "p_": 1, "c_": 2, "vx": 3, "vy": 4, "vz": 5, "t_": 6, "mass_": 7,
                "Density": 0, "Pressure": 1, "SoundSpeed": 2, "VelocityX": 3, "VelocityY": 4, "VelocityZ": 5,
                "Temperature": 6, "Mass": 7}
KERNELS = {"CubicSpline": 0, "Gaussian": 1, "WendlandC2": 2, "WendlandC4": 3}
SOLVE_FLUID_WALL = 0
SOLVE_FLUID_THERMOSTATIC_WALL = 1
SOLVE_FLUID_COMPULSIVE_THERMOSTATIC_WALL = 2
SOLVE_FLUID_VELOCITY_WALL = 3
SOLVE_FLUID_INLET_OUTLET_WALL = 4
WALL_COMPULSIVE = 0
WALL_STATIC_VELOCITY = 1
WALL_THERMOSTATIC = 2
PRECISION_FP64 = 0
PRECISION_FP32_COMPENSATED = 1
# momentum lanes codes SPH_LANES_LIST + t (t in 1, 2, 4, -1) read the neighbour list
LANES_LIST = 16
NUM_STAGES = 6
STAGE_NAMES = ["cell_count", "scan", "sort", "continuity", "momentum", "reinit"]


class SphParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("kernel", C.c_int32), ("solve", C.c_int32), ("precision", C.c_int32),
        ("influence_radius", C.c_double), ("h", C.c_double), ("sigma", C.c_double), ("kernel_0", C.c_double),
        ("rho_0", C.c_double), ("c_0", C.c_double), ("p_0", C.c_double),
        ("gamma", C.c_int32), ("thermal", C.c_int32),
        ("b", C.c_double), ("mu_0", C.c_double), ("nu_0", C.c_double), ("body_force", C.c_double * 3),
        ("t_0", C.c_double), ("kappa_0", C.c_double), ("cp", C.c_double), ("beta", C.c_double),
        ("dt", C.c_double), ("total_step", C.c_int64), ("output_interval", C.c_int64),
        ("check_interval", C.c_int64), ("density_reinitialized_interval", C.c_int64),
        ("check_enabled", C.c_int32), ("periodic_x", C.c_int32),
        ("check_lo", C.c_double * 3), ("check_hi", C.c_double * 3),
        ("domain_lo", C.c_double * 3), ("domain_hi", C.c_double * 3),
        ("nan_check", C.c_int32), ("cell_subdivision", C.c_int32),
    ]


class SphBufferRules(C.Structure):
    """SphBufferRules (include/ethersph_gpu.h): the plane tests of the inlet/outlet solve."""
    _fields_ = [("inlet_normal", C.c_double * 3), ("inlet_offset", C.c_double), ("inlet_shift", C.c_double * 3),
                ("outlet_normal", C.c_double * 3), ("outlet_offset", C.c_double),
                ("drop_normal", C.c_double * 3), ("drop_offset", C.c_double)]


class SphStats(C.Structure):
    _fields_ = [
        ("n_fluid", C.c_int64), ("n_wall", C.c_int64), ("steps_done", C.c_int64),
        ("total_mass", C.c_double), ("kinetic_energy", C.c_double), ("max_speed", C.c_double),
        ("status_flags", C.c_int32), ("reserved0", C.c_int32),
    ]


_DP = C.POINTER(C.c_double)
_H = C.c_void_p

# symbol -> (restype, argtypes); every entry point of include/ethersph_gpu.h
SIGNATURES = {
    "sph_version": (C.c_int32, []),
    "sph_create": (C.c_int32, [C.POINTER(SphParams), C.c_int64, C.c_int64, C.POINTER(C.c_void_p)]),
    "sph_upload_fluid": (C.c_int32, [_H, C.c_int64] + [_DP] * 10),
    "sph_upload_walls": (C.c_int32, [_H, C.c_int32, C.c_int64] + [_DP] * 6),
    "sph_step": (C.c_int32, [_H, C.c_int64, C.c_int64]),
    "sph_step_async": (C.c_int32, [_H, C.c_int64, C.c_int64]),
    "sph_synchronize": (C.c_int32, [_H]),
    "sph_download_fluid": (C.c_int32, [_H, C.c_int64, C.POINTER(C.c_int64)] + [_DP] * 10),
    "sph_download_ids": (C.c_int32, [_H, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "sph_stats": (C.c_int32, [_H, C.POINTER(SphStats)]),
    "sph_count_pairs": (C.c_int32, [_H, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "sph_download_cell_keys": (C.c_int32, [_H, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int32)]),
    "sph_download_neighbours": (C.c_int32, [_H, C.c_int64, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                            C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "sph_get_stream": (C.c_int32, [_H, C.POINTER(C.c_void_p)]),
    "sph_time_stages": (C.c_int32, [_H, C.c_int32, _DP]),
    "sph_output_open": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32, C.c_int32,
                                    C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_char_p]),
    "sph_scene_footprint": (C.c_int32, [C.POINTER(SphParams), C.c_int64, C.c_int64, C.POINTER(C.c_int64)]),
    "sph_upload_buffers": (C.c_int32, [C.c_void_p, C.POINTER(SphBufferRules), C.c_int64, C.c_int64] + [C.c_void_p] * 7
                           + [C.c_int64] + [C.c_void_p] * 7),
    "sph_set_buffer_velocity": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p]),
    "sph_download_buffers": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_int64)] + [C.c_void_p] * 7),
    "sph_probe": (C.c_int32, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_double,
                              C.c_void_p]),
    "sph_output_write": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double]),
    "sph_output_flush": (C.c_int32, [C.c_void_p]),
    "sph_count_pairs_noalloc": (C.c_int32, [C.POINTER(SphParams), C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                            C.c_void_p, C.c_void_p]),
    "sph_batch_create": (C.c_int32, [C.POINTER(SphParams), C.c_int64, C.c_int64, C.c_int64, C.c_int32,
                                     C.POINTER(C.c_void_p)]),
    "sph_batch_add_scene": (C.c_int32, [_H, C.POINTER(SphParams), C.c_int64, C.c_int64, C.c_int64] + [_DP] * 10 +
                            [C.c_int64, C.POINTER(C.c_int32)] + [_DP] * 6 + [C.POINTER(C.c_int32)]),
    "sph_batch_step": (C.c_int32, [_H, C.c_int64]),
    "sph_batch_scene_info": (C.c_int32, [_H, C.c_int32, C.POINTER(C.c_int64)]),
    "sph_batch_download_scene": (C.c_int32, [_H, C.c_int32, C.c_int64, C.POINTER(C.c_int64)] + [_DP] * 10),
    "sph_batch_retire": (C.c_int32, [_H, C.c_int32]),
    "sph_batch_free": (C.c_int32, [_H, C.POINTER(C.c_int64)]),
    "sph_autotune": (C.c_int32, [_H, C.c_int32, C.POINTER(C.c_int32)]),
    "sph_set_launch_shape": (C.c_int32, [_H, C.POINTER(C.c_int32)]),
    "sph_set_stencil_pruning": (C.c_int32, [_H, C.c_int32]),
    "sph_last_error": (C.c_char_p, [_H]),
    "sph_destroy": (C.c_int32, [_H]),
}

_lib = None


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with ethersphcpu.jl_gb300/build.py "
                          "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.sph_version() != ABI_VERSION:
        raise ImportError(f"{p}: ABI version {lib.sph_version()} != {ABI_VERSION}")
    if path is None:
        _lib = lib
    return lib


def check(lib: C.CDLL, handle, rc: int) -> None:
    if rc != SPH_OK:
        msg = lib.sph_last_error(handle)
        raise SphError(rc, msg.decode() if msg else "")


def dptr(a: np.ndarray | None):
    """Pointer to a C-contiguous float64 array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_DP)
