"""Many scenes in one set of kernel launches (the batch entry points of the C ABI).

A `Batch` holds independent scenes of one kind (dim, kernel, solve variant, form,
thermal flag) with any geometry and physical constants.  Each scene keeps its own step
counter and step budget; scenes are added and retired between steps, which is what the
serving loop (serve.py) builds on.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi

MAX_CELLS = 4096 * 1024 * 16      # what one three-level scan covers
MAX_PARTICLES = (2**31 - 1) // 8  # int32 indices with up to 8 lanes per particle


def merged_walls(scene):
    """The scene's wall groups as one set with a kind per particle."""
    if not scene.walls:
        d = scene.kernel.dim_
        z = np.zeros((0, d))
        return dict(x=z, normal=z, gap=np.zeros(0), t=np.zeros(0), kappa=np.zeros(0), v=z,
                    kind=np.zeros(0, dtype=np.int32))
    cat = lambda a: np.ascontiguousarray(np.concatenate(a))
    xs, ns, gs, ts, ks, vs, kinds = [], [], [], [], [], [], []
    for w in scene.walls:
        m = len(w)
        xs.append(w.x_vec_)
        ns.append(w.normal_vec_)
        gs.append(w.gap_)
        ts.append(getattr(w, "t_", np.zeros(m)))
        ks.append(getattr(w, "kappa_", np.zeros(m)))
        vs.append(getattr(w, "v_vec_", np.zeros((m, w.dim))))
        kinds.append(np.full(m, w.wall_kind, dtype=np.int32))
    return dict(x=cat(xs), normal=cat(ns), gap=cat(gs), t=cat(ts), kappa=cat(ks), v=cat(vs), kind=cat(kinds))


def cells_per_cutoff(cell_subdivision: int, precision: int, dim: int) -> int:
    """The library's cell subdivision (its default: 3 cells per r_cut)."""
    return cell_subdivision if cell_subdivision else 3


def grid_cells(scene, cell_subdivision: int = 0, precision: int = _abi.PRECISION_FP64) -> int:
    """Cells of the scene's grid as the library builds it (edge r_cut (1 + 1e-9) / m)."""
    m = cells_per_cutoff(cell_subdivision, precision, scene.kernel.dim_)
    edge = scene.kernel.influence_radius_ * (1.0 + 1e-9) / m
    n = 1
    for a in range(scene.kernel.dim_):
        L = scene.domain_hi[a] - scene.domain_lo[a]
        if a == 0 and scene.periodic_x:
            n *= int(math.floor(L / edge))
        else:
            n *= max(1, int(math.ceil(L / edge)))
    return n


def footprint(scene, precision: int = _abi.PRECISION_FP64) -> tuple[int, int, int]:
    """(particles, cells incl. the scene's sentinel cell, walls) the scene occupies."""
    return scene.n_fluid, grid_cells(scene, 0, precision) + 1, scene.n_wall


def bytes_per(dim: int, thermal: bool, precision: int) -> tuple[int, int, int]:
    """Device bytes per particle, per cell and per wall particle of a batch handle."""
    vec = 16 if dim == 2 else 32
    scal = 7 + (3 if thermal else 0)
    per_sorted = 2 * vec + 8 * scal + 8
    if precision == _abi.PRECISION_FP32_COMPENSATED:
        per_sorted += 3 * 16 + 4 + 4 + 8
    particle = 2 * per_sorted + 2 * vec + 8 + (8 if thermal else 0) + 12
    cell = 4 * 3 + 1
    wall = 3 * vec + 3 * 8 + 4 + (48 if precision == _abi.PRECISION_FP32_COMPENSATED else 0)
    return particle, cell, wall


class Batch:
    def __init__(self, prototype: _abi.SphParams, particle_capacity: int, cell_capacity: int, wall_capacity: int,
                 scene_capacity: int, lib=None):
        self.lib = lib or _abi.load_library()
        self.dim = prototype.dim
        self.thermal = bool(prototype.thermal)
        self.precision = prototype.precision
        h = C.c_void_p()
        _abi.check(self.lib, None, self.lib.sph_batch_create(C.byref(prototype), particle_capacity, cell_capacity,
                                                             wall_capacity, scene_capacity, C.byref(h)))
        self.h = h
        self.capacity = (particle_capacity, cell_capacity, wall_capacity, scene_capacity)

    @classmethod
    def for_budget(cls, prototype: _abi.SphParams, budget_bytes: int, scene_capacity: int = 4096,
                   cells_per_particle: float = 1.0, walls_per_particle: float = 0.5, lib=None):
        """Size a batch to a device memory budget."""
        bp, bc, bw = bytes_per(prototype.dim, bool(prototype.thermal), prototype.precision)
        unit = bp + cells_per_particle * bc + walls_per_particle * bw
        n = min(int(budget_bytes / unit), MAX_PARTICLES)
        cells = max(2, min(int(n * cells_per_particle), MAX_CELLS))
        return cls(prototype, n, cells, int(n * walls_per_particle), scene_capacity, lib=lib)

    def close(self):
        if self.h:
            self.lib.sph_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _abi.check(self.lib, self.h, rc)

    def add_scene(self, scene, first_step: int = 1, nsteps: int | None = None) -> int:
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        fl = scene.fluid
        prm = scene.params(precision=self.precision)
        nsteps = scene.td.total_step_ if nsteps is None else nsteps
        arrs = [f(fl.x_vec_), f(fl.v_vec_), f(fl.rho_), f(fl.p_), f(fl.c_), f(fl.mass_), f(fl.gap_)]
        arrs += [f(fl.t_), f(fl.kappa_), f(fl.cp_)] if self.thermal else [None, None, None]
        w = merged_walls(scene)
        wk = np.ascontiguousarray(w["kind"], dtype=np.int32)
        warrs = [f(w["x"]), f(w["normal"]), f(w["gap"]), f(w["t"]), f(w["kappa"]), f(w["v"])]
        sid = C.c_int32()
        self._check(self.lib.sph_batch_add_scene(
            self.h, C.byref(prm), first_step, nsteps, len(fl), *[_abi.dptr(a) for a in arrs], len(wk),
            wk.ctypes.data_as(C.POINTER(C.c_int32)), *[_abi.dptr(a) for a in warrs], C.byref(sid)))
        return sid.value

    def step(self, nsteps: int) -> None:
        self._check(self.lib.sph_batch_step(self.h, nsteps))

    def synchronize(self) -> None:
        self._check(self.lib.sph_synchronize(self.h))

    def info(self, sid: int) -> dict:
        out = (C.c_int64 * 4)()
        self._check(self.lib.sph_batch_scene_info(self.h, sid, out))
        return dict(n_fluid=out[0], steps_done=out[1], finished=bool(out[2]), next_step=out[3])

    def download(self, sid: int, capacity: int | None = None) -> dict:
        cap = capacity if capacity is not None else self.info(sid)["n_fluid"]
        d = self.dim
        out = {k: np.empty((cap, d)) for k in ("x", "v")}
        names = ["rho", "p", "c", "mass", "gap"] + (["t", "kappa", "cp"] if self.thermal else [])
        for k in names:
            out[k] = np.empty(cap)
        n = C.c_int64()
        ptr = lambda k: _abi.dptr(out[k]) if k in out else None
        self._check(self.lib.sph_batch_download_scene(self.h, sid, cap, C.byref(n), ptr("x"), ptr("v"), ptr("rho"),
                                                      ptr("p"), ptr("c"), ptr("mass"), ptr("gap"), ptr("t"),
                                                      ptr("kappa"), ptr("cp")))
        return {k: a[: n.value] for k, a in out.items()}

    def retire(self, sid: int) -> None:
        self._check(self.lib.sph_batch_retire(self.h, sid))

    def free(self) -> dict:
        out = (C.c_int64 * 4)()
        self._check(self.lib.sph_batch_free(self.h, out))
        return dict(particles=out[0], cells=out[1], walls=out[2], scenes=out[3])

    def fits(self, scene) -> bool:
        p, c, w = footprint(scene, self.precision)
        fr = self.free()
        return p <= fr["particles"] and c <= fr["cells"] and w <= fr["walls"] and fr["scenes"] >= 1

    def set_launch_shape(self, continuity: int, momentum: int, reinit: int, block: int) -> None:
        shape = (C.c_int32 * 4)(continuity, momentum, reinit, block)
        self._check(self.lib.sph_set_launch_shape(self.h, shape))

    def set_stencil_pruning(self, on: bool) -> None:
        """FP32 walks skip neighbour cells beyond r_cut (default: 3D on, 2D off); the
        results are bitwise the same either way."""
        self._check(self.lib.sph_set_stencil_pruning(self.h, 1 if on else 0))

    def autotune(self, reps: int = 3) -> tuple:
        out = (C.c_int32 * 4)()
        self._check(self.lib.sph_autotune(self.h, reps, out))
        return tuple(out)

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.sph_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def stats(self) -> _abi.SphStats:
        s = _abi.SphStats()
        self._check(self.lib.sph_stats(self.h, C.byref(s)))
        return s

    def time_stages(self, reps: int = 10) -> dict:
        ms = np.zeros(_abi.NUM_STAGES)
        self._check(self.lib.sph_time_stages(self.h, reps, _abi.dptr(ms)))
        return dict(zip(_abi.STAGE_NAMES, ms.tolist()))
