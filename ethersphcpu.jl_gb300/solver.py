"""`solve` and the handle around the C ABI.

`solve` mirrors the `solve!` methods of EtherSPHCPU.jl (src/Solve/*.jl): the wall
argument types select the eachStep! variant exactly as Julia's dispatch does:

  solve(fluid, walls, kernel, model, td, ...)                 FluidWallSolve.jl:85-140
      walls: CompulsiveWallParticles (or any wall type)
  solve(fluid, thermostatic_walls, kernel, thermal_model, ...) FluidThermostaticWallSolve.jl:127-173
  solve(fluid, compulsive, thermostatic, kernel, thermal_model, ...)
                                                              FluidCompulsiveThermostaticWallSolve.jl:154-233
  solve(fluid, static_velocity_walls, kernel, model, ...)     FluidVelocitySolve.jl:104-168

The fluid container is updated in place (positions, velocities, density, pressure,
sound speed, temperature; particles removed by the check are dropped), like the Julia
vector after solve!.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from .types import (AABBCheck, CompulsiveWallParticles, StaticVelocityWallParticles, ThermostaticWallParticles,
                    isCheckStep, isOutputStep)


def make_params(kernel, model, td, *, solve: int, precision: int = _abi.PRECISION_FP64, check: AABBCheck | None = None,
                domain_lo=None, domain_hi=None, periodic_x: bool = False, nan_check: bool = True,
                cell_subdivision: int = 0) -> _abi.SphParams:
    """Fill the C parameter block from the Julia-mirror objects."""
    p = _abi.SphParams()
    p.dim = kernel.dim_
    p.kernel = kernel.kind.code
    p.solve = solve
    p.precision = precision
    p.influence_radius = kernel.influence_radius_
    p.h = kernel.h_
    p.sigma = kernel.sigma_
    p.kernel_0 = kernel.kernel_0_
    p.rho_0 = model.rho_0_
    p.c_0 = model.c_0_
    p.p_0 = model.p_0_
    p.gamma = model.gamma_
    p.thermal = 1 if model.thermal else 0
    p.b = model.b_
    p.mu_0 = model.mu_0_
    p.nu_0 = model.nu_0_
    for k in range(3):
        p.body_force[k] = float(model.body_force_vec_[k]) if k < len(model.body_force_vec_) else 0.0
    if model.thermal:
        p.t_0 = model.t_0_
        p.kappa_0 = model.kappa_0_
        p.cp = model.cp_
        p.beta = model.beta_
    p.dt = td.dt_
    p.total_step = td.total_step_
    p.output_interval = td.output_interval_
    p.check_interval = td.check_interval_
    p.density_reinitialized_interval = td.density_reinitialized_interval_
    p.check_enabled = 1 if check is not None else 0
    chk = check or AABBCheck()
    for k in range(3):
        p.check_lo[k] = chk.lo[k] if k < len(chk.lo) else -math.inf
        p.check_hi[k] = chk.hi[k] if k < len(chk.hi) else math.inf
    for k in range(3):
        p.domain_lo[k] = domain_lo[k] if domain_lo is not None and k < len(domain_lo) else 0.0
        p.domain_hi[k] = domain_hi[k] if domain_hi is not None and k < len(domain_hi) else 1.0
    p.periodic_x = 1 if periodic_x else 0
    p.nan_check = 1 if nan_check else 0
    p.cell_subdivision = cell_subdivision
    return p


class Simulation:
    """One device-resident scene behind an ``SphHandle``."""

    def __init__(self, params: _abi.SphParams, fluid_capacity: int, wall_capacity: int, lib=None):
        self.lib = lib or _abi.load_library()
        self.params = params
        self.dim = params.dim
        self.thermal = bool(params.thermal)
        h = C.c_void_p()
        _abi.check(self.lib, None, self.lib.sph_create(C.byref(params), fluid_capacity, max(wall_capacity, 0),
                                                       C.byref(h)))
        self.h = h
        self._fluid_capacity = fluid_capacity

    # -- lifetime
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

    # -- data
    def upload_fluid(self, fluid) -> None:
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        n = len(fluid)
        args = [f(fluid.x_vec_), f(fluid.v_vec_), f(fluid.rho_), f(fluid.p_), f(fluid.c_), f(fluid.mass_),
                f(fluid.gap_)]
        if self.thermal:
            args += [f(fluid.t_), f(fluid.kappa_), f(fluid.cp_)]
        else:
            args += [None, None, None]
        self._keep = args
        self._check(self.lib.sph_upload_fluid(self.h, n, *[_abi.dptr(a) for a in args]))

    def upload_walls(self, walls) -> None:
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        n = len(walls)
        kind = walls.wall_kind
        t = f(walls.t_) if kind == _abi.WALL_THERMOSTATIC else None
        kap = f(walls.kappa_) if kind == _abi.WALL_THERMOSTATIC else None
        v = f(walls.v_vec_) if kind == _abi.WALL_STATIC_VELOCITY else None
        self._check(self.lib.sph_upload_walls(self.h, kind, n, _abi.dptr(f(walls.x_vec_)),
                                              _abi.dptr(f(walls.normal_vec_)), _abi.dptr(f(walls.gap_)),
                                              _abi.dptr(t), _abi.dptr(kap), _abi.dptr(v)))

    # -- inlet/outlet buffers (SPH_SOLVE_FLUID_INLET_OUTLET_WALL)
    def upload_buffers(self, rules, inlet, outlet, capacity: int | None = None) -> None:
        """Inlet and outlet particles (CommonLiquidParticles) and the transfer rules
        (InletOutletRules); capacity: room for all buffer particles (default: inlet +
        outlet + as many as the fluid)."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        cap = capacity if capacity is not None else len(inlet) + len(outlet) + self._fluid_capacity
        arrays = lambda g: [_abi.dptr(f(getattr(g, k))) for k in ("x_vec_", "v_vec_", "rho_", "p_", "c_", "mass_",
                                                                   "gap_")]
        r = rules.c_struct()
        self._keep = (inlet, outlet)
        self._check(self.lib.sph_upload_buffers(self.h, C.byref(r), cap, len(inlet), *arrays(inlet), len(outlet),
                                                *arrays(outlet)))

    def download_buffers(self, which: int) -> dict:
        """Inlet (0) or outlet (1) particles in the reference's vector order."""
        n = C.c_int64()
        self.lib.sph_download_buffers(self.h, which, 0, C.byref(n), *([None] * 7))  # the count
        out = {k: np.empty((n.value, self.dim)) for k in ("x", "v")}
        for k in ("rho", "p", "c", "mass", "gap"):
            out[k] = np.empty(n.value)
        names = ("x", "v", "rho", "p", "c", "mass", "gap")
        self._check(self.lib.sph_download_buffers(self.h, which, n.value, C.byref(n),
                                                  *[_abi.dptr(out[k]) for k in names]))
        return out

    def set_buffer_velocity(self, which: int, v) -> None:
        vv = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, self.dim)
        self._check(self.lib.sph_set_buffer_velocity(self.h, which, len(vv), vv.ctypes.data))

    def step(self, first_step: int, nsteps: int) -> None:
        self._check(self.lib.sph_step(self.h, first_step, nsteps))

    def download(self, capacity: int | None = None, out: dict | None = None) -> dict:
        """The live fluid in ascending upload index.  `out` (optional): caller arrays to
        write into (x, v: (capacity, dim); rho p c mass gap [t kappa cp]: (capacity,),
        C-contiguous float64); the returned arrays are views of their first n rows."""
        cap = capacity if capacity is not None else self.stats().n_fluid
        d = self.dim
        names = ["rho", "p", "c", "mass", "gap"] + (["t", "kappa", "cp"] if self.thermal else [])
        if out is None:
            out = {k: np.empty((cap, d)) for k in ("x", "v")}
            for k in names:
                out[k] = np.empty(cap)
        else:
            for k in ("x", "v"):
                assert out[k].shape[0] >= cap and out[k].shape[1:] == (d,), k
            for k in names:
                assert out[k].shape[0] >= cap, k
        n = C.c_int64()
        ptr = lambda k: _abi.dptr(out[k]) if k in out else None
        self._check(self.lib.sph_download_fluid(self.h, cap, C.byref(n), ptr("x"), ptr("v"), ptr("rho"), ptr("p"),
                                                ptr("c"), ptr("mass"), ptr("gap"), ptr("t"), ptr("kappa"),
                                                ptr("cp")))
        return {k: a[: n.value] for k, a in out.items()}

    def download_into(self, fluid) -> None:
        """The live fluid into `fluid`'s own arrays (the library writes them directly), then
        `fluid` is cut to the live count (deleted particles removed, upload order kept)."""
        fields = {"x": "x_vec_", "v": "v_vec_", "rho": "rho_", "p": "p_", "c": "c_", "mass": "mass_", "gap": "gap_"}
        if self.thermal:
            fields.update(t="t_", kappa="kappa_", cp="cp_")
        out = {k: getattr(fluid, f) for k, f in fields.items()}
        if all(a.dtype == np.float64 and a.flags.c_contiguous for a in out.values()):
            n = len(self.download(len(fluid), out=out)["rho"])
            fluid.resize(n)
            return
        r = self.download(len(fluid))
        fluid.resize(len(r["rho"]))
        for k, f in fields.items():
            getattr(fluid, f)[:] = r[k]

    def download_ids(self) -> np.ndarray:
        """Original indices (of the last upload) of the live particles, ascending."""
        cap = self.stats().n_fluid
        ids = np.zeros(max(cap, 1), dtype=np.int64)
        n = C.c_int64()
        self._check(self.lib.sph_download_ids(self.h, cap, C.byref(n), ids.ctypes.data_as(C.POINTER(C.c_int64))))
        return ids[: n.value]

    def autotune(self, reps: int = 5) -> tuple:
        """Pick the fastest FP32 launch shape on the current state (state unchanged)."""
        out = (C.c_int32 * 4)()
        self._check(self.lib.sph_autotune(self.h, reps, out))
        return tuple(out)

    def set_launch_shape(self, continuity: int, momentum: int, reinit: int, block: int) -> None:
        shape = (C.c_int32 * 4)(continuity, momentum, reinit, block)
        self._check(self.lib.sph_set_launch_shape(self.h, shape))

    def set_stencil_pruning(self, on: bool) -> None:
        """FP32 walks skip neighbour cells beyond r_cut (default: 3D on, 2D off); the
        results are bitwise the same either way."""
        self._check(self.lib.sph_set_stencil_pruning(self.h, 1 if on else 0))

    def stats(self) -> _abi.SphStats:
        s = _abi.SphStats()
        self._check(self.lib.sph_stats(self.h, C.byref(s)))
        return s

    def count_pairs(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        self._check(self.lib.sph_count_pairs(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def cell_keys(self) -> tuple[np.ndarray, tuple]:
        """Cell of every live fluid particle as the step's sort assigns it (scene-local
        index cx + nx (cy + ny cz)), rows in download order; and the grid (nx, ny, nz)."""
        n = C.c_int64()
        grid = (C.c_int32 * 3)()
        self._check(self.lib.sph_download_cell_keys(self.h, 0, C.byref(n), None, grid))
        keys = np.zeros(n.value, dtype=np.int64)
        self._check(self.lib.sph_download_cell_keys(self.h, n.value, C.byref(n),
                                                    keys.ctypes.data_as(C.POINTER(C.c_int64)), grid))
        return keys, tuple(grid)

    def neighbour_lists(self) -> tuple[np.ndarray, np.ndarray]:
        """Fluid neighbours each live particle's gathers accept, as (offsets[n+1], ids):
        the ids of row q are those of particle q of download(), ascending."""
        P64 = C.POINTER(C.c_int64)
        n, total = C.c_int64(), C.c_int64()
        cap = int(self.stats().n_fluid) + 1
        offsets = np.zeros(cap, dtype=np.int64)
        self._check(self.lib.sph_download_neighbours(self.h, cap, 0, C.byref(n), C.byref(total),
                                                     offsets.ctypes.data_as(P64), None))
        ids = np.zeros(max(total.value, 1), dtype=np.int64)
        self._check(self.lib.sph_download_neighbours(self.h, cap, total.value, C.byref(n), C.byref(total),
                                                     offsets.ctypes.data_as(P64), ids.ctypes.data_as(P64)))
        return offsets[:n.value + 1], ids[:total.value]

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.sph_get_stream(self.h, C.byref(s)))
        return s.value or 0

    # -- SPH interpolation at points (sph_probe)
    def probe(self, points, fields=("rho_",), none_value: float = math.nan) -> np.ndarray:
        """kernelValueInterpolation (VTPToDataFrame.jl:93-142) of the fluid on the
        device: points (n, dim); fields: particle symbols (rho_, p_, c_, t_, mass_,
        vx, vy, vz) or VTP column names (Density, VelocityX, ...).  Returns
        (len(fields), n)."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, self.dim)
        codes = (C.c_int32 * len(fields))(*[_abi.PROBE_FIELDS[str(f).lstrip(":")] for f in fields])
        out = np.empty((len(fields), len(pts)))
        self._check(self.lib.sph_probe(self.h, len(pts), pts.ctypes.data, len(fields), codes, float(none_value),
                                       out.ctypes.data))
        return out

    # -- VTP output staged off the step stream (sph_output_*)
    def output_open(self, vtp_io, wall_time: str | None = None) -> None:
        """Write files of `vtp_io` (VTPIO) from the library: sph_output_write copies the
        state on the device and a host thread writes the file while later steps run."""
        syms = (C.c_char_p * max(1, len(vtp_io.field_symbols_)))(*[s.encode() for s in vtp_io.field_symbols_])
        names = (C.c_char_p * max(1, len(vtp_io.field_names_)))(*[s.encode() for s in vtp_io.field_names_])
        self._check(self.lib.sph_output_open(self.h, vtp_io.dir_path_.encode(), vtp_io.file_name_.encode(),
                                             vtp_io.file_suffix_.encode(), vtp_io.step_digit_,
                                             len(vtp_io.field_symbols_), syms, names,
                                             None if wall_time is None else wall_time.encode()))

    def output_write(self, file_step: int, time: float) -> None:
        self._check(self.lib.sph_output_write(self.h, file_step, float(time)))

    def output_flush(self) -> None:
        self._check(self.lib.sph_output_flush(self.h))

    def time_stages(self, reps: int = 10) -> dict:
        ms = np.zeros(_abi.NUM_STAGES)
        self._check(self.lib.sph_time_stages(self.h, reps, _abi.dptr(ms)))
        return dict(zip(_abi.STAGE_NAMES, ms.tolist()))


def _variant(walls):
    if len(walls) == 2:
        return _abi.SOLVE_FLUID_COMPULSIVE_THERMOSTATIC_WALL
    w = walls[0]
    if isinstance(w, ThermostaticWallParticles):
        return _abi.SOLVE_FLUID_THERMOSTATIC_WALL
    if isinstance(w, StaticVelocityWallParticles):
        return _abi.SOLVE_FLUID_VELOCITY_WALL
    return _abi.SOLVE_FLUID_WALL


class ParticleView:
    """One fluid particle of a downloaded state, with the field names of the reference's
    particle structs (x_vec_, v_vec_, rho_, p_, c_, mass_, gap_, and t_, kappa_, cp_ for
    thermal particles): what a `check(p)` closure of solve! reads (CollapseDry.jl:119-127)."""

    __slots__ = ("_d", "_q")
    _names = {"x_vec_": "x", "v_vec_": "v", "rho_": "rho", "p_": "p", "c_": "c", "mass_": "mass", "gap_": "gap",
              "t_": "t", "kappa_": "kappa", "cp_": "cp"}

    def __init__(self, d: dict, q: int):
        self._d = d
        self._q = q

    def __getattr__(self, name):
        try:
            return self._d[ParticleView._names[name]][self._q]
        except KeyError:
            raise AttributeError(name) from None


def _host_check(sim, check, fluid_type, dim) -> int:
    """Apply a `check(p) -> Bool` closure on the host at a check step (FluidWallSolve.jl:
    73-81: every fluid particle with !check(p) is deleted): download the live fluid, keep
    the particles the closure accepts and, when some fail, upload the survivors in their
    order (their ids stay ascending, so the sort order and the continuation of the run are
    unchanged).  Returns the number of particles deleted."""
    d = sim.download()
    n = len(d["rho"])
    keep = np.fromiter((bool(check(ParticleView(d, q))) for q in range(n)), dtype=bool, count=n)
    dropped = int(n - np.count_nonzero(keep))
    if dropped:
        sub = fluid_type(int(np.count_nonzero(keep)), dim)
        for f, k in ParticleView._names.items():
            if k in d and hasattr(sub, f):
                getattr(sub, f)[:] = d[k][keep]
        sim.upload_fluid(sub)
    return dropped


def solve(fluid, *args, check=None, vtp_io=None, precision: int = _abi.PRECISION_FP64,
          domain_lo=None, domain_hi=None, periodic_x: bool = False, first_step: int = 1, nsteps: int | None = None,
          staged_output: bool = True, wall_time: str | None = None, autotune: bool = False):
    """GPU counterpart of solve!(fluid, walls..., kernel, model, td, vtp_io; check).

    `check`: an AABBCheck (evaluated on the device, in the step's momentum epilogue) or
    any callable check(p) -> bool over one particle (a ParticleView: p.x_vec_, p.rho_,
    ...), which runs on the host at every check step (isCheckStep), as the reference runs
    its closure (FluidWallSolve.jl:73-81): the run stops after each check step, the
    closure sees the end-of-step state, and the particles it rejects are removed.

    Runs steps first_step .. td.total_step_ (or `nsteps` steps), writes VTP files at
    step 0 and at output steps when `vtp_io` is given (FluidWallSolve.jl:95,133-136),
    and leaves the final state in `fluid`.  With `staged_output` the library writes the
    files from device snapshots while the next steps run; otherwise every output step
    downloads the state and writes the file here.  `domain_lo/hi` bound the cell grid
    (default: the particles' bounding box grown by two cut-off radii; particles leaving
    it are clamped into the edge cells, which stays exact but slower).  `autotune` picks
    the FP32-compensated form's launch shape on the uploaded scene (sph_autotune); the
    form's results depend on the shape in the last bits, so it is off by default.
    """
    *walls, kernel, model, td = args
    for w in walls:
        assert isinstance(w, (CompulsiveWallParticles, ThermostaticWallParticles, StaticVelocityWallParticles))
    variant = _variant(walls)
    if domain_lo is None or domain_hi is None:
        pts = np.concatenate([fluid.x_vec_] + [w.x_vec_ for w in walls if len(w)])
        pad = 2.0 * kernel.influence_radius_
        domain_lo = pts.min(axis=0) - pad if domain_lo is None else domain_lo
        domain_hi = pts.max(axis=0) + pad if domain_hi is None else domain_hi
    host_check = check if (check is not None and not isinstance(check, AABBCheck)) else None
    params = make_params(kernel, model, td, solve=variant, precision=precision,
                         check=None if host_check is not None else check,
                         domain_lo=list(domain_lo), domain_hi=list(domain_hi), periodic_x=periodic_x)
    nw = sum(len(w) for w in walls)
    with Simulation(params, max(len(fluid), 1), nw) as sim:
        for w in walls:
            sim.upload_walls(w)
        sim.upload_fluid(fluid)
        if autotune and precision == _abi.PRECISION_FP32_COMPENSATED:
            sim.autotune(3)
        staged = vtp_io is not None and staged_output
        if staged:
            sim.output_open(vtp_io, wall_time)
            sim.output_write(0, 0.0)
        elif vtp_io is not None:
            vtp_io.write(0, 0.0, fluid, walls, wall_time=wall_time)
        last = td.total_step_ if nsteps is None else first_step + nsteps - 1
        step = first_step
        while step <= last:
            # run up to the next output step (isOutputStep, TimeDiscretization.jl:13-18) or,
            # with a host closure, the next check step (isCheckStep, :20-25)
            nxt = step
            while nxt < last and not (vtp_io is not None and isOutputStep(nxt, td)) and \
                    not (host_check is not None and isCheckStep(nxt, td)):
                nxt += 1
            if staged:
                _abi.check(sim.lib, sim.h, sim.lib.sph_step_async(sim.h, step, nxt - step + 1))
            else:
                sim.step(step, nxt - step + 1)
            step = nxt + 1
            if host_check is not None and isCheckStep(nxt, td):  # deleteat! before writeVTP
                if staged:
                    _abi.check(sim.lib, sim.h, sim.lib.sph_synchronize(sim.h))
                _host_check(sim, host_check, type(fluid), sim.dim)
            if vtp_io is not None and isOutputStep(nxt, td):
                if staged:
                    sim.output_write(nxt // td.output_interval_, nxt * td.dt_)
                else:
                    sim.download_into(fluid)
                    vtp_io.write(nxt // td.output_interval_, nxt * td.dt_, fluid, walls, wall_time=wall_time)
        if staged:
            _abi.check(sim.lib, sim.h, sim.lib.sph_synchronize(sim.h))
            sim.output_flush()
        sim.download_into(fluid)
    return fluid


def solve_inlet_outlet(fluid, inlet, outlet, walls, kernel, model, td, vtp_io=None, *, rules,
                       user_defined_function=None, udf_interval: int = 1, precision: int = _abi.PRECISION_FP64,
                       domain_lo=None, domain_hi=None, first_step: int = 1, nsteps: int | None = None,
                       fluid_capacity: int | None = None, buffer_capacity: int | None = None,
                       staged_output: bool = True, wall_time: str | None = None):
    """GPU counterpart of the inlet/outlet solve!(fluid, inlet, outlet, walls, kernel,
    model, td, vtp_io; checks..., user_defined_function) (FluidInletOutletWallSolve.jl:
    264-340).  rules: InletOutletRules (the check/modify closures as planes).
    user_defined_function(sim, t) runs on the host every `udf_interval` steps (the
    reference calls it after every step, :258); it typically sets the buffer velocities
    with sim.set_buffer_velocity.  VTP files hold [fluid, inlet, outlet, walls] (:282,
    :331-336).  fluid, inlet and outlet are left holding the final state."""
    if domain_lo is None or domain_hi is None:
        pts = np.concatenate([g.x_vec_ for g in (fluid, inlet, outlet, walls) if len(g)])
        pad = 2.0 * kernel.influence_radius_
        domain_lo = pts.min(axis=0) - pad if domain_lo is None else domain_lo
        domain_hi = pts.max(axis=0) + pad if domain_hi is None else domain_hi
    params = make_params(kernel, model, td, solve=_abi.SOLVE_FLUID_INLET_OUTLET_WALL, precision=precision,
                         domain_lo=list(domain_lo), domain_hi=list(domain_hi))
    last = td.total_step_ if nsteps is None else first_step + nsteps - 1
    # room for the fluid to grow while more enters than leaves (reported if exceeded)
    cap = fluid_capacity if fluid_capacity is not None else 2 * len(fluid) + 64 * len(inlet)

    def write(step_file, t):
        if vtp_io is None:
            return
        if staged_output:  # the library copies the state and writes the file meanwhile
            sim.output_write(step_file, t)
            return
        _buffers_into(sim, inlet, 0)
        _buffers_into(sim, outlet, 1)
        _fluid_into(sim, fluid)
        vtp_io.write(step_file, t, fluid, [inlet, outlet, walls], wall_time=wall_time)

    with Simulation(params, cap, len(walls)) as sim:
        sim.upload_walls(walls)
        sim.upload_fluid(fluid)
        sim.upload_buffers(rules, inlet, outlet, buffer_capacity)
        if vtp_io is not None and staged_output:
            sim.output_open(vtp_io, wall_time)
        write(0, 0.0)
        step = first_step
        while step <= last:
            nxt = step
            while nxt < last and (nxt - first_step + 1) % udf_interval != 0 and \
                    not (vtp_io is not None and isOutputStep(nxt, td)):
                nxt += 1
            sim.step(step, nxt - step + 1)
            step = nxt + 1
            if user_defined_function is not None:
                user_defined_function(sim, nxt * td.dt_)
            if vtp_io is not None and isOutputStep(nxt, td):
                write(nxt // td.output_interval_, nxt * td.dt_)
        if vtp_io is not None and staged_output:
            sim.output_flush()
        _fluid_into(sim, fluid)
        _buffers_into(sim, inlet, 0)
        _buffers_into(sim, outlet, 1)
    return fluid, inlet, outlet


def _fluid_into(sim, fluid):
    """The live fluid into `fluid` (its length follows the device: the inlet adds)."""
    _replace(fluid, sim.download(), sim.dim)


def _buffers_into(sim, group, which):
    _replace(group, sim.download_buffers(which), sim.dim)


def _replace(group, d, dim):
    n = len(d["rho"])
    fresh = type(group)(n, dim)
    fresh.x_vec_[:] = d["x"]
    fresh.v_vec_[:] = d["v"]
    for k, f in (("rho", "rho_"), ("p", "p_"), ("c", "c_"), ("mass", "mass_"), ("gap", "gap_")):
        getattr(fresh, f)[:] = d[k]
    for f in fresh._vector_fields + fresh._scalar_fields:
        setattr(group, f, getattr(fresh, f))


def kernelValueInterpolation(points, sim: Simulation, field, none_value: float = math.nan) -> np.ndarray:
    """Reference-named form of Simulation.probe for one field (VTPToDataFrame.jl:122-142):
    the interpolated values at `points` (n, dim) from the live fluid of `sim`."""
    return sim.probe(points, (field,), none_value)[0]
