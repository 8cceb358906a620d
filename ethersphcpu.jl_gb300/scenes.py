"""Scene builders for the benchmark workloads, following the lattice recipes of the
reference examples (particle k of a row at origin + (k - 1/2) dx):

  dam_break_2d            examples/CollapseDry/CollapseDry.jl:10-127
  natural_convection_2d   examples/NaturalConvectionCavityNormalization/NaturalConvectionCavityNormalization.jl:17-135
  dam_break_3d            examples/Cruchaga3D/Cruchaga3D.jl:63-160 (y vertical)
  poiseuille_periodic_2d  examples/PoiseuilleFlow2D/PoiseuilleFlow2D.jl:10-45 (periodic in x instead of
                          the reference's inlet/outlet buffers)

A Scene carries everything `solve` and `Simulation` need.  The artificial viscosity
alpha of the dam-break workloads maps onto the reference's only (laminar) viscosity
through nu0 = alpha h c0 / (2 (d + 2)).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .solver import make_params
from .types import (AABBCheck, CommonLiquidParticles, CommonWeaklyCompressibleLiquidModel, CompulsiveWallParticles,
                    DensityReinitializedFixedTimeIntervalForwardEuler, SmoothKernel, ThermalLiquidParticles,
                    ThermalWeaklyCompressibleLiquidModel, ThermostaticWallParticles)


@dataclass
class Scene:
    name: str
    fluid: object
    walls: list
    kernel: SmoothKernel
    model: object
    td: DensityReinitializedFixedTimeIntervalForwardEuler
    solve: int
    check: AABBCheck | None
    domain_lo: tuple
    domain_hi: tuple
    periodic_x: bool = False
    meta: dict = field(default_factory=dict)

    def params(self, precision: int = _abi.PRECISION_FP64, nan_check: bool = True,
               cell_subdivision: int = 0) -> _abi.SphParams:
        return make_params(self.kernel, self.model, self.td, solve=self.solve, precision=precision,
                           check=self.check, domain_lo=self.domain_lo, domain_hi=self.domain_hi,
                           periodic_x=self.periodic_x, nan_check=nan_check, cell_subdivision=cell_subdivision)

    @property
    def n_fluid(self) -> int:
        return len(self.fluid)

    @property
    def n_wall(self) -> int:
        return sum(len(w) for w in self.walls)


def lattice_2d(x0, y0, nx, ny, dx):
    """createRectangleParticles (CollapseDry.jl:51-58): row-major, x fastest."""
    j, i = np.meshgrid(np.arange(nx), np.arange(ny))
    x = x0 + j.ravel() * dx + dx / 2
    y = y0 + i.ravel() * dx + dx / 2
    return np.stack([x, y], axis=1)


def lattice_3d(x0, y0, z0, nx, ny, nz, dx):
    """createBoxParticles (Cruchaga3D.jl:69-76): x fastest, then y, then z."""
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = x0 + i.ravel() * dx + dx / 2
    y = y0 + j.ravel() * dx + dx / 2
    z = z0 + k.ravel() * dx + dx / 2
    return np.stack([x, y, z], axis=1)


def _walls(cls, x, normal, gap):
    w = cls(len(x), x.shape[1])
    w.x_vec_[:] = x
    w.normal_vec_[:] = np.broadcast_to(np.asarray(normal, dtype=np.float64), x.shape)
    w.gap_[:] = gap
    return w


def _rho_hydrostatic(p, b, gamma, rho0):
    # (p/b + 1)^(1/gamma) * rho0   (CollapseDry.jl:67)
    return (p / b + 1.0) ** (1.0 / gamma) * rho0


def _eos(rho, model):
    # updatePressure! (UpdatePressure.jl:8-16) for the initial p, c
    rr = rho / model.rho_0_
    p = model.b_ * (rr ** model.gamma_ - 1.0) + model.p_0_
    c = model.c_0_ * np.sqrt(rr ** (model.gamma_ - 1))
    return p, c


def dam_break_2d(dx=0.02, water_w=1.0, water_h=2.0, box_w=4.0, box_h=3.0, alpha=0.1, gamma=1, c0=None,
                 reinit=30, check_interval=5, total_step=2000, g=9.81, kernel="CubicSpline", name="dam_break_2d"):
    """2D dry dam break (CollapseDry.jl), the 5,000-particle FP64 workload by default."""
    dim = 2
    rc = 3.0 * dx
    kernel = SmoothKernel(rc, dim, kernel)
    if c0 is None:
        c0 = 10.0 * math.sqrt(2.0 * g * water_h)
    nu0 = alpha * kernel.h_ * c0 / (2.0 * (dim + 2))
    rho0 = 1000.0
    model = CommonWeaklyCompressibleLiquidModel(rho0, c0, 0.0, gamma, nu0 * rho0, np.array([0.0, -g]))
    dt = 0.1 * kernel.h_ / c0
    td = DensityReinitializedFixedTimeIntervalForwardEuler(dt, total_step, 100, check_interval, reinit)
    nrow, ncol = int(round(water_h / dx)), int(round(water_w / dx))
    fluid = CommonLiquidParticles(nrow * ncol, dim)
    fluid.x_vec_[:] = lattice_2d(0.0, 0.0, ncol, nrow, dx)
    p = rho0 * g * (water_h + dx - fluid.x_vec_[:, 1])  # CollapseDry.jl:66
    fluid.rho_[:] = _rho_hydrostatic(p, model.b_, gamma, rho0)
    fluid.p_[:], fluid.c_[:] = _eos(fluid.rho_, model)
    fluid.mass_[:] = fluid.rho_ * (dx * dx)
    fluid.gap_[:] = dx
    t = 3
    nbw, nbh = int(round(box_w / dx)), int(round(box_h / dx))
    walls = CompulsiveWallParticles.vcat(
        _walls(CompulsiveWallParticles, lattice_2d(0.0, -t * dx, nbw, t, dx), [0.0, 1.0], dx),
        _walls(CompulsiveWallParticles, lattice_2d(-t * dx, 0.0, t, nbh, dx), [1.0, 0.0], dx),
        _walls(CompulsiveWallParticles, lattice_2d(box_w, 0.0, t, nbh, dx), [-1.0, 0.0], dx),
        _walls(CompulsiveWallParticles, lattice_2d(-t * dx, -t * dx, t, t, dx),
               np.array([1.0, 1.0]) / math.sqrt(2.0), dx),
        _walls(CompulsiveWallParticles, lattice_2d(box_w, -t * dx, t, t, dx),
               np.array([-1.0, 1.0]) / math.sqrt(2.0), dx),
    )
    check = AABBCheck(hi=(box_w, box_h))  # CollapseDry.jl:119-127
    lo = (-t * dx - rc, -t * dx - rc)
    hi = (box_w + t * dx + rc, box_h + rc)
    return Scene(name, fluid, [walls], kernel, model, td, _abi.SOLVE_FLUID_WALL, check, lo, hi,
                 meta=dict(dx=dx, water_w=water_w, water_h=water_h, box_w=box_w, box_h=box_h))


def natural_convection_2d(n=256, prandtl=0.71, rayleigh=1e5, c0_factor=10.0, reinit=30, total_step=20000,
                          kernel="WendlandC2", seed=0, noise=1e-3, name="natural_convection_2d"):
    """2D differentially heated square cavity (NaturalConvectionCavityNormalization.jl).

    Normalisation rho0 = g = kappa = L = 1, nu = Pr/sqrt(Ra), cp = Pr kappa / mu0,
    beta = Ra nu alpha / (g dT L^3) (:17-39), c0 = c0_factor * sqrt(g beta dT L),
    p0 = 0.02 rho0 c0^2, gamma = 7, dt = 0.1 r_cut / c0 (:48).  Left wall T = 1, right
    T = 0 (ThermostaticWallParticle), adiabatic top/bottom CompulsiveWallParticle; the
    initial temperature is 0.5 + U(-noise, noise) from a seeded generator.
    """
    dim = 2
    L = 1.0
    dr = L / n
    rc = 3.0 * dr
    kernel = SmoothKernel(rc, dim, kernel)
    rho0, g, kappa = 1.0, 1.0, 1.0
    nu0 = prandtl / math.sqrt(rayleigh)
    mu0 = rho0 * nu0
    alpha = nu0 / prandtl
    t_left, t_right = 1.0, 0.0
    dT = t_left - t_right
    t0 = (t_left + t_right) / 2
    cp = prandtl * kappa / mu0
    beta = rayleigh * nu0 * alpha / g / dT / (L * L * L)
    c0 = c0_factor * math.sqrt(g * beta * dT * L)
    p0 = 0.02 * rho0 * c0 * c0
    model = ThermalWeaklyCompressibleLiquidModel(rho0, c0, p0, 7, mu0, np.array([0.0, -g]),
                                                 t_0_=t0, kappa_0_=kappa, cp_=cp, beta_=beta)
    dt = 0.1 * rc / c0
    td = DensityReinitializedFixedTimeIntervalForwardEuler(dt, total_step, 100, 100, reinit)
    fluid = ThermalLiquidParticles(n * n, dim)
    fluid.x_vec_[:] = lattice_2d(0.0, 0.0, n, n, dr)
    fluid.rho_[:] = rho0
    fluid.p_[:] = p0
    fluid.c_[:] = c0
    rng = np.random.default_rng(seed)
    fluid.t_[:] = t0 + rng.uniform(-noise, noise, n * n)
    fluid.mass_[:] = rho0 * (dr * dr)
    fluid.gap_[:] = dr
    fluid.kappa_[:] = kappa
    fluid.cp_[:] = cp
    t = 3

    def thermo(x0, temp, nrm):
        w = _walls(ThermostaticWallParticles, lattice_2d(x0, -rc, t, n + 2 * t, dr), nrm, dr)
        w.t_[:] = temp
        w.kappa_[:] = kappa
        return w

    thermostat = ThermostaticWallParticles.vcat(thermo(-rc, t_left, [1.0, 0.0]), thermo(L, t_right, [-1.0, 0.0]))
    compulsive = CompulsiveWallParticles.vcat(
        _walls(CompulsiveWallParticles, lattice_2d(0.0, -rc, n, t, dr), [0.0, 1.0], dr),
        _walls(CompulsiveWallParticles, lattice_2d(0.0, L, n, t, dr), [0.0, -1.0], dr),
    )
    lo = (-2 * rc, -2 * rc)
    hi = (L + 2 * rc, L + 2 * rc)
    return Scene(name, fluid, [compulsive, thermostat], kernel, model, td,
                 _abi.SOLVE_FLUID_COMPULSIVE_THERMOSTATIC_WALL, None, lo, hi,
                 meta=dict(n=n, prandtl=prandtl, rayleigh=rayleigh, dx=dr))


def dam_break_3d(dx=0.005, tank=(3.2, 1.0, 1.0), column=(0.6, 0.6, 1.2), wall_height=None, alpha=0.05, gamma=7,
                 reinit=30, total_step=5000, g=9.81, kernel="WendlandC4", name="dam_break_3d"):
    """3D dam break, y vertical as in Cruchaga3D.jl.  tank = (length x, width z, height y),
    column = (length x, width z, height y).  The side walls are open-topped and reach
    max(tank height, 1.05 column height) so a column taller than the tank stays
    enclosed; no particle is deleted (check = true, Cruchaga3D.jl:162)."""
    dim = 3
    rc = 3.0 * dx
    kernel = SmoothKernel(rc, dim, kernel)
    lx, lz, ly = tank
    cx, cz, cy = column
    c0 = 10.0 * math.sqrt(2.0 * g * cy)
    nu0 = alpha * kernel.h_ * c0 / (2.0 * (dim + 2))
    rho0 = 1000.0
    model = CommonWeaklyCompressibleLiquidModel(rho0, c0, 0.0, gamma, nu0 * rho0, np.array([0.0, -g, 0.0]))
    dt = 0.1 * kernel.h_ / c0
    td = DensityReinitializedFixedTimeIntervalForwardEuler(dt, total_step, 100, 1000, reinit)
    nx, ny, nz = int(round(cx / dx)), int(round(cy / dx)), int(round(cz / dx))
    fluid = CommonLiquidParticles(nx * ny * nz, dim)
    fluid.x_vec_[:] = lattice_3d(0.0, 0.0, 0.0, nx, ny, nz, dx)
    p = rho0 * g * (cy - fluid.x_vec_[:, 1])  # Cruchaga3D.jl:79
    fluid.rho_[:] = _rho_hydrostatic(p, model.b_, gamma, rho0)
    fluid.p_[:], fluid.c_[:] = _eos(fluid.rho_, model)
    fluid.mass_[:] = fluid.rho_ * (dx * dx * dx)
    fluid.gap_[:] = dx
    t = 3
    wh = wall_height if wall_height is not None else max(ly, 1.05 * cy)
    bx, by, bz = int(round(lx / dx)), int(round(wh / dx)), int(round(lz / dx))
    W = CompulsiveWallParticles
    walls = W.vcat(
        _walls(W, lattice_3d(-t * dx, -t * dx, -t * dx, bx + 2 * t, t, bz + 2 * t, dx), [0.0, 1.0, 0.0], dx),
        _walls(W, lattice_3d(-t * dx, 0.0, -t * dx, bx + 2 * t, by, t, dx), [0.0, 0.0, 1.0], dx),
        _walls(W, lattice_3d(-t * dx, 0.0, bz * dx, bx + 2 * t, by, t, dx), [0.0, 0.0, -1.0], dx),
        _walls(W, lattice_3d(-t * dx, 0.0, 0.0, t, by, bz, dx), [1.0, 0.0, 0.0], dx),
        _walls(W, lattice_3d(bx * dx, 0.0, 0.0, t, by, bz, dx), [-1.0, 0.0, 0.0], dx),
    )
    lo = (-t * dx - rc, -t * dx - rc, -t * dx - rc)
    hi = (lx + t * dx + rc, max(wh, cy) + 2 * rc, lz + t * dx + rc)
    return Scene(name, fluid, [walls], kernel, model, td, _abi.SOLVE_FLUID_WALL, None, lo, hi,
                 meta=dict(dx=dx))


def poiseuille_periodic_2d(H=1e-3, length_factor=4.0, nu=1e-6, reynolds=0.5, n_across=40, total_step=5000,
                           reinit=30, kernel="WendlandC2", rho0=1000.0, name="poiseuille_periodic_2d"):
    """Plane Poiseuille flow between two compulsive walls, periodic in x (new: the
    reference drives this flow with inlet/outlet buffers, PoiseuilleFlow2D.jl).  Body
    force f = 8 nu^2 Re / H^3 so that U_max = f H^2 / (8 nu) = Re nu / H."""
    dim = 2
    dx = H / n_across
    rc = 3.0 * dx
    kernel = SmoothKernel(rc, dim, kernel)
    f = 8.0 * nu * nu * reynolds / (H * H * H)
    umax = f * H * H / (8.0 * nu)
    c0 = 10.0 * umax
    p0 = 0.02 * rho0 * c0 * c0
    model = CommonWeaklyCompressibleLiquidModel(rho0, c0, p0, 7, nu * rho0, np.array([f, 0.0]))
    # acoustic limit of the example (PoiseuilleFlow2D.jl:46) and the viscous limit
    # 0.1 h^2 / nu, which governs at millimetre channel heights
    dt = min(0.1 * rc / c0, 0.1 * kernel.h_ * kernel.h_ / nu)
    td = DensityReinitializedFixedTimeIntervalForwardEuler(dt, total_step, 100, 100, reinit)
    L = length_factor * H
    nxl = int(round(L / dx))
    fluid = CommonLiquidParticles(nxl * n_across, dim)
    fluid.x_vec_[:] = lattice_2d(0.0, 0.0, nxl, n_across, dx)
    fluid.rho_[:] = rho0
    fluid.p_[:], fluid.c_[:] = _eos(fluid.rho_, model)
    fluid.mass_[:] = rho0 * dx * dx
    fluid.gap_[:] = dx
    t = 3
    W = CompulsiveWallParticles
    walls = W.vcat(_walls(W, lattice_2d(0.0, -t * dx, nxl, t, dx), [0.0, 1.0], dx),
                   _walls(W, lattice_2d(0.0, H, nxl, t, dx), [0.0, -1.0], dx))
    lo = (0.0, -t * dx - rc)
    hi = (L, H + t * dx + rc)
    # wall terms as in FluidInletOutletWallSolve.jl:112-124 (no wall pressure)
    return Scene(name, fluid, [walls], kernel, model, td, _abi.SOLVE_FLUID_WALL, None, lo, hi,
                 periodic_x=True, meta=dict(H=H, nu=nu, f=f, umax=umax, dx=dx, L=L))


def poiseuille_inlet_outlet_2d(H=1e-2, length_factor=4.0, nu=1e-6, f=8e-5, n_across=20, total_step=2000,
                               reinit=5, kernel="WendlandC2", rho0=1000.0, start="steady",
                               name="poiseuille_inlet_outlet_2d"):
    """The reference's channel flow with inlet and outlet buffers (PoiseuilleFlow2D.jl):
    channel H x 4H, 3 layers of inlet particles upstream of x = 0 and of outlet particles
    downstream of x = 4H, 3 wall layers below and above reaching 6 layers past both ends,
    WendlandC2 with r_cut = 3 dx, body force f, U_max = f H^2 / (8 nu), c0 = 10 U_max,
    p0 = 0.02 rho0 c0^2, gamma = 7, dt = 0.1 r_cut / c0.  The example starts from the
    transient profile at t = 0 (at rest) and lets a host callback set the buffers to the
    analytic profile every step; start="steady" starts every particle on the steady
    profile instead, so that particles cross the inlet and outlet from the first steps.
    meta holds the inlet and outlet particles and the InletOutletRules."""
    from .types import InletOutletRules
    dim = 2
    dx = H / n_across
    rc = 3.0 * dx
    kernel = SmoothKernel(rc, dim, kernel)
    umax = f / 2.0 / nu / 4.0 * H * H
    c0 = 10.0 * umax
    p0 = 0.02 * rho0 * c0 * c0
    model = CommonWeaklyCompressibleLiquidModel(rho0, c0, p0, 7, nu * rho0, np.array([f, 0.0]))
    dt = min(0.1 * rc / c0, 0.1 * kernel.h_ * kernel.h_ / nu)
    td = DensityReinitializedFixedTimeIntervalForwardEuler(dt, total_step, 100, reinit, reinit)
    L = length_factor * H
    nxl = int(round(L / dx))
    t = 3

    def block(x0, ncol):
        g = CommonLiquidParticles(ncol * n_across, dim)
        g.x_vec_[:] = lattice_2d(x0, 0.0, ncol, n_across, dx)
        g.rho_[:] = rho0
        g.p_[:] = p0
        g.c_[:] = c0
        g.mass_[:] = rho0 * dx * dx
        g.gap_[:] = dx
        y = g.x_vec_[:, 1]
        g.v_vec_[:, 0] = (f / 2.0 / nu * y * (H - y) if start == "steady"
                          else poiseuille_ux_theory(y, 0.0, H, nu, f))
        return g

    fluid = block(0.0, nxl)
    inlet = block(-t * dx, t)
    outlet = block(L, t)
    W = CompulsiveWallParticles
    more = 3
    wcols = nxl + 2 * (t + more)
    walls = W.vcat(_walls(W, lattice_2d(-(t + more) * dx, -t * dx, wcols, t, dx), [0.0, 1.0], dx),
                   _walls(W, lattice_2d(-(t + more) * dx, H, wcols, t, dx), [0.0, -1.0], dx))
    lo = (-(t + more) * dx - rc, -t * dx - rc)
    hi = (L + (t + more) * dx + rc, H + t * dx + rc)
    rules = InletOutletRules(inlet_normal=(1.0, 0.0), inlet_offset=0.0, inlet_shift=(-t * dx, 0.0),
                             outlet_normal=(1.0, 0.0), outlet_offset=L,
                             drop_normal=(1.0, 0.0), drop_offset=L + t * dx)
    return Scene(name, fluid, [walls], kernel, model, td, _abi.SOLVE_FLUID_INLET_OUTLET_WALL, None, lo, hi,
                 meta=dict(H=H, nu=nu, f=f, umax=umax, dx=dx, L=L, inlet=inlet, outlet=outlet, rules=rules))


def poiseuille_ux_theory(y, t, H, nu, f, order=10):
    """Transient plane Poiseuille profile (the series of PoiseuilleFlow2D.jl:28-35)."""
    y = np.asarray(y, dtype=np.float64)
    ux = f / 2.0 / nu * y * (H - y)
    for n in range(order + 1):
        k = 2 * n + 1
        ux = ux - 4.0 * f * H * H / nu / math.pi ** 3 / k ** 3 * np.sin(math.pi * y / H * k) * \
            np.exp(-(k * k) * math.pi ** 2 * nu * t / (H * H))
    return ux


def lid_driven_cavity_2d(n=100, reynolds=100.0, lid_velocity=1.0, reinit=100, total_step=5000,
                         kernel="WendlandC2", name="lid_driven_cavity_2d"):
    """Lid-driven cavity with StaticVelocityWallParticle walls (LidDrivenCavity.jl:10-145),
    the FluidVelocitySolve workload: rho0 = 1, mu0 = L rho0 U / Re, c0 = 10 U,
    p0 = 0.001 rho0 c0^2, gamma = 7, dt = 0.1 r_cut / c0, 3 wall layers, moving lid and
    its two corners at (U, 0)."""
    from .types import StaticVelocityWallParticles as SV
    dim = 2
    L = 1.0
    dr = L / n
    rc = 3.0 * dr
    kernel = SmoothKernel(rc, dim, kernel)
    rho0 = 1.0
    mu0 = L * rho0 * lid_velocity / reynolds
    c0 = 10.0 * lid_velocity
    p0 = 0.001 * rho0 * c0 * c0
    model = CommonWeaklyCompressibleLiquidModel(rho0, c0, p0, 7, mu0, np.array([0.0, 0.0]))
    dt = 0.1 * rc / c0
    td = DensityReinitializedFixedTimeIntervalForwardEuler(dt, total_step, 100, 100, reinit)
    fluid = CommonLiquidParticles(n * n, dim)
    fluid.x_vec_[:] = lattice_2d(0.0, 0.0, n, n, dr)
    fluid.rho_[:] = rho0
    fluid.p_[:], fluid.c_[:] = _eos(fluid.rho_, model)
    fluid.mass_[:] = rho0 * dr * dr
    fluid.gap_[:] = dr
    t = 3
    s2 = 1.0 / math.sqrt(2.0)

    def sv(x0, y0, nx, ny, nrm, vel):
        w = _walls(SV, lattice_2d(x0, y0, nx, ny, dr), nrm, dr)
        w.v_vec_[:] = vel
        return w

    U = [lid_velocity, 0.0]
    Z = [0.0, 0.0]
    walls = SV.vcat(
        sv(0.0, L, n, t, [0.0, -1.0], U),
        sv(-t * dr, 0.0, t, n, [1.0, 0.0], Z),
        sv(L, 0.0, t, n, [-1.0, 0.0], Z),
        sv(0.0, -t * dr, n, t, [0.0, 1.0], Z),
        sv(-t * dr, -t * dr, t, t, [s2, s2], Z),
        sv(L, -t * dr, t, t, [-s2, s2], Z),
        sv(-t * dr, L, t, t, [s2, -s2], U),
        sv(L, L, t, t, [-s2, -s2], U),
    )
    lo = (-t * dr - rc, -t * dr - rc)
    hi = (L + t * dr + rc, L + t * dr + rc)
    return Scene(name, fluid, [walls], kernel, model, td, _abi.SOLVE_FLUID_VELOCITY_WALL, None, lo, hi,
                 meta=dict(n=n, reynolds=reynolds, dx=dr))


# ---------------------------------------------------------------- batched and served workloads
def random_dam_break_2d(rng, dx=0.01, total_step=1000, kernel="CubicSpline", name="dam_break"):
    """One scene of the batched distribution: column width W ~ U[0.3, 1.5] m, height/width
    ~ U[0.5, 3], tank 4W x 1.5 H, the physics of dam_break_2d (c0 = 10 sqrt(2 g H))."""
    W = float(rng.uniform(0.3, 1.5))
    H = float(rng.uniform(0.5, 3.0)) * W
    return dam_break_2d(dx=dx, water_w=W, water_h=H, box_w=4.0 * W, box_h=1.5 * H, total_step=total_step,
                        kernel=kernel, name=name)


def batched_dam_breaks(n_scenes=512, seed=0, dx=0.01, total_step=1000, kernel="CubicSpline"):
    """The batched workload: n_scenes seeded 2D dam breaks (about 450 to 67,500 fluid
    particles each) for one launch of the batch kernels."""
    rng = np.random.default_rng(seed)
    return [random_dam_break_2d(rng, dx, total_step, kernel, name=f"dam_break_{k}") for k in range(n_scenes)]


def random_poiseuille_2d(rng, total_step=1000, kernel="CubicSpline", name="poiseuille"):
    """Served Poiseuille channel: H = 1 mm, L = 4H, nu = 1e-6, Re ~ U[0.01, 1],
    dx = H / U{20..80}, periodic in x."""
    return poiseuille_periodic_2d(H=1e-3, length_factor=4.0, nu=1e-6, reynolds=float(rng.uniform(0.01, 1.0)),
                                  n_across=int(rng.integers(20, 81)), total_step=total_step, kernel=kernel,
                                  name=name)


def random_dam_break_3d(rng, total_step=1000, kernel="WendlandC4", name="dam_break_3d"):
    """Served 3D dam break: dx ~ U[0.01, 0.02] m, a 0.4 x 0.4 x 0.65 m column (about 13k
    to 110k particles) in a 1.6 x 0.4 x 0.8 m tank."""
    dx = float(rng.uniform(0.01, 0.02))
    return dam_break_3d(dx=dx, tank=(1.6, 0.4, 0.8), column=(0.4, 0.4, 0.65), total_step=total_step, kernel=kernel,
                        name=name)


@dataclass
class Request:
    t_arrival: float
    kind: str       # "dam_break_2d" | "poiseuille_2d" | "dam_break_3d"
    nsteps: int
    seed: int

    def build(self):
        rng = np.random.default_rng(self.seed)
        if self.kind == "dam_break_2d":
            return random_dam_break_2d(rng, total_step=self.nsteps, name=f"req{self.seed}")
        if self.kind == "poiseuille_2d":
            return random_poiseuille_2d(rng, total_step=self.nsteps, name=f"req{self.seed}")
        return random_dam_break_3d(rng, total_step=self.nsteps, name=f"req{self.seed}")


def poisson_stream(rate, count, seed=0, steps=(500, 5000), kinds=("dam_break_2d", "poiseuille_2d", "dam_break_3d")):
    """A served request stream: Poisson arrivals at `rate` per second, kinds drawn with
    equal probability, step budgets ~ U{steps[0]..steps[1]}."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    kind = rng.integers(0, len(kinds), count)
    nsteps = rng.integers(steps[0], steps[1] + 1, count)
    return [Request(float(t[k]), kinds[int(kind[k])], int(nsteps[k]), seed * 1_000_003 + k) for k in range(count)]
