"""Host-side mirror of the EtherSPHCPU.jl type tree used by ``solve``.

Same names, fields and constructor arguments as the Julia structs, held as
structure-of-arrays numpy containers (the layout the C ABI copies in):

  SmoothKernel(influence_radius, dim, CubicSpline|Gaussian|WendlandC2|WendlandC4)
      src/SPHKernel/SmoothKernel/SmoothKernel.jl:15-48
  CommonLiquidParticles / ThermalLiquidParticles          LiquidParticle.jl:8-101
  CompulsiveWallParticles / StaticVelocityWallParticles /
  ThermostaticWallParticles                                WallParticle.jl:8-51
  CommonWeaklyCompressibleLiquidModel /
  ThermalWeaklyCompressibleLiquidModel                     LiquidModel.jl:10-66
  DensityReinitializedFixedTimeIntervalForwardEuler        FixedTimeIntervalDiscretization.jl:10-23
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# ---------------------------------------------------------------- SPHKernel
class CubicSpline:
    radius_ratio = 2.0
    sigma_table = (2.0 / 3.0, 10.0 / 7.0 / math.pi, 1.0 / math.pi)
    code = 0


class Gaussian:
    radius_ratio = 3.0
    sigma_table = (1.0 / math.sqrt(math.pi), 1.0 / math.pi, 1.0 / math.sqrt(math.pi * math.pi * math.pi))
    code = 1


class WendlandC2:
    radius_ratio = 2.0
    sigma_table = (0.0, 7.0 / 4.0 / math.pi, 21.0 / 16.0 / math.pi)
    code = 2


class WendlandC4:
    radius_ratio = 2.0
    sigma_table = (5.0 / 8.0, 9.0 / 4.0 / math.pi, 495.0 / 256.0 / math.pi)
    code = 3


KERNEL_TYPES = {"CubicSpline": CubicSpline, "Gaussian": Gaussian, "WendlandC2": WendlandC2, "WendlandC4": WendlandC4}


@dataclass(frozen=True)
class SmoothKernel:
    """SmoothKernel(influence_radius, dim, kind) — SmoothKernel.jl:37-48.

    h = r_cut / ratio; sigma = table[dim] / h^dim (Julia's h^dim with an integer dim is
    h*h in 2D and h*h*h in 3D); kernel_0 = sigma.
    """

    kind: type
    h_: float
    dim_: int
    radius_ratio_: float
    influence_radius_: float
    sigma_: float
    kernel_0_: float

    def __init__(self, influence_radius: float, dim: int, kind):
        if isinstance(kind, str):
            kind = KERNEL_TYPES[kind]
        assert dim in (1, 2, 3)
        h = influence_radius / kind.radius_ratio
        hd = h if dim == 1 else (h * h if dim == 2 else h * h * h)
        sigma = kind.sigma_table[dim - 1] / hd
        object.__setattr__(self, "kind", kind)
        object.__setattr__(self, "h_", h)
        object.__setattr__(self, "dim_", dim)
        object.__setattr__(self, "radius_ratio_", kind.radius_ratio)
        object.__setattr__(self, "influence_radius_", influence_radius)
        object.__setattr__(self, "sigma_", sigma)
        object.__setattr__(self, "kernel_0_", sigma)


# ---------------------------------------------------------------- particles
def _zeros(n, dim=None):
    return np.zeros((n, dim) if dim else n, dtype=np.float64)


class _Particles:
    _scalar_fields: tuple = ()
    _vector_fields: tuple = ()

    def __init__(self, n: int, dim: int):
        self.dim = dim
        for f in self._vector_fields:
            setattr(self, f, _zeros(n, dim))
        for f in self._scalar_fields:
            setattr(self, f, _zeros(n))

    def __len__(self):
        return len(getattr(self, self._vector_fields[0]))

    def resize(self, n: int) -> None:
        for f in self._vector_fields + self._scalar_fields:
            a = getattr(self, f)
            setattr(self, f, np.ascontiguousarray(a[:n]))

    @classmethod
    def vcat(cls, *groups):
        out = cls(0, groups[0].dim)
        for f in cls._vector_fields + cls._scalar_fields:
            setattr(out, f, np.ascontiguousarray(np.concatenate([getattr(g, f) for g in groups])))
        return out


class CommonLiquidParticles(_Particles):
    """Vector of CommonLiquidParticle (LiquidParticle.jl:8-35) as arrays."""

    _vector_fields = ("x_vec_", "v_vec_")
    _scalar_fields = ("rho_", "p_", "c_", "mass_", "gap_")
    thermal = False


class ThermalLiquidParticles(_Particles):
    """Vector of ThermalLiquidParticle (LiquidParticle.jl:43-95) as arrays."""

    _vector_fields = ("x_vec_", "v_vec_")
    _scalar_fields = ("rho_", "p_", "c_", "mass_", "gap_", "t_", "kappa_", "cp_")
    thermal = True


class CompulsiveWallParticles(_Particles):
    """Vector of CompulsiveWallParticle (WallParticle.jl:8-19)."""

    _vector_fields = ("x_vec_", "normal_vec_")
    _scalar_fields = ("gap_",)
    wall_kind = 0


class StaticVelocityWallParticles(_Particles):
    """Vector of StaticVelocityWallParticle (WallParticle.jl:21-34)."""

    _vector_fields = ("x_vec_", "normal_vec_", "v_vec_")
    _scalar_fields = ("gap_",)
    wall_kind = 1


class ThermostaticWallParticles(_Particles):
    """Vector of ThermostaticWallParticle (WallParticle.jl:36-51)."""

    _vector_fields = ("x_vec_", "normal_vec_")
    _scalar_fields = ("gap_", "t_", "kappa_")
    wall_kind = 2


# ---------------------------------------------------------------- equation models
@dataclass
class CommonWeaklyCompressibleLiquidModel:
    """LiquidModel.jl:10-33: b = c0^2 rho0 / gamma, nu0 = mu0 / rho0."""

    rho_0_: float
    c_0_: float
    p_0_: float
    gamma_: int
    mu_0_: float
    body_force_vec_: np.ndarray
    b_: float = field(init=False)
    nu_0_: float = field(init=False)
    thermal = False

    def __post_init__(self):
        self.gamma_ = int(self.gamma_)
        self.body_force_vec_ = np.asarray(self.body_force_vec_, dtype=np.float64)
        self.b_ = self.c_0_ * self.c_0_ * self.rho_0_ / self.gamma_
        self.nu_0_ = self.mu_0_ / self.rho_0_


@dataclass
class ThermalWeaklyCompressibleLiquidModel(CommonWeaklyCompressibleLiquidModel):
    """LiquidModel.jl:35-66: adds t_0, kappa_0, cp, beta (Boussinesq)."""

    t_0_: float = 0.0
    kappa_0_: float = 0.0
    cp_: float = 0.0
    beta_: float = 0.0
    thermal = True


def CommonWeaklyCompressibleLiquidModelJL(rho_0, c_0, p_0, gamma, mu_0, body_force_vec):
    """Positional constructor with the Julia argument order."""
    return CommonWeaklyCompressibleLiquidModel(rho_0, c_0, p_0, gamma, mu_0, body_force_vec)


def ThermalWeaklyCompressibleLiquidModelJL(rho_0, c_0, p_0, gamma, mu_0, body_force_vec, t_0, kappa_0, cp, beta):
    """Positional constructor with the Julia argument order (LiquidModel.jl:45-60)."""
    return ThermalWeaklyCompressibleLiquidModel(rho_0, c_0, p_0, gamma, mu_0, body_force_vec,
                                                t_0_=t_0, kappa_0_=kappa_0, cp_=cp, beta_=beta)


# ---------------------------------------------------------------- time discretisation
@dataclass(frozen=True)
class DensityReinitializedFixedTimeIntervalForwardEuler:
    """FixedTimeIntervalDiscretization.jl:10-16 — positional order
    (dt, total_step, output_interval, check_interval, density_reinitialized_interval)."""

    dt_: float
    total_step_: int
    output_interval_: int
    check_interval_: int
    density_reinitialized_interval_: int


def isDensityReinitializedStep(step: int, td) -> bool:  # FixedTimeIntervalDiscretization.jl:18-23
    return step % td.density_reinitialized_interval_ == 0


def isOutputStep(step: int, td) -> bool:  # TimeDiscretization.jl:13-18
    return step % td.output_interval_ == 0


def isCheckStep(step: int, td) -> bool:  # TimeDiscretization.jl:20-25
    return step % td.check_interval_ == 0


# ---------------------------------------------------------------- check predicate
@dataclass(frozen=True)
class AABBCheck:
    """Device form of the `check::Function` keyword of solve!: a fluid particle survives
    a check step iff lo <= x <= hi componentwise (NaN survives, as `>` is false).
    Unbounded sides are +-inf.  CollapseDry.jl:119-127 is AABBCheck(hi=(box_w, box_h))."""

    lo: tuple = (-math.inf, -math.inf, -math.inf)
    hi: tuple = (math.inf, math.inf, math.inf)

    def __call__(self, x: np.ndarray) -> np.ndarray:
        d = x.shape[1]
        lo = np.asarray(self.lo[:d])
        hi = np.asarray(self.hi[:d])
        return ~np.any((x > hi) | (x < lo), axis=1)


@dataclass(frozen=True)
class InletOutletRules:
    """The keyword closures of the inlet/outlet solve! (FluidInletOutletWallSolve.jl:
    inlet_into_calculation_domain_check, inlet_into_calculation_domain_modify,
    outlet_out_calculation_domain_check, outlet_out_check) as the plane tests the
    example's closures are (PoiseuilleFlow2D.jl:146-151): a particle passes when
    normal . x > offset; an inlet particle that entered the fluid is moved by
    inlet_shift."""

    inlet_normal: tuple
    inlet_offset: float
    inlet_shift: tuple
    outlet_normal: tuple
    outlet_offset: float
    drop_normal: tuple
    drop_offset: float

    def c_struct(self):
        from . import _abi
        pad = lambda v: tuple(float(a) for a in v) + (0.0,) * (3 - len(v))
        r = _abi.SphBufferRules()
        r.inlet_normal[:] = pad(self.inlet_normal)
        r.inlet_offset = float(self.inlet_offset)
        r.inlet_shift[:] = pad(self.inlet_shift)
        r.outlet_normal[:] = pad(self.outlet_normal)
        r.outlet_offset = float(self.outlet_offset)
        r.drop_normal[:] = pad(self.drop_normal)
        r.drop_offset = float(self.drop_offset)
        return r
