"""Pins of the CPU restatement (oracle/) — no GPU needed.

1. The reference's own tests (test/SPHKernel.jl, test/EquationModel.jl,
   test/Neighbour.jl, test/Particle.jl), restated.
2. Known-answer tests of every kernel against its closed form, normalisation,
   Julia's integer power, the NaN guard of the gradient.
3. Cell-list pair enumeration equals brute force on lattices and jittered sets.
4. Step-level self-consistency: the half-list atomic-scatter mode (the reference's
   algorithm) and the full-list gather mode (the GPU's order) agree to rounding;
   mass is conserved exactly.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

KINDS = {"CubicSpline": 0, "Gaussian": 1, "WendlandC2": 2, "WendlandC4": 3}


# ---------------------------------------------------------------- reference tests
def test_reference_smooth_kernel_h(orc):
    # test/SPHKernel.jl:10-19
    r = 1.0
    assert math.isclose(orc.smooth_kernel(0, 2, r)[0], r / 2.0)
    assert math.isclose(orc.smooth_kernel(1, 2, r)[0], r / 3.0)
    assert math.isclose(orc.smooth_kernel(2, 2, r)[0], r / 2.0)
    assert math.isclose(orc.smooth_kernel(3, 2, r)[0], r / 2.0)


def test_reference_equation_model(pkg):
    # test/EquationModel.jl:10-23
    m = pkg.CommonWeaklyCompressibleLiquidModel(1.0, 1.0, 1.0, 7, 0.1, [0.0, 0.0, -9.8])
    assert math.isclose(m.nu_0_, 0.1 / 1.0)
    t = pkg.ThermalWeaklyCompressibleLiquidModel(1.0, 1.0, 1.0, 7, 0.1, [0.0, 0.0, -9.8],
                                                 t_0_=1.0, kappa_0_=1.0, cp_=1.0, beta_=1.0)
    assert math.isclose(t.b_, 1.0 * 1.0 * 1.0 / 7)


def test_reference_neighbour_r(orc):
    # test/Neighbour.jl:9-21: tuple (1, 1, 5.0) with x_i = (3, 4), x_j = 0 gives r_ = 5
    nb = orc.neighbour(0, 2, 10.0, [3.0, 4.0], [0.0, 0.0], [0.0, 0.0], [0.0, 0.0], 5.0)
    assert np.allclose(nb["r_vec"], [3.0, 4.0])
    # the pair record keeps the tuple's r; its kernel values follow from it
    assert nb["W"] == orc.kernel_value(0, 2, 10.0, 5.0)


def test_reference_particle_defaults(pkg):
    # test/Particle.jl:10-16
    assert pkg.CompulsiveWallParticles(1, 2).gap_[0] == 0.0
    assert np.all(pkg.StaticVelocityWallParticles(1, 2).v_vec_[0] == [0.0, 0.0])
    assert pkg.ThermostaticWallParticles(1, 2).t_[0] == 0.0
    assert pkg.CommonLiquidParticles(1, 2).mass_[0] == 0.0
    assert pkg.ThermalLiquidParticles(1, 2).t_[0] == 0.0


def test_host_mirror_matches_oracle_kernel_constants(pkg, orc):
    for name, code in KINDS.items():
        for dim in (1, 2, 3):
            if name == "WendlandC2" and dim == 1:
                continue
            k = pkg.SmoothKernel(0.03, dim, name)
            h, s, k0 = orc.smooth_kernel(code, dim, 0.03)
            assert (k.h_, k.sigma_, k.kernel_0_) == (h, s, k0), (name, dim)


# ---------------------------------------------------------------- kernel KATs
def closed_form(name, q, sigma, h):
    """W and dW/dr straight from the formulas of the reference docstrings."""
    if name == "CubicSpline":
        if q < 1:
            return sigma / 4 * (3 * q * q * (q - 2) + 4), sigma / h * 0.75 * q * (3 * q - 4)
        if q < 2:
            return sigma / 4 * (2 - q) ** 3, -sigma / h * 0.75 * (2 - q) ** 2
        return 0.0, 0.0
    if name == "Gaussian":
        if q < 3:
            return sigma * math.exp(-q * q), -2 * sigma / h * q * math.exp(-q * q)
        return 0.0, 0.0
    if name == "WendlandC2":
        if q < 2:
            return sigma * (2 - q) ** 4 * (1 + 2 * q) / 16, -sigma / h * 5 / 8 * q * (2 - q) ** 3
        return 0.0, 0.0
    if q < 2:
        return (sigma * (2 - q) ** 6 * (35 * q * q + 36 * q + 12) / 768,
                -sigma / h * (35 / 96 * q * q + 7 / 48 * q) * (2 - q) ** 5)
    return 0.0, 0.0


@pytest.mark.parametrize("name", list(KINDS))
@pytest.mark.parametrize("dim", [2, 3])
def test_kernel_known_answers(orc, name, dim):
    rc = 0.03
    h, sigma, _ = orc.smooth_kernel(KINDS[name], dim, rc)
    for q in (0.0, 0.25, 0.5, 0.999, 1.0, 1.5, 1.999, 2.0, 2.5, 3.0):
        r = q * h
        W = orc.kernel_value(KINDS[name], dim, rc, r)
        dW = orc.kernel_gradient(KINDS[name], dim, rc, r)
        Wc, dWc = closed_form(name, r / h, sigma, h)
        assert W == pytest.approx(Wc, rel=1e-13, abs=1e-13 * sigma), (q, W, Wc)
        assert dW == pytest.approx(dWc, rel=1e-13, abs=1e-13 * sigma / h), (q, dW, dWc)
    # W(0) = kernel_0 = sigma
    assert orc.kernel_value(KINDS[name], dim, rc, 0.0) == pytest.approx(sigma, rel=1e-15)


@pytest.mark.parametrize("name", list(KINDS))
@pytest.mark.parametrize("dim", [2, 3])
def test_kernel_normalisation(orc, name, dim):
    # integral of W over the plane/space is 1 (Gaussian: truncated at q = 3)
    rc = 1.0
    h, _, _ = orc.smooth_kernel(KINDS[name], dim, rc)
    r = np.linspace(0.0, rc, 20001)
    W = np.array([orc.kernel_value(KINDS[name], dim, rc, x) for x in r])
    shell = 2 * math.pi * r if dim == 2 else 4 * math.pi * r * r
    integral = np.trapezoid(W * shell, r)
    expected = 1.0
    if name == "Gaussian":  # mass inside q < 3 of the untruncated Gaussian
        expected = 1.0 - math.exp(-9.0) if dim == 2 else math.erf(3.0) - 6.0 / math.sqrt(math.pi) * math.exp(-9.0)
    assert integral == pytest.approx(expected, abs=1e-6)


def test_kernel_gradient_is_derivative(orc):
    for name, code in KINDS.items():
        rc = 1.0
        h, _, _ = orc.smooth_kernel(code, 2, rc)
        for r in np.linspace(0.05, 0.95, 13) * rc:
            eps = 1e-6
            num = (orc.kernel_value(code, 2, rc, r + eps) - orc.kernel_value(code, 2, rc, r - eps)) / (2 * eps)
            assert orc.kernel_gradient(code, 2, rc, r) == pytest.approx(num, rel=1e-6, abs=1e-7)


def test_julia_integer_power_is_faithful(orc):
    rng = np.random.default_rng(0)
    for x in rng.uniform(0.5, 2.0, 200):
        for n in (1, 2, 3, 4, 5, 6, 7):
            got = orc.powi(float(x), n)
            exact = Fraction(float(x)) ** n
            err = abs(Fraction(got) - exact) / exact
            assert float(err) <= 2.3e-16  # within one ulp
            if n == 2:
                assert got == float(x) * float(x)
            if n == 3:
                assert got == float(x) * float(x) * float(x)
    assert orc.powi(1.7, 0) == 1.0


def test_gradient_nan_guard(orc):
    # coincident particles: normalize(0-vector) is NaN, set to 0 (Neighbour.jl:79-84)
    nb = orc.neighbour(0, 2, 1.0, [0.5, 0.5], [0.5, 0.5], [1.0, 0.0], [0.0, 0.0], 0.0)
    assert np.all(nb["grad"] == 0.0)
    nb = orc.neighbour(2, 3, 1.0, [0.1, 0.2, 0.3], [0.0, 0.0, 0.0], [0, 0, 0], [0, 0, 0], math.sqrt(0.14))
    g = nb["dW"] * np.array([0.1, 0.2, 0.3]) * (1.0 / math.sqrt(0.14))
    assert np.allclose(nb["grad"], g, rtol=1e-15)


# ---------------------------------------------------------------- pair enumeration
def _bruteforce_counts(x, wx, rc):
    d = x[:, None, :] - x[None, :, :]
    d2 = (d * d).sum(-1) if x.shape[1] == 2 else None
    n = len(x)
    ff = 0
    fw = 0
    for i in range(n):
        rv = x[i] - x[i + 1:]
        s = rv[:, 0] * rv[:, 0] + rv[:, 1] * rv[:, 1]
        if x.shape[1] == 3:
            s = s + rv[:, 2] * rv[:, 2]
        ff += int(np.count_nonzero(s <= rc * rc))
        if wx is not None:
            rw = x[i] - wx
            s = rw[:, 0] * rw[:, 0] + rw[:, 1] * rw[:, 1]
            if x.shape[1] == 3:
                s = s + rw[:, 2] * rw[:, 2]
            fw += int(np.count_nonzero(s <= rc * rc))
    del d2
    return ff, fw


@pytest.mark.parametrize("jitter", [0.0, 0.3])
def test_cell_list_pairs_equal_bruteforce_2d(pkg, orc, jitter):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_2d(dx=0.05)
    rng = np.random.default_rng(1)
    x = s.fluid.x_vec_ + jitter * 0.05 * rng.uniform(-1, 1, s.fluid.x_vec_.shape)
    wx = s.walls[0].x_vec_
    prm = s.params()
    got = orc.neighbour_counts(prm, x, wx)
    assert got == _bruteforce_counts(x, wx, s.kernel.influence_radius_)
    pairs = orc.pair_list_bruteforce(x, s.kernel.influence_radius_)
    assert len(pairs) == got[0]
    if jitter == 0.0:
        # on the lattice, interior particles have 28 neighbours within 3 dx (<= keeps the 4 at exactly 3 dx)
        nb = np.bincount(pairs.ravel(), minlength=len(x))
        assert nb.max() == 28


def test_cell_list_pairs_equal_bruteforce_3d(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_3d(dx=0.05, tank=(0.8, 0.4, 0.4), column=(0.3, 0.2, 0.4))
    rng = np.random.default_rng(2)
    x = s.fluid.x_vec_ + 0.2 * 0.05 * rng.uniform(-1, 1, s.fluid.x_vec_.shape)
    wx = s.walls[0].x_vec_
    got = orc.neighbour_counts(s.params(), x, wx)
    assert got == _bruteforce_counts(x, wx, s.kernel.influence_radius_)


def test_periodic_pairs_use_minimum_image(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.poiseuille_periodic_2d(n_across=10)
    prm = s.params()
    x = s.fluid.x_vec_
    ff, _ = orc.neighbour_counts(prm, x, None)
    L = s.meta["L"]
    rc = s.kernel.influence_radius_
    cnt = 0
    for i in range(len(x)):
        rv = x[i] - x[i + 1:]
        rv[:, 0] = np.where(rv[:, 0] > L / 2, rv[:, 0] - L, np.where(rv[:, 0] < -L / 2, rv[:, 0] + L, rv[:, 0]))
        cnt += int(np.count_nonzero(rv[:, 0] * rv[:, 0] + rv[:, 1] * rv[:, 1] <= rc * rc))
    assert ff == cnt


@pytest.mark.parametrize("case", ["lattice_2d", "jitter_2d", "jitter_3d", "periodic", "clamped"])
def test_neighbour_lists_equal_bruteforce(pkg, orc, case):
    # or_neighbour_lists (the per-particle pin the GPU's sets are compared with) against
    # an all-pairs restatement with the same rounding: d^2 = sum of products, k ascending
    from ethersph_gb300 import scenes
    rng = np.random.default_rng(3)
    period = None
    if case == "periodic":
        s = scenes.poiseuille_periodic_2d(n_across=10)
        period = s.meta["L"]
        x = s.fluid.x_vec_
    elif case == "jitter_3d":
        s = scenes.dam_break_3d(dx=0.05, tank=(0.8, 0.4, 0.4), column=(0.3, 0.2, 0.4))
        x = s.fluid.x_vec_ + 0.3 * 0.05 * rng.uniform(-1, 1, s.fluid.x_vec_.shape)
    else:
        s = scenes.dam_break_2d(dx=0.05)
        x = s.fluid.x_vec_ + (0.0 if case == "lattice_2d" else 0.3 * 0.05 * rng.uniform(-1, 1, s.fluid.x_vec_.shape))
    prm = s.params()
    if case == "clamped":  # the grid ends inside the fluid: keys clamped into the top cells
        prm.domain_hi[1] = 0.6
    x = np.ascontiguousarray(x)
    offsets, ids = orc.neighbour_lists(prm, x)
    rc = s.kernel.influence_radius_
    for i in range(len(x)):
        rv = x[i] - x
        if period is not None:
            rv[:, 0] = np.where(rv[:, 0] > period / 2, rv[:, 0] - period,
                                np.where(rv[:, 0] < -period / 2, rv[:, 0] + period, rv[:, 0]))
        d2 = rv[:, 0] * rv[:, 0] + rv[:, 1] * rv[:, 1]
        if x.shape[1] == 3:
            d2 = d2 + rv[:, 2] * rv[:, 2]
        expect = np.flatnonzero(d2 <= rc * rc)
        expect = expect[expect != i]
        assert np.array_equal(ids[offsets[i]:offsets[i + 1]], expect), i
    if case == "lattice_2d":  # interior particles: 28 neighbours within 3 dx (4 at exactly 3 dx)
        assert np.diff(offsets).max() == 28


# ---------------------------------------------------------------- step-level
def _run_both(orc, scene, steps):
    prm = scene.params()
    fluid, walls = orc.scene_arrays(scene)
    a = orc.run(prm, fluid, walls, 1, steps, mode=orc.GATHER, threads=1)
    b = orc.run(prm, fluid, walls, 1, steps, mode=orc.SCATTER, threads=1)
    return a, b


def _rel(a, b):
    """max |a - b| relative to the field's magnitude (L-inf norm)."""
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_scatter_and_gather_agree_dam_break(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_2d(dx=0.05)
    a, b = _run_both(orc, s, 31)  # crosses a density re-initialisation (step 30)
    assert len(a["rho"]) == len(b["rho"])
    for k in ("x", "v", "rho", "p"):
        assert _rel(a[k], b[k]) < 1e-11, k


def test_scatter_and_gather_agree_thermal_cavity(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.natural_convection_2d(n=24)
    a, b = _run_both(orc, s, 31)
    for k in ("x", "v", "rho", "t"):
        assert _rel(a[k], b[k]) < 1e-11, k


def test_scatter_and_gather_agree_3d(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_3d(dx=0.05, tank=(0.8, 0.4, 0.4), column=(0.3, 0.2, 0.4))
    a, b = _run_both(orc, s, 5)
    for k in ("x", "v", "rho"):
        assert _rel(a[k], b[k]) < 1e-11, k


def test_gather_threads_bitwise(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_2d(dx=0.05)
    prm = s.params()
    fluid, walls = orc.scene_arrays(s)
    a = orc.run(prm, fluid, walls, 1, 12, mode=orc.GATHER, threads=1)
    b = orc.run(prm, fluid, walls, 1, 12, mode=orc.GATHER, threads=4)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_mass_conserved_and_check_deletes(pkg, orc):
    from ethersph_gb300 import scenes
    s = scenes.dam_break_2d(dx=0.05)
    # a box that cuts the top rows of the column: they are removed at the check step
    s.check = pkg.AABBCheck(hi=(4.0, 1.5))
    prm = s.params()
    fluid, walls = orc.scene_arrays(s)
    out = orc.run(prm, fluid, walls, 1, 5, mode=orc.GATHER, threads=1)
    keep_expected = np.count_nonzero(fluid["x"][:, 1] <= 1.5 + 1e-3)
    assert len(out["rho"]) < len(fluid["rho"])
    assert abs(len(out["rho"]) - keep_expected) <= 20
    assert out["mass"].sum() == pytest.approx(fluid["mass"][: len(out["mass"])].sum(), rel=0.05)
    # without deletions the mass is conserved exactly (masses never change)
    out = orc.run(s.params(), fluid, walls, 1, 4, mode=orc.GATHER, threads=1)
    assert np.array_equal(np.sort(out["mass"]), np.sort(fluid["mass"]))


def test_hydrostatic_column_stays_near_rest(pkg, orc):
    # A settled column in a closed tank: 60 steps move nothing by more than a fraction of dx.
    from ethersph_gb300 import scenes
    s = scenes.dam_break_2d(dx=0.05, water_w=4.0, water_h=1.0, box_w=4.0, box_h=3.0)
    fluid, walls = orc.scene_arrays(s)
    out = orc.run(s.params(), fluid, walls, 1, 60, mode=orc.GATHER, threads=2)
    disp = np.abs(out["x"] - fluid["x"]).max()
    assert disp < 0.2 * 0.05


def test_cell_subdivisions_enumerate_the_same_pairs(pkg, orc):
    from ethersph_gb300 import scenes
    for s in (scenes.dam_break_2d(dx=0.05), scenes.dam_break_3d(dx=0.05, tank=(0.8, 0.4, 0.4),
                                                                 column=(0.3, 0.2, 0.4))):
        wx = s.walls[0].x_vec_
        a = orc.neighbour_counts(s.params(cell_subdivision=1), s.fluid.x_vec_, wx)
        for sub in (2, 3):
            assert orc.neighbour_counts(s.params(cell_subdivision=sub), s.fluid.x_vec_, wx) == a
        fluid, walls = orc.scene_arrays(s)
        ra = orc.run(s.params(cell_subdivision=1), fluid, walls, 1, 6, mode=orc.GATHER, threads=2)
        for sub in (2, 3):
            rb = orc.run(s.params(cell_subdivision=sub), fluid, walls, 1, 6, mode=orc.GATHER, threads=2)
            for k in ("x", "v", "rho"):
                assert _rel(ra[k], rb[k]) < 1e-12, (sub, k)


# ---------------------------------------------------------------- probe interpolation
def _probe_numpy(orc, kind, dim, rc, pts, x, m, rho, fields, none_value, period=0.0):
    # kernelValueInterpolation (VTPToDataFrame.jl:93-142) restated with Python loops
    out = np.full((len(fields), len(pts)), none_value)
    for i, p in enumerate(pts):
        kw, wv = 0.0, [0.0] * len(fields)
        for j in range(len(x)):
            rv = p - x[j]
            if period:
                rv[0] = rv[0] - period if rv[0] > period / 2 else (rv[0] + period if rv[0] < -period / 2 else rv[0])
            d2 = float(sum(rv[k] * rv[k] for k in range(dim)))
            if d2 > rc * rc:
                continue
            t = orc.kernel_value(kind, dim, rc, math.sqrt(d2)) * m[j] / rho[j]
            kw += t
            for f in range(len(fields)):
                wv[f] += t * fields[f][j]
        if kw > 0:
            out[:, i] = [w / kw for w in wv]
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_probe_oracle_matches_python_restatement(orc, dim):
    rng = np.random.default_rng(7)
    n, rc = 300, 0.3
    x = rng.uniform(0, 1, (n, dim))
    m = rng.uniform(0.5, 1.5, n)
    rho = rng.uniform(900, 1100, n)
    f1, f2 = rng.normal(size=n), x[:, 0] * 2.0 + 1.0
    pts = rng.uniform(-0.2, 1.2, (40, dim))
    got = orc.probe(2, dim, rc, pts, x, m, rho, [f1, f2], none_value=-7.0)
    ref = _probe_numpy(orc, 2, dim, rc, pts, x, m, rho, [f1, f2], -7.0)
    assert np.allclose(got, ref, rtol=1e-13, atol=0)
    far = orc.probe(2, dim, rc, np.full((1, dim), 10.0), x, m, rho, [f1], none_value=-7.0)
    assert far[0, 0] == -7.0  # no particle in range: none_value (VTPToDataFrame.jl:132-138)


def test_probe_oracle_reproduces_constants_and_wraps(orc):
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, (400, 2))
    m, rho = np.full(400, 2.0), rng.uniform(1, 2, 400)
    pts = rng.uniform(0.2, 0.8, (30, 2))
    c = orc.probe(0, 2, 0.2, pts, x, m, rho, [np.full(400, 3.25)])
    assert np.allclose(c, 3.25, rtol=1e-14)  # Shepard-normalised: constants are exact
    # periodic x: a point at x = 0.01 sees particles near x = 0.99 through the wrap
    edge = np.array([[0.01, 0.5]])
    plain = orc.probe(0, 2, 0.2, edge, x, m, rho, [x[:, 0]])
    wrapped = orc.probe(0, 2, 0.2, edge, x, m, rho, [x[:, 0]], periodic_x=True, period=1.0)
    ref = _probe_numpy(orc, 0, 2, 0.2, edge, x, m, rho, [x[:, 0]], float("nan"), period=1.0)
    assert np.allclose(wrapped, ref, rtol=1e-13) and wrapped[0, 0] > plain[0, 0]
