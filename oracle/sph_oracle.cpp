// sph_oracle.cpp — CPU restatement of the EtherSPHCPU.jl WCSPH time step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library and the
// timed CPU baseline; no product code path links, loads or calls it.
//
// It restates, in IEEE FP64 with the reference's expression order (compiled with
// -ffp-contract=off so that no a*b+c is fused), the Julia sources of the hot path
// (paths inside the EtherSPHCPU.jl project):
//   src/SPHKernel/SmoothKernel/{SmoothKernel,CubicSpline,Gaussian,WendlandC2,WendlandC4}.jl
//   src/Neighbour/Neighbour.jl
//   src/ParticleAction/Interaction/*.jl, SelfAction/*.jl, GroupAction/ReconstructValue.jl
//   src/Solve/{FluidWallSolve,FluidThermostaticWallSolve,
//              FluidCompulsiveThermostaticWallSolve,FluidVelocitySolve,
//              FluidInletOutletWallSolve}.jl (eachStep!)
//
// Two summation modes:
//   ORACLE_SCATTER: a half pair list (i<j, the CellListMap convention) with
//     materialised CommonNeighbour records and atomic scatter to both particles, as
//     the reference's @floop loops do.  With threads > 1 the summation order is
//     nondeterministic, exactly like the reference.  This is the CPU baseline.
//   ORACLE_GATHER: every particle sums its own full neighbour list, cells visited
//     in (z, y, x) order and particles inside a cell in ascending id.  This is the
//     GPU library's deterministic order, so the two can be compared bit for bit.
//
// Parity status: the reference's own tests pin only SmoothKernel.h_, the model's
// b_ and nu_0_, and CommonNeighbour.r_ (test/*.jl); they are reproduced in
// tests/test_oracle.py.  Step-level results are parity unpinned against the Julia
// code itself: no Julia toolchain exists here, and neighbour enumeration lives in
// the un-vendored, unpinned CellListMap.jl, restated here as d^2 <= r_cut^2 with
// d^2 = sum_k (x_ik - x_jk)^2, k ascending.
//
// Third-party numerics restated (Julia Base; Project.toml compat julia = "1.8"):
//   integer powers x^n with a non-literal or literal n >= 4 use Base's compensated
//   power by squaring (error-free products through fma); literal x^2 and x^3 are
//   x*x and x*x*x (Base.literal_pow).
//   LinearAlgebra.normalize(v) = v .* inv(norm(v)) with generic_norm2 (length < 32)
//   and the small-norm rescaling branch of __normalize!.
//   LinearAlgebra.dot on 2/3-vectors is restated as an ordered unfused sum.

#include "../include/ethersph_gpu.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
enum { ORACLE_GATHER = 0, ORACLE_SCATTER = 1 };
}

namespace {

// ---------------------------------------------------------------- Julia numerics
// Base ^(x::Float64, n::Integer): compensated power by squaring.  x is carried as
// an unevaluated sum (x, xnlo) and the running product as (y, ynlo); exact
// products come from fma.
double jl_powi(double x, int64_t n) {
    if (n == 0) return 1.0;
    if (n == 3) return x * x * x;
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    if (n < 0) {
        const double rx = 1.0 / x;
        if (n == -2) return rx * rx;
        if (std::isfinite(x)) xnlo = -std::fma(x, rx, -1.0) * rx;
        x = rx;
        n = -n;
    }
    while (n > 1) {
        if (n & 1) {
            const double err = std::fma(y, xnlo, x * ynlo);
            const double yh = x * y;
            const double yl = std::fma(x, y, -yh);
            y = yh;
            ynlo = yl + err;
        }
        const double err = x * 2.0 * xnlo;
        const double xh = x * x;
        const double xl = std::fma(x, x, -xh);
        x = xh;
        xnlo = xl + err;
        n >>= 1;
    }
    const double err = std::fma(y, xnlo, x * ynlo);
    return (std::isfinite(x) && std::isfinite(err)) ? std::fma(x, y, err) : x * y;
}

double jl_max0(double v) {  // Julia max(0, v) for Float64 v (WallForce.jl:16)
    if (std::isnan(v)) return v;
    return v > 0.0 ? v : 0.0;
}

// ---------------------------------------------------------------- SPHKernel
struct Kern {
    int kind;
    int dim;
    double rc, h, sigma, k0;
};

// SmoothKernel.jl:15-20 (table) and :37-48 (constructor)
bool make_kernel(int kind, int dim, double rc, Kern* k) {
    if (dim < 1 || dim > 3) return false;
    const double pi = M_PI;
    double ratio, c[3];
    switch (kind) {
        case SPH_KERNEL_CUBIC_SPLINE:
            ratio = 2.0; c[0] = 2.0 / 3.0; c[1] = 10.0 / 7.0 / pi; c[2] = 1.0 / pi; break;
        case SPH_KERNEL_GAUSSIAN:
            ratio = 3.0; c[0] = 1.0 / std::sqrt(pi); c[1] = 1.0 / pi; c[2] = 1.0 / std::sqrt(pi * pi * pi); break;
        case SPH_KERNEL_WENDLAND_C2:
            ratio = 2.0; c[0] = 0.0; c[1] = 7.0 / 4.0 / pi; c[2] = 21.0 / 16.0 / pi; break;
        case SPH_KERNEL_WENDLAND_C4:
            ratio = 2.0; c[0] = 5.0 / 8.0; c[1] = 9.0 / 4.0 / pi; c[2] = 495.0 / 256.0 / pi; break;
        default: return false;
    }
    k->kind = kind;
    k->dim = dim;
    k->rc = rc;
    k->h = rc / ratio;
    k->sigma = c[dim - 1] / jl_powi(k->h, dim);
    k->k0 = k->sigma;
    return true;
}

double kernel_value(double r, const Kern& k) {
    const double q = r / k.h;
    switch (k.kind) {
        case SPH_KERNEL_CUBIC_SPLINE:  // CubicSpline.jl:39-50
            if (q < 1.0) return k.sigma / 4.0 * (3.0 * (q * q) * (q - 2.0) + 4.0);
            if (q < 2.0) { const double t = 2.0 - q; return k.sigma / 4.0 * (t * t * t); }
            return 0.0;
        case SPH_KERNEL_GAUSSIAN:  // Gaussian.jl:31-38
            if (q < 3.0) return k.sigma * std::exp(-(q * q));
            return 0.0;
        case SPH_KERNEL_WENDLAND_C2:  // WendlandC2.jl:38-45
            if (q < 2.0) return k.sigma * jl_powi(2.0 - q, 4) * (1.0 + 2.0 * q) / 16.0;
            return 0.0;
        case SPH_KERNEL_WENDLAND_C4:  // WendlandC4.jl:38-45
            if (q < 2.0) return k.sigma * jl_powi(2.0 - q, 6) * (35.0 * (q * q) + 36.0 * q + 12.0) / 768.0;
            return 0.0;
    }
    return 0.0;
}

double kernel_gradient(double r, const Kern& k) {
    const double q = r / k.h;
    switch (k.kind) {
        case SPH_KERNEL_CUBIC_SPLINE:  // CubicSpline.jl:64-73
            if (q < 1.0) return k.sigma / k.h * 3.0 / 4.0 * q * (3.0 * q - 4.0);
            if (q < 2.0) { const double t = 2.0 - q; return -k.sigma / k.h * 3.0 / 4.0 * (t * t); }
            return 0.0;
        case SPH_KERNEL_GAUSSIAN:  // Gaussian.jl:49-56
            if (q < 3.0) return -2.0 * k.sigma / k.h * q * std::exp(-(q * q));
            return 0.0;
        case SPH_KERNEL_WENDLAND_C2:  // WendlandC2.jl:56-63
            if (q < 2.0) { const double t = 2.0 - q; return -k.sigma / k.h * 5.0 / 8.0 * q * (t * t * t); }
            return 0.0;
        case SPH_KERNEL_WENDLAND_C4:  // WendlandC4.jl:47-54
            if (q < 2.0) return -k.sigma / k.h * (35.0 / 96.0 * (q * q) + 7.0 / 48.0 * q) * jl_powi(2.0 - q, 5);
            return 0.0;
    }
    return 0.0;
}

// ---------------------------------------------------------------- small vectors
double dotv(const double* a, const double* b, int dim) {
    double s = a[0] * b[0];
    for (int k = 1; k < dim; ++k) s += a[k] * b[k];
    return s;
}

// LinearAlgebra.norm -> generic_norm2 for short vectors.
double jl_norm2(const double* a, int dim) {
    double maxabs = 0.0;
    for (int k = 0; k < dim; ++k) {
        const double v = std::fabs(a[k]);
        if (std::isnan(v)) return v;
        maxabs = v > maxabs ? v : maxabs;
    }
    if (maxabs == 0.0 || std::isinf(maxabs)) return maxabs;
    if (std::isfinite(dim * maxabs * maxabs) && maxabs * maxabs != 0.0) {
        double s = a[0] * a[0];
        for (int k = 1; k < dim; ++k) s += a[k] * a[k];
        return std::sqrt(s);
    }
    double s = 0.0;
    for (int k = 0; k < dim; ++k) { const double t = a[k] / maxabs; s += t * t; }
    return maxabs * std::sqrt(s);
}

// kernel_gradient * normalize(r_vec) with the NaN guard (Neighbour.jl:76-84).
void grad_vec(double dW, const double* rv, int dim, double* g) {
    const double nrm = jl_norm2(rv, dim);
    const double delta = 1.0 / 1.7976931348623157e308;  // inv(prevfloat(typemax(Float64)))
    double a[3];
    if (nrm >= delta) {
        const double inv = 1.0 / nrm;
        for (int k = 0; k < dim; ++k) a[k] = rv[k] * inv;
    } else {
        const double ed = DBL_EPSILON / delta;
        const double inv = 1.0 / (nrm * ed);
        for (int k = 0; k < dim; ++k) a[k] = (rv[k] * ed) * inv;
    }
    for (int k = 0; k < dim; ++k) {
        g[k] = dW * a[k];
        if (std::isnan(g[k])) g[k] = 0.0;
    }
}

// ---------------------------------------------------------------- scene state
struct Model {
    int solve, thermal, gamma, dim;
    double rho0, c0, p0, b, nu0, g[3], t0, kappa0, cp, beta, dt;
    int64_t reinit_interval, check_interval;
    int check_enabled, periodic_x;
    int cells_per_rc;  // grid cells per r_cut along each axis
    double lo[3], hi[3];
    double dlo[3], dhi[3];
};

struct Fluid {
    int64_t n = 0;
    std::vector<double> x, v, rho, p, c, m, gap, T, kappa, cp;
    std::vector<int64_t> id;
    std::vector<double> drho, dv, dT, sw, sws;
};

struct Walls {
    int64_t n = 0;
    std::vector<double> x, nrm, gap, T, kappa, v;
    std::vector<int32_t> kind;
};

// Cell grid shared by both modes.  Cell edge = r_cut * (1 + 1e-9) (the margin keeps
// every pair with d <= r_cut in adjacent cells under rounding); a periodic x axis is
// cut into floor(L / edge) equal cells.  Out-of-grid coordinates clamp to the edge
// cells, which keeps adjacency (clamping is monotone and 1-Lipschitz on cells).
struct Grid {
    int dim;
    int m;  // neighbour cells within +-m
    double lo[3], inv[3];
    int64_t n[3];
    int periodic_x;
    double period;
    int64_t ncells() const { return n[0] * n[1] * n[2]; }
    int64_t coord(double x, int a) const {
        const double u = (x - lo[a]) * inv[a];
        if (!(u >= 0.0)) return 0;
        const double f = std::floor(u);
        if (f >= (double)(n[a] - 1)) return n[a] - 1;
        return (int64_t)f;
    }
    int64_t key(const double* x) const {
        int64_t c[3] = {0, 0, 0};
        for (int a = 0; a < dim; ++a) c[a] = coord(x[a], a);
        return (c[2] * n[1] + c[1]) * n[0] + c[0];
    }
};

Grid make_grid(const Model& M, double rc) {
    Grid G;
    G.dim = M.dim;
    G.periodic_x = M.periodic_x;
    G.period = M.dhi[0] - M.dlo[0];
    G.m = M.cells_per_rc;
    const double edge = rc * (1.0 + 1e-9) / (double)G.m;
    for (int a = 0; a < 3; ++a) {
        G.lo[a] = M.dlo[a];
        if (a >= M.dim) { G.n[a] = 1; G.inv[a] = 0.0; continue; }
        if (a == 0 && M.periodic_x) {
            int64_t nx = (int64_t)std::floor(G.period / edge);
            if (nx < 2 * G.m + 1) nx = 0;  // rejected by load_model: too few periodic cells
            G.n[a] = nx;
            G.inv[a] = 1.0 / (G.period / (double)nx);
        } else {
            int64_t na = (int64_t)std::ceil((M.dhi[a] - M.dlo[a]) / edge);
            if (na < 1) na = 1;
            G.n[a] = na;
            G.inv[a] = 1.0 / edge;
        }
    }
    return G;
}

// r_vec = x_i - x_j, with the minimum image along a periodic x axis.
void rvec(const Grid& G, const double* xi, const double* xj, int dim, double* rv) {
    for (int k = 0; k < dim; ++k) rv[k] = xi[k] - xj[k];
    if (G.periodic_x) {
        const double half = 0.5 * G.period;
        if (rv[0] > half) rv[0] -= G.period;
        else if (rv[0] < -half) rv[0] += G.period;
    }
}

double dist2(const double* rv, int dim) {
    double s = rv[0] * rv[0];
    for (int k = 1; k < dim; ++k) s += rv[k] * rv[k];
    return s;
}

// Neighbour cells of cell (cx, cy, cz) in visiting order: z, then y, then x, each
// -m .. +m; cells off the grid are skipped, a periodic x axis wraps.
constexpr int kMaxCells = 343;  // (2 m + 1)^3 for m = 3
int neighbour_cells(const Grid& G, const int64_t c[3], int64_t out[kMaxCells]) {
    int cnt = 0;
    const int m = G.m;
    const int zr = G.dim == 3 ? m : 0;
    for (int dz = -zr; dz <= zr; ++dz) {
        const int64_t z = c[2] + dz;
        if (z < 0 || z >= G.n[2]) continue;
        for (int dy = -m; dy <= m; ++dy) {
            const int64_t y = c[1] + dy;
            if (y < 0 || y >= G.n[1]) continue;
            for (int dx = -m; dx <= m; ++dx) {
                int64_t x = c[0] + dx;
                if (G.periodic_x) {
                    x = (x + G.n[0]) % G.n[0];  // n[0] >= 2m+1, so no cell repeats
                } else if (x < 0 || x >= G.n[0]) {
                    continue;
                }
                out[cnt++] = (z * G.n[1] + y) * G.n[0] + x;
            }
        }
    }
    return cnt;
}

struct CellList {
    std::vector<int64_t> start;  // ncells + 1
    std::vector<int64_t> order;  // particle indices sorted by (cell, id)
};

CellList build_cells(const Grid& G, int64_t n, const double* x, int dim, const int64_t* id) {
    CellList L;
    const int64_t nc = G.ncells();
    std::vector<int64_t> key(n);
    for (int64_t i = 0; i < n; ++i) key[i] = G.key(x + i * dim);
    L.order.resize(n);
    for (int64_t i = 0; i < n; ++i) L.order[i] = i;
    std::sort(L.order.begin(), L.order.end(), [&](int64_t a, int64_t b) {
        if (key[a] != key[b]) return key[a] < key[b];
        return id ? id[a] < id[b] : a < b;
    });
    L.start.assign(nc + 1, 0);
    for (int64_t i = 0; i < n; ++i) L.start[key[i] + 1]++;
    for (int64_t c = 0; c < nc; ++c) L.start[c + 1] += L.start[c];
    return L;
}

void cell_of(const Grid& G, const double* x, int64_t c[3]) {
    c[0] = c[1] = c[2] = 0;
    for (int a = 0; a < G.dim; ++a) c[a] = G.coord(x[a], a);
}

// ---------------------------------------------------------------- pair physics
// One fluid-fluid pair seen from particle i (Neighbour.jl:63-86 values).
struct PairGeom {
    double r, rv[3], vv[3], W, dW, g[3];
};

void pair_geom(const Grid& G, const Kern& K, const double* xi, const double* xj, const double* vi,
               const double* vj, double d2, PairGeom* P) {
    const int dim = K.dim;
    P->r = std::sqrt(d2);
    rvec(G, xi, xj, dim, P->rv);
    for (int k = 0; k < dim; ++k) P->vv[k] = vi[k] - vj[k];
    P->W = kernel_value(P->r, K);
    P->dW = kernel_gradient(P->r, K);
    grad_vec(P->dW, P->rv, dim, P->g);
}

// pressureForce! fluid-fluid, PressureForce.jl:8-21: contribution to dv_i.
void pressure_ff(double pi_, double rhoi, double pj, double rhoj, double gapi, double gapj, double mj,
                 const PairGeom& P, const Kern& K, double* dvi) {
    double prho2 = pi_ / (rhoi * rhoi) + pj / (rhoj * rhoj);
    prho2 += std::fabs(prho2) * 0.01 * P.W / kernel_value((gapi + gapj) / 2.0, K);
    for (int k = 0; k < K.dim; ++k) dvi[k] += -mj * prho2 * P.g[k];
}

// viscosityForce! fluid-fluid, ViscosityForce.jl:8-25: contribution to dv_i.
void viscosity_ff(double rhoi, double rhoj, double mj, const PairGeom& P, const Kern& K, const Model& M,
                  double* dvi) {
    const double sum_rho = rhoi + rhoj;
    const double mui = M.nu0 * rhoi;
    const double muj = M.nu0 * rhoj;
    const double f = 4.0 * (mui + muj) * P.r * P.dW / (sum_rho * sum_rho) / (P.r * P.r + 0.01 * (K.h * K.h));
    for (int k = 0; k < K.dim; ++k) dvi[k] += mj * f * P.vv[k];
}

// thermalConduction! fluid-fluid, ThermalConduction.jl:8-22: contribution to dT_i.
double thermal_ff(double kappai, double kappaj, double rhoi, double rhoj, double Ti, double Tj, double mj,
                  double cpi, const PairGeom& P, const Kern& K) {
    const double keq = 2.0 * kappai * kappaj / (kappai + kappaj);
    const double dq = 2.0 * keq * P.r * P.dW / rhoi / rhoj / (P.r * P.r + 0.01 * (K.h * K.h)) * (Ti - Tj);
    return dq * mj / cpi;
}

// All wall terms for fluid particle i and wall particle w.
// wallForce!       WallForce.jl:8-30
// pressureForce!   PressureForce.jl:23-35 (not in FluidWallSolve, FluidWallSolve.jl:53-62)
// viscosityForce!  ViscosityForce.jl:27-46
// thermalConduction! ThermalConduction.jl:24-36 (thermostatic walls of thermal solves)
void wall_terms(const Grid& G, const Kern& K, const Model& M, const double* xi, const double* vi, double rhoi,
                double pi_, double ci, double mi, double gapi, double Ti, double kappai, const Walls& W, int64_t w,
                double d2, double* dvi, double* dTi) {
    const int dim = K.dim;
    PairGeom P;
    const double* vw = &W.v[w * dim];
    pair_geom(G, K, xi, &W.x[w * dim], vi, vw, d2, &P);  // relativeVelocityVector: v_i - v_w (v_w = 0 if fixed)
    const double* n = &W.nrm[w * dim];
    const double gw = W.gap[w];
    // wallForce!
    {
        const double psi = std::fabs(dotv(P.rv, n, dim));
        const double xi_ = std::sqrt(jl_max0(P.r * P.r - psi * psi));
        const double q = psi / gw;
        if (!(q > 1.0 || xi_ > gw)) {
            const double pxi = std::fabs((1.0 + std::cos(M_PI * xi_ / gw)) / 2.0);
            const double vert = dotv(P.vv, n, dim);
            const double beta = vert > 0.0 ? 0.0 : 1.0;
            const double rpsi = (0.01 * (ci * ci) + beta * ci * std::fabs(vert)) / K.h * std::fabs(1.0 - q) / std::sqrt(q);
            const double wf = rpsi * pxi;
            for (int k = 0; k < dim; ++k) dvi[k] += wf * n[k];
        }
    }
    // background pressure against the wall
    // (neither in the inlet/outlet solve, FluidInletOutletWallSolve.jl:121-124)
    if (M.solve != SPH_SOLVE_FLUID_WALL && M.solve != SPH_SOLVE_FLUID_INLET_OUTLET_WALL) {
        double prho2 = pi_ / (rhoi * rhoi) + M.p0 / (M.rho0 * M.rho0);
        prho2 += std::fabs(prho2) * 0.01 * P.W / kernel_value(gapi, K);
        for (int k = 0; k < dim; ++k) dvi[k] += -mi * prho2 * P.g[k];
    }
    // viscosity against the wall (tangential part)
    {
        const double sum_rho = 2.0 * rhoi;
        const double mui = M.nu0 * rhoi;
        const double f = 8.0 * mui * P.r * P.dW / (sum_rho * sum_rho) / (P.r * P.r + 0.01 * (K.h * K.h));
        const double vert = dotv(P.vv, n, dim);
        for (int k = 0; k < dim; ++k) dvi[k] += mi * f * (P.vv[k] - vert * n[k]);
    }
    // heat from a thermostatic wall
    if (M.thermal && W.kind[w] == SPH_WALL_THERMOSTATIC) {
        const double dq = 1.0 / M.cp * (kappai + W.kappa[w]) * P.r * P.dW / rhoi / M.rho0 /
                          (P.r * P.r + 0.01 * (K.h * K.h)) * (Ti - W.T[w]);
        *dTi += dq * mi;
    }
}

// ---------------------------------------------------------------- self actions
// updateDensity! UpdateDensity.jl:8-12 and updatePressure! UpdatePressure.jl:8-16
void density_pressure(Fluid& F, int64_t i, const Model& M) {
    F.rho[i] += F.drho[i] * M.dt;
    F.drho[i] = 0.0;
    const double rr = F.rho[i] / M.rho0;
    F.p[i] = M.b * (jl_powi(rr, M.gamma) - 1.0) + M.p0;
    F.c[i] = M.c0 * std::sqrt(jl_powi(rr, M.gamma - 1));
}

// updateTemperature! UpdateTemperature.jl:8-12, updateVelocity! UpdateVelocity.jl:15-23
// (body force g, or -g*beta*(T-T0) in thermal solves,
// FluidCompulsiveThermostaticWallSolve.jl:134-138), updatePosition! UpdatePosition.jl:8-14.
void integrate(Fluid& F, int64_t i, const Model& M, const Grid& G) {
    const int dim = M.dim;
    const double dt = M.dt;
    double body[3];
    if (M.thermal) {
        F.T[i] += dt * F.dT[i];
        F.dT[i] = 0.0;
        for (int k = 0; k < dim; ++k) body[k] = -M.g[k] * M.beta * (F.T[i] - M.t0);
    } else {
        for (int k = 0; k < dim; ++k) body[k] = M.g[k];
    }
    double* v = &F.v[i * dim];
    double* x = &F.x[i * dim];
    double* dv = &F.dv[i * dim];
    for (int k = 0; k < dim; ++k) v[k] += body[k] * dt;
    for (int k = 0; k < dim; ++k) v[k] += dv[k] * dt;
    for (int k = 0; k < dim; ++k) {
        x[k] += v[k] * dt - dv[k] * (dt * dt) / 2.0;
        dv[k] = 0.0;
    }
    if (G.periodic_x) {  // new feature: wrap into [lo, lo + L)
        if (x[0] >= G.lo[0] + G.period) x[0] -= G.period;
        else if (x[0] < G.lo[0]) x[0] += G.period;
    }
}

bool keep(const Model& M, const double* x) {
    if (!M.check_enabled) return true;
    for (int k = 0; k < M.dim; ++k)
        if (x[k] > M.hi[k] || x[k] < M.lo[k]) return false;
    return true;
}

void delete_outside(Fluid& F, const Model& M) {
    const int dim = M.dim;
    int64_t w = 0;
    for (int64_t i = 0; i < F.n; ++i) {
        if (!keep(M, &F.x[i * dim])) continue;
        if (w != i) {
            for (int k = 0; k < dim; ++k) {
                F.x[w * dim + k] = F.x[i * dim + k];
                F.v[w * dim + k] = F.v[i * dim + k];
            }
            F.rho[w] = F.rho[i]; F.p[w] = F.p[i]; F.c[w] = F.c[i]; F.m[w] = F.m[i]; F.gap[w] = F.gap[i];
            F.T[w] = F.T[i]; F.kappa[w] = F.kappa[i]; F.cp[w] = F.cp[i]; F.id[w] = F.id[i];
        }
        ++w;
    }
    F.n = w;
}

// ---------------------------------------------------------------- scatter mode
struct Nb {
    int64_t i, j;
    double d2;
    PairGeom P;
};

inline void atomic_add(double* a, double v) {
#pragma omp atomic
    *a += v;
}

// CellListMap-like half list (unique i<j) of fluid pairs and the full fluid-wall
// bipartite list, then findNeighbours! (Neighbour.jl:88-128).
void build_lists(const Grid& G, const Kern& K, const Fluid& F, const Walls& W, const CellList& CL,
                 const CellList& WL, std::vector<Nb>& ff, std::vector<Nb>& fw) {
    const int dim = K.dim;
    const double rc2 = K.rc * K.rc;
    const int64_t n = F.n;
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    std::vector<std::vector<Nb>> tff(nthreads), tfw(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const double* xi = &F.x[i * dim];
        int64_t c[3];
        cell_of(G, xi, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        for (int q = 0; q < nc; ++q) {
            for (int64_t s = CL.start[cells[q]]; s < CL.start[cells[q] + 1]; ++s) {
                const int64_t j = CL.order[s];
                if (j <= i) continue;
                double rv[3];
                rvec(G, xi, &F.x[j * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (d2 <= rc2) tff[tid].push_back(Nb{i, j, d2, {}});
            }
            if (W.n == 0) continue;
            for (int64_t s = WL.start[cells[q]]; s < WL.start[cells[q] + 1]; ++s) {
                const int64_t w = WL.order[s];
                double rv[3];
                rvec(G, xi, &W.x[w * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (d2 <= rc2) tfw[tid].push_back(Nb{i, w, d2, {}});
            }
        }
    }
    ff.clear();
    fw.clear();
    for (int t = 0; t < nthreads; ++t) {
        ff.insert(ff.end(), tff[t].begin(), tff[t].end());
        fw.insert(fw.end(), tfw[t].begin(), tfw[t].end());
    }
    const int64_t nff = (int64_t)ff.size(), nfw = (int64_t)fw.size();
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nff; ++q) {
        Nb& b = ff[q];
        pair_geom(G, K, &F.x[b.i * dim], &F.x[b.j * dim], &F.v[b.i * dim], &F.v[b.j * dim], b.d2, &b.P);
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nfw; ++q) {
        Nb& b = fw[q];
        pair_geom(G, K, &F.x[b.i * dim], &W.x[b.j * dim], &F.v[b.i * dim], &W.v[b.j * dim], b.d2, &b.P);
    }
}

void step_scatter(const Grid& G, const Kern& K, const Model& M, Fluid& F, const Walls& W, const CellList& WL,
                  int64_t step) {
    const int dim = K.dim;
    const int64_t n = F.n;
    CellList CL = build_cells(G, n, F.x.data(), dim, nullptr);
    std::vector<Nb> ff, fw;
    build_lists(G, K, F, W, CL, WL, ff, fw);
    const int64_t nff = (int64_t)ff.size(), nfw = (int64_t)fw.size();
    // continuity!  Continuity.jl:8-17
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nff; ++q) {
        const Nb& b = ff[q];
        const double drho = dotv(b.P.vv, b.P.g, dim);
        atomic_add(&F.drho[b.i], drho * F.m[b.j]);
        atomic_add(&F.drho[b.j], drho * F.m[b.i]);
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) density_pressure(F, i, M);
    // momentum (and heat) over fluid pairs: both particles of each pair
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nff; ++q) {
        const Nb& b = ff[q];
        const int64_t i = b.i, j = b.j;
        const PairGeom& P = b.P;
        double prho2 = F.p[i] / (F.rho[i] * F.rho[i]) + F.p[j] / (F.rho[j] * F.rho[j]);
        prho2 += std::fabs(prho2) * 0.01 * P.W / kernel_value((F.gap[i] + F.gap[j]) / 2.0, K);
        for (int k = 0; k < dim; ++k) {
            atomic_add(&F.dv[i * dim + k], -F.m[j] * prho2 * P.g[k]);
            atomic_add(&F.dv[j * dim + k], F.m[i] * prho2 * P.g[k]);
        }
        const double sum_rho = F.rho[i] + F.rho[j];
        const double mui = M.nu0 * F.rho[i], muj = M.nu0 * F.rho[j];
        const double f = 4.0 * (mui + muj) * P.r * P.dW / (sum_rho * sum_rho) / (P.r * P.r + 0.01 * (K.h * K.h));
        for (int k = 0; k < dim; ++k) {
            atomic_add(&F.dv[i * dim + k], F.m[j] * f * P.vv[k]);
            atomic_add(&F.dv[j * dim + k], -F.m[i] * f * P.vv[k]);
        }
        if (M.thermal) {
            const double keq = 2.0 * F.kappa[i] * F.kappa[j] / (F.kappa[i] + F.kappa[j]);
            const double dq = 2.0 * keq * P.r * P.dW / F.rho[i] / F.rho[j] / (P.r * P.r + 0.01 * (K.h * K.h)) *
                              (F.T[i] - F.T[j]);
            atomic_add(&F.dT[i], dq * F.m[j] / F.cp[i]);
            atomic_add(&F.dT[j], -dq * F.m[i] / F.cp[j]);
        }
    }
    // wall terms (one-sided)
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nfw; ++q) {
        const Nb& b = fw[q];
        const int64_t i = b.i;
        double dv[3] = {0, 0, 0}, dT = 0.0;
        wall_terms(G, K, M, &F.x[i * dim], &F.v[i * dim], F.rho[i], F.p[i], F.c[i], F.m[i], F.gap[i], F.T[i],
                   F.kappa[i], W, b.j, b.d2, dv, &dT);
        for (int k = 0; k < dim; ++k) atomic_add(&F.dv[i * dim + k], dv[k]);
        if (M.thermal) atomic_add(&F.dT[i], dT);
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) integrate(F, i, M, G);
    // reconstructScalar!(fluid, :rho_, fluid_neighbours)  ReconstructValue.jl:22-57
    if (M.reinit_interval > 0 && step % M.reinit_interval == 0) {
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < nff; ++q) {
            const Nb& b = ff[q];
            const int64_t i = b.i, j = b.j;
            atomic_add(&F.sw[i], b.P.W * F.m[j] / F.rho[j]);
            atomic_add(&F.sws[i], b.P.W * F.m[j] / F.rho[j] * F.rho[j]);
            atomic_add(&F.sw[j], b.P.W * F.m[i] / F.rho[i]);
            atomic_add(&F.sws[j], b.P.W * F.m[i] / F.rho[i] * F.rho[i]);
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            F.sw[i] += K.k0 * F.m[i] / F.rho[i];
            F.sws[i] += K.k0 * F.m[i] / F.rho[i] * F.rho[i];
            F.rho[i] = F.sws[i] / F.sw[i];
            F.sw[i] = 0.0;
            F.sws[i] = 0.0;
        }
    }
    if (M.check_enabled && M.check_interval > 0 && step % M.check_interval == 0) delete_outside(F, M);
}

// ---------------------------------------------------------------- gather mode
void permute(Fluid& F, const std::vector<int64_t>& order, int dim) {
    const int64_t n = F.n;
    auto perm1 = [&](std::vector<double>& a) {
        std::vector<double> b(n);
        for (int64_t k = 0; k < n; ++k) b[k] = a[order[k]];
        std::copy(b.begin(), b.end(), a.begin());
    };
    auto permd = [&](std::vector<double>& a) {
        std::vector<double> b((size_t)n * dim);
        for (int64_t k = 0; k < n; ++k)
            for (int q = 0; q < dim; ++q) b[k * dim + q] = a[order[k] * dim + q];
        std::copy(b.begin(), b.end(), a.begin());
    };
    permd(F.x); permd(F.v);
    perm1(F.rho); perm1(F.p); perm1(F.c); perm1(F.m); perm1(F.gap);
    perm1(F.T); perm1(F.kappa); perm1(F.cp);
    std::vector<int64_t> id(n);
    for (int64_t k = 0; k < n; ++k) id[k] = F.id[order[k]];
    std::copy(id.begin(), id.end(), F.id.begin());
}

void step_gather(const Grid& G, const Kern& K, const Model& M, Fluid& F, const Walls& W, const CellList& WL,
                 int64_t step) {
    const int dim = K.dim;
    const double rc2 = K.rc * K.rc;
    // sort by (cell, id): the GPU's storage order
    {
        CellList tmp = build_cells(G, F.n, F.x.data(), dim, F.id.data());
        permute(F, tmp.order, dim);
    }
    const int64_t n = F.n;
    CellList CL = build_cells(G, n, F.x.data(), dim, F.id.data());  // identity order now
    std::vector<double> x0(F.x);  // start-of-step positions (kernel values of the reinit)
    std::vector<double> v0(F.v);
    // continuity + density + EOS
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const double* xi = &x0[i * dim];
        int64_t c[3];
        cell_of(G, xi, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        double drho = 0.0;
        for (int q = 0; q < nc; ++q)
            for (int64_t j = CL.start[cells[q]]; j < CL.start[cells[q] + 1]; ++j) {
                if (j == i) continue;
                double rv[3];
                rvec(G, xi, &x0[j * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (!(d2 <= rc2)) continue;
                PairGeom P;
                pair_geom(G, K, xi, &x0[j * dim], &v0[i * dim], &v0[j * dim], d2, &P);
                drho += dotv(P.vv, P.g, dim) * F.m[j];
            }
        F.drho[i] = drho;
    }
    for (int64_t i = 0; i < n; ++i) density_pressure(F, i, M);
    // momentum + heat
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const double* xi = &x0[i * dim];
        int64_t c[3];
        cell_of(G, xi, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        double dv[3] = {0, 0, 0}, dT = 0.0;
        for (int q = 0; q < nc; ++q)
            for (int64_t j = CL.start[cells[q]]; j < CL.start[cells[q] + 1]; ++j) {
                if (j == i) continue;
                double rv[3];
                rvec(G, xi, &x0[j * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (!(d2 <= rc2)) continue;
                PairGeom P;
                pair_geom(G, K, xi, &x0[j * dim], &v0[i * dim], &v0[j * dim], d2, &P);
                pressure_ff(F.p[i], F.rho[i], F.p[j], F.rho[j], F.gap[i], F.gap[j], F.m[j], P, K, dv);
                viscosity_ff(F.rho[i], F.rho[j], F.m[j], P, K, M, dv);
                if (M.thermal) dT += thermal_ff(F.kappa[i], F.kappa[j], F.rho[i], F.rho[j], F.T[i], F.T[j], F.m[j],
                                                F.cp[i], P, K);
            }
        if (W.n > 0)
            for (int q = 0; q < nc; ++q)
                for (int64_t s = WL.start[cells[q]]; s < WL.start[cells[q] + 1]; ++s) {
                    const int64_t w = WL.order[s];
                    double rv[3];
                    rvec(G, xi, &W.x[w * dim], dim, rv);
                    const double d2 = dist2(rv, dim);
                    if (!(d2 <= rc2)) continue;
                    wall_terms(G, K, M, xi, &v0[i * dim], F.rho[i], F.p[i], F.c[i], F.m[i], F.gap[i], F.T[i],
                               F.kappa[i], W, w, d2, dv, &dT);
                }
        for (int k = 0; k < dim; ++k) F.dv[i * dim + k] = dv[k];
        F.dT[i] = dT;
    }
    // the heat of particle j must be read before any T changes: integrate afterwards
    for (int64_t i = 0; i < n; ++i) integrate(F, i, M, G);
    if (M.reinit_interval > 0 && step % M.reinit_interval == 0) {
        std::vector<double> rho_new(n);
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            const double* xi = &x0[i * dim];
            int64_t c[3];
            cell_of(G, xi, c);
            int64_t cells[kMaxCells];
            const int nc = neighbour_cells(G, c, cells);
            double sw = 0.0, sws = 0.0;
            for (int q = 0; q < nc; ++q)
                for (int64_t j = CL.start[cells[q]]; j < CL.start[cells[q] + 1]; ++j) {
                    if (j == i) continue;
                    double rv[3];
                    rvec(G, xi, &x0[j * dim], dim, rv);
                    const double d2 = dist2(rv, dim);
                    if (!(d2 <= rc2)) continue;
                    const double Wij = kernel_value(std::sqrt(d2), K);
                    sw += Wij * F.m[j] / F.rho[j];
                    sws += Wij * F.m[j] / F.rho[j] * F.rho[j];
                }
            sw += K.k0 * F.m[i] / F.rho[i];
            sws += K.k0 * F.m[i] / F.rho[i] * F.rho[i];
            rho_new[i] = sws / sw;
        }
        std::copy(rho_new.begin(), rho_new.end(), F.rho.begin());
    }
    if (M.check_enabled && M.check_interval > 0 && step % M.check_interval == 0) delete_outside(F, M);
}

// ---------------------------------------------------------------- inlet / outlet
// FluidInletOutletWallSolve.jl:8-262 in gather mode.  Buffer particles (inlet and
// outlet) are neighbours of the fluid in continuity and momentum with their own, frozen
// rho, p, c; after the step they move by x += v dt (updatePosition! with dv = 0).  The
// closures of the reference's keywords are restated as plane tests n.x > d (what the
// example's closures express, PoiseuilleFlow2D.jl:146-151), the modify closure as a
// shift.  Visiting order: fluid neighbours, then buffer neighbours (cells z, y, x; inside
// a cell by order), then walls, as the GPU sums them.
constexpr int64_t kOutletBit = int64_t(1) << 62;

struct Buffers {
    int64_t n = 0;
    std::vector<double> x, v, rho, p, c, m, gap;
    std::vector<int64_t> order;  // inlet k: k; outlet: kOutletBit | ...
};

struct BufRules {
    double in_n[3], in_d, in_shift[3], out_n[3], out_d, drop_n[3], drop_d;
    int64_t n_inlet, id_base, first_step;
};

bool beyond(const double* n, double d, const double* x, int dim) {
    double s = n[0] * x[0];
    for (int k = 1; k < dim; ++k) s = s + n[k] * x[k];
    return s > d;
}

void permute_buffers(Buffers& B, const std::vector<int64_t>& order, int dim) {
    const int64_t n = B.n;
    auto p1 = [&](std::vector<double>& a) {
        std::vector<double> b(n);
        for (int64_t k = 0; k < n; ++k) b[k] = a[order[k]];
        a.swap(b);
    };
    auto pd = [&](std::vector<double>& a) {
        std::vector<double> b((size_t)n * dim);
        for (int64_t k = 0; k < n; ++k)
            for (int q = 0; q < dim; ++q) b[k * dim + q] = a[order[k] * dim + q];
        a.swap(b);
    };
    pd(B.x); pd(B.v);
    p1(B.rho); p1(B.p); p1(B.c); p1(B.m); p1(B.gap);
    std::vector<int64_t> o(n);
    for (int64_t k = 0; k < n; ++k) o[k] = B.order[order[k]];
    B.order.swap(o);
}

void step_gather_io(const Grid& G, const Kern& K, const Model& M, Fluid& F, const Walls& W, const CellList& WL,
                    Buffers& B, const BufRules& R, int64_t step) {
    const int dim = K.dim;
    const double rc2 = K.rc * K.rc;
    {
        CellList tmp = build_cells(G, F.n, F.x.data(), dim, F.id.data());
        permute(F, tmp.order, dim);
        CellList tb = build_cells(G, B.n, B.x.data(), dim, B.order.data());
        permute_buffers(B, tb.order, dim);
    }
    const int64_t n = F.n;
    CellList CL = build_cells(G, n, F.x.data(), dim, F.id.data());
    CellList BL = build_cells(G, B.n, B.x.data(), dim, B.order.data());
    std::vector<double> x0(F.x), v0(F.v);
    // continuity: fluid, then buffer neighbours (FluidInletOutletWallSolve.jl:59-72)
    for (int64_t i = 0; i < n; ++i) {
        const double* xi = &x0[i * dim];
        int64_t c[3];
        cell_of(G, xi, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        double drho = 0.0;
        for (int q = 0; q < nc; ++q)
            for (int64_t j = CL.start[cells[q]]; j < CL.start[cells[q] + 1]; ++j) {
                if (j == i) continue;
                double rv[3];
                rvec(G, xi, &x0[j * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (!(d2 <= rc2)) continue;
                PairGeom P;
                pair_geom(G, K, xi, &x0[j * dim], &v0[i * dim], &v0[j * dim], d2, &P);
                drho += dotv(P.vv, P.g, dim) * F.m[j];
            }
        for (int q = 0; q < nc; ++q)
            for (int64_t b = BL.start[cells[q]]; b < BL.start[cells[q] + 1]; ++b) {
                double rv[3];
                rvec(G, xi, &B.x[b * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (!(d2 <= rc2)) continue;
                PairGeom P;
                pair_geom(G, K, xi, &B.x[b * dim], &v0[i * dim], &B.v[b * dim], d2, &P);
                drho += dotv(P.vv, P.g, dim) * B.m[b];
            }
        F.drho[i] = drho;
    }
    for (int64_t i = 0; i < n; ++i) density_pressure(F, i, M);
    // momentum: fluid, buffers (:125-158), walls (wallForce! + viscosity, :111-124)
    for (int64_t i = 0; i < n; ++i) {
        const double* xi = &x0[i * dim];
        int64_t c[3];
        cell_of(G, xi, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        double dv[3] = {0, 0, 0}, dT = 0.0;
        for (int q = 0; q < nc; ++q)
            for (int64_t j = CL.start[cells[q]]; j < CL.start[cells[q] + 1]; ++j) {
                if (j == i) continue;
                double rv[3];
                rvec(G, xi, &x0[j * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (!(d2 <= rc2)) continue;
                PairGeom P;
                pair_geom(G, K, xi, &x0[j * dim], &v0[i * dim], &v0[j * dim], d2, &P);
                pressure_ff(F.p[i], F.rho[i], F.p[j], F.rho[j], F.gap[i], F.gap[j], F.m[j], P, K, dv);
                viscosity_ff(F.rho[i], F.rho[j], F.m[j], P, K, M, dv);
            }
        for (int q = 0; q < nc; ++q)
            for (int64_t b = BL.start[cells[q]]; b < BL.start[cells[q] + 1]; ++b) {
                double rv[3];
                rvec(G, xi, &B.x[b * dim], dim, rv);
                const double d2 = dist2(rv, dim);
                if (!(d2 <= rc2)) continue;
                PairGeom P;
                pair_geom(G, K, xi, &B.x[b * dim], &v0[i * dim], &B.v[b * dim], d2, &P);
                pressure_ff(F.p[i], F.rho[i], B.p[b], B.rho[b], F.gap[i], B.gap[b], B.m[b], P, K, dv);
                viscosity_ff(F.rho[i], B.rho[b], B.m[b], P, K, M, dv);
            }
        if (W.n > 0)
            for (int q = 0; q < nc; ++q)
                for (int64_t s = WL.start[cells[q]]; s < WL.start[cells[q] + 1]; ++s) {
                    const int64_t w = WL.order[s];
                    double rv[3];
                    rvec(G, xi, &W.x[w * dim], dim, rv);
                    const double d2 = dist2(rv, dim);
                    if (!(d2 <= rc2)) continue;
                    wall_terms(G, K, M, xi, &v0[i * dim], F.rho[i], F.p[i], F.c[i], F.m[i], F.gap[i], F.T[i],
                               F.kappa[i], W, w, d2, dv, &dT);
                }
        for (int k = 0; k < dim; ++k) F.dv[i * dim + k] = dv[k];
    }
    for (int64_t i = 0; i < n; ++i) integrate(F, i, M, G);
    if (M.reinit_interval > 0 && step % M.reinit_interval == 0) {  // fluid neighbours only
        std::vector<double> rho_new(n);
        for (int64_t i = 0; i < n; ++i) {
            const double* xi = &x0[i * dim];
            int64_t c[3];
            cell_of(G, xi, c);
            int64_t cells[kMaxCells];
            const int nc = neighbour_cells(G, c, cells);
            double sw = 0.0, sws = 0.0;
            for (int q = 0; q < nc; ++q)
                for (int64_t j = CL.start[cells[q]]; j < CL.start[cells[q] + 1]; ++j) {
                    if (j == i) continue;
                    double rv[3];
                    rvec(G, xi, &x0[j * dim], dim, rv);
                    const double d2 = dist2(rv, dim);
                    if (!(d2 <= rc2)) continue;
                    const double Wij = kernel_value(std::sqrt(d2), K);
                    sw += Wij * F.m[j] / F.rho[j];
                    sws += Wij * F.m[j] / F.rho[j] * F.rho[j];
                }
            sw += K.k0 * F.m[i] / F.rho[i];
            sws += K.k0 * F.m[i] / F.rho[i] * F.rho[i];
            rho_new[i] = sws / sw;
        }
        std::copy(rho_new.begin(), rho_new.end(), F.rho.begin());
    }
    if (M.check_enabled && M.check_interval > 0 && step % M.check_interval == 0) delete_outside(F, M);
    // transfers (:162-257), decided on the state at the end of the step
    const int64_t srel = step - R.first_step;
    std::vector<char> to_outlet(F.n, 0);
    for (int64_t i = 0; i < F.n; ++i) to_outlet[i] = beyond(R.out_n, R.out_d, &F.x[i * dim], dim);
    Buffers NB;  // buffers after the move: survivors in place, then the fluid arrivals
    Fluid add;   // fluid copies of inlet particles
    for (int64_t b = 0; b < B.n; ++b) {
        double xn[3];
        for (int k = 0; k < dim; ++k) xn[k] = B.x[b * dim + k] + B.v[b * dim + k] * M.dt;
        if (!(B.order[b] & kOutletBit)) {
            if (beyond(R.in_n, R.in_d, xn, dim)) {
                for (int k = 0; k < dim; ++k) {
                    add.x.push_back(xn[k]);
                    add.v.push_back(B.v[b * dim + k]);
                }
                add.rho.push_back(B.rho[b]); add.p.push_back(B.p[b]); add.c.push_back(B.c[b]);
                add.m.push_back(B.m[b]); add.gap.push_back(B.gap[b]);
                add.id.push_back(R.id_base + srel * R.n_inlet + B.order[b]);
                ++add.n;
                for (int k = 0; k < dim; ++k) xn[k] += R.in_shift[k];
            }
        } else if (beyond(R.drop_n, R.drop_d, xn, dim)) {
            continue;  // out of the outlet
        }
        for (int k = 0; k < dim; ++k) {
            NB.x.push_back(xn[k]);
            NB.v.push_back(B.v[b * dim + k]);
        }
        NB.rho.push_back(B.rho[b]); NB.p.push_back(B.p[b]); NB.c.push_back(B.c[b]);
        NB.m.push_back(B.m[b]); NB.gap.push_back(B.gap[b]); NB.order.push_back(B.order[b]);
        ++NB.n;
    }
    Fluid keep;
    for (int64_t i = 0; i < F.n; ++i) {
        if (to_outlet[i]) {
            for (int k = 0; k < dim; ++k) {
                NB.x.push_back(F.x[i * dim + k]);
                NB.v.push_back(F.v[i * dim + k]);
            }
            NB.rho.push_back(F.rho[i]); NB.p.push_back(F.p[i]); NB.c.push_back(F.c[i]);
            NB.m.push_back(F.m[i]); NB.gap.push_back(F.gap[i]);
            NB.order.push_back(kOutletBit | ((srel + 1) << 32) | F.id[i]);
            ++NB.n;
            continue;
        }
        for (int k = 0; k < dim; ++k) {
            keep.x.push_back(F.x[i * dim + k]);
            keep.v.push_back(F.v[i * dim + k]);
        }
        keep.rho.push_back(F.rho[i]); keep.p.push_back(F.p[i]); keep.c.push_back(F.c[i]);
        keep.m.push_back(F.m[i]); keep.gap.push_back(F.gap[i]); keep.id.push_back(F.id[i]);
        ++keep.n;
    }
    for (int64_t a = 0; a < add.n; ++a) {
        for (int k = 0; k < dim; ++k) {
            keep.x.push_back(add.x[a * dim + k]);
            keep.v.push_back(add.v[a * dim + k]);
        }
        keep.rho.push_back(add.rho[a]); keep.p.push_back(add.p[a]); keep.c.push_back(add.c[a]);
        keep.m.push_back(add.m[a]); keep.gap.push_back(add.gap[a]); keep.id.push_back(add.id[a]);
        ++keep.n;
    }
    F.n = keep.n;
    F.x.swap(keep.x); F.v.swap(keep.v); F.rho.swap(keep.rho); F.p.swap(keep.p); F.c.swap(keep.c);
    F.m.swap(keep.m); F.gap.swap(keep.gap); F.id.swap(keep.id);
    F.T.assign(F.n, 0.0); F.kappa.assign(F.n, 0.0); F.cp.assign(F.n, 0.0);
    B = NB;
}

bool load_model(const SphParams* p, Model* M, Kern* K) {
    if (!p || (p->dim != 2 && p->dim != 3)) return false;
    if (!make_kernel(p->kernel, p->dim, p->influence_radius, K)) return false;
    // the handle's SmoothKernel fields are authoritative (they come from the Julia struct)
    K->h = p->h;
    K->sigma = p->sigma;
    K->k0 = p->kernel_0;
    M->solve = p->solve;
    M->thermal = p->thermal;
    M->gamma = p->gamma;
    M->dim = p->dim;
    M->rho0 = p->rho_0; M->c0 = p->c_0; M->p0 = p->p_0; M->b = p->b; M->nu0 = p->nu_0;
    for (int k = 0; k < 3; ++k) {
        M->g[k] = p->body_force[k];
        M->lo[k] = p->check_lo[k]; M->hi[k] = p->check_hi[k];
        M->dlo[k] = p->domain_lo[k]; M->dhi[k] = p->domain_hi[k];
    }
    M->t0 = p->t_0; M->kappa0 = p->kappa_0; M->cp = p->cp; M->beta = p->beta; M->dt = p->dt;
    M->reinit_interval = p->density_reinitialized_interval;
    M->check_interval = p->check_interval;
    M->check_enabled = p->check_enabled;
    M->periodic_x = p->periodic_x;
    // the library's default: 3 cells per r_cut
    M->cells_per_rc = p->cell_subdivision != 0 ? p->cell_subdivision : 3;
    if (M->cells_per_rc < 1 || M->cells_per_rc > 3) return false;
    if (M->periodic_x) {
        const double edge = K->rc * (1.0 + 1e-9) / (double)M->cells_per_rc;
        if (!(std::floor((M->dhi[0] - M->dlo[0]) / edge) >= 2.0 * M->cells_per_rc + 1.0)) return false;
    }
    return true;
}

}  // namespace

// ==================================================================== C entry points
extern "C" {

int or_smooth_kernel(int kind, int dim, double rc, double* h, double* sigma, double* k0) {
    Kern K;
    if (!make_kernel(kind, dim, rc, &K)) return 1;
    *h = K.h; *sigma = K.sigma; *k0 = K.k0;
    return 0;
}

double or_kernel_value(int kind, int dim, double rc, double r) {
    Kern K;
    if (!make_kernel(kind, dim, rc, &K)) return NAN;
    return kernel_value(r, K);
}

double or_kernel_gradient(int kind, int dim, double rc, double r) {
    Kern K;
    if (!make_kernel(kind, dim, rc, &K)) return NAN;
    return kernel_gradient(r, K);
}

double or_powi(double x, int64_t n) { return jl_powi(x, n); }

// CommonNeighbour! (Neighbour.jl:63-86) for one tuple (i, j, r): fills r_vec, v_vec,
// W, W', grad W.
int or_neighbour(int kind, int dim, double rc, const double* xi, const double* xj, const double* vi, const double* vj,
                 double r, double* rvec_out, double* vvec_out, double* W, double* dW, double* g) {
    Kern K;
    if (!make_kernel(kind, dim, rc, &K)) return 1;
    for (int k = 0; k < dim; ++k) {
        rvec_out[k] = xi[k] - xj[k];
        vvec_out[k] = vi[k] - vj[k];
    }
    *W = kernel_value(r, K);
    *dW = kernel_gradient(r, K);
    grad_vec(*dW, rvec_out, dim, g);
    return 0;
}

// Half pair list by brute force (all i<j with d^2 <= rc^2): the pair-set pin.
int64_t or_pair_list_bruteforce(int dim, int64_t n, const double* x, double rc, int64_t cap, int64_t* pairs) {
    const double rc2 = rc * rc;
    int64_t cnt = 0;
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i + 1; j < n; ++j) {
            double rv[3];
            for (int k = 0; k < dim; ++k) rv[k] = x[i * dim + k] - x[j * dim + k];
            if (dist2(rv, dim) <= rc2) {
                if (cnt < cap) { pairs[2 * cnt] = i; pairs[2 * cnt + 1] = j; }
                ++cnt;
            }
        }
    return cnt;
}

// Cell keys of the shared grid definition (the cell-assignment pin).
int or_cell_keys(const SphParams* prm, int64_t n, const double* x, int64_t* keys, int64_t* ncells) {
    Model M;
    Kern K;
    if (!load_model(prm, &M, &K)) return 1;
    Grid G = make_grid(M, K.rc);
    for (int64_t i = 0; i < n; ++i) keys[i] = G.key(x + i * M.dim);
    if (ncells) *ncells = G.ncells();
    return 0;
}

// Full neighbour list of every particle (all j != i with d^2 <= r_cut^2 at the positions
// x, minimum image along a periodic x axis), ids ascending, in CSR form: offsets[n + 1],
// ids[offsets[n]].  The per-particle pair-set pin of the neighbour search
// (CellListMap.neighborlist! + findNeighbours!, Neighbour.jl:88-128, turned into the
// full list each particle gathers over).  Returns the total, or -1 on a bad parameter
// block; ids are written only when the total fits cap.
int64_t or_neighbour_lists(const SphParams* prm, int64_t n, const double* x, int64_t cap, int64_t* offsets,
                           int64_t* ids) {
    Model M;
    Kern K;
    if (!load_model(prm, &M, &K)) return -1;
    Grid G = make_grid(M, K.rc);
    const int dim = M.dim;
    const double rc2 = K.rc * K.rc;
    CellList CL = build_cells(G, n, x, dim, nullptr);
    std::vector<std::vector<int64_t>> rows((size_t)n);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c[3];
        cell_of(G, x + i * dim, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        std::vector<int64_t>& row = rows[(size_t)i];
        for (int q = 0; q < nc; ++q)
            for (int64_t s = CL.start[cells[q]]; s < CL.start[cells[q] + 1]; ++s) {
                const int64_t j = CL.order[s];
                if (j == i) continue;
                double rv[3];
                rvec(G, x + i * dim, x + j * dim, dim, rv);
                if (dist2(rv, dim) <= rc2) row.push_back(j);
            }
        std::sort(row.begin(), row.end());
    }
    offsets[0] = 0;
    for (int64_t i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + (int64_t)rows[(size_t)i].size();
    const int64_t total = offsets[n];
    if (ids && total <= cap)
        for (int64_t i = 0; i < n; ++i) std::copy(rows[(size_t)i].begin(), rows[(size_t)i].end(), ids + offsets[i]);
    return total;
}

// Number of fluid neighbours (full list) of every particle and fluid-wall neighbours.
int or_neighbour_counts(const SphParams* prm, int64_t n, const double* x, int64_t nw, const double* wx,
                        int64_t* ff_pairs, int64_t* fw_pairs) {
    Model M;
    Kern K;
    if (!load_model(prm, &M, &K)) return 1;
    Grid G = make_grid(M, K.rc);
    const int dim = M.dim;
    const double rc2 = K.rc * K.rc;
    CellList CL = build_cells(G, n, x, dim, nullptr);
    CellList WL = build_cells(G, nw, wx, dim, nullptr);
    int64_t a = 0, b = 0;
#pragma omp parallel for reduction(+ : a, b) schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c[3];
        cell_of(G, x + i * dim, c);
        int64_t cells[kMaxCells];
        const int nc = neighbour_cells(G, c, cells);
        for (int q = 0; q < nc; ++q) {
            for (int64_t s = CL.start[cells[q]]; s < CL.start[cells[q] + 1]; ++s) {
                const int64_t j = CL.order[s];
                if (j <= i) continue;
                double rv[3];
                rvec(G, x + i * dim, x + j * dim, dim, rv);
                if (dist2(rv, dim) <= rc2) ++a;
            }
            if (nw)
                for (int64_t s = WL.start[cells[q]]; s < WL.start[cells[q] + 1]; ++s) {
                    double rv[3];
                    rvec(G, x + i * dim, wx + WL.order[s] * dim, dim, rv);
                    if (dist2(rv, dim) <= rc2) ++b;
                }
        }
    }
    *ff_pairs = a;
    *fw_pairs = b;
    return 0;
}

// Run steps first_step .. first_step+nsteps-1.  Fluid arrays are in/out in the
// caller's order (ids 0..n-1 on entry); deleted particles are removed and the
// survivors kept in their original relative order.  x, v: dim x n packed.
int or_run(const SphParams* prm, int mode, int threads, int64_t* n_fluid, double* x, double* v, double* rho, double* p,
           double* c, double* mass, double* gap, double* t, double* kappa, double* cp, int64_t n_wall,
           const double* wx, const double* wnormal, const double* wgap, const double* wt, const double* wkappa,
           const double* wv, const int32_t* wkind, int64_t first_step, int64_t nsteps) {
    Model M;
    Kern K;
    if (!load_model(prm, &M, &K)) return 1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const int dim = M.dim;
    Grid G = make_grid(M, K.rc);
    Fluid F;
    const int64_t n = *n_fluid;
    F.n = n;
    F.x.assign(x, x + n * dim);
    F.v.assign(v, v + n * dim);
    F.rho.assign(rho, rho + n);
    F.p.assign(p, p + n);
    F.c.assign(c, c + n);
    F.m.assign(mass, mass + n);
    F.gap.assign(gap, gap + n);
    if (M.thermal) {
        F.T.assign(t, t + n);
        F.kappa.assign(kappa, kappa + n);
        F.cp.assign(cp, cp + n);
    } else {
        F.T.assign(n, 0.0);
        F.kappa.assign(n, 0.0);
        F.cp.assign(n, 0.0);
    }
    F.id.resize(n);
    for (int64_t i = 0; i < n; ++i) F.id[i] = i;
    F.drho.assign(n, 0.0);
    F.dv.assign(n * dim, 0.0);
    F.dT.assign(n, 0.0);
    F.sw.assign(n, 0.0);
    F.sws.assign(n, 0.0);

    Walls W;
    W.n = n_wall;
    if (n_wall > 0) {
        W.x.assign(wx, wx + n_wall * dim);
        W.nrm.assign(wnormal, wnormal + n_wall * dim);
        W.gap.assign(wgap, wgap + n_wall);
        W.T.assign(n_wall, 0.0);
        W.kappa.assign(n_wall, 0.0);
        W.v.assign(n_wall * dim, 0.0);
        W.kind.assign(wkind, wkind + n_wall);
        for (int64_t w = 0; w < n_wall; ++w) {
            if (W.kind[w] == SPH_WALL_THERMOSTATIC) {
                W.T[w] = wt ? wt[w] : 0.0;
                W.kappa[w] = wkappa ? wkappa[w] : 0.0;
            }
            if (W.kind[w] == SPH_WALL_STATIC_VELOCITY && wv)
                for (int k = 0; k < dim; ++k) W.v[w * dim + k] = wv[w * dim + k];
        }
    }
    std::vector<int64_t> wid(n_wall);
    for (int64_t w = 0; w < n_wall; ++w) wid[w] = w;
    CellList WL = build_cells(G, n_wall, W.x.data(), dim, wid.data());

    for (int64_t s = first_step; s < first_step + nsteps; ++s) {
        if (mode == ORACLE_SCATTER) step_scatter(G, K, M, F, W, WL, s);
        else step_gather(G, K, M, F, W, WL, s);
        F.drho.assign(F.n, 0.0);
        F.dv.assign(F.n * dim, 0.0);
        F.dT.assign(F.n, 0.0);
        F.sw.assign(F.n, 0.0);
        F.sws.assign(F.n, 0.0);
    }
    // back to ascending id (the caller's order with deletions removed)
    std::vector<int64_t> order(F.n);
    for (int64_t k = 0; k < F.n; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return F.id[a] < F.id[b]; });
    permute(F, order, dim);
    *n_fluid = F.n;
    std::copy(F.x.begin(), F.x.begin() + F.n * dim, x);
    std::copy(F.v.begin(), F.v.begin() + F.n * dim, v);
    std::copy(F.rho.begin(), F.rho.begin() + F.n, rho);
    std::copy(F.p.begin(), F.p.begin() + F.n, p);
    std::copy(F.c.begin(), F.c.begin() + F.n, c);
    std::copy(F.m.begin(), F.m.begin() + F.n, mass);
    std::copy(F.gap.begin(), F.gap.begin() + F.n, gap);
    if (M.thermal) {
        std::copy(F.T.begin(), F.T.begin() + F.n, t);
        std::copy(F.kappa.begin(), F.kappa.begin() + F.n, kappa);
        std::copy(F.cp.begin(), F.cp.begin() + F.n, cp);
    }
    return 0;
}

// The inlet/outlet solve in gather mode.  Fluid (x, v: dim x cap; rho, p, c, mass,
// gap: cap) is replaced by the fluid at the end, in ascending id (uploaded ids 0..n-1,
// inlet copies after them); inlet arrays (n_in) by the inlet particles in index order;
// outlet arrays (capacity out_cap) by the outlet particles in arrival order; ids_out (cap)
// receives the fluid ids.  Returns 1 on bad parameters, 2 when a capacity is too small.
int or_run_io(const SphParams* prm, int64_t* n_fluid, int64_t cap, double* x, double* v, double* rho, double* p,
              double* c, double* mass, double* gap, int64_t n_wall, const double* wx, const double* wnormal,
              const double* wgap, const int32_t* wkind, const SphBufferRules* rules, int64_t n_in, double* ix,
              double* iv, double* irho, double* ip, double* ic, double* imass, double* igap, int64_t* n_out,
              int64_t out_cap, double* ox, double* ov, double* orho, double* op, double* oc, double* omass,
              double* ogap, int64_t first_step, int64_t nsteps, int64_t* ids_out) {
    Model M;
    Kern K;
    if (!load_model(prm, &M, &K) || M.thermal || !rules) return 1;
    const int dim = M.dim;
    Grid G = make_grid(M, K.rc);
    Fluid F;
    const int64_t n = *n_fluid;
    F.n = n;
    F.x.assign(x, x + n * dim); F.v.assign(v, v + n * dim);
    F.rho.assign(rho, rho + n); F.p.assign(p, p + n); F.c.assign(c, c + n);
    F.m.assign(mass, mass + n); F.gap.assign(gap, gap + n);
    F.T.assign(n, 0.0); F.kappa.assign(n, 0.0); F.cp.assign(n, 0.0);
    F.id.resize(n);
    for (int64_t i = 0; i < n; ++i) F.id[i] = i;
    Walls W;
    W.n = n_wall;
    if (n_wall > 0) {
        W.x.assign(wx, wx + n_wall * dim);
        W.nrm.assign(wnormal, wnormal + n_wall * dim);
        W.gap.assign(wgap, wgap + n_wall);
        W.T.assign(n_wall, 0.0);
        W.kappa.assign(n_wall, 0.0);
        W.v.assign(n_wall * dim, 0.0);
        W.kind.assign(wkind, wkind + n_wall);
    }
    std::vector<int64_t> wid(n_wall);
    for (int64_t w = 0; w < n_wall; ++w) wid[w] = w;
    CellList WL = build_cells(G, n_wall, W.x.data(), dim, wid.data());
    Buffers B;
    const int64_t no = *n_out;
    B.n = n_in + no;
    for (int64_t b = 0; b < n_in; ++b) {
        for (int k = 0; k < dim; ++k) { B.x.push_back(ix[b * dim + k]); B.v.push_back(iv[b * dim + k]); }
        B.rho.push_back(irho[b]); B.p.push_back(ip[b]); B.c.push_back(ic[b]); B.m.push_back(imass[b]);
        B.gap.push_back(igap[b]); B.order.push_back(b);
    }
    for (int64_t b = 0; b < no; ++b) {
        for (int k = 0; k < dim; ++k) { B.x.push_back(ox[b * dim + k]); B.v.push_back(ov[b * dim + k]); }
        B.rho.push_back(orho[b]); B.p.push_back(op[b]); B.c.push_back(oc[b]); B.m.push_back(omass[b]);
        B.gap.push_back(ogap[b]); B.order.push_back(kOutletBit | b);
    }
    BufRules R;
    for (int k = 0; k < 3; ++k) {
        R.in_n[k] = rules->inlet_normal[k]; R.in_shift[k] = rules->inlet_shift[k];
        R.out_n[k] = rules->outlet_normal[k]; R.drop_n[k] = rules->drop_normal[k];
    }
    R.in_d = rules->inlet_offset; R.out_d = rules->outlet_offset; R.drop_d = rules->drop_offset;
    R.n_inlet = n_in; R.id_base = n; R.first_step = first_step;
    for (int64_t s = first_step; s < first_step + nsteps; ++s) {
        F.drho.assign(F.n, 0.0); F.dv.assign(F.n * dim, 0.0); F.dT.assign(F.n, 0.0);
        F.sw.assign(F.n, 0.0); F.sws.assign(F.n, 0.0);
        step_gather_io(G, K, M, F, W, WL, B, R, s);
    }
    std::vector<int64_t> ord(F.n);
    for (int64_t k = 0; k < F.n; ++k) ord[k] = k;
    std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return F.id[a] < F.id[b]; });
    permute(F, ord, dim);
    std::vector<int64_t> bo(B.n);
    for (int64_t k = 0; k < B.n; ++k) bo[k] = k;
    std::sort(bo.begin(), bo.end(), [&](int64_t a, int64_t b) { return B.order[a] < B.order[b]; });
    permute_buffers(B, bo, dim);
    int64_t n_inlet_end = 0;
    while (n_inlet_end < B.n && !(B.order[n_inlet_end] & kOutletBit)) ++n_inlet_end;
    const int64_t n_outlet_end = B.n - n_inlet_end;
    *n_fluid = F.n;
    *n_out = n_outlet_end;
    if (F.n > cap || n_outlet_end > out_cap || n_inlet_end != n_in) return 2;
    std::copy(F.x.begin(), F.x.end(), x); std::copy(F.v.begin(), F.v.end(), v);
    std::copy(F.rho.begin(), F.rho.end(), rho); std::copy(F.p.begin(), F.p.end(), p);
    std::copy(F.c.begin(), F.c.end(), c); std::copy(F.m.begin(), F.m.end(), mass);
    std::copy(F.gap.begin(), F.gap.end(), gap);
    if (ids_out) std::copy(F.id.begin(), F.id.end(), ids_out);
    for (int64_t b = 0; b < B.n; ++b) {
        const bool in = b < n_inlet_end;
        const int64_t q = in ? b : b - n_inlet_end;
        double* xs = in ? ix : ox;
        double* vs = in ? iv : ov;
        for (int k = 0; k < dim; ++k) { xs[q * dim + k] = B.x[b * dim + k]; vs[q * dim + k] = B.v[b * dim + k]; }
        (in ? irho : orho)[q] = B.rho[b];
        (in ? ip : op)[q] = B.p[b];
        (in ? ic : oc)[q] = B.c[b];
        (in ? imass : omass)[q] = B.m[b];
        (in ? igap : ogap)[q] = B.gap[b];
    }
    return 0;
}

// kernelValueInterpolation (src/DataIO/VTPToDataFrame.jl:93-142) by brute force over
// the fluid: for every point i and every particle j with d(i, j)^2 <= rc^2,
//   kw_i += W m_j / rho_j,  wv_i += W m_j / rho_j * f_j  (VTPToDataFrame.jl:115-120),
// result wv_i / kw_i, or none_value where kw_i is not > 0 (:132-138).  A periodic x axis
// takes the nearest image, as the step's pair search does.  fields: n_fields arrays of
// n values; out: n_fields x np.
int or_probe(int kind, int dim, double rc, int periodic_x, double period, int64_t np, const double* pts, int64_t n,
             const double* x, const double* mass, const double* rho, int n_fields, const double* const* fields,
             double none_value, double* out) {
    Kern K;
    if (!make_kernel(kind, dim, rc, &K) || n_fields < 0) return 1;
    const double rc2 = rc * rc;
    std::vector<double> wv((size_t)n_fields);
    for (int64_t i = 0; i < np; ++i) {
        double kw = 0.0;
        std::fill(wv.begin(), wv.end(), 0.0);
        for (int64_t j = 0; j < n; ++j) {
            double rv[3];
            for (int k = 0; k < dim; ++k) rv[k] = pts[i * dim + k] - x[j * dim + k];
            if (periodic_x) {
                if (rv[0] > 0.5 * period) rv[0] -= period;
                else if (rv[0] < -0.5 * period) rv[0] += period;
            }
            const double d2 = dist2(rv, dim);
            if (!(d2 <= rc2)) continue;
            const double t = kernel_value(std::sqrt(d2), K) * mass[j] / rho[j];
            kw += t;
            for (int f = 0; f < n_fields; ++f) wv[(size_t)f] += t * fields[f][j];
        }
        for (int f = 0; f < n_fields; ++f) out[f * np + i] = kw > 0.0 ? wv[(size_t)f] / kw : none_value;
    }
    return 0;
}

}  // extern "C"
