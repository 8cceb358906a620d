// sph_physics.cuh — FP64 pair physics of the WCSPH step, in the reference's IEEE
// operation order.  Compiled with -fmad=false so that no a*b+c is contracted; with
// the sequential per-particle neighbour order this makes a step reproducible bit for
// bit across runs and comparable bit for bit with a CPU restatement (up to the last
// ulp of cos/exp, the only library functions on the path).
#pragma once

#include "sph_device.cuh"

namespace sph {

// ---------------------------------------------------------------- SPHKernel
// W(r) and dW/dr.  CubicSpline.jl:39-73, Gaussian.jl:31-56, WendlandC2.jl:38-63,
// WendlandC4.jl:38-54.  q = r/h is formed once (the reference forms the same value
// twice).  kw_a / kg_a are the leading constant products of each formula, formed on
// the host in the same order.
template <int KK>
__device__ __forceinline__ void kernel_wdw(double r, const SceneDev& S, double& W, double& dW) {
    const double q = r / S.h;
    if (KK == SPH_KERNEL_CUBIC_SPLINE) {
        if (q < 1.0) {
            W = S.kw_a * (3.0 * (q * q) * (q - 2.0) + 4.0);
            dW = S.kg_a * q * (3.0 * q - 4.0);
        } else if (q < 2.0) {
            const double t = 2.0 - q;
            W = S.kw_a * (t * t * t);
            dW = -S.kg_a * (t * t);
        } else {
            W = 0.0;
            dW = 0.0;
        }
    } else if (KK == SPH_KERNEL_GAUSSIAN) {
        if (q < 3.0) {
            const double e = exp(-(q * q));
            W = S.kw_a * e;
            dW = S.kg_a * q * e;
        } else {
            W = 0.0;
            dW = 0.0;
        }
    } else if (KK == SPH_KERNEL_WENDLAND_C2) {
        if (q < 2.0) {
            const double t = 2.0 - q;
            W = S.kw_a * jl_powi(t, 4) * (1.0 + 2.0 * q) * 0.0625;  // /16 is exact as *2^-4
            dW = S.kg_a * q * (t * t * t);
        } else {
            W = 0.0;
            dW = 0.0;
        }
    } else {  // WendlandC4
        if (q < 2.0) {
            const double t = 2.0 - q;
            W = S.kw_a * jl_powi(t, 6) * (35.0 * (q * q) + 36.0 * q + 12.0) / 768.0;
            dW = S.kg_a * (35.0 / 96.0 * (q * q) + 7.0 / 48.0 * q) * jl_powi(t, 5);
        } else {
            W = 0.0;
            dW = 0.0;
        }
    }
}

template <int KK>
__device__ __forceinline__ double kernel_w(double r, const SceneDev& S) {
    const double q = r / S.h;
    if (KK == SPH_KERNEL_CUBIC_SPLINE) {
        if (q < 1.0) return S.kw_a * (3.0 * (q * q) * (q - 2.0) + 4.0);
        if (q < 2.0) {
            const double t = 2.0 - q;
            return S.kw_a * (t * t * t);
        }
        return 0.0;
    } else if (KK == SPH_KERNEL_GAUSSIAN) {
        if (q < 3.0) return S.kw_a * exp(-(q * q));
        return 0.0;
    } else if (KK == SPH_KERNEL_WENDLAND_C2) {
        if (q < 2.0) return S.kw_a * jl_powi(2.0 - q, 4) * (1.0 + 2.0 * q) * 0.0625;
        return 0.0;
    } else {
        if (q < 2.0) return S.kw_a * jl_powi(2.0 - q, 6) * (35.0 * (q * q) + 36.0 * q + 12.0) / 768.0;
        return 0.0;
    }
}

// ---------------------------------------------------------------- pair geometry
template <int DIM>
struct Pair {
    double rv[DIM];
    double d2;
};

template <int DIM, typename V>
__device__ __forceinline__ void make_rvec(const V& xi, const V& xj, const SceneDev& S, double rv[DIM]) {
    rv[0] = xi.x - xj.x;
    rv[1] = xi.y - xj.y;
    if (DIM == 3) rv[DIM - 1] = comp(xi, DIM - 1) - comp(xj, DIM - 1);
    if (S.periodic_x) {
        if (rv[0] > S.half_period) rv[0] -= S.period;
        else if (rv[0] < -S.half_period) rv[0] += S.period;
    }
}

// |r|^2 = sum over k ascending of r_k^2, each product and sum rounded on its own (no
// fused multiply-add in any translation unit): the pair predicate d^2 <= r_cut^2 then
// decides every pair as the reference's restatement does, also on lattices where pairs
// sit at exactly r_cut.
template <int DIM>
__device__ __forceinline__ double norm_sq(const double rv[DIM]) {
    double s = __dadd_rn(__dmul_rn(rv[0], rv[0]), __dmul_rn(rv[1], rv[1]));
    if (DIM == 3) s = __dadd_rn(s, __dmul_rn(rv[DIM - 1], rv[DIM - 1]));
    return s;
}

// grad W = dW * normalize(r_vec), NaN components -> 0 (Neighbour.jl:76-84).
// normalize: LinearAlgebra generic_norm2 + __normalize!; for ordinary magnitudes
// the norm is sqrt(d2) = r bit for bit.
template <int DIM>
__device__ __forceinline__ void grad_vec(double dW, double r, const double rv[DIM], double g[DIM]) {
    double maxabs = fabs(rv[0]);
    bool nan_in = isnan(rv[0]);
#pragma unroll
    for (int k = 1; k < DIM; ++k) {
        const double a = fabs(rv[k]);
        nan_in |= isnan(a);
        maxabs = a > maxabs ? a : maxabs;
    }
    double nrm;
    if (nan_in) {
        nrm = CUDART_NAN;
    } else if (maxabs == 0.0 || isinf(maxabs)) {
        nrm = maxabs;
    } else if (isfinite((double)DIM * maxabs * maxabs) && maxabs * maxabs != 0.0) {
        nrm = r;
    } else {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            const double t = rv[k] / maxabs;
            s += t * t;
        }
        nrm = maxabs * sqrt(s);
    }
    const double delta = 1.0 / 1.7976931348623157e308;
    double a[DIM];
    if (nrm >= delta) {
        const double inv = 1.0 / nrm;
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] = rv[k] * inv;
    } else {
        const double ed = 2.220446049250313e-16 / delta;
        const double inv = 1.0 / (nrm * ed);
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] = (rv[k] * ed) * inv;
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        const double gk = dW * a[k];
        g[k] = isnan(gk) ? 0.0 : gk;
    }
}

template <int DIM>
__device__ __forceinline__ double dotd(const double a[DIM], const double b[DIM]) {
    double s = a[0] * b[0] + a[1] * b[1];
    if (DIM == 3) s += a[DIM - 1] * b[DIM - 1];
    return s;
}

// ---------------------------------------------------------------- neighbour walk
// Visits the neighbour cells of cell c (within +-reach cells on every axis) in (z, y, x)
// order, each x-run of up to 2 reach + 1 cells as one contiguous range of the sorted
// arrays (cells of a row are adjacent in key space).  A periodic x axis visits its cells
// one by one (wrapping; it has at least 2 reach + 1 cells, so none repeats).
template <int DIM, typename F>
__device__ __forceinline__ void walk_cells(const SceneDev& S, const int32_t* __restrict__ start, const int32_t c[3],
                                           F&& f) {
    const int m = S.reach;
    const int zr = DIM == 3 ? m : 0;
    for (int dz = -zr; dz <= zr; ++dz) {
        const int z = c[2] + dz;
        if (DIM == 3 && (z < 0 || z >= S.n[2])) continue;
        for (int dy = -m; dy <= m; ++dy) {
            const int y = c[1] + dy;
            if (y < 0 || y >= S.n[1]) continue;
            const int row = S.cell_off + (z * S.n[1] + y) * S.n[0];
            if (!S.periodic_x) {
                const int x0 = c[0] > m ? c[0] - m : 0;
                const int x1 = c[0] + m < S.n[0] ? c[0] + m : S.n[0] - 1;
                f(__ldg(start + row + x0), __ldg(start + row + x1 + 1));
            } else {
                for (int dx = -m; dx <= m; ++dx) {
                    int x = c[0] + dx;
                    x = x < 0 ? x + S.n[0] : (x >= S.n[0] ? x - S.n[0] : x);
                    f(__ldg(start + row + x), __ldg(start + row + x + 1));
                }
            }
        }
    }
}

// The same walk for the gathers of the FP64 form, with stencil pruning: in each neighbour
// row only the x cells whose extent comes within r_cut of the particle are visited, and a
// row whose y (and z) extent lies beyond r_cut is skipped.  fu is the particle's position
// in cell units relative to its cell c (FP32: the bounds cost a few FP32 operations a row,
// where FP64 work is 64 times slower on GB300), and the test keeps a relative margin of
// 1e-4 on r_cut^2, far above the FP32 rounding of positions within a few cells.  Only
// candidates the distance test would reject are left out, in a walk that keeps the order
// of the others: the sums are bitwise those of walk_cells.  Rows on the y/z grid boundary
// and the grid's first and last x cells may hold particles clamped from outside the grid
// (beyond their cell's extent) and are never trimmed; a periodic axis is walked whole.
template <int DIM, typename F>
__device__ __forceinline__ void walk_cells_pruned(const SceneDev& S, const int32_t* __restrict__ start,
                                                  const int32_t c[3], const float fu[3], F&& f) {
    if (S.periodic_x) {
        walk_cells<DIM>(S, start, c, f);
        return;
    }
    const int m = S.reach;
    const int zr = DIM == 3 ? m : 0;
    const float r2 = S.rc2_f * 1.0001f;
    const float ey = S.cell_f[1], ez = S.cell_f[2];
    const float inv_ex = S.inv_cell_fx;
    for (int dz = -zr; dz <= zr; ++dz) {
        const int z = c[2] + dz;
        if (DIM == 3 && (z < 0 || z >= S.n[2])) continue;
        float gz2 = 0.f;
        if (DIM == 3 && z > 0 && z < S.n[2] - 1) {
            const float gz = fmaxf(fmaxf((float)dz - fu[2], fu[2] - (float)(dz + 1)), 0.f) * ez;
            gz2 = gz * gz;
        }
        for (int dy = -m; dy <= m; ++dy) {
            const int y = c[1] + dy;
            if (y < 0 || y >= S.n[1]) continue;
            const int row = S.cell_off + (z * S.n[1] + y) * S.n[0];
            int x0 = c[0] > m ? c[0] - m : 0;
            int x1 = c[0] + m < S.n[0] ? c[0] + m : S.n[0] - 1;
            const bool edge_row = y == 0 || y == S.n[1] - 1 || (DIM == 3 && (z == 0 || z == S.n[2] - 1));
            if (!edge_row) {
                const float gy = fmaxf(fmaxf((float)dy - fu[1], fu[1] - (float)(dy + 1)), 0.f) * ey;
                const float rem = r2 - (gy * gy + gz2);
                if (rem < 0.f) continue;
                const float wu = sqrtf(rem) * inv_ex;  // half-width in x cells
                // cells entirely left of x - w or right of x + w hold no candidate within
                // r_cut; the grid's first and last cells stay when the stencil reaches them
                const bool keep_first = x0 == 0, keep_last = x1 == S.n[0] - 1;
                int a = x0, e = x1;
                const int al = c[0] + (int)floorf(fu[0] - wu), eh = c[0] + (int)floorf(fu[0] + wu);
                if (!keep_first && al > a) a = al < x1 + 1 ? al : x1 + 1;
                if (!keep_last && eh < e) e = eh > x0 - 1 ? eh : x0 - 1;
                if (keep_first && e < 0) e = 0;
                if (keep_last && a > S.n[0] - 1) a = S.n[0] - 1;
                if (a > e) continue;
                x0 = a;
                x1 = e;
            }
            f(__ldg(start + row + x0), __ldg(start + row + x1 + 1));
        }
    }
}

// The position of x in cell units relative to its cell c (FP64 once, then FP32 for the
// pruning bounds of walk_cells_pruned).
template <int DIM, typename V>
__device__ __forceinline__ void cell_units(const V& x, const SceneDev& S, const int32_t c[3], float fu[3]) {
    // a particle clamped from far outside the grid keeps a bounded value (the pruning
    // decisions are the same for any distance beyond the stencil)
    fu[0] = (float)fmin(fmax((x.x - S.lo[0]) * S.inv_cell[0] - (double)c[0], -1e6), 1e6);
    fu[1] = (float)fmin(fmax((x.y - S.lo[1]) * S.inv_cell[1] - (double)c[1], -1e6), 1e6);
    fu[2] = DIM == 3 ? (float)fmin(fmax((comp(x, DIM - 1) - S.lo[2]) * S.inv_cell[2] - (double)c[2], -1e6), 1e6)
                     : 0.f;
}

template <int DIM, typename V>
__device__ __forceinline__ void cell_of(const V& x, const SceneDev& S, int32_t c[3]) {
    c[0] = cell_coord(x.x, S, 0);
    c[1] = cell_coord(x.y, S, 1);
    c[2] = DIM == 3 ? cell_coord(comp(x, DIM - 1), S, 2) : 0;
}

template <int DIM, typename V>
__device__ __forceinline__ int32_t cell_key(const V& x, const SceneDev& S) {
    int32_t c[3];
    cell_of<DIM>(x, S, c);
    return S.cell_off + (c[2] * S.n[1] + c[1]) * S.n[0] + c[0];
}

__device__ __forceinline__ bool is_step(int64_t step, int64_t interval) {
    return interval > 0 && step % interval == 0;
}

// A scene takes part in the physics of a step while it is active and has steps left.
__device__ __forceinline__ bool scene_runs(const SceneDev& S, int64_t step) { return S.active && step <= S.last_step; }

// The momentum kernel's work for a particle of a scene that does not run this step:
// carry the state unchanged into the step outputs and hash it for the next sort (or
// drop it when the scene was retired).
template <int DIM>
__device__ __forceinline__ void carry_frozen(int i, const SceneDev& S, const SortedState& st, const NextState& nx,
                                             const SortScratch& sc) {
    using V = typename VecT<DIM>::T;
    if (!S.active) {
        sc.key[i] = kDeadKey;
        return;
    }
    const V x = ((const V*)st.x)[i];
    ((V*)nx.x)[i] = x;
    ((V*)nx.v)[i] = ((const V*)st.v)[i];
    nx.rho[i] = st.rho[i];
    if (nx.T) nx.T[i] = st.T[i];
    cell_arrival(sc, i, cell_key<DIM>(x, S));
}

// ---------------------------------------------------------------- buffer neighbours
// Sums of a fluid particle over the inlet/outlet buffer particles within r_cut, in FP64
// (FluidInletOutletWallSolve.jl:59-72 continuity, :125-158 pressure and viscosity): the
// FP32 form adds them to its compensated sums after the lane reduction.
template <int DIM, int KK, typename V>
__device__ __forceinline__ double buffer_drho(const SceneDev& S, const BufferState& bf, const int32_t c[3],
                                              const V& xi, const V& vi) {
    const V* __restrict__ bx = (const V*)bf.x;
    const V* __restrict__ bv = (const V*)bf.v;
    double drho = 0.0;
    walk_cells<DIM>(S, bf.start, c, [&](int jb, int je) {
        for (int b = jb; b < je; ++b) {
            double rv[DIM];
            make_rvec<DIM>(xi, bx[b], S, rv);
            const double d2 = norm_sq<DIM>(rv);
            if (!(d2 <= S.rc2)) continue;
            const double r = sqrt(d2);
            double W, dW;
            kernel_wdw<KK>(r, S, W, dW);
            double g[DIM];
            grad_vec<DIM>(dW, r, rv, g);
            const V vb = bv[b];
            double vv[DIM];
            vv[0] = vi.x - vb.x;
            vv[1] = vi.y - vb.y;
            if (DIM == 3) vv[DIM - 1] = comp(vi, DIM - 1) - comp(vb, DIM - 1);
            drho += dotd<DIM>(vv, g) * bf.m[b];
        }
    });
    return drho;
}

template <int DIM, int KK, typename V>
__device__ __forceinline__ void buffer_dv(const SceneDev& S, const BufferState& bf, const int32_t c[3], const V& xi,
                                          const V& vi, double rho_i, double P_i, double gap_i, double Wg_i,
                                          double mu_i, double dv[DIM]) {
    const V* __restrict__ bx = (const V*)bf.x;
    const V* __restrict__ bv = (const V*)bf.v;
    walk_cells<DIM>(S, bf.start, c, [&](int jb, int je) {
        for (int b = jb; b < je; ++b) {
            double rv[DIM];
            make_rvec<DIM>(xi, bx[b], S, rv);
            const double d2 = norm_sq<DIM>(rv);
            if (!(d2 <= S.rc2)) continue;
            const double r = sqrt(d2);
            double W, dW;
            kernel_wdw<KK>(r, S, W, dW);
            double g[DIM];
            grad_vec<DIM>(dW, r, rv, g);
            const V vb = bv[b];
            double vv[DIM];
            vv[0] = vi.x - vb.x;
            vv[1] = vi.y - vb.y;
            if (DIM == 3) vv[DIM - 1] = comp(vi, DIM - 1) - comp(vb, DIM - 1);
            const double rho_b = bf.rho[b];
            const double m_b = bf.m[b];
            const double gap_b = bf.gap[b];
            double prho2 = P_i + bf.p[b] / (rho_b * rho_b);
            const double Wg = gap_b == gap_i ? Wg_i : kernel_w<KK>((gap_i + gap_b) / 2.0, S);
            prho2 += fabs(prho2) * 0.01 * W / Wg;
#pragma unroll
            for (int k = 0; k < DIM; ++k) dv[k] += -m_b * prho2 * g[k];
            const double sum_rho = rho_i + rho_b;
            const double f = 4.0 * (mu_i + S.nu0 * rho_b) * r * dW / (sum_rho * sum_rho) / (r * r + S.hh001);
#pragma unroll
            for (int k = 0; k < DIM; ++k) dv[k] += m_b * f * vv[k];
        }
    });
}

}  // namespace sph
