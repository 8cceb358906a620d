// sph_fp64.cu — plain FP64 gather kernels of the WCSPH step (compiled -fmad=false).
//
// K4 continuity + updateDensity! + updatePressure!   (Continuity.jl:8-17,
//    UpdateDensity.jl:8-12, UpdatePressure.jl:8-16)
// K5 momentum (pressure, viscosity, compulsive wall, heat) + updateTemperature! +
//    updateVelocity! + updatePosition!, fused with the out-of-domain check and the
//    cell hash of the next step's sort   (PressureForce.jl, ViscosityForce.jl,
//    WallForce.jl, ThermalConduction.jl, SelfAction/*.jl, FluidWallSolve.jl:37-81)
// On a re-initialisation step K5 also forms the Shepard sums of reconstructScalar!
//    (ReconstructValue.jl:22-57) over the same fluid neighbours, in the same order, at
//    the same start-of-step positions, and writes the re-initialised density: the update
//    and the re-initialisation are one kernel (FluidWallSolve.jl:64-72).
//
// One thread per fluid particle in sorted (cell, id) order; each thread sums its own
// full neighbour list in a fixed order (cells z, y, x; particles by id), so there are
// no atomics on the physics and results are deterministic.  Walls are visited after
// fluid neighbours.  The reference scatters each unordered pair to both particles
// with atomics; every pair term here is the bitwise same number the reference adds
// (the pair formulas are antisymmetric under exact negation), only the order of the
// additions differs.
#include "sph_physics.cuh"
#include "sph_kernels.h"

namespace sph {

// Solve variants: which wall terms and which body force.
enum { kModeFluidWall = 0, kModeWallPressure = 1, kModeThermal = 2, kModeBuffers = 3 };

template <int DIM, int KK>
__global__ void __launch_bounds__(128) k_continuity_fp64(const SceneDev* __restrict__ scenes, SortedState st,
                                                         SortScratch sc, int32_t cap, BufferState bf) {
    using V = typename VecT<DIM>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || i >= *sc.n_live) return;
    const int32_t s = st.scene[i];
    const SceneDev& S = scenes[s];
    if (!scene_runs(S, sc.scene_step[s])) return;
    const int32_t* __restrict__ start = sc.start;
    const V* __restrict__ x = (const V*)st.x;
    const V* __restrict__ v = (const V*)st.v;
    const V xi = x[i];
    const V vi = v[i];
    int32_t c[3];
    cell_of<DIM>(xi, S, c);
    float xd[3];
    cell_units<DIM>(xi, S, c, xd);
    double drho = 0.0;
    walk_cells_pruned<DIM>(S, start, c, xd, [&](int jb, int je) {
        for (int j = jb; j < je; ++j) {
            if (j == i) continue;
            const V xj = x[j];
            double rv[DIM];
            make_rvec<DIM>(xi, xj, S, rv);
            const double d2 = norm_sq<DIM>(rv);
            if (!(d2 <= S.rc2)) continue;
            const double r = sqrt(d2);
            double W, dW;
            kernel_wdw<KK>(r, S, W, dW);
            double g[DIM];
            grad_vec<DIM>(dW, r, rv, g);
            const V vj = v[j];
            double vv[DIM];
            vv[0] = vi.x - vj.x;
            vv[1] = vi.y - vj.y;
            if (DIM == 3) vv[DIM - 1] = comp(vi, DIM - 1) - comp(vj, DIM - 1);
            drho += dotd<DIM>(vv, g) * st.m[j];
        }
    });
    if (bf.n) {  // inlet/outlet buffer neighbours (FluidInletOutletWallSolve.jl:59-72)
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
                drho += dotd<DIM>(vv, g) * bf.m[b];
            }
        });
    }
    double rho = st.rho[i];
    rho += drho * S.dt;  // written to rhoc, so the kernel can be re-run on the same input
    const double rr = rho / S.rho0;
    const double p = S.b * (jl_powi(rr, S.gamma) - 1.0) + S.p0;
    const double cs = S.c0 * sqrt(jl_powi(rr, S.gamma - 1));
    st.rhoc[i] = rho;
    st.p[i] = p;
    st.c[i] = cs;
    st.P[i] = p / (rho * rho);
}

// SHEP: the momentum gather of density re-initialisation steps, for the particles of the
// scenes whose step re-initialises (every running scene when `sel` is set).  Without SHEP,
// `sel` set leaves those particles to the SHEP launch of the same step (a batch whose
// scenes re-initialise at different steps runs both).
template <int DIM, int KK, int MODE, bool SHEP>
__global__ void __launch_bounds__(128) k_momentum_fp64(const SceneDev* __restrict__ scenes, SortedState st,
                                                       NextState nx, WallState wl, SortScratch sc,
                                                       int32_t cap, BufferState bf, BufferScratch bs,
                                                       BufferRules br, int sel) {
    using V = typename VecT<DIM>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || i >= *sc.n_live) return;
    const int32_t s = st.scene[i];
    const SceneDev& S = scenes[s];
    const int64_t step = sc.scene_step[s];
    const bool runs = scene_runs(S, step);
    const bool reinit_scene = runs && is_step(step, S.reinit_interval);
    if (SHEP ? !(runs && (sel || reinit_scene)) : (sel && reinit_scene)) return;
    if (!runs) {
        carry_frozen<DIM>(i, S, st, nx, sc);
        return;
    }
    const V* __restrict__ x = (const V*)st.x;
    const V* __restrict__ v = (const V*)st.v;
    const V xi = x[i];
    const V vi = v[i];
    const double rho_i = st.rhoc[i];
    const double P_i = st.P[i];
    const double m_i = st.m[i];
    const double gap_i = st.gap[i];
    const double c_i = st.c[i];
    const double mu_i = S.nu0 * rho_i;
    double T_i = 0.0, kap_i = 0.0, cp_i = 1.0;
    if (MODE == kModeThermal) {
        T_i = st.T[i];
        kap_i = st.kappa[i];
        cp_i = st.cp[i];
    }
    // W((gap_i + gap_j)/2) of the tensile term; with uniform gaps it is W(gap_i).
    const double Wg_i = kernel_w<KK>(gap_i, S);
    int32_t c[3];
    cell_of<DIM>(xi, S, c);
    float xd[3];
    cell_units<DIM>(xi, S, c, xd);
    double dv[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) dv[k] = 0.0;
    double dT = 0.0;
    // Shepard sums (ReconstructValue.jl:28-50): sum W m_j/rho_j and sum W m_j/rho_j rho_j
    // over the fluid neighbours, with the post-continuity densities
    double sw = 0.0, sws = 0.0;

    // ---- fluid neighbours: pressureForce! + viscosityForce! (+ thermalConduction!)
    walk_cells_pruned<DIM>(S, sc.start, c, xd, [&](int jb, int je) {
        for (int j = jb; j < je; ++j) {
            if (j == i) continue;
            const V xj = x[j];
            double rv[DIM];
            make_rvec<DIM>(xi, xj, S, rv);
            const double d2 = norm_sq<DIM>(rv);
            if (!(d2 <= S.rc2)) continue;
            const double r = sqrt(d2);
            double W, dW;
            kernel_wdw<KK>(r, S, W, dW);
            double g[DIM];
            grad_vec<DIM>(dW, r, rv, g);
            const V vj = v[j];
            double vv[DIM];
            vv[0] = vi.x - vj.x;
            vv[1] = vi.y - vj.y;
            if (DIM == 3) vv[DIM - 1] = comp(vi, DIM - 1) - comp(vj, DIM - 1);
            const double rho_j = st.rhoc[j];
            const double m_j = st.m[j];
            if (SHEP) {
                sw += W * m_j / rho_j;
                sws += W * m_j / rho_j * rho_j;
            }
            // PressureForce.jl:14-19
            double prho2 = P_i + st.P[j];
            const double Wg = S.uniform_gap ? Wg_i : kernel_w<KK>((gap_i + st.gap[j]) / 2.0, S);
            prho2 += fabs(prho2) * 0.01 * W / Wg;
#pragma unroll
            for (int k = 0; k < DIM; ++k) dv[k] += -m_j * prho2 * g[k];
            // ViscosityForce.jl:15-23
            const double sum_rho = rho_i + rho_j;
            const double mu_j = S.nu0 * rho_j;
            const double f = 4.0 * (mu_i + mu_j) * r * dW / (sum_rho * sum_rho) / (r * r + S.hh001);
#pragma unroll
            for (int k = 0; k < DIM; ++k) dv[k] += m_j * f * vv[k];
            if (MODE == kModeThermal) {  // ThermalConduction.jl:15-21
                const double kap_j = st.kappa[j];
                const double keq = 2.0 * kap_i * kap_j / (kap_i + kap_j);
                const double dq = 2.0 * keq * r * dW / rho_i / rho_j / (r * r + S.hh001) * (T_i - st.T[j]);
                dT += dq * m_j / cp_i;
            }
        }
    });

    // ---- inlet/outlet buffer neighbours: pressureForce! + viscosityForce! with the
    // buffer particle's frozen density and pressure (FluidInletOutletWallSolve.jl:125-158)
    if (MODE == kModeBuffers && bf.n) {
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
                const double mu_b = S.nu0 * rho_b;
                const double f = 4.0 * (mu_i + mu_b) * r * dW / (sum_rho * sum_rho) / (r * r + S.hh001);
#pragma unroll
                for (int k = 0; k < DIM; ++k) dv[k] += m_b * f * vv[k];
            }
        });
    }

    // ---- walls: wallForce! (+ background pressureForce!) + viscosityForce! (+ heat)
    if (wl.n > 0) {
        const V* __restrict__ wx = (const V*)wl.x;
        const V* __restrict__ wn = (const V*)wl.nrm;
        const V* __restrict__ wv = (const V*)wl.v;
        const double Wgap_bg = Wg_i;  // kernelValue(p_i.gap_) of PressureForce.jl:30
        walk_cells_pruned<DIM>(S, wl.start, c, xd, [&](int jb, int je) {
            for (int w = jb; w < je; ++w) {
                const V xw = wx[w];
                double rv[DIM];
                make_rvec<DIM>(xi, xw, S, rv);
                const double d2 = norm_sq<DIM>(rv);
                if (!(d2 <= S.rc2)) continue;
                const double r = sqrt(d2);
                double W, dW;
                kernel_wdw<KK>(r, S, W, dW);
                double g[DIM];
                grad_vec<DIM>(dW, r, rv, g);
                const V vw = wv[w];
                const V nw = wn[w];
                double vv[DIM], n[DIM];
                vv[0] = vi.x - vw.x;
                vv[1] = vi.y - vw.y;
                n[0] = nw.x;
                n[1] = nw.y;
                if (DIM == 3) {
                    vv[DIM - 1] = comp(vi, DIM - 1) - comp(vw, DIM - 1);
                    n[DIM - 1] = comp(nw, DIM - 1);
                }
                const double gw = wl.gap[w];
                // WallForce.jl:15-28 (Rogers & Dalrymple 2008)
                {
                    const double psi = fabs(dotd<DIM>(rv, n));
                    double t = r * r - psi * psi;
                    t = isnan(t) ? t : (t > 0.0 ? t : 0.0);
                    const double xi_ = sqrt(t);
                    const double q = psi / gw;
                    if (!(q > 1.0 || xi_ > gw)) {
                        const double pxi = fabs((1.0 + cos(CUDART_PI * xi_ / gw)) / 2.0);
                        const double vert = dotd<DIM>(vv, n);
                        const double beta = vert > 0.0 ? 0.0 : 1.0;
                        const double rpsi =
                            (0.01 * (c_i * c_i) + beta * c_i * fabs(vert)) / S.h * fabs(1.0 - q) / sqrt(q);
                        const double wf = rpsi * pxi;
#pragma unroll
                        for (int k = 0; k < DIM; ++k) dv[k] += wf * n[k];
                    }
                }
                if (MODE == kModeWallPressure || MODE == kModeThermal) {  // PressureForce.jl:29-33
                    double prho2 = P_i + S.P_bg;
                    prho2 += fabs(prho2) * 0.01 * W / Wgap_bg;
#pragma unroll
                    for (int k = 0; k < DIM; ++k) dv[k] += -m_i * prho2 * g[k];
                }
                {  // ViscosityForce.jl:34-44
                    const double sum_rho = 2.0 * rho_i;
                    const double f = 8.0 * mu_i * r * dW / (sum_rho * sum_rho) / (r * r + S.hh001);
                    const double vert = dotd<DIM>(vv, n);
#pragma unroll
                    for (int k = 0; k < DIM; ++k) dv[k] += m_i * f * (vv[k] - vert * n[k]);
                }
                if (MODE == kModeThermal && wl.kind[w] == SPH_WALL_THERMOSTATIC) {  // ThermalConduction.jl:31-35
                    const double dq = S.inv_cp_d * (kap_i + wl.kappa[w]) * r * dW / rho_i / S.rho0 /
                                      (r * r + S.hh001) * (T_i - wl.T[w]);
                    dT += dq * m_i;
                }
            }
        });
    }

    // ---- updateTemperature!, updateVelocity!, updatePosition!
    const double dt = S.dt;
    double body[DIM];
    if (MODE == kModeThermal) {
        T_i += dt * dT;
#pragma unroll
        for (int k = 0; k < DIM; ++k) body[k] = S.bous[k] * (T_i - S.t0);
        nx.T[i] = T_i;
    } else {
        if (nx.T) nx.T[i] = st.T[i];  // thermal particles in a solve without heat terms
#pragma unroll
        for (int k = 0; k < DIM; ++k) body[k] = S.g[k];
    }
    double vn[DIM], xn[DIM];
    vn[0] = vi.x;
    vn[1] = vi.y;
    xn[0] = xi.x;
    xn[1] = xi.y;
    if (DIM == 3) {
        vn[DIM - 1] = comp(vi, DIM - 1);
        xn[DIM - 1] = comp(xi, DIM - 1);
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) vn[k] += body[k] * dt;
#pragma unroll
    for (int k = 0; k < DIM; ++k) vn[k] += dv[k] * dt;
#pragma unroll
    for (int k = 0; k < DIM; ++k) xn[k] += vn[k] * dt - dv[k] * S.dtdt / 2.0;
    if (S.periodic_x) {
        if (xn[0] >= S.wrap_hi) xn[0] -= S.period;
        else if (xn[0] < S.lo[0]) xn[0] += S.period;
    }
    V xo, vo;
    xo.x = xn[0];
    xo.y = xn[1];
    vo.x = vn[0];
    vo.y = vn[1];
    if constexpr (DIM == 3) {
        xo.z = xn[2];
        xo.w = 0.0;
        vo.z = vn[2];
        vo.w = 0.0;
    }
    ((V*)nx.x)[i] = xo;
    ((V*)nx.v)[i] = vo;
    if (SHEP) {  // the particle's own W(0) term, then the Shepard quotient
        sw += S.k0 * m_i / rho_i;
        sws += S.k0 * m_i / rho_i * rho_i;
        nx.rho[i] = sws / sw;
    } else {
        nx.rho[i] = rho_i;
    }

    // ---- non-finite state, out-of-domain check, next step's cell hash
    bool finite = isfinite(rho_i);
#pragma unroll
    for (int k = 0; k < DIM; ++k) finite &= isfinite(xn[k]) & isfinite(vn[k]);
    if (!finite && S.nan_check) atomicOr(sc.status, kStatusNonFinite);
    bool dead = false;
    if (S.check_enabled && is_step(step, S.check_interval)) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) dead |= (xn[k] > S.check_hi[k]) | (xn[k] < S.check_lo[k]);
    }
    if (dead) {
        sc.key[i] = kDeadKey;
    } else if (MODE == kModeBuffers && bs.npend && beyond_plane<DIM>(br.out_n, br.out_d, xn)) {
        // outlet_out_calculation_domain_check: leaves the fluid, joins the outlet
        sc.key[i] = kDeadKey;
        const int32_t k = atomicAdd(bs.npend, 1);
        if (k < bs.cap) bs.pend[k] = i;
        else atomicOr(sc.status, kStatusBufferOverflow);
    } else {
        cell_arrival(sc, i, cell_key<DIM>(xo, S));
    }
}

// ---------------------------------------------------------------- launchers
namespace {
template <int DIM, int KK>
void launch_k4(const LaunchCtx& L) {
    const int grid = (L.cap + 127) / 128;
    k_continuity_fp64<DIM, KK><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.sc, L.cap, L.bf);
}
template <int DIM, int KK, int MODE>
void launch_k5(const LaunchCtx& L) {
    const int grid = (L.cap + 127) / 128;
    if (L.shepard)
        k_momentum_fp64<DIM, KK, MODE, true><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.nx, L.wl, L.sc, L.cap,
                                                                          L.bf, L.bs, L.br, L.force_reinit);
    else
        k_momentum_fp64<DIM, KK, MODE, false><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.nx, L.wl, L.sc, L.cap,
                                                                           L.bf, L.bs, L.br, L.skip_reinit);
}

template <int DIM>
void dispatch_kk(int kk, int stage, int mode, const LaunchCtx& L) {
#define SPH_KK_CASE(KKV)                                                        \
    case KKV:                                                                   \
        if (stage == 0) launch_k4<DIM, KKV>(L);                                 \
        else if (mode == kModeFluidWall) launch_k5<DIM, KKV, kModeFluidWall>(L); \
        else if (mode == kModeWallPressure) launch_k5<DIM, KKV, kModeWallPressure>(L); \
        else if (mode == kModeBuffers) launch_k5<DIM, KKV, kModeBuffers>(L);    \
        else launch_k5<DIM, KKV, kModeThermal>(L);                              \
        break;
    switch (kk) {
        SPH_KK_CASE(SPH_KERNEL_CUBIC_SPLINE)
        SPH_KK_CASE(SPH_KERNEL_GAUSSIAN)
        SPH_KK_CASE(SPH_KERNEL_WENDLAND_C2)
        SPH_KK_CASE(SPH_KERNEL_WENDLAND_C4)
    }
#undef SPH_KK_CASE
}
}  // namespace

void launch_physics_fp64(int stage, const LaunchCtx& L) {
    if (L.dim == 2) dispatch_kk<2>(L.kernel, stage, L.mode, L);
    else dispatch_kk<3>(L.kernel, stage, L.mode, L);
}

}  // namespace sph
