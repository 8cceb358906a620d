// sph_fp32.cuh — FP32-compensated form of the continuity, momentum and Shepard gathers
//
// Pair arithmetic runs in FP32 on cell-relative positions: every particle carries
// (x - origin of its cell) as floats, and a neighbour in the cell offset (dx, dy, dz)
// sits at xr_j + (dx, dy, dz) * edge in the frame of particle i's cell, so r_vec is
// formed from numbers of magnitude <= 2 r_cut with an absolute error of a few 1e-9 r_cut.
// Continuity and force sums are Kahan-compensated FP32 accumulators; the result
// (sum - compensation) goes to FP64 before the forward-Euler update, which runs in FP64
// on the FP64 master position / velocity / density / temperature.  The Shepard sums
// accumulate in FP64 (FP32 kernel values times FP64 volumes and masses).
//
// Each particle's neighbour walk is split over TPP consecutive lanes of a warp: lane t
// takes candidates t, t+TPP, ... of every neighbour row (the x-cells of a row are one
// virtual range), keeps its own compensated partial sums, and the lanes combine them
// with an xor butterfly (FP32 TwoSum of the sums, the rounding errors joining the
// compensations) — every lane ends with the bitwise same total, so results are
// deterministic for a given TPP.  TPP and the block size are launch parameters picked by
// the autotuner (more lanes per particle = more warps in flight to hide the dependent
// neighbour loads).  With the neighbour-list shapes the continuity gather records each
// particle's accepted neighbours (NbrList) and the momentum gather reads them instead of
// walking the cells again; the walks may skip cells of a row beyond r_cut (row_span).
// On a re-initialisation step the momentum gather also forms the Shepard sums over the
// same neighbours (FP32 kernel values, FP64 sums) and writes the re-initialised density:
// the update and the re-initialisation are one kernel.
//
// Same terms, order of walls after fluid, and solve variants as sph_fp64.cu; the
// formulas follow Continuity.jl, PressureForce.jl, ViscosityForce.jl, WallForce.jl,
// ThermalConduction.jl, SelfAction/*.jl and ReconstructValue.jl.
#pragma once

#include <climits>
#include <type_traits>

#include "sph_physics.cuh"
#include "sph_kernels.h"

namespace sph {

namespace {

enum { kModeFluidWall = 0, kModeWallPressure = 1, kModeThermal = 2, kModeBuffers = 3 };

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// x^n for n >= 0 by repeated squaring, without the compensation of jl_powi.
__device__ __forceinline__ double powi_plain(double x, int n) {
    double y = 1.0;
    while (n > 0) {
        if (n & 1) y *= x;
        x *= x;
        n >>= 1;
    }
    return y;
}

template <int TPP>
__device__ __forceinline__ unsigned group_mask() {
    if (TPP == 32) return 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    return ((1u << TPP) - 1u) << (lane & ~(unsigned)(TPP - 1));
}

// Combine the compensated sums of a particle's TPP lanes in place: the lanes' (s, c)
// pairs are merged in FP32 (the sums by an error-free TwoSum whose rounding error joins
// the compensations); every lane ends with the same bits, and one lane converts the
// result with value() (FP64 work is slow on GB300: done once per particle).
template <int TPP>
__device__ __forceinline__ void group_combine(Kahan& k, unsigned mask) {
#pragma unroll
    for (int o = TPP / 2; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(mask, k.s, o);
        const float c2 = __shfl_xor_sync(mask, k.c, o);
        const float t = k.s + s2;
        const float bp = t - k.s;
        const float e = (k.s - (t - bp)) + (s2 - bp);
        k.s = t;
        k.c = (k.c + c2) - e;
    }
}

// Non-finite test on the exponent bits (integer work instead of FP64 compares).
__device__ __forceinline__ bool bits_finite(double x) {
    return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000;
}

template <int TPP>
__device__ __forceinline__ double group_sum(double v, unsigned mask) {
#pragma unroll
    for (int o = TPP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
}

// W and dW/dr in FP32 (same polynomials as sph_physics.cuh).
template <int KK>
__device__ __forceinline__ void kernel_wdw_f(float q, const SceneDev& S, float& W, float& dW) {
    if (KK == SPH_KERNEL_CUBIC_SPLINE) {
        if (q < 1.f) {
            W = S.kw_a_f * (3.f * q * q * (q - 2.f) + 4.f);
            dW = S.kg_a_f * q * (3.f * q - 4.f);
        } else if (q < 2.f) {
            const float t = 2.f - q;
            W = S.kw_a_f * t * t * t;
            dW = -S.kg_a_f * t * t;
        } else {
            W = 0.f;
            dW = 0.f;
        }
    } else if (KK == SPH_KERNEL_GAUSSIAN) {
        if (q < 3.f) {
            const float e = __expf(-q * q);
            W = S.kw_a_f * e;
            dW = S.kg_a_f * q * e;
        } else {
            W = 0.f;
            dW = 0.f;
        }
    } else if (KK == SPH_KERNEL_WENDLAND_C2) {
        if (q < 2.f) {
            const float t = 2.f - q;
            const float t3 = t * t * t;
            W = S.kw_a_f * (t3 * t) * (1.f + 2.f * q) * 0.0625f;
            dW = S.kg_a_f * q * t3;
        } else {
            W = 0.f;
            dW = 0.f;
        }
    } else {
        if (q < 2.f) {
            const float t = 2.f - q;
            const float t2 = t * t;
            const float t5 = t2 * t2 * t;
            W = S.kw_a_f * (t5 * t) * (35.f * q * q + 36.f * q + 12.f) * (1.f / 768.f);
            dW = S.kg_a_f * (35.f / 96.f * q * q + 7.f / 48.f * q) * t5;
        } else {
            W = 0.f;
            dW = 0.f;
        }
    }
}

template <int KK>
__device__ __forceinline__ float kernel_w_f(float q, const SceneDev& S) {
    float W, dW;
    kernel_wdw_f<KK>(q, S, W, dW);
    return W;
}

// Neighbour rows in (z, y) order (within +-reach cells); inside a row the cells
// x-reach .. x+reach (wrapping on a periodic axis, skipped off the grid) form one virtual
// range that the TPP lanes share.  The callback gets the sorted index j and the offset
// of j's cell from i's cell in metres.
// A neighbour row whose cells x-m .. x+m do not wrap is one contiguous run of the
// sorted arrays, [b, e); the cell of a candidate follows from the interior cell
// boundaries (at most 2m = 6 of them): dx = dx0 + #(boundaries <= j).
struct RowRun {
    int b, e, dx0;
    int bnd[6];
};

__device__ __forceinline__ bool row_run(const SceneDev& S, const int32_t* __restrict__ start, int row, int cx,
                                        int xlo, int xhi, RowRun& R) {
    // a row whose full stencil wraps takes the cell-by-cell path whatever its pruned
    // span: each row keeps one code path (one inlined copy of the pair terms, one rounding)
    const int m = S.reach;
    if (S.periodic_x && (cx - m < 0 || cx + m >= S.n[0])) return false;
    const int x0 = cx + xlo < 0 ? 0 : cx + xlo;
    const int x1 = cx + xhi >= S.n[0] ? S.n[0] - 1 : cx + xhi;
    R.b = __ldg(start + row + x0);
    R.e = __ldg(start + row + x1 + 1);
    R.dx0 = x0 - cx;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const int cell = x0 + 1 + q;
        R.bnd[q] = cell <= x1 ? __ldg(start + row + cell) : INT_MAX;
    }
    return true;
}

// The cells of neighbour row (dy, dz) that can hold a particle within r_cut of particle i
// (cell-relative position xi): offsets [xlo, xhi] in x, or false when none can.  Bounds
// are taken from the cell extents with a relative margin of 1e-5 on r_cut^2 (far above
// the FP32 rounding of the pair distance), so only candidates the distance test would
// reject are skipped and the walk visits the accepted ones in the same order.  Particles
// outside the domain are clamped into the grid's first and last cells with their true
// positions: rows on the y/z grid boundary are kept whole, and the first and last x cells
// are never trimmed away.
template <int DIM>
__device__ __forceinline__ bool row_span(const SceneDev& S, const int32_t c[3], const float xi[3], int y, int z,
                                         int dy, int dz, int& xlo, int& xhi) {
    const int m = S.reach;
    xlo = -m;
    xhi = m;
    if (!S.prune) return true;
    if (y == 0 || y == S.n[1] - 1 || (DIM == 3 && (z == 0 || z == S.n[2] - 1))) return true;
    const float ey = S.cell_f[1];
    const float gy = fmaxf(fmaxf((float)dy * ey - xi[1], xi[1] - (float)(dy + 1) * ey), 0.f);
    float g2 = gy * gy;
    if (DIM == 3) {
        const float ez = S.cell_f[2];
        const float gz = fmaxf(fmaxf((float)dz * ez - xi[2], xi[2] - (float)(dz + 1) * ez), 0.f);
        g2 += gz * gz;
    }
    const float rem = S.rc2_prune - g2;
    if (rem < 0.f) return false;
    const float w = sqrtf(rem);
    int lo = (int)floorf((xi[0] - w) * S.inv_cell_fx);
    int hi = (int)floorf((xi[0] + w) * S.inv_cell_fx);
    lo = lo < -m ? -m : lo;
    hi = hi > m ? m : hi;
    if (!S.periodic_x) {
        if (c[0] - m <= 0) {
            lo = -m;
            hi = hi < -c[0] ? -c[0] : hi;
        }
        if (c[0] + m >= S.n[0] - 1) {
            hi = m;
            lo = lo > S.n[0] - 1 - c[0] ? S.n[0] - 1 - c[0] : lo;
        }
    }
    xlo = lo;
    xhi = hi;
    return lo <= hi;
}

__device__ __forceinline__ int run_dx(const RowRun& R, int j) {
    return R.dx0 + (j >= R.bnd[0]) + (j >= R.bnd[1]) + (j >= R.bnd[2]) + (j >= R.bnd[3]) + (j >= R.bnd[4]) +
           (j >= R.bnd[5]);
}

// Cell offset of a candidate in metres, and its neighbour-list code (see NbrList).
// The product is rounded on its own (no contraction into the caller's subtraction), so
// the cell walk and the list walk form bitwise the same pair vectors.
__device__ __forceinline__ float cell_offset(int d, float edge) { return __fmul_rn((float)d, edge); }
__device__ __forceinline__ int row_code(int dy, int dz, int m) { return ((dz + m) << 6) | ((dy + m) << 3); }

// |r|^2 with a fixed rounding sequence: the continuity gather's test and the momentum
// gather's test agree bit for bit, so the neighbour list holds exactly the pairs the
// momentum walk would accept.
__device__ __forceinline__ float dist2(float rx, float ry, float rz) {
    return __fmaf_rn(rx, rx, __fmaf_rn(ry, ry, __fmul_rn(rz, rz)));
}

template <int DIM, int TPP, typename F>
__device__ __forceinline__ void walk_lanes(const SceneDev& S, const int32_t* __restrict__ start, const int32_t c[3],
                                           const float xi[3], int lane, F&& f) {
    const int m = S.reach;
    const int zr = DIM == 3 ? m : 0;
    for (int dz = -zr; dz <= zr; ++dz) {
        const int z = c[2] + dz;
        if (DIM == 3 && (z < 0 || z >= S.n[2])) continue;
        for (int dy = -m; dy <= m; ++dy) {
            const int y = c[1] + dy;
            if (y < 0 || y >= S.n[1]) continue;
            const int row = S.cell_off + (z * S.n[1] + y) * S.n[0];
            const float oy = cell_offset(dy, S.cell_f[1]);
            const float oz = DIM == 3 ? cell_offset(dz, S.cell_f[2]) : 0.f;
            const int rc = row_code(dy, dz, m) + m;
            int xlo, xhi;
            if (!row_span<DIM>(S, c, xi, y, z, dy, dz, xlo, xhi)) continue;
            // the row's cells are one virtual range v = 0 .. (sum of lengths)-1; lane t
            // takes v = t, t+TPP, ...
            RowRun R;
            if (row_run(S, start, row, c[0], xlo, xhi, R)) {
                for (int j = R.b + lane; j < R.e; j += TPP) {
                    const int dx = run_dx(R, j);
                    f(j, cell_offset(dx, S.cell_f[0]), oy, oz, rc + dx);
                }
                continue;
            }
            int prefix = 0;  // a wrapping row of a periodic axis: cell by cell
            for (int dx = xlo; dx <= xhi; ++dx) {
                int x = c[0] + dx;
                x = x < 0 ? x + S.n[0] : (x >= S.n[0] ? x - S.n[0] : x);
                const int b = __ldg(start + row + x);
                const int e = __ldg(start + row + x + 1);
                const float ox = cell_offset(dx, S.cell_f[0]);
                const int first = (lane - prefix) & (TPP - 1);
                for (int j = b + first; j < e; j += TPP) f(j, ox, oy, oz, rc + dx);
                prefix += e - b;
            }
        }
    }
}

// The same walk, software-pipelined: the loads of a lane's next candidate (load(j)) are
// issued before the current candidate is processed (f(j, data, ...)), so the memory
// latency of one overlaps the arithmetic of the other.  Few warps per scheduler (small
// scenes) cannot hide that latency by switching warps.
template <int DIM, int TPP, typename L, typename F>
__device__ __forceinline__ void walk_lanes_pf(const SceneDev& S, const int32_t* __restrict__ start,
                                              const int32_t c[3], const float xi[3], int lane, L&& load, F&& f) {
    const int m = S.reach;
    const int zr = DIM == 3 ? m : 0;
    for (int dz = -zr; dz <= zr; ++dz) {
        const int z = c[2] + dz;
        if (DIM == 3 && (z < 0 || z >= S.n[2])) continue;
        for (int dy = -m; dy <= m; ++dy) {
            const int y = c[1] + dy;
            if (y < 0 || y >= S.n[1]) continue;
            const int row = S.cell_off + (z * S.n[1] + y) * S.n[0];
            const float oy = cell_offset(dy, S.cell_f[1]);
            const float oz = DIM == 3 ? cell_offset(dz, S.cell_f[2]) : 0.f;
            const int rc = row_code(dy, dz, m) + m;
            int xlo, xhi;
            if (!row_span<DIM>(S, c, xi, y, z, dy, dz, xlo, xhi)) continue;
            RowRun R;
            if (row_run(S, start, row, c[0], xlo, xhi, R)) {
                int j = R.b + lane;
                if (j >= R.e) continue;
                auto d = load(j);
                for (;;) {
                    const int jn = j + TPP;
                    const bool more = jn < R.e;
                    decltype(d) dn = d;
                    if (more) dn = load(jn);
                    const int dx = run_dx(R, j);
                    f(j, d, cell_offset(dx, S.cell_f[0]), oy, oz, rc + dx);
                    if (!more) break;
                    j = jn;
                    d = dn;
                }
                continue;
            }
            int prefix = 0;  // a wrapping row of a periodic axis: cell by cell
            for (int dx = xlo; dx <= xhi; ++dx) {
                int x = c[0] + dx;
                x = x < 0 ? x + S.n[0] : (x >= S.n[0] ? x - S.n[0] : x);
                const int b = __ldg(start + row + x);
                const int e = __ldg(start + row + x + 1);
                const float ox = cell_offset(dx, S.cell_f[0]);
                int j = b + ((lane - prefix) & (TPP - 1));
                prefix += e - b;
                if (j >= e) continue;
                auto d = load(j);
                for (;;) {
                    const int jn = j + TPP;
                    const bool more = jn < e;
                    decltype(d) dn = d;
                    if (more) dn = load(jn);
                    f(j, d, ox, oy, oz, rc + dx);
                    if (!more) break;
                    j = jn;
                    d = dn;
                }
            }
        }
    }
}

// Walk with (PF) or without software pipelining; body(j, load(j), ox, oy, oz, code).
template <int DIM, int TPP, bool PF, typename L, typename F>
__device__ __forceinline__ void walk(const SceneDev& S, const int32_t* __restrict__ start, const int32_t c[3],
                                     const float xi[3], int lane, L&& load, F&& body) {
    if constexpr (PF) {
        walk_lanes_pf<DIM, TPP>(S, start, c, xi, lane, load, body);
    } else {
        walk_lanes<DIM, TPP>(S, start, c, xi, lane, [&](int j, float ox, float oy, float oz, int code) {
            body(j, load(j), ox, oy, oz, code);
        });
    }
}

// Entry k of particle i.
__device__ __forceinline__ const int32_t* list_entry(const NbrList& nl, int k, int i) {
    return nl.e + (int64_t)k * nl.stride + i;
}

// Walk of particle i's neighbour list (cnt entries, NbrList): lane t takes entries t,
// t+TPP, ...; the PF form loads the next entry and its neighbour's data before the
// current neighbour is processed.  body as for walk().
template <int DIM, int TPP, bool PF, typename L, typename F>
__device__ __forceinline__ void walk_list(const SceneDev& S, const NbrList& nl, int i, int cnt, int lane, L&& load,
                                          F&& body) {
    const int m = S.reach;
    // the list is entries [0, front) followed by entries kmax - 1 down to kmax - back
    const int front = cnt & 0xffff, back = cnt >> 16;
    cnt = front + back;
    auto entry = [&](int k) { return __ldg(list_entry(nl, k < front ? k : nl.kmax - 1 - (k - front), i)); };
    auto off = [&](int32_t x, float& ox, float& oy, float& oz) {
        ox = cell_offset((x & 7) - m, S.cell_f[0]);
        oy = cell_offset(((x >> 3) & 7) - m, S.cell_f[1]);
        oz = DIM == 3 ? cell_offset(((x >> 6) & 7) - m, S.cell_f[2]) : 0.f;
    };
    if constexpr (PF) {
        int k = lane;
        if (k >= cnt) return;
        int32_t x = entry(k);
        int j = i + (x >> 9);
        auto d = load(j);
        for (;;) {
            const int kn = k + TPP;
            const bool more = kn < cnt;
            int32_t xn = x;
            int jn = j;
            decltype(d) dn = d;
            if (more) {
                xn = entry(kn);
                jn = i + (xn >> 9);
                dn = load(jn);
            }
            float ox, oy, oz;
            off(x, ox, oy, oz);
            body(j, d, ox, oy, oz, 0);
            if (!more) break;
            k = kn;
            x = xn;
            j = jn;
            d = dn;
        }
    } else {
        // the next entry is loaded while the current neighbour is processed, so only the
        // neighbour's own load stays on each iteration's chain of memory round trips
        int k = lane;
        if (k >= cnt) return;
        int32_t x = entry(k);
        for (;;) {
            const int kn = k + TPP;
            const bool more = kn < cnt;
            const int32_t xn = more ? entry(kn) : 0;
            const int j = i + (x >> 9);
            float ox, oy, oz;
            off(x, ox, oy, oz);
            body(j, load(j), ox, oy, oz, 0);
            if (!more) break;
            k = kn;
            x = xn;
        }
    }
}

struct Cand2 {
    float4 a, b;
};
struct Cand3 {
    float4 a, b, c;
};
struct WallCand {
    float4 a, b, c;
    int kind;
};
// A fluid candidate of the momentum gather on a re-initialisation step: the FP32
// shadows plus the FP64 volume m/rho and mass of the Shepard sums.
struct Cand3S {
    float4 a, b, c;
    double vol, m;
};

__device__ __forceinline__ void decode_cell(int32_t key, const SceneDev& S, int32_t c[3]) {
    const int32_t k = key - S.cell_off;
    c[0] = k % S.n[0];
    c[1] = (k / S.n[0]) % S.n[1];
    c[2] = k / (S.n[0] * S.n[1]);
}

// -------------------------------------------------------------------- K4 (FP32)
// LIST (one lane per particle): also records the neighbours within r_cut in nl.
template <int DIM, int KK, int TPP, bool PF, bool LIST>
__global__ void k_continuity_f32(const SceneDev* __restrict__ scenes, SortedState st, SortScratch sc, int32_t cap,
                                 BufferState bf, NbrList nl) {
    pdl_wait();
    static_assert(!LIST || TPP <= 2, "the neighbour list is written by one or two lanes per particle");
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / TPP, lane = t % TPP;
    if (i >= cap || i >= *sc.n_live) return;
    const int32_t s = st.scene[i];
    const SceneDev& S = scenes[s];
    if (!scene_runs(S, sc.scene_step[s])) return;
    const int32_t* __restrict__ start = sc.start;
    const float4 ai = st.fa[i];
    float xi[3], vi[3];
    if (DIM == 2) {
        xi[0] = ai.x; xi[1] = ai.y; xi[2] = 0.f;
        vi[0] = ai.z; vi[1] = ai.w; vi[2] = 0.f;
    } else {
        const float4 bi = st.fb[i];
        xi[0] = ai.x; xi[1] = ai.y; xi[2] = ai.z;
        vi[0] = bi.x; vi[1] = bi.y; vi[2] = bi.z;
    }
    int32_t c[3];
    decode_cell(st.cell[i], S, c);
    Kahan drho;
    int cnt = 0;
    bool list_ok = !LIST || S.reach <= 3;
    // lane 0 fills the particle's list from entry 0 up, lane 1 (two-lane writer) from
    // entry kmax - 1 down; the count word holds both counts (NbrList)
    int32_t* lp = LIST ? nl.e + (lane == 0 ? (int64_t)0 : (int64_t)(nl.kmax - 1) * nl.stride) + i : nullptr;
    const int64_t lstep = lane == 0 ? nl.stride : -nl.stride;
    if (LIST) {  // every candidate lies between the first and the last neighbour row
        const int m = S.reach;
        const int zl = DIM == 3 ? max(c[2] - m, 0) : 0, zh = DIM == 3 ? min(c[2] + m, S.n[2] - 1) : 0;
        const int lo = __ldg(start + S.cell_off + (zl * S.n[1] + max(c[1] - m, 0)) * S.n[0]);
        const int hi = __ldg(start + S.cell_off + (zh * S.n[1] + min(c[1] + m, S.n[1] - 1) + 1) * S.n[0]);
        list_ok &= i - lo < kListDelta && hi - i <= kListDelta;
    }
    auto load = [&](int j) { return Cand2{st.fa[j], st.fb[j]}; };
    walk<DIM, TPP, PF>(S, start, c, xi, lane, load, [&](int j, const Cand2& cd, float ox, float oy, float oz, int code) {
        if (j == i) return;
        const float4 aj = cd.a;
        const float4 bj = cd.b;
        const float rx = xi[0] - ox - aj.x, ry = xi[1] - oy - aj.y;
        const float rz = DIM == 3 ? xi[2] - oz - aj.z : 0.f;
        const float d2 = dist2(rx, ry, rz);
        if (!(d2 <= S.rc2_f)) return;
        if (LIST) {  // coincident neighbours are listed too: the Shepard sums count them
            if (cnt < nl.kmax) {
                *lp = (int32_t)(((uint32_t)(j - i) << 9) | (uint32_t)code);
                lp += lstep;
            } else {
                list_ok = false;
            }
            ++cnt;
        }
        // a coincident neighbour (d2 == 0) gets 1/r = 0, hence r = 0, dW = 0 and no
        // continuity term, without a branch in the walk
        const float inv_r = d2 > 0.f ? rsqrtf(d2) : 0.f;
        const float r = d2 * inv_r;
        float W, dW;
        kernel_wdw_f<KK>(r * S.inv_h_f, S, W, dW);
        const float s = dW * inv_r;
        float vx, vy, vz, mj;
        if (DIM == 2) {
            vx = vi[0] - aj.z;
            vy = vi[1] - aj.w;
            vz = 0.f;
            mj = bj.x;
        } else {
            vx = vi[0] - bj.x;
            vy = vi[1] - bj.y;
            vz = vi[2] - bj.z;
            mj = aj.w;
        }
        drho.add(mj * s * (vx * rx + vy * ry + vz * rz));
    });
    group_combine<TPP>(drho, group_mask<TPP>());
    int n_back = 0;  // entries of lane 1 (two-lane writer)
    if (LIST && TPP == 2) {
        n_back = __shfl_xor_sync(group_mask<TPP>(), cnt, 1);
        list_ok &= __shfl_xor_sync(group_mask<TPP>(), (int)list_ok, 1) != 0;
    }
    if (lane != 0) return;
    double dr = drho.value();
    if (LIST) {
        list_ok &= cnt + n_back <= nl.kmax;
        nl.n[i] = list_ok ? (cnt | (n_back << 16)) : kListWalk;
    }
    if (bf.n) {  // inlet/outlet buffer neighbours, FP64
        using V = typename VecT<DIM>::T;
        dr += buffer_drho<DIM, KK>(S, bf, c, ((const V*)st.x)[i], ((const V*)st.v)[i]);
    }
    // Tait equation of state (UpdatePressure.jl:8-16) with one FP64 division and plain
    // powers: FP64 is slow on GB300, and these values feed FP32 pair terms (P, c) or FP64
    // sums (vol) where their last-bit differences from the reference's rounding do not show.
    // (Evaluated in FP32 instead, on the relative change rho/rho0 - 1, it took 4 more
    // registers and fewer resident warps: slower on GB300.)
    // loads first: stores to the state arrays would otherwise order them (possible aliasing)
    double rho = st.rho[i];
    const double m_i = st.m[i];
    const float4 fb_i = st.fb[i];
    const float4 fc_i = DIM == 3 ? st.fc[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    rho += dr * S.dt;
    const double inv_rho = 1.0 / rho;
    const double rr = rho * S.inv_rho0;
    const double p = S.b * (powi_plain(rr, S.gamma) - 1.0) + S.p0;
    const double cs =
        S.c0 * ((S.gamma & 1) ? powi_plain(rr, (S.gamma - 1) >> 1) : sqrt(powi_plain(rr, S.gamma - 1)));
    const double P = p * inv_rho * inv_rho;
    st.rhoc[i] = rho;
    st.p[i] = p;
    st.c[i] = cs;
    st.P[i] = P;
    st.vol[i] = m_i * inv_rho;
    if (DIM == 2) {
        st.fb[i] = make_float4(fb_i.x, (float)rho, (float)P, fb_i.w);
    } else {
        st.fb[i] = make_float4(fb_i.x, fb_i.y, fb_i.z, (float)rho);
        st.fc[i] = make_float4((float)P, fc_i.y, fc_i.z, fc_i.w);
    }
}

// -------------------------------------------------------------------- K5 (FP32)
// The walks without software pipelining are held to 64 registers (1024 threads x 64 =
// one SM's register file): 32 resident warps instead of 24 hide more of the dependent
// neighbour loads on large scenes (about 10% faster at 1M particles), at the cost of a
// few spilled bytes in the thermal variant.  The pipelined walk keeps its registers (its
// prefetched candidate would spill) and is therefore limited to blocks of 256 threads.
// LIST: the fluid neighbours come from the list the continuity gather recorded (the
// cell walk for a particle whose list did not fit).
// SHEP: the momentum gather of density re-initialisation steps.  It takes the particles
// of the scenes whose step re-initialises (every running scene when `sel` is set): the
// fluid walk also sums W m_j/rho_j and W m_j (ReconstructValue.jl:28-50) in FP64, and the
// particle's density leaves the step as the Shepard quotient instead of the continuity
// update.  Without SHEP, `sel` set leaves those particles to the SHEP launch of the same
// step (a batch whose scenes re-initialise at different steps runs both): every particle
// goes through the kernel of its own scene's step kind, so a scene's result does not
// depend on the other scenes of its batch.
template <int DIM, int KK, int MODE, int TPP, bool PF, bool LIST, bool SHEP>
__global__ void __launch_bounds__(PF ? 256 : 1024) k_momentum_f32(const SceneDev* __restrict__ scenes, SortedState st, NextState nx, WallState wl,
                               SortScratch sc, int32_t cap, BufferState bf, BufferScratch bs, BufferRules br,
                               NbrList nl, int sel) {
    pdl_wait();
    using V = typename VecT<DIM>::T;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / TPP, lane = t % TPP;
    if (i >= cap || i >= *sc.n_live) return;
    const int32_t s = st.scene[i];
    const SceneDev& S = scenes[s];
    const int64_t step_s = sc.scene_step[s];
    const bool runs = scene_runs(S, step_s);
    const bool reinit_scene = runs && is_step(step_s, S.reinit_interval);
    if constexpr (SHEP) {
        if (!(runs && (sel || reinit_scene))) return;
    } else {
        if (sel && reinit_scene) return;
    }
    if (!runs) {
        if (lane == 0) carry_frozen<DIM>(i, S, st, nx, sc);
        return;
    }
    const float4 ai = st.fa[i];
    const float4 bi = st.fb[i];
    float xi[3], vi[3], m_i, rho_i, P_i, gap_i;
    float T_i = 0.f, kap_i = 0.f, cp_i = 1.f;
    if (DIM == 2) {
        xi[0] = ai.x; xi[1] = ai.y; xi[2] = 0.f;
        vi[0] = ai.z; vi[1] = ai.w; vi[2] = 0.f;
        m_i = bi.x; rho_i = bi.y; P_i = bi.z; gap_i = bi.w;
        if (MODE == kModeThermal) {
            const float4 ci = st.fc[i];
            T_i = ci.x; kap_i = ci.y; cp_i = ci.z;
        }
    } else {
        xi[0] = ai.x; xi[1] = ai.y; xi[2] = ai.z; m_i = ai.w;
        vi[0] = bi.x; vi[1] = bi.y; vi[2] = bi.z; rho_i = bi.w;
        const float4 ci = st.fc[i];
        P_i = ci.x; gap_i = ci.y;
        if (MODE == kModeThermal) {
            T_i = ci.z; kap_i = ci.w; cp_i = st.fd[i];
        }
    }
    const float c_i = (float)st.c[i];
    const float mu_i = S.nu0_f * rho_i;
    const float inv_h = S.inv_h_f;
    const float inv_Wg_i = 1.f / kernel_w_f<KK>(gap_i * inv_h, S);
    const float inv_cp_i = 1.f / cp_i;
    int32_t c[3];
    decode_cell(st.cell[i], S, c);
    Kahan dv[3], dT;
    double sw = 0.0, sws = 0.0;  // Shepard sums (FP64)

    // every load of a candidate is issued before its distance test (one memory round
    // trip per candidate), and before the previous candidate is processed
    using CandF = std::conditional_t<SHEP, Cand3S, Cand3>;
    auto load_f = [&](int j) {
        CandF d;
        d.a = st.fa[j];
        d.b = st.fb[j];
        d.c = (DIM == 3 || MODE == kModeThermal) ? st.fc[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (SHEP) {
            d.vol = st.vol[j];
            d.m = st.m[j];
        }
        return d;
    };
    auto pair = [&](int j, const CandF& cd, float ox, float oy, float oz, int) {
        if (j == i) return;
        const float4 aj = cd.a;
        const float4 bj = cd.b;
        const float4 cj = cd.c;
        const float rx = xi[0] - ox - aj.x, ry = xi[1] - oy - aj.y;
        const float rz = DIM == 3 ? xi[2] - oz - aj.z : 0.f;
        const float d2 = dist2(rx, ry, rz);
        if (!(d2 <= S.rc2_f)) return;
        if (d2 == 0.f) {  // a coincident neighbour: no force, W(0) in the Shepard sums
            if constexpr (SHEP) {
                const double W0 = (double)kernel_w_f<KK>(0.f, S);
                sw += W0 * cd.vol;
                sws += W0 * cd.m;
            }
            return;
        }
        const float inv_r = rsqrtf(d2);
        const float r = d2 * inv_r;
        float W, dW;
        kernel_wdw_f<KK>(r * inv_h, S, W, dW);
        if constexpr (SHEP) {
            sw += (double)W * cd.vol;
            sws += (double)W * cd.m;
        }
        float vx, vy, vz, m_j, rho_j, P_j, gap_j;
        float T_j = 0.f, kap_j = 0.f;
        if (DIM == 2) {
            vx = vi[0] - aj.z; vy = vi[1] - aj.w; vz = 0.f;
            m_j = bj.x; rho_j = bj.y; P_j = bj.z; gap_j = bj.w;
            if (MODE == kModeThermal) {
                T_j = cj.x; kap_j = cj.y;
            }
        } else {
            vx = vi[0] - bj.x; vy = vi[1] - bj.y; vz = vi[2] - bj.z;
            m_j = aj.w; rho_j = bj.w;
            P_j = cj.x; gap_j = cj.y;
            if (MODE == kModeThermal) {
                T_j = cj.z; kap_j = cj.w;
            }
        }
        // pressure (PressureForce.jl:14-19), tensile term included
        float prho2 = P_i + P_j;
        const float inv_Wg = S.uniform_gap ? inv_Wg_i : 1.f / kernel_w_f<KK>(0.5f * (gap_i + gap_j) * inv_h, S);
        prho2 += fabsf(prho2) * 0.01f * W * inv_Wg;
        // viscosity (ViscosityForce.jl:15-23)
        const float sum_rho = rho_i + rho_j;
        const float f = __fdividef(4.f * (mu_i + S.nu0_f * rho_j) * r * dW, sum_rho * sum_rho * (r * r + S.hh001_f));
        const float gp = -m_j * prho2 * dW * inv_r;  // pressure term along r_vec
        const float gv = m_j * f;                    // viscosity term along v_ij
        dv[0].add(gp * rx + gv * vx);
        dv[1].add(gp * ry + gv * vy);
        if (DIM == 3) dv[2].add(gp * rz + gv * vz);
        if (MODE == kModeThermal) {  // ThermalConduction.jl:15-21
            const float keq = __fdividef(2.f * kap_i * kap_j, kap_i + kap_j);
            const float dq = __fdividef(2.f * keq * r * dW, rho_i * rho_j * (r * r + S.hh001_f)) * (T_i - T_j);
            dT.add(dq * m_j * inv_cp_i);
        }
    };
    if constexpr (LIST) {
        const int cnt = nl.n[i];
        if (cnt != kListWalk) walk_list<DIM, TPP, PF>(S, nl, i, cnt, lane, load_f, pair);
        else walk<DIM, TPP, PF>(S, sc.start, c, xi, lane, load_f, pair);
    } else {
        walk<DIM, TPP, PF>(S, sc.start, c, xi, lane, load_f, pair);
    }

    if (wl.n > 0 && wl.near[st.cell[i]]) {  // walls only where a wall cell is within reach
        auto load_w = [&](int w) {
            WallCand d;
            d.a = wl.fa[w];
            d.b = wl.fb[w];
            d.c = (DIM == 3 || MODE == kModeThermal) ? wl.fc[w] : make_float4(0.f, 0.f, 0.f, 0.f);
            d.kind = (DIM == 3 && MODE == kModeThermal) ? wl.kind[w] : 0;
            return d;
        };
        walk<DIM, TPP, PF>(S, wl.start, c, xi, lane, load_w, [&](int w, const WallCand& cd, float ox, float oy,
                                                                   float oz, int) {
            const float4 wa = cd.a;
            const float4 wb = cd.b;
            const float4 wc = cd.c;
            float rv[3], n[3], vv[3], gw, Tw = 0.f, kw = 0.f;
            bool thermo = false;
            if (DIM == 2) {
                rv[0] = xi[0] - ox - wa.x; rv[1] = xi[1] - oy - wa.y; rv[2] = 0.f;
                n[0] = wa.z; n[1] = wa.w; n[2] = 0.f;
                vv[0] = vi[0] - wb.x; vv[1] = vi[1] - wb.y; vv[2] = 0.f;
                gw = wb.z;
                if (MODE == kModeThermal) {
                    Tw = wb.w; kw = wc.x; thermo = wc.y != 0.f;
                }
            } else {
                rv[0] = xi[0] - ox - wa.x; rv[1] = xi[1] - oy - wa.y; rv[2] = xi[2] - oz - wa.z;
                gw = wa.w;
                n[0] = wb.x; n[1] = wb.y; n[2] = wb.z;
                vv[0] = vi[0] - wc.x; vv[1] = vi[1] - wc.y; vv[2] = vi[2] - wc.z;
                if (MODE == kModeThermal) {
                    Tw = wb.w; kw = wc.w; thermo = cd.kind == SPH_WALL_THERMOSTATIC;
                }
            }
            const float d2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
            if (!(d2 <= S.rc2_f)) return;
            const float inv_r = d2 > 0.f ? rsqrtf(d2) : 0.f;
            const float r = d2 * inv_r;
            float W, dW;
            kernel_wdw_f<KK>(r * inv_h, S, W, dW);
            const float vert = vv[0] * n[0] + vv[1] * n[1] + vv[2] * n[2];
            float acc[3] = {0.f, 0.f, 0.f};
            {  // WallForce.jl:15-28
                const float psi = fabsf(rv[0] * n[0] + rv[1] * n[1] + rv[2] * n[2]);
                const float xi_ = sqrtf(fmaxf(r * r - psi * psi, 0.f));
                const float q = psi / gw;
                if (!(q > 1.f || xi_ > gw)) {
                    const float pxi = fabsf((1.f + cospif(xi_ / gw)) * 0.5f);
                    const float beta = vert > 0.f ? 0.f : 1.f;
                    const float rpsi =
                        (0.01f * c_i * c_i + beta * c_i * fabsf(vert)) * inv_h * fabsf(1.f - q) * rsqrtf(q);
                    const float wf = rpsi * pxi;
                    acc[0] += wf * n[0];
                    acc[1] += wf * n[1];
                    acc[2] += wf * n[2];
                }
            }
            if (MODE == kModeWallPressure || MODE == kModeThermal) {  // PressureForce.jl:29-33
                float prho2 = P_i + S.P_bg_f;
                prho2 += fabsf(prho2) * 0.01f * W * inv_Wg_i;
                const float gp = -m_i * prho2 * dW * inv_r;
                acc[0] += gp * rv[0];
                acc[1] += gp * rv[1];
                acc[2] += gp * rv[2];
            }
            {  // ViscosityForce.jl:34-44
                const float sum_rho = 2.f * rho_i;
                const float f = __fdividef(8.f * mu_i * r * dW, sum_rho * sum_rho * (r * r + S.hh001_f));
                const float gv = m_i * f;
                acc[0] += gv * (vv[0] - vert * n[0]);
                acc[1] += gv * (vv[1] - vert * n[1]);
                acc[2] += gv * (vv[2] - vert * n[2]);
            }
            dv[0].add(acc[0]);
            dv[1].add(acc[1]);
            if (DIM == 3) dv[2].add(acc[2]);
            if (MODE == kModeThermal && thermo) {  // ThermalConduction.jl:31-35
                const float dq =
                    __fdividef(S.inv_cp_f * (kap_i + kw) * r * dW * S.inv_rho0_f, rho_i * (r * r + S.hh001_f)) *
                    (T_i - Tw);
                dT.add(dq * m_i);
            }
        });
    }

    const unsigned mask = group_mask<TPP>();
#pragma unroll
    for (int k = 0; k < DIM; ++k) group_combine<TPP>(dv[k], mask);
    if (MODE == kModeThermal) group_combine<TPP>(dT, mask);
    if constexpr (SHEP) {
        sw = group_sum<TPP>(sw, mask);
        sws = group_sum<TPP>(sws, mask);
    }
    if (lane != 0) return;
    double dvd[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) dvd[k] = dv[k].value();
    const double dTd = MODE == kModeThermal ? dT.value() : 0.0;

    // ---- FP64 forward Euler on the masters (UpdateTemperature/Velocity/Position.jl)
    const int64_t step = sc.scene_step[s];
    const V x0 = ((const V*)st.x)[i];
    const V v0 = ((const V*)st.v)[i];
    const double rho_d = st.rhoc[i];  // loaded before the stores below (possible aliasing)
    if constexpr (SHEP) {  // the particle's own W(0) term (ReconstructValue.jl:51-55)
        sw += S.k0 * st.vol[i];
        sws += S.k0 * st.m[i];
    }
    if (MODE == kModeBuffers && bf.n) {  // inlet/outlet buffer neighbours, FP64
        const double gap_d = st.gap[i];
        buffer_dv<DIM, KK>(S, bf, c, x0, v0, rho_d, st.P[i], gap_d, kernel_w<KK>(gap_d, S), S.nu0 * rho_d, dvd);
    }
    const double dt = S.dt;
    double body[DIM];
    if (MODE == kModeThermal) {
        const double Tn = st.T[i] + dt * dTd;
#pragma unroll
        for (int k = 0; k < DIM; ++k) body[k] = S.bous[k] * (Tn - S.t0);
        nx.T[i] = Tn;
    } else {
        if (nx.T) nx.T[i] = st.T[i];
#pragma unroll
        for (int k = 0; k < DIM; ++k) body[k] = S.g[k];
    }
    double vn[DIM], xn[DIM];
    vn[0] = v0.x; vn[1] = v0.y;
    xn[0] = x0.x; xn[1] = x0.y;
    if (DIM == 3) {
        vn[DIM - 1] = comp(v0, DIM - 1);
        xn[DIM - 1] = comp(x0, DIM - 1);
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
        vn[k] += body[k] * dt;
        vn[k] += dvd[k] * dt;
        xn[k] += vn[k] * dt - dvd[k] * S.half_dtdt;  // dv dt^2 / 2
    }
    if (S.periodic_x) {
        if (xn[0] >= S.wrap_hi) xn[0] -= S.period;
        else if (xn[0] < S.lo[0]) xn[0] += S.period;
    }
    V xo, vo;
    xo.x = xn[0]; xo.y = xn[1];
    vo.x = vn[0]; vo.y = vn[1];
    if constexpr (DIM == 3) {
        xo.z = xn[2]; xo.w = 0.0;
        vo.z = vn[2]; vo.w = 0.0;
    }
    ((V*)nx.x)[i] = xo;
    ((V*)nx.v)[i] = vo;
    nx.rho[i] = SHEP ? sws / sw : rho_d;

    bool finite = bits_finite(rho_d);
#pragma unroll
    for (int k = 0; k < DIM; ++k) finite &= bits_finite(xn[k]) & bits_finite(vn[k]);
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

// -------------------------------------------------------------------- launchers
// SHEP selects the momentum gather of re-initialisation steps; its instantiations live in
// translation units of their own (the *_shep.cu files), so the two sets compile in parallel.
template <int DIM, int KK, int MODE, int TPP, bool PF, bool LIST, bool SHEP>
void launch_momentum(const LaunchCtx& L, int grid, int block) {
    launch_dep(k_momentum_f32<DIM, KK, MODE, TPP, PF, LIST, SHEP>, grid, block, L.stream, L.scenes, L.st, L.nx, L.wl,
               L.sc, L.cap, L.bf, L.bs, L.br, L.nl, SHEP ? L.force_reinit : L.skip_reinit);
}

template <int DIM, int KK, int TPP, bool PF, bool LIST, bool SHEP>
void launch_tpp(int stage, int mode, const LaunchCtx& L) {
    const int block = L.block > 0 ? L.block : 128;
    const int grid = (int)(((int64_t)L.cap * TPP + block - 1) / block);
    if (stage == 0) {
        if constexpr (!SHEP && (!LIST || TPP <= 2))
            launch_dep(k_continuity_f32<DIM, KK, TPP, PF, LIST>, grid, block, L.stream, L.scenes, L.st, L.sc, L.cap,
                       L.bf, L.nl);
    } else if (mode == kModeFluidWall) {
        launch_momentum<DIM, KK, kModeFluidWall, TPP, PF, LIST, SHEP>(L, grid, block);
    } else if (mode == kModeWallPressure) {
        launch_momentum<DIM, KK, kModeWallPressure, TPP, PF, LIST, SHEP>(L, grid, block);
    } else if (mode == kModeBuffers) {
        launch_momentum<DIM, KK, kModeBuffers, TPP, PF, LIST, SHEP>(L, grid, block);
    } else {
        launch_momentum<DIM, KK, kModeThermal, TPP, PF, LIST, SHEP>(L, grid, block);
    }
}

// Lanes code: 1, 2, 4, 8 lanes per particle; -1: one lane with a software-pipelined
// candidate loop (pays off when few warps are resident, i.e. small scenes).  The cell
// walks (LIST false) take every code for every stage; with the neighbour list (LIST
// true) continuity runs one or two lanes (1, -1 or 2; the two-lane list writer loads
// each lane's next candidate ahead, as -1 does: on GB300 5-22% faster than without in
// 2D and 3D) and momentum 1, 2, 4 or -1 lanes (there two pipelined lanes were 30-60%
// slower: the prefetched candidate of three float4 costs the occupancy).
template <int DIM, int KK, bool LIST, bool SHEP>
void launch_kk(int stage, const LaunchCtx& L) {
    const int tpp = stage == 0 ? L.tpp_continuity : L.tpp_momentum;
    if constexpr (LIST) {
        if (stage == 0) {
            if (tpp == -1) launch_tpp<DIM, KK, 1, true, true, SHEP>(stage, L.mode, L);
            else if (tpp == 2) launch_tpp<DIM, KK, 2, true, true, SHEP>(stage, L.mode, L);
            else launch_tpp<DIM, KK, 1, false, true, SHEP>(stage, L.mode, L);
            return;
        }
        switch (tpp) {
            case -1: launch_tpp<DIM, KK, 1, true, true, SHEP>(stage, L.mode, L); break;
            case 1: launch_tpp<DIM, KK, 1, false, true, SHEP>(stage, L.mode, L); break;
            case 2: launch_tpp<DIM, KK, 2, false, true, SHEP>(stage, L.mode, L); break;
            default: launch_tpp<DIM, KK, 4, false, true, SHEP>(stage, L.mode, L); break;
        }
    } else {
        switch (tpp) {
            case -1: launch_tpp<DIM, KK, 1, true, false, SHEP>(stage, L.mode, L); break;
            case 1: launch_tpp<DIM, KK, 1, false, false, SHEP>(stage, L.mode, L); break;
            case 2: launch_tpp<DIM, KK, 2, false, false, SHEP>(stage, L.mode, L); break;
            case 8: launch_tpp<DIM, KK, 8, false, false, SHEP>(stage, L.mode, L); break;
            default: launch_tpp<DIM, KK, 4, false, false, SHEP>(stage, L.mode, L); break;
        }
    }
}

template <int DIM, bool LIST, bool SHEP>
void dispatch(int stage, const LaunchCtx& L) {
    switch (L.kernel) {
        case SPH_KERNEL_CUBIC_SPLINE: launch_kk<DIM, SPH_KERNEL_CUBIC_SPLINE, LIST, SHEP>(stage, L); break;
        case SPH_KERNEL_GAUSSIAN: launch_kk<DIM, SPH_KERNEL_GAUSSIAN, LIST, SHEP>(stage, L); break;
        case SPH_KERNEL_WENDLAND_C2: launch_kk<DIM, SPH_KERNEL_WENDLAND_C2, LIST, SHEP>(stage, L); break;
        default: launch_kk<DIM, SPH_KERNEL_WENDLAND_C4, LIST, SHEP>(stage, L); break;
    }
}

}  // namespace

}  // namespace sph
