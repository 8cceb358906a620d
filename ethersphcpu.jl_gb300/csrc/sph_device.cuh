// sph_device.cuh — device-side types and math shared by the GB300 SPH kernels.
//
// Layout in HBM (one "scene table" entry per independent simulation; a single-scene
// handle is a table of one):
//   sorted state S (double-buffered, S <-> S' each step), index = position in
//   (cell, id) order:  x, v (double2 in 2D, 32-byte aligned double4 in 3D, w unused), rho, p, c,
//   P = p / rho^2, mass, gap, T, kappa, cp, id, scene
//   step outputs N (unsorted, same index as S): x', v', T', rho'
//   cell list: count[cells], start[cells + 1] (exclusive scan), key/slot per particle
//   walls (static, sorted once by (cell, wall index) on the host): x, normal, gap, T,
//   kappa, v, kind, wall_start[cells + 1]
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "../../include/ethersph_gpu.h"

namespace sph {

constexpr int32_t kDeadKey = 0x7fffffff;

// Programmatic dependent launch between the kernels of a step (launch_dep): the next
// kernel's launch is prepared while its predecessor in the stream finishes; pdl_wait()
// blocks until the predecessor grid has completed and its writes are visible (a no-op
// when the kernel was launched without the attribute).  Every step kernel calls it first,
// before it touches device memory.  No kernel triggers its dependents early: blocks of the
// next kernel parked on the wait took SM slots from the tail of the current one (a
// 65k-particle step on GB300: 0.0652 ms with an early trigger, 0.0642 ms without
// programmatic launches, 0.0622 ms with the trigger at block exit, as here).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Status bits written by kernels (atomicOr) and read by the host after a step.
enum : int32_t { kStatusNonFinite = 1, kStatusClamped = 2, kStatusBufferOverflow = 4 };

// Per-scene constants.  Every derived constant is formed on the host with the same
// IEEE operation sequence the Julia code would use at the point of use, so using the
// constant inside a kernel rounds exactly like recomputing it there.
struct SceneDev {
    // cell grid
    double lo[3];
    double inv_cell[3];
    double cell_d[3];   // cell edge per axis; cell c starts at lo + c * cell_d
    int32_t n[3];
    int32_t reach;      // neighbour cells within +-reach (cells per r_cut)
    int32_t prune;      // 1: the FP32 walks skip neighbour cells beyond r_cut (row_span)
    int32_t cell_off;   // first global cell of this scene
    int32_t ncells;
    int32_t periodic_x;
    double period;      // domain_hi[0] - domain_lo[0]
    double half_period; // 0.5 * period
    double wrap_hi;     // lo[0] + period

    // SmoothKernel
    double h, sigma, k0, rc2;
    double kw_a;   // CubicSpline: sigma/4; Gaussian: sigma; WendlandC2: sigma; WendlandC4: sigma
    double kg_a;   // gradient prefactor (see kernel_wdw)
    double hh001;  // 0.01 * (h * h)

    // model
    double rho0, c0, p0, b, nu0, t0, cp, beta, P_bg;  // P_bg = p0 / (rho0 * rho0)
    double inv_cp_d;  // 1.0 / cp
    double g[3];
    double bous[3];  // -g[k] * beta (Boussinesq prefactor)
    int32_t gamma;
    int32_t thermal;
    int32_t wall_pressure;
    int32_t uniform_gap;
    int32_t check_enabled;
    int32_t nan_check;
    double dt, half_dtdt;  // half_dtdt = dt * dt * 0.5 (scaling by 0.5 is exact)
    double dtdt;     // dt * dt
    int64_t reinit_interval;
    int64_t check_interval;
    int64_t last_step;  // the scene is frozen (state kept, no physics) after this step
    int32_t active;     // 0: retired, its particles are dropped at the next sort
    int32_t pad_active;
    double check_lo[3];
    double check_hi[3];
    double inv_rho0;  // 1 / rho0 (FP32-compensated form's equation of state)

    // FP32-compensated form
    float cell_f[3];   // cell edge per axis (float)
    float h_f, rc2_f, hh001_f, nu0_f, P_bg_f;
    float kw_a_f, kg_a_f, inv_h_f, c0_f, rho0_f, inv_cp_f, inv_rho0_f;
    float rc2_prune;    // rc2_f * (1 + 1e-5): conservative bound for the stencil pruning
    float inv_cell_fx;  // 1 / cell_f[0]
    float pad_f;
};

// ---------------------------------------------------------------- vector types
template <int DIM> struct VecT;
template <> struct VecT<2> { using T = double2; };
template <> struct VecT<3> { using T = double4_32a; };  // 32-byte aligned: one 256-bit access

template <int DIM> struct FVec;
template <> struct FVec<2> { using T = float2; };
template <> struct FVec<3> { using T = float4; };

__device__ __forceinline__ double comp(const double2& a, int k) { return k == 0 ? a.x : a.y; }
__device__ __forceinline__ double comp(const double4_32a& a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// ---------------------------------------------------------------- state buffers
struct SortedState {
    void* x;
    void* v;
    double* rho;   // density at the start of the step
    double* rhoc;  // density after the continuity update (K4 output)
    double* p;
    double* c;
    double* P;
    double* m;
    double* gap;
    double* T;
    double* kappa;
    double* cp;
    int32_t* id;
    int32_t* scene;
    // FP32 shadows (allocated only for the compensated form)
    float4* fa;   // 2D: (xr, yr, vx, vy)      3D: (xr, yr, zr, m)
    float4* fb;   // 2D: (m, rho, P, gap)      3D: (vx, vy, vz, rho)
    float4* fc;   // 2D: (T, kappa, cp, -)     3D: (P, gap, T, kappa)
    float* fd;    // 3D: cp
    int32_t* cell;  // cell key of the particle (global)
    double* vol;    // m / rho after continuity (FP32 form: FP64 Shepard weights)
};

struct NextState {
    void* x;
    void* v;
    double* T;
    double* rho;
};

struct WallState {
    void* x;       // VecT
    void* nrm;     // VecT
    void* v;       // VecT
    double* gap;
    double* T;
    double* kappa;
    int32_t* kind;
    int32_t* start;  // global cells + 1
    uint8_t* near;   // global cells: 1 where a wall particle lies within +-reach cells
    float4* fa;      // FP32: 2D (xr, yr, nx, ny)    3D (xr, yr, zr, gap)
    float4* fb;      // FP32: 2D (vx, vy, gap, T)    3D (nx, ny, nz, T)
    float4* fc;      // FP32: 2D (kappa, kind, -, -) 3D (vx, vy, vz, kappa)
    int32_t* cell;
    int64_t n;
};

// Neighbour list of the FP32 form: the continuity gather records, in its walk order,
// every neighbour within r_cut of each particle; the momentum gather of the same step
// reads it instead of walking the cells again (the pairs are the same: positions do not
// change between the two gathers).  Entry k of particle i is e[k * stride + i] =
// (j - i) << 9 | (dz + m) << 6 | (dy + m) << 3 | (dx + m): j the sorted index of the
// neighbour, (dx, dy, dz) the offset of j's cell from i's cell, m the reach in cells.
// A one-lane writer fills entries 0, 1, ...; with two lanes, lane 0 fills them from 0 up
// and lane 1 from kmax - 1 down.  n[i] = front | back << 16 (the entries written by the
// two lanes), or kListWalk when they do not fit (more than kmax neighbours, j - i outside
// 23 bits, or m > 3): momentum then walks the cells for i.  The list of i reads as
// entries 0 .. front - 1, then kmax - 1 down to kmax - back.
struct NbrList {
    int32_t* e;
    int32_t* n;
    int32_t kmax;
    int64_t stride;
};
constexpr int32_t kListWalk = 0x7fffffff;
constexpr int32_t kListDelta = 1 << 22;  // |j - i| < kListDelta

struct SortScratch {
    int32_t* key;    // per particle (unsorted index): global cell key or kDeadKey
    int32_t* slot;   // per particle: arrival slot inside its cell
    int32_t* count;  // per cell
    int32_t* start;  // per cell + 1: exclusive scan of count
    int32_t* tmp;    // per sorted position: id by arrival slot
    int32_t* block_sums;
    int32_t* n_live;    // device scalar: live particles after the last sort
    int32_t* status;    // device scalar: status bits
    int64_t* scene_step;  // per scene: number of the step being run
    // non-null in a step whose scan runs over 1,024-cell tiles: the momentum epilogue adds
    // each particle's arrival to its tile's sum here (the scan then skips its tile pass)
    int32_t* tile_acc;
};

constexpr int32_t kScanTileCells = 1024;  // cells of a tile of the two-launch scan

// Warp-aggregated count of arrivals per scan tile: the lanes that reach this call
// together (a coalesced group, whatever branch brought them here) are partitioned by
// tile, and one lane per tile adds the partition's size.
__device__ __forceinline__ void count_tile(int32_t* tile_acc, int32_t key) {
    if (!tile_acc) return;
    const int tile = key / kScanTileCells;
    const cooperative_groups::coalesced_group here = cooperative_groups::coalesced_threads();
    const cooperative_groups::coalesced_group peers = cooperative_groups::labeled_partition(here, tile);
    if (peers.thread_rank() == 0) atomicAdd(tile_acc + tile, (int32_t)peers.size());
}

// A particle arrives in cell `key` for the next sort: its key, its arrival slot in the
// cell and, when the step's scan reads tile sums (sc.tile_acc), its tile's count.  Every
// site that adds to sc.count goes through here, so the tile sums can never miss one.
__device__ __forceinline__ void cell_arrival(const SortScratch& sc, int32_t i, int32_t key) {
    sc.key[i] = key;
    sc.slot[i] = atomicAdd(sc.count + key, 1);
    count_tile(sc.tile_acc, key);
}

// ---------------------------------------------------------------- inlet/outlet buffers
// Buffer particles (FluidInletOutletWallSolve.jl:8-262): fluid particles of the inlet and
// outlet regions.  They are neighbours of the fluid in continuity and momentum but are
// not updated by them: they move with their own velocity (x += v dt) and keep their
// density, pressure and sound speed.  Sorted by (cell, order) like the fluid by (cell, id).
// order: bit 62 = outlet; inlet particle k: k; outlet particle uploaded as k:
// kOutletBit | k; fluid particle id moved to the outlet at step first_step + r:
// kOutletBit | (r + 1) << 32 | id.  Ascending order is the reference's vector order.
constexpr int64_t kOutletBit = int64_t(1) << 62;

struct BufferState {
    void* x;  // V
    void* v;  // V
    double* rho;
    double* p;
    double* c;
    double* m;
    double* gap;
    int64_t* order;
    const int32_t* start;  // cell starts of the buffer particles (scene grid, ncells + 1)
    const int32_t* n;      // device scalar: live buffer particles; null when the handle has none
};

struct BufferScratch {
    int32_t* key;
    int32_t* slot;
    int32_t* count;    // per cell
    int32_t* start;    // per cell + 1 (the next step's BufferState::start)
    int64_t* tmp;      // order by arrival slot
    int32_t* block_sums;
    int32_t* pend;     // fluid particles moving to the outlet this step
    int32_t* npend;    // device scalar
    int32_t cap;       // buffer capacity (also the capacity of pend)
};

// Transfer rules: plane tests n.x > d (the example's checks compare one coordinate with a
// bound, PoiseuilleFlow2D.jl:146-151), the inlet shift of the modify step, and the id
// arithmetic of fluid particles created from the inlet.
struct BufferRules {
    double in_n[3], in_d, in_shift[3];  // inlet_into_calculation_domain_check / _modify
    double out_n[3], out_d;             // outlet_out_calculation_domain_check
    double drop_n[3], drop_d;           // outlet_out_check
    int64_t n_inlet;                    // inlet particles (their count never changes)
    int64_t id_base;                    // id of the first fluid particle made from the inlet
    int64_t first_step;                 // step of the buffer upload
};

// n.x > d, products and sums rounded one by one, x ascending (no contraction, so every
// form and the CPU restatement take the same decisions).
template <int DIM>
__device__ __forceinline__ bool beyond_plane(const double n[3], double d, const double x[DIM]) {
    double s = __dmul_rn(n[0], x[0]);
    s = __dadd_rn(s, __dmul_rn(n[1], x[1]));
    if (DIM == 3) s = __dadd_rn(s, __dmul_rn(n[2], x[DIM - 1]));
    return s > d;
}

// ---------------------------------------------------------------- grid
__device__ __forceinline__ int32_t cell_coord(double x, const SceneDev& S, int a) {
    const double u = (x - S.lo[a]) * S.inv_cell[a];
    if (!(u >= 0.0)) return 0;
    const double f = floor(u);
    if (f >= (double)(S.n[a] - 1)) return S.n[a] - 1;
    return (int32_t)f;
}

// Whether coordinate lies outside the grid (the particle was clamped into an edge cell).
__device__ __forceinline__ bool outside_grid(double x, const SceneDev& S, int a) {
    const double u = (x - S.lo[a]) * S.inv_cell[a];
    return !(u >= 0.0) || u >= (double)S.n[a];
}

// ---------------------------------------------------------------- Julia numerics
// Base ^(x::Float64, n::Integer) (compensated power by squaring; exact products by fma).
__device__ __forceinline__ double jl_powi(double x, int n) {
    if (n == 0) return 1.0;
    if (n == 3) return __dmul_rn(__dmul_rn(x, x), x);
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    if (n < 0) {
        const double rx = 1.0 / x;
        if (n == -2) return __dmul_rn(rx, rx);
        if (isfinite(x)) xnlo = __dmul_rn(-fma(x, rx, -1.0), rx);
        x = rx;
        n = -n;
    }
    while (n > 1) {
        if (n & 1) {
            const double err = fma(y, xnlo, __dmul_rn(x, ynlo));
            const double yh = __dmul_rn(x, y);
            const double yl = fma(x, y, -yh);
            y = yh;
            ynlo = __dadd_rn(yl, err);
        }
        const double err = __dmul_rn(__dmul_rn(x, 2.0), xnlo);
        const double xh = __dmul_rn(x, x);
        const double xl = fma(x, x, -xh);
        x = xh;
        xnlo = __dadd_rn(xl, err);
        n >>= 1;
    }
    const double err = fma(y, xnlo, __dmul_rn(x, ynlo));
    return (isfinite(x) && isfinite(err)) ? fma(x, y, err) : __dmul_rn(x, y);
}

}  // namespace sph
