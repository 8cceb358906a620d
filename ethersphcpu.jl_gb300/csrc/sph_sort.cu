// sph_sort.cu — the per-step cell list: hash, exclusive scan, stable (cell, id)
// placement with the SoA reorder, plus FP64 reductions and the pair counter.
//
// Replaces CellListMap.update!/neighborlist! + findNeighbours! (Neighbour.jl:88-128,
// FluidWallSolve.jl:21-35): instead of a materialised pair list, particles are kept
// physically sorted by (cell key, id) and every gather kernel walks the 9 (2D) or 27
// (3D) neighbour cells.  Counting sort:
//   1. hash: key = cell of the position, slot = atomicAdd(count[key]) (fused into the
//      momentum kernel for every step after the first)
//   2. exclusive scan of count -> start (3 kernels: tile sums, top scan, tile scan)
//   3. fill: tmp[start[key] + slot] = id       (arrival order, nondeterministic)
//   4. place: rank = #ids in the cell smaller than mine -> destination start[key]+rank,
//      copy every field there (deterministic: the order is (cell, id) whatever the
//      arrival order was)
#include "sph_physics.cuh"
#include "sph_kernels.h"

namespace sph {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // cells per tile
constexpr int kScanTopThreads = 1024;
constexpr int kScanTopItems = 16;

int scan_max_cells() { return kScanTile * kScanTopThreads * kScanTopItems; }

// ---------------------------------------------------------------- hash (after upload)
template <int DIM>
__global__ void k_hash(const SceneDev* __restrict__ scenes, NextState nx, SortedState st, SortScratch sc,
                       int32_t cap) {
    using V = typename VecT<DIM>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || i >= *sc.n_live) return;
    const SceneDev& S = scenes[st.scene[i]];
    if (!S.active) {  // retired scene: dropped by this sort
        sc.key[i] = kDeadKey;
        return;
    }
    const V x = ((const V*)nx.x)[i];
    cell_arrival(sc, i, cell_key<DIM>(x, S));
}

// ---------------------------------------------------------------- scan
// Block-wide exclusive scan of one value per thread; returns the prefix, *total gets
// the block sum.
template <int THREADS>
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* warp_sums, int32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        constexpr int NW = THREADS / 32;
        int32_t w = lane < NW ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < NW) warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    const int32_t warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0;
    *total = warp_sums[THREADS / 32 - 1];
    return warp_prefix + inc - v;
}

template <int ITEMS>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t* __restrict__ count, int32_t n,
                                                            int32_t* __restrict__ tile_sums) {
    pdl_wait();
    __shared__ int32_t red[kScanThreads / 32];
    const int base = blockIdx.x * kScanThreads * ITEMS;
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = base + k * kScanThreads + threadIdx.x;
        s += idx < n ? count[idx] : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
        tile_sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kScanTopThreads) k_scan_top(int32_t* __restrict__ tile_sums, int32_t ntiles,
                                                             int32_t* __restrict__ start_total,
                                                             int32_t* __restrict__ n_next,
                                                             int64_t* __restrict__ scene_step, int32_t nscenes,
                                                             int advance) {
    pdl_wait();
    __shared__ int32_t warp_sums[kScanTopThreads / 32];
    int32_t v[kScanTopItems];
    int32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanTopItems; ++k) {
        const int idx = threadIdx.x * kScanTopItems + k;
        v[k] = idx < ntiles ? tile_sums[idx] : 0;
        local += v[k];
    }
    int32_t total;
    int32_t run = block_exclusive_scan<kScanTopThreads>(local, warp_sums, &total);
#pragma unroll
    for (int k = 0; k < kScanTopItems; ++k) {
        const int idx = threadIdx.x * kScanTopItems + k;
        if (idx < ntiles) tile_sums[idx] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) {
        *start_total = total;
        *n_next = total;
    }
    if (advance)
        for (int s = threadIdx.x; s < nscenes; s += blockDim.x) scene_step[s] += 1;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const int32_t* __restrict__ count, int32_t n,
                                                           const int32_t* __restrict__ tile_offsets,
                                                           int32_t* __restrict__ start) {
    pdl_wait();
    __shared__ int32_t tile[kScanTile];
    __shared__ int32_t warp_sums[kScanThreads / 32];
    const int base = blockIdx.x * kScanTile;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int idx = k * kScanThreads + threadIdx.x;
        tile[idx] = base + idx < n ? count[base + idx] : 0;
    }
    __syncthreads();
    int32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) local += tile[threadIdx.x * kScanItems + k];
    int32_t total;
    int32_t run = block_exclusive_scan<kScanThreads>(local, warp_sums, &total) + tile_offsets[blockIdx.x];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int idx = threadIdx.x * kScanItems + k;
        const int32_t c = tile[idx];
        tile[idx] = run;
        run += c;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int idx = k * kScanThreads + threadIdx.x;
        if (base + idx < n) start[base + idx] = tile[idx];
    }
}

// Down-sweep that forms its tile's offset itself from the tile sums of k_scan_tiles (a
// block reduction over the tiles before it): two launches instead of three for grids of
// at most kScanDirectTiles tiles of kScanDirectItems x 256 cells (small tiles: many
// blocks in flight on a small grid).  Block 0 also writes the total and advances the
// steps.
constexpr int kScanDirectItems = kScanTileCells / kScanThreads;
constexpr int kScanDirectTile = kScanThreads * kScanDirectItems;
constexpr int kScanDirectTiles = 256;

__global__ void __launch_bounds__(kScanThreads) k_scan_down_direct(const int32_t* __restrict__ count, int32_t n,
                                                                  const int32_t* __restrict__ tile_sums,
                                                                  int32_t ntiles, int32_t* __restrict__ start,
                                                                  int32_t* __restrict__ n_next,
                                                                  int64_t* __restrict__ scene_step, int32_t nscenes,
                                                                  int advance) {
    pdl_wait();
    constexpr int ITEMS = kScanDirectItems;
    __shared__ int32_t tile[kScanDirectTile];
    __shared__ int32_t warp_sums[kScanThreads / 32];
    __shared__ int32_t offset;
    const int base = blockIdx.x * kScanDirectTile;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = k * kScanThreads + threadIdx.x;
        tile[idx] = base + idx < n ? count[base + idx] : 0;
    }
    if (threadIdx.x < 32) {  // offset of this tile: sum of the tile sums before it
        const int upto = blockIdx.x == 0 ? ntiles : blockIdx.x;  // block 0: the total
        int32_t t = 0;
        for (int q = threadIdx.x; q < upto; q += 32) t += tile_sums[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) {
            offset = blockIdx.x == 0 ? 0 : t;
            if (blockIdx.x == 0) {
                start[n] = t;
                *n_next = t;
            }
        }
    }
    if (blockIdx.x == 0 && advance)
        for (int q = threadIdx.x; q < nscenes; q += blockDim.x) scene_step[q] += 1;
    __syncthreads();
    int32_t local = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) local += tile[threadIdx.x * ITEMS + k];
    int32_t total;
    int32_t run = block_exclusive_scan<kScanThreads>(local, warp_sums, &total) + offset;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = threadIdx.x * ITEMS + k;
        const int32_t c = tile[idx];
        tile[idx] = run;
        run += c;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = k * kScanThreads + threadIdx.x;
        if (base + idx < n) start[base + idx] = tile[idx];
    }
}

// ---------------------------------------------------------------- placement
__global__ void k_fill(SortScratch sc, const int32_t* __restrict__ id, int32_t cap) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || i >= *sc.n_live) return;
    const int32_t key = sc.key[i];
    if (key == kDeadKey) return;
    sc.tmp[sc.start[key] + sc.slot[i]] = id[i];
}

// CARRY (FP32 shadows of a step): the FP32 copies of the per-particle constants (m, gap,
// kappa, cp) are taken from the particle's current shadows instead of being converted from
// FP64 again (the FP64 pipe is 1/64 of the FP32 rate on GB300); after an upload the
// shadows do not exist yet and are converted.
template <int DIM, bool THERMAL, bool SHADOW, bool CARRY>
__global__ void k_place(const SceneDev* __restrict__ scenes, SortedState src, NextState nx, SortedState dst,
                        SortScratch sc, int32_t cap, int32_t ncells) {
    pdl_wait();
    using V = typename VecT<DIM>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // count[] and the tile sums have been scanned: clear them for the next step's arrivals
    for (int k = i; k < ncells; k += gridDim.x * blockDim.x) sc.count[k] = 0;
    for (int k = i; k < ncells / kScanTileCells + 1; k += gridDim.x * blockDim.x) sc.block_sums[k] = 0;
    if (i >= cap || i >= *sc.n_live) return;
    const int32_t key = sc.key[i];
    if (key == kDeadKey) return;
    // every source element is loaded before the first store: the compiler cannot prove
    // that the destination arrays do not alias the sources, and would otherwise order
    // each load after the previous store (one memory round trip per field)
    const V x = ((const V*)nx.x)[i];
    const V v = ((const V*)nx.v)[i];
    const double rho = nx.rho[i], p = src.p[i], c = src.c[i], m = src.m[i], gap = src.gap[i];
    const int32_t myid = src.id[i], scn = src.scene[i];
    double T = 0.0, kap = 0.0, cpv = 1.0;
    if (THERMAL) {
        T = nx.T[i];
        kap = src.kappa[i];
        cpv = src.cp[i];
    }
    // FP32 constants: carried from the current shadows, or converted
    float m_f, gap_f, kap_f = 0.f, cp_f = 1.f;
    if constexpr (SHADOW && CARRY) {
        if constexpr (DIM == 2) {
            const float4 b = src.fb[i];
            m_f = b.x;
            gap_f = b.w;
            if (THERMAL) {
                const float4 cc = src.fc[i];
                kap_f = cc.y;
                cp_f = cc.z;
            }
        } else {
            const float4 a = src.fa[i];
            const float4 cc = src.fc[i];
            m_f = a.w;
            gap_f = cc.y;
            if (THERMAL) {
                kap_f = cc.w;
                cp_f = src.fd[i];
            }
        }
    } else {
        m_f = (float)m;
        gap_f = (float)gap;
        if (THERMAL) {
            kap_f = (float)kap;
            cp_f = (float)cpv;
        }
    }
    const int32_t b = sc.start[key], e = sc.start[key + 1];
    int32_t rank = 0;
    for (int32_t t = b; t < e; ++t) rank += sc.tmp[t] < myid;
    const int32_t d = b + rank;
    ((V*)dst.x)[d] = x;
    ((V*)dst.v)[d] = v;
    dst.rho[d] = rho;
    dst.p[d] = p;
    dst.c[d] = c;
    dst.m[d] = m;
    dst.gap[d] = gap;
    dst.id[d] = myid;
    dst.scene[d] = scn;
    if (THERMAL) {
        dst.T[d] = T;
        dst.kappa[d] = kap;
        dst.cp[d] = cpv;
    }
    if (SHADOW) {  // FP32 shadows: position relative to the origin of the particle's cell
        const SceneDev& S = scenes[scn];
        const int32_t k = key - S.cell_off;
        const int32_t cx = k % S.n[0], cy = (k / S.n[0]) % S.n[1], cz = k / (S.n[0] * S.n[1]);
        const float xr = (float)(x.x - __dadd_rn(S.lo[0], __dmul_rn((double)cx, S.cell_d[0])));
        const float yr = (float)(x.y - __dadd_rn(S.lo[1], __dmul_rn((double)cy, S.cell_d[1])));
        dst.cell[d] = key;
        if constexpr (DIM == 2) {
            dst.fa[d] = make_float4(xr, yr, (float)v.x, (float)v.y);
            dst.fb[d] = make_float4(m_f, (float)rho, 0.f, gap_f);
            dst.fc[d] = make_float4((float)T, kap_f, cp_f, 0.f);
        } else {
            const float zr = (float)(x.z - __dadd_rn(S.lo[2], __dmul_rn((double)cz, S.cell_d[2])));
            dst.fa[d] = make_float4(xr, yr, zr, m_f);
            dst.fb[d] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)rho);
            dst.fc[d] = make_float4(0.f, gap_f, (float)T, kap_f);
            dst.fd[d] = cp_f;
        }
    }
}

// ---------------------------------------------------------------- reductions
constexpr int kStatThreads = 256;
constexpr int kStatBlocks = 152;

template <int DIM>
__global__ void __launch_bounds__(kStatThreads) k_stats_partial(SortedState st, const int32_t* __restrict__ n_live,
                                                               double* __restrict__ partials) {
    using V = typename VecT<DIM>::T;
    __shared__ double sm[3][kStatThreads];
    const int n = *n_live;
    double m = 0.0, ke = 0.0, vmax = 0.0;
    for (int i = blockIdx.x * kStatThreads + threadIdx.x; i < n; i += gridDim.x * kStatThreads) {
        const V v = ((const V*)st.v)[i];
        double v2 = v.x * v.x + v.y * v.y;
        if (DIM == 3) v2 += comp(v, DIM - 1) * comp(v, DIM - 1);
        m += st.m[i];
        ke += 0.5 * st.m[i] * v2;
        vmax = fmax(vmax, sqrt(v2));
    }
    sm[0][threadIdx.x] = m;
    sm[1][threadIdx.x] = ke;
    sm[2][threadIdx.x] = vmax;
    __syncthreads();
    for (int s = kStatThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sm[0][threadIdx.x] += sm[0][threadIdx.x + s];
            sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
            sm[2][threadIdx.x] = fmax(sm[2][threadIdx.x], sm[2][threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x + 0] = sm[0][0];
        partials[3 * blockIdx.x + 1] = sm[1][0];
        partials[3 * blockIdx.x + 2] = sm[2][0];
    }
}

__global__ void k_stats_final(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double m = 0.0, ke = 0.0, vmax = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        m += partials[3 * b];
        ke += partials[3 * b + 1];
        vmax = fmax(vmax, partials[3 * b + 2]);
    }
    out[0] = m;
    out[1] = ke;
    out[2] = vmax;
}

template <int DIM>
__global__ void k_count_pairs(const SceneDev* __restrict__ scenes, SortedState st, WallState wl, SortScratch sc,
                              int32_t cap, unsigned long long* counts) {
    using V = typename VecT<DIM>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap || i >= *sc.n_live) return;
    const SceneDev& S = scenes[st.scene[i]];
    const V* x = (const V*)st.x;
    const V xi = x[i];
    int32_t c[3];
    cell_of<DIM>(xi, S, c);
    unsigned long long a = 0, b = 0;
    walk_cells<DIM>(S, sc.start, c, [&](int jb, int je) {
        for (int j = jb; j < je; ++j) {
            if (j <= i) continue;
            double rv[DIM];
            make_rvec<DIM>(xi, x[j], S, rv);
            a += norm_sq<DIM>(rv) <= S.rc2;
        }
    });
    if (wl.n > 0) {
        const V* wx = (const V*)wl.x;
        walk_cells<DIM>(S, wl.start, c, [&](int jb, int je) {
            for (int w = jb; w < je; ++w) {
                double rv[DIM];
                make_rvec<DIM>(xi, wx[w], S, rv);
                b += norm_sq<DIM>(rv) <= S.rc2;
            }
        });
    }
    atomicAdd(counts, a);
    atomicAdd(counts + 1, b);
}

// ---------------------------------------------------------------- launchers
void launch_hash(const LaunchCtx& L) {
    const int grid = (L.cap + 127) / 128;
    if (L.dim == 2) k_hash<2><<<grid, 128, 0, L.stream>>>(L.scenes, L.nx, L.st, L.sc, L.cap);
    else k_hash<3><<<grid, 128, 0, L.stream>>>(L.scenes, L.nx, L.st, L.sc, L.cap);
}

// Whole scan in one block, chunk by chunk (1024 x 16 cells each) with a running carry,
// when the grid has at most kScanSingleChunks chunks: one launch.  One block moves the
// whole array through one SM, so more chunks are faster as two launches over many SMs
// (about 3.4 us per chunk against 10 us for two or three launches on GB300).
constexpr int kScanChunk = kScanTopThreads * kScanTopItems;
constexpr int kScanSingleChunks = 1;

__global__ void __launch_bounds__(kScanTopThreads) k_scan_single(const int32_t* __restrict__ count, int32_t n,
                                                                int32_t* __restrict__ start,
                                                                int32_t* __restrict__ n_next,
                                                                int64_t* __restrict__ scene_step, int32_t nscenes,
                                                                int advance) {
    pdl_wait();
    __shared__ int32_t warp_sums[kScanTopThreads / 32];
    int32_t carry = 0;
    for (int base = 0; base < n; base += kScanChunk) {
        // a thread's 16 cells are 64 contiguous bytes: four 16-byte loads and stores
        // (count and start are cudaMalloc'd, the thread's first cell a multiple of 16)
        const int first = base + threadIdx.x * kScanTopItems;
        const bool whole = first + kScanTopItems <= n;
        int32_t v[kScanTopItems];
        int32_t local = 0;
        if (whole) {
#pragma unroll
            for (int q = 0; q < kScanTopItems / 4; ++q) {
                const int4 w = reinterpret_cast<const int4*>(count + first)[q];
                v[4 * q] = w.x;
                v[4 * q + 1] = w.y;
                v[4 * q + 2] = w.z;
                v[4 * q + 3] = w.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < kScanTopItems; ++k) v[k] = first + k < n ? count[first + k] : 0;
        }
#pragma unroll
        for (int k = 0; k < kScanTopItems; ++k) local += v[k];
        int32_t total;
        int32_t run = block_exclusive_scan<kScanTopThreads>(local, warp_sums, &total) + carry;
#pragma unroll
        for (int k = 0; k < kScanTopItems; ++k) {
            const int32_t c = v[k];
            v[k] = run;
            run += c;
        }
        if (whole) {
#pragma unroll
            for (int q = 0; q < kScanTopItems / 4; ++q)
                reinterpret_cast<int4*>(start + first)[q] = make_int4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else {
#pragma unroll
            for (int k = 0; k < kScanTopItems; ++k)
                if (first + k < n) start[first + k] = v[k];
        }
        carry += total;
        __syncthreads();  // warp_sums is rewritten by the next chunk
    }
    if (threadIdx.x == 0) {
        start[n] = carry;
        *n_next = carry;
    }
    if (advance)
        for (int s = threadIdx.x; s < nscenes; s += blockDim.x) scene_step[s] += 1;
}

bool scan_uses_tiles(int n) {
    return n > kScanSingleChunks * kScanChunk && (n + kScanDirectTile - 1) / kScanDirectTile <= kScanDirectTiles;
}

void launch_scan(const LaunchCtx& L, int advance, bool tiles_ready) {
    const int n = L.total_cells;
    if (n <= kScanSingleChunks * kScanChunk) {
        launch_dep(k_scan_single, 1, kScanTopThreads, L.stream, L.sc.count, n, L.sc.start, L.n_next, L.sc.scene_step,
                   L.nscenes, advance);
        return;
    }
    const int dtiles = (n + kScanDirectTile - 1) / kScanDirectTile;
    if (dtiles <= kScanDirectTiles) {
        if (!tiles_ready)
            launch_dep(k_scan_tiles<kScanDirectItems>, dtiles, kScanThreads, L.stream, L.sc.count, n, L.sc.block_sums);
        launch_dep(k_scan_down_direct, dtiles, kScanThreads, L.stream, L.sc.count, n, L.sc.block_sums, dtiles,
                   L.sc.start, L.n_next, L.sc.scene_step, L.nscenes, advance);
        return;
    }
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    launch_dep(k_scan_tiles<kScanItems>, ntiles, kScanThreads, L.stream, L.sc.count, n, L.sc.block_sums);
    launch_dep(k_scan_top, 1, kScanTopThreads, L.stream, L.sc.block_sums, ntiles, L.sc.start + n, L.n_next,
               L.sc.scene_step, L.nscenes, advance);
    launch_dep(k_scan_down, ntiles, kScanThreads, L.stream, L.sc.count, n, L.sc.block_sums, L.sc.start);
}

// Rows of a download in the caller's order: row q takes sorted particle b + order[q];
// out = x (n x dim), v (n x dim), then one n-array per requested field.
template <int DIM>
__global__ void k_gather_rows(const int32_t* __restrict__ order, int64_t n, int32_t b, const void* __restrict__ x,
                              const void* __restrict__ v, DownloadFields F, double* __restrict__ out) {
    using V = typename VecT<DIM>::T;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int64_t k = b + order[q];
    double* o = out;
    if (F.x) {
        const V xv = ((const V*)x)[k];
        o[q * DIM] = xv.x;
        o[q * DIM + 1] = xv.y;
        if constexpr (DIM == 3) o[q * DIM + 2] = xv.z;
        o += n * DIM;
    }
    if (F.v) {
        const V vv = ((const V*)v)[k];
        o[q * DIM] = vv.x;
        o[q * DIM + 1] = vv.y;
        if constexpr (DIM == 3) o[q * DIM + 2] = vv.z;
        o += n * DIM;
    }
    for (int f = 0; f < F.n; ++f) o[f * n + q] = F.src[f][k];
}

// Rows of a download when the scene's ids are a permutation of 0 .. n-1 (no particle
// deleted or created since the upload): sorted particle b + k goes to row id[b + k], the
// caller's original order, with no order computed on the host.
template <int DIM>
__global__ void k_scatter_rows(const int32_t* __restrict__ id, int64_t n, int32_t b, const void* __restrict__ x,
                               const void* __restrict__ v, DownloadFields F, double* __restrict__ out) {
    using V = typename VecT<DIM>::T;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t q = id[b + k];
    double* o = out;
    if (F.x) {
        const V xv = ((const V*)x)[b + k];
        o[q * DIM] = xv.x;
        o[q * DIM + 1] = xv.y;
        if constexpr (DIM == 3) o[q * DIM + 2] = xv.z;
        o += n * DIM;
    }
    if (F.v) {
        const V vv = ((const V*)v)[b + k];
        o[q * DIM] = vv.x;
        o[q * DIM + 1] = vv.y;
        if constexpr (DIM == 3) o[q * DIM + 2] = vv.z;
        o += n * DIM;
    }
    for (int f = 0; f < F.n; ++f) o[f * n + q] = F.src[f][b + k];
}

void launch_scatter_rows(cudaStream_t stream, int dim, const int32_t* id, int64_t n, int32_t b, const void* x,
                         const void* v, const DownloadFields& F, double* out) {
    const int grid = (int)((n + 255) / 256);
    if (dim == 2) k_scatter_rows<2><<<grid, 256, 0, stream>>>(id, n, b, x, v, F, out);
    else k_scatter_rows<3><<<grid, 256, 0, stream>>>(id, n, b, x, v, F, out);
}

// Upload of fluid particles [o, o + n) of scene s: ids 0 .. n-1 in upload order and the
// scene index; in 3D the caller's n x 3 positions and velocities (staged on the device)
// widen to the 32-byte records of the state.
__global__ void k_upload_ids(int32_t* __restrict__ id, int32_t* __restrict__ scene, int64_t n, int32_t s) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    id[i] = (int32_t)i;
    scene[i] = s;
}

__global__ void k_widen3(const double* __restrict__ x3, const double* __restrict__ v3, double4_32a* __restrict__ x,
                         double4_32a* __restrict__ v, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a a, w;
    a.x = x3[3 * i]; a.y = x3[3 * i + 1]; a.z = x3[3 * i + 2]; a.w = 0.0;
    w.x = v3[3 * i]; w.y = v3[3 * i + 1]; w.z = v3[3 * i + 2]; w.w = 0.0;
    x[i] = a;
    v[i] = w;
}

void launch_upload_ids(cudaStream_t stream, int32_t* id, int32_t* scene, int64_t n, int32_t s) {
    if (n > 0) k_upload_ids<<<(int)((n + 255) / 256), 256, 0, stream>>>(id, scene, n, s);
}

void launch_widen3(cudaStream_t stream, const double* x3, const double* v3, void* x, void* v, int64_t n) {
    if (n > 0)
        k_widen3<<<(int)((n + 255) / 256), 256, 0, stream>>>(x3, v3, (double4_32a*)x, (double4_32a*)v, n);
}

void launch_gather_rows(cudaStream_t stream, int dim, const int32_t* order, int64_t n, int32_t b, const void* x,
                        const void* v, const DownloadFields& F, double* out) {
    const int grid = (int)((n + 255) / 256);
    if (dim == 2) k_gather_rows<2><<<grid, 256, 0, stream>>>(order, n, b, x, v, F, out);
    else k_gather_rows<3><<<grid, 256, 0, stream>>>(order, n, b, x, v, F, out);
}

void launch_place(const LaunchCtx& L, bool carry_shadows) {
    const int grid = (L.cap + 127) / 128;
    launch_dep(k_fill, grid, 128, L.stream, L.sc, L.st.id, L.cap);
#define SPH_PLACE(D, T, SH, CA) \
    launch_dep(k_place<D, T, SH, CA>, grid, 128, L.stream, L.scenes, L.st, L.nx, L.st2, L.sc, L.cap, L.total_cells)
#define SPH_PLACE_SH(D, T) \
    do { if (!sh) SPH_PLACE(D, T, false, false); else if (carry_shadows) SPH_PLACE(D, T, true, true); \
         else SPH_PLACE(D, T, true, false); } while (0)
    const bool sh = L.precision == SPH_PRECISION_FP32_COMPENSATED;
    if (L.dim == 2) {
        if (L.thermal) SPH_PLACE_SH(2, true);
        else SPH_PLACE_SH(2, false);
    } else {
        if (L.thermal) SPH_PLACE_SH(3, true);
        else SPH_PLACE_SH(3, false);
    }
#undef SPH_PLACE_SH
#undef SPH_PLACE
}

void launch_stats(const LaunchCtx& L, double* d_partials, double* d_out) {
    if (L.dim == 2) k_stats_partial<2><<<kStatBlocks, kStatThreads, 0, L.stream>>>(L.st, L.sc.n_live, d_partials);
    else k_stats_partial<3><<<kStatBlocks, kStatThreads, 0, L.stream>>>(L.st, L.sc.n_live, d_partials);
    k_stats_final<<<1, 32, 0, L.stream>>>(d_partials, kStatBlocks, d_out);
}

void launch_count_pairs(const LaunchCtx& L, unsigned long long* d_counts) {
    const int grid = (L.cap + 127) / 128;
    if (L.dim == 2) k_count_pairs<2><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.wl, L.sc, L.cap, d_counts);
    else k_count_pairs<3><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.wl, L.sc, L.cap, d_counts);
}

}  // namespace sph
