// sph_noalloc.cu — pair counting that allocates no device memory.
//
// sph_count_pairs_noalloc() is for callers that cannot let a library call cudaMalloc:
// code running while another framework's stream-ordered memory pool owns the device
// memory, a Julia task that must not trigger a device-wide synchronisation (cudaMalloc
// and cudaFree can synchronise the device), or code enqueued between the kernels of a
// caller-managed stream.  The caller passes its own device buffers and stream; the
// cell list the kernel needs lives in the file-scope array below, which is part of the
// library's module and stays resident on every GPU that loaded the library until the
// process exits.
//
// Limits: at most kMaxParticles fluid and kMaxParticles wall particles and at most
// kMaxCells cells in the grid derived from the parameter block; larger inputs are
// rejected with SPH_ERR_ARG.  Every call uses the same array and leaves its contents
// behind (only the counters are cleared at the start of a call), so calls whose work
// overlaps on the GPU race with each other: serialise them on one stream.
#include <cuda.h>

#include <mutex>
#include <string>

#include "sph_physics.cuh"
#include "sph_kernels.h"

namespace sph {
namespace {

constexpr int64_t kMaxParticles = 262144;
constexpr int64_t kMaxCells = 262144;
constexpr size_t kIdxBytes = kMaxParticles * sizeof(int32_t);
constexpr size_t kCellBytes = (kMaxCells + 64) * sizeof(int32_t);  // + the scan's total
// key, slot, perm for fluid and walls, then count and start for fluid and walls
constexpr size_t kScratchBytes = 6 * kIdxBytes + 4 * kCellBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct Scratch {
    int32_t *f_key, *f_slot, *f_perm, *w_key, *w_slot, *w_perm;
    int32_t *f_count, *f_start, *w_count, *w_start;
};

Scratch carve(unsigned char* base) {
    Scratch s;
    int32_t** idx[] = {&s.f_key, &s.f_slot, &s.f_perm, &s.w_key, &s.w_slot, &s.w_perm};
    size_t off = 0;
    for (int32_t** p : idx) {
        *p = (int32_t*)(base + off);
        off += kIdxBytes;
    }
    int32_t** cells[] = {&s.f_count, &s.f_start, &s.w_count, &s.w_start};
    for (int32_t** p : cells) {
        *p = (int32_t*)(base + off);
        off += kCellBytes;
    }
    return s;
}

template <int DIM>
__device__ __forceinline__ int32_t packed_key(const double* __restrict__ x, int64_t i, const SceneDev& S) {
    int32_t c[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < DIM; ++a) c[a] = cell_coord(x[i * DIM + a], S, a);
    return S.cell_off + (c[2] * S.n[1] + c[1]) * S.n[0] + c[0];
}

template <int DIM>
__global__ void k_na_hash(SceneDev S, int32_t n, const double* __restrict__ x, int32_t* __restrict__ key,
                          int32_t* __restrict__ slot, int32_t* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t k = packed_key<DIM>(x, i, S);
    key[i] = k;
    slot[i] = atomicAdd(count + k, 1);
}

// Exclusive scan of count[0..n) into start[0..n] by one block.
__global__ void __launch_bounds__(1024) k_na_scan(const int32_t* __restrict__ count, int32_t n,
                                                  int32_t* __restrict__ start) {
    __shared__ int32_t warp_sums[32];
    __shared__ int32_t carry;
    constexpr int kItems = 8;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024 * kItems) {
        int32_t v[kItems];
        int32_t local = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int idx = base + threadIdx.x * kItems + k;
            v[k] = idx < n ? count[idx] : 0;
            local += v[k];
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        int32_t inc = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) warp_sums[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            int32_t w = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        int32_t run = carry + (warp > 0 ? warp_sums[warp - 1] : 0) + inc - local;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int idx = base + threadIdx.x * kItems + k;
            if (idx < n) start[idx] = run;
            run += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sums[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) start[n] = carry;
}

__global__ void k_na_place(int32_t n, const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                           const int32_t* __restrict__ start, int32_t* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[start[key[i]] + slot[i]] = i;
}

template <int DIM>
__device__ __forceinline__ double packed_d2(const double* __restrict__ a, int64_t i, const double* __restrict__ b,
                                            int64_t j, const SceneDev& S) {
    double rv[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) rv[k] = a[i * DIM + k] - b[j * DIM + k];
    if (S.periodic_x) {
        if (rv[0] > S.half_period) rv[0] -= S.period;
        else if (rv[0] < -S.half_period) rv[0] += S.period;
    }
    return norm_sq<DIM>(rv);
}

// The counting kernel: unique fluid pairs (i < j by input index) and fluid-wall pairs
// within r_cut, through the cell lists held in the scratch array.
template <int DIM>
__global__ void k_na_count(SceneDev S, int32_t n, const double* __restrict__ x, const int32_t* __restrict__ f_start,
                           const int32_t* __restrict__ f_perm, int32_t nw, const double* __restrict__ wx,
                           const int32_t* __restrict__ w_start, const int32_t* __restrict__ w_perm,
                           unsigned long long* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t c[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < DIM; ++a) c[a] = cell_coord(x[(int64_t)i * DIM + a], S, a);
    unsigned long long a = 0, b = 0;
    walk_cells<DIM>(S, f_start, c, [&](int jb, int je) {
        for (int s = jb; s < je; ++s) {
            const int j = f_perm[s];
            if (j <= i) continue;
            a += packed_d2<DIM>(x, i, x, j, S) <= S.rc2;
        }
    });
    if (nw > 0)
        walk_cells<DIM>(S, w_start, c, [&](int jb, int je) {
            for (int s = jb; s < je; ++s) b += packed_d2<DIM>(x, i, wx, w_perm[s], S) <= S.rc2;
        });
    if (a) atomicAdd(out, a);
    if (b) atomicAdd(out + 1, b);
}

template <int DIM>
void enqueue(const SceneDev& S, const Scratch& s, int32_t n, const double* x, int32_t nw, const double* wx,
             unsigned long long* out, cudaStream_t st) {
    const int nc = S.ncells;
    if (n > 0) k_na_hash<DIM><<<(n + 255) / 256, 256, 0, st>>>(S, n, x, s.f_key, s.f_slot, s.f_count);
    k_na_scan<<<1, 1024, 0, st>>>(s.f_count, nc, s.f_start);
    if (n > 0) k_na_place<<<(n + 255) / 256, 256, 0, st>>>(n, s.f_key, s.f_slot, s.f_start, s.f_perm);
    if (nw > 0) {
        k_na_hash<DIM><<<(nw + 255) / 256, 256, 0, st>>>(S, nw, wx, s.w_key, s.w_slot, s.w_count);
        k_na_scan<<<1, 1024, 0, st>>>(s.w_count, nc, s.w_start);
        k_na_place<<<(nw + 255) / 256, 256, 0, st>>>(nw, s.w_key, s.w_slot, s.w_start, s.w_perm);
    }
    if (n > 0)
        k_na_count<DIM><<<(n + 127) / 128, 128, 0, st>>>(S, n, x, s.f_start, s.f_perm, nw, wx, s.w_start, s.w_perm,
                                                          out);
}

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // unique id of the context the address belongs to

// Unique id (for the life of the process) of the calling thread's current CUDA context,
// through the driver's cuCtxGetCurrent / cuCtxGetId reached by the runtime's entry-point
// query (no link against the driver library); false when there is none or the query fails.
bool current_context_id(unsigned long long* id) {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)f;
        cudaGetLastError();
        resolved = true;
    }
    CUcontext ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

int32_t reject(int32_t code, const std::string& msg) {
    set_global_error(msg);
    return code;
}

}  // namespace
}  // namespace sph

extern "C" int32_t sph_count_pairs_noalloc(const SphParams* params, int64_t n, const double* x, int64_t n_wall,
                                           const double* wall_x, int64_t* counts, void* stream) {
    using namespace sph;
    if (!params || !counts) return reject(SPH_ERR_ARG, "sph_count_pairs_noalloc: null params or counts");
    if (n < 0 || n > kMaxParticles || n_wall < 0 || n_wall > kMaxParticles)
        return reject(SPH_ERR_ARG, "sph_count_pairs_noalloc: at most 262144 fluid and 262144 wall particles");
    if ((n > 0 && !x) || (n_wall > 0 && !wall_x))
        return reject(SPH_ERR_ARG, "sph_count_pairs_noalloc: null position array");
    SceneDev S;
    std::string err;
    if (!scene_from_params(*params, S, err)) return reject(SPH_ERR_ARG, "sph_count_pairs_noalloc: " + err);
    if ((int64_t)S.ncells > kMaxCells)
        return reject(SPH_ERR_ARG, "sph_count_pairs_noalloc: the cell grid has " + std::to_string(S.ncells) +
                                       " cells, more than the limit of 262144");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return reject(SPH_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return reject(SPH_ERR_ARG, "sph_count_pairs_noalloc: device index too large");
    unsigned char* base;
    {
        // set-up, once per device and context, with that device current: the device
        // address of the scratch array (its name in host code is not a device address).
        // The address is cached with the id of the context it was taken in; a call from
        // another context (after cudaDeviceReset, or under a context a caller made current
        // through the driver API) looks it up again.
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        unsigned long long ctx = 0;
        const bool known = current_context_id(&ctx);
        if (!g_scratch_addr[dev] || !known || g_scratch_ctx[dev] != ctx) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return reject(SPH_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = (unsigned char*)p;
            g_scratch_ctx[dev] = current_context_id(&ctx) ? ctx : 0;
        }
        base = g_scratch_addr[dev];
    }
    const Scratch s = carve(base);
    cudaStream_t st = (cudaStream_t)stream;
    if ((e = cudaMemsetAsync(counts, 0, 2 * sizeof(int64_t), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(s.f_count, 0, sizeof(int32_t) * (size_t)S.ncells, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(s.w_count, 0, sizeof(int32_t) * (size_t)S.ncells, st)) != cudaSuccess)
        return reject(SPH_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    if (params->dim == 2)
        enqueue<2>(S, s, (int32_t)n, x, (int32_t)n_wall, wall_x, (unsigned long long*)counts, st);
    else
        enqueue<3>(S, s, (int32_t)n, x, (int32_t)n_wall, wall_x, (unsigned long long*)counts, st);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return reject(SPH_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return SPH_OK;
}
