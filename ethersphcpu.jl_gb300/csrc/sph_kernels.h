// sph_kernels.h — host-side launch interface of the device kernels (internal).
#pragma once

#include <utility>

#include "sph_device.cuh"

namespace sph {

// Everything one stage launch needs.  Filled by the engine for the current buffer
// parity; plain values, so a captured CUDA graph bakes them in.
struct LaunchCtx {
    cudaStream_t stream;
    int dim;
    int kernel;   // SPH_KERNEL_*
    int mode;     // 0 fluid-wall, 1 wall pressure, 2 thermal
    int thermal;
    int precision;
    int32_t cap;          // particle capacity (grid size of per-particle kernels)
    int32_t total_cells;  // cells over all scenes
    int32_t nscenes;
    const SceneDev* scenes;
    SortedState st;   // current sorted state
    SortedState st2;  // the other sorted buffer (output of the sort)
    NextState nx;
    WallState wl;
    SortScratch sc;
    int32_t* n_next;  // live count after the sort being built
    // shepard = 1: the momentum launch of re-initialisation steps (it also forms the Shepard
    // sums and writes the re-initialised density), for the particles of the scenes whose
    // step re-initialises; force_reinit = 1 with it: of every running scene, whatever its
    // step (stage timing).  skip_reinit = 1 with shepard = 0: the ordinary momentum launch
    // leaves those particles to the shepard launch of the same step.
    int shepard;
    int force_reinit;
    int skip_reinit;
    // launch shape of the FP32 gathers (lanes per particle, threads per block)
    int block;
    int tpp_continuity, tpp_momentum;
    // list_momentum != 0: continuity (one or two lanes) records the neighbour list and momentum
    // reads it (tpp_momentum lanes per particle)
    int list_momentum;
    NbrList nl;
    // inlet/outlet buffers (bf.n == nullptr: none): current and next sorted buffers
    BufferState bf, bf2;
    BufferScratch bs;
    BufferRules br;
    int32_t* bn_next;  // live buffer particles after the buffer sort being built
};

// Launch a step kernel with programmatic stream serialisation: its launch is prepared
// while the previous kernel of the stream finishes (it calls pdl_wait first).  Captured
// into the step graphs as programmatic edges.
template <typename... P, typename... A>
inline void launch_dep(void (*kernel)(P...), int grid, int block, cudaStream_t stream, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// stage 0: continuity + EOS; 1: momentum + integrate (+ next hash; + Shepard re-init when
// L.shepard is set)
void launch_physics_fp64(int stage, const LaunchCtx& L);
void launch_physics_fp32(int stage, const LaunchCtx& L);
void launch_physics_fp32_2d(int stage, const LaunchCtx& L);
void launch_physics_fp32_3d(int stage, const LaunchCtx& L);
void launch_physics_fp32_list_2d(int stage, const LaunchCtx& L);
void launch_physics_fp32_list_3d(int stage, const LaunchCtx& L);
// the momentum gathers of re-initialisation steps (L.shepard set)
void launch_momentum_fp32_2d_shep(const LaunchCtx& L);
void launch_momentum_fp32_3d_shep(const LaunchCtx& L);
void launch_momentum_fp32_list_2d_shep(const LaunchCtx& L);
void launch_momentum_fp32_list_3d_shep(const LaunchCtx& L);

// Buffer particles after the gathers of a step (K4-K5): move them, copy inlet particles
// that crossed into the fluid, move the fluid particles K5 marked to the outlet, drop
// outlet particles, and sort the buffers by (cell, order) into L.bf2.
void launch_buffers(const LaunchCtx& L);

// Cell hash of the unsorted positions in L.nx.x (used once after an upload).
void launch_hash(const LaunchCtx& L);
// Exclusive scan of sc.count into sc.start; writes the live total to *L.n_next.
// When advance != 0 it also increments every scene's step counter.
// tiles_ready: the step's momentum epilogue already summed the arrivals per 1,024-cell
// tile (sc.tile_acc) and the two-launch scan skips its tile pass.
void launch_scan(const LaunchCtx& L, int advance, bool tiles_ready = false);
// True when a scan over n cells runs as tile sums + down-sweep over 1,024-cell tiles.
bool scan_uses_tiles(int n);
// Stable (cell, id) placement: tmp fill, then rank + copy of every field into L.st2.
// carry_shadows: the current state's FP32 shadows are valid (a step), so the FP32 copies
// of the per-particle constants are carried over instead of converted from FP64.
void launch_place(const LaunchCtx& L, bool carry_shadows = false);
// Fields of a download: x and v (flags) and up to 8 FP64 per-particle arrays.
struct DownloadFields {
    int x, v;
    int n;
    const double* src[8];
};
// Gather rows b + order[q], q < n, of the sorted state into out (device): x (n x dim)
// and v (n x dim) when flagged, then one n-array per field.
void launch_gather_rows(cudaStream_t stream, int dim, const int32_t* order, int64_t n, int32_t b, const void* x,
                        const void* v, const DownloadFields& F, double* out);
// The same rows when the ids of [b, b + n) are a permutation of 0 .. n-1: row id[b + k]
// takes sorted particle b + k (no row order needed).
void launch_scatter_rows(cudaStream_t stream, int dim, const int32_t* id, int64_t n, int32_t b, const void* x,
                         const void* v, const DownloadFields& F, double* out);
// Upload helpers: ids 0 .. n-1 and scene s for [id, id + n); 3D positions and velocities
// (n x 3, device) widened into the state's 32-byte records.
void launch_upload_ids(cudaStream_t stream, int32_t* id, int32_t* scene, int64_t n, int32_t s);
void launch_widen3(cudaStream_t stream, const double* x3, const double* v3, void* x, void* v, int64_t n);
// FP64 reductions: out[0] = sum m, out[1] = sum m|v|^2/2, out[2] = max |v|.
void launch_stats(const LaunchCtx& L, double* d_partials, double* d_out);
// Unique fluid pairs (sorted j > i) and fluid-wall pairs within r_cut.
void launch_count_pairs(const LaunchCtx& L, unsigned long long* d_counts);

int scan_max_cells();

// Diagnostics of the cell list (sph_diag.cu) over the sorted particles [b, e) of one
// scene: the scene-local cell key of each; the number of fluid neighbours each one's
// gathers accept (counts != null) or their ids written from ids[rows[i - b]] on.
void launch_cell_keys(const LaunchCtx& L, int32_t b, int32_t e, int32_t* keys);
void launch_neighbours(const LaunchCtx& L, int32_t b, int32_t e, int32_t* counts, const int64_t* rows,
                       int32_t* ids);

// Fields interpolated by launch_probe (SPH_PROBE_* codes), at most kMaxProbeFields.
constexpr int kMaxProbeFields = 8;
struct ProbeFields {
    int n;
    int code[kMaxProbeFields];
};
// SPH interpolation of fluid fields of scene 0 at np device points (dim x np packed)
// into out (n_fields x np), device arrays.
void launch_probe(const LaunchCtx& L, int64_t np, const double* pts, const ProbeFields& F, double none_value,
                  double* out);

}  // namespace sph

#include <string>

namespace sph {
// Parameter block -> scene constants (defined in sph_api.cu).
bool scene_from_params(const SphParams& p, SceneDev& S, std::string& err);
// Text returned by sph_last_error(NULL).
void set_global_error(const std::string& msg);
}  // namespace sph
