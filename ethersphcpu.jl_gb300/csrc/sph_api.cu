// sph_api.cu — host engine and C ABI (include/ethersph_gpu.h).
//
// One handle = one CUDA stream + the device state of one scene.  Step pipeline
// (FluidWallSolve.jl:8-83 and its siblings), all on the handle's stream:
//   K4 continuity+EOS -> K5 momentum+integrate(+check, +next hash; on a re-initialisation
//   step + the Shepard density) -> scan -> fill+place (stable (cell, id) reorder into the
//   other buffer, count reset) -> swap.
// Bundles of steps are captured once as CUDA graphs and replayed.
//
// Host arithmetic in this file (parameter constants, the EOS for uploads without
// p/c, wall cell keys) must round exactly like the device and CPU restatement, so
// the file is compiled with -ffp-contract=off.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "sph_kernels.h"
#include "sph_output.h"

namespace {
// NVTX range around a host entry point (shown by Nsight Systems; free without a tool).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
}  // namespace

using namespace sph;

namespace {

thread_local std::string g_create_error;

double host_powi(double x, int64_t n) {  // Julia Base ^(Float64, Integer); see sph_device.cuh
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

int mode_of(int solve) {
    switch (solve) {
        case SPH_SOLVE_FLUID_WALL: return 0;
        case SPH_SOLVE_FLUID_VELOCITY_WALL: return 1;
        case SPH_SOLVE_FLUID_INLET_OUTLET_WALL: return 3;
        default: return 2;
    }
}

// Parameter block -> per-scene device constants.  Grid: cell edge r_cut*(1+1e-9)
// (a periodic x axis is cut into floor(L/edge) equal cells), origin domain_lo.
bool build_scene(const SphParams& p, SceneDev& S, std::string& err) {
    std::memset(&S, 0, sizeof(S));
    if (p.dim != 2 && p.dim != 3) { err = "dim must be 2 or 3"; return false; }
    if (p.kernel < 0 || p.kernel > 3) { err = "unknown kernel"; return false; }
    if (p.solve < 0 || p.solve > 4) { err = "unknown solve variant"; return false; }
    if (p.solve == SPH_SOLVE_FLUID_INLET_OUTLET_WALL && p.thermal) {
        err = "the inlet/outlet solve has no thermal model"; return false;
    }
    if (p.precision != SPH_PRECISION_FP64 && p.precision != SPH_PRECISION_FP32_COMPENSATED) {
        err = "unknown precision"; return false;
    }
    if ((p.solve == SPH_SOLVE_FLUID_THERMOSTATIC_WALL || p.solve == SPH_SOLVE_FLUID_COMPULSIVE_THERMOSTATIC_WALL) &&
        !p.thermal) {
        err = "thermostatic solves need the thermal model"; return false;
    }
    if (!(p.influence_radius > 0.0) || !(p.h > 0.0) || !(p.dt > 0.0) || !(p.rho_0 > 0.0)) {
        err = "influence_radius, h, dt and rho_0 must be positive"; return false;
    }
    const double rc = p.influence_radius;
    // cells per r_cut; default 3: cells of r_cut/3 leave fewer candidates beyond r_cut
    // than r_cut/2 (the walks' candidate tests fall by 20-27%; measured on GB300: the
    // FP32-compensated step 6-7% faster on 2D cavities of 65k and 1 M particles and on a
    // 432k-particle 3D dam break), and a row of cells is walked as one contiguous run
    const int m = p.cell_subdivision != 0 ? p.cell_subdivision : 3;
    if (m < 1 || m > 3) { err = "cell_subdivision must be 0, 1, 2 or 3"; return false; }
    S.reach = m;
    // cell edge r_cut (1 + 1e-9) / m: a pair with d <= r_cut is at most m cells apart
    // even after rounding
    const double edge = rc * (1.0 + 1e-9) / (double)m;
    int64_t ncells = 1;
    for (int a = 0; a < 3; ++a) {
        if (a >= p.dim) { S.n[a] = 1; S.lo[a] = 0.0; S.inv_cell[a] = 0.0; continue; }
        if (!(p.domain_hi[a] > p.domain_lo[a])) { err = "domain_hi must exceed domain_lo"; return false; }
        S.lo[a] = p.domain_lo[a];
        int64_t na;
        if (a == 0 && p.periodic_x) {
            const double L = p.domain_hi[0] - p.domain_lo[0];
            na = (int64_t)std::floor(L / edge);
            if (na < 2 * m + 1) { err = "a periodic axis needs at least 2 m + 1 cells"; return false; }
            S.cell_d[a] = L / (double)na;
            S.inv_cell[a] = 1.0 / S.cell_d[a];
        } else {
            na = (int64_t)std::ceil((p.domain_hi[a] - p.domain_lo[a]) / edge);
            if (na < 1) na = 1;
            S.cell_d[a] = edge;
            S.inv_cell[a] = 1.0 / edge;
        }
        if (na > (1 << 24)) { err = "cell grid too large"; return false; }
        S.n[a] = (int32_t)na;
        ncells *= na;
    }
    if (ncells > (int64_t)scan_max_cells()) { err = "cell grid too large for the scan"; return false; }
    S.cell_off = 0;
    S.ncells = (int32_t)ncells;
    S.periodic_x = p.periodic_x;
    S.period = p.domain_hi[0] - p.domain_lo[0];
    S.half_period = 0.5 * S.period;
    S.wrap_hi = S.lo[0] + S.period;

    S.h = p.h;
    S.sigma = p.sigma;
    S.k0 = p.kernel_0;
    S.rc2 = rc * rc;
    switch (p.kernel) {  // leading constants of CubicSpline.jl / Gaussian.jl / WendlandC2.jl / WendlandC4.jl
        case SPH_KERNEL_CUBIC_SPLINE: S.kw_a = p.sigma / 4.0; S.kg_a = p.sigma / p.h * 3.0 / 4.0; break;
        case SPH_KERNEL_GAUSSIAN: S.kw_a = p.sigma; S.kg_a = -2.0 * p.sigma / p.h; break;
        case SPH_KERNEL_WENDLAND_C2: S.kw_a = p.sigma; S.kg_a = -p.sigma / p.h * 5.0 / 8.0; break;
        default: S.kw_a = p.sigma; S.kg_a = -p.sigma / p.h; break;
    }
    S.hh001 = 0.01 * (p.h * p.h);

    S.rho0 = p.rho_0;
    S.c0 = p.c_0;
    S.p0 = p.p_0;
    S.b = p.b;
    S.nu0 = p.nu_0;
    S.t0 = p.t_0;
    S.cp = p.cp;
    S.beta = p.beta;
    S.P_bg = p.p_0 / (p.rho_0 * p.rho_0);
    S.inv_cp_d = p.thermal ? 1.0 / p.cp : 0.0;
    for (int k = 0; k < 3; ++k) {
        S.g[k] = p.body_force[k];
        S.bous[k] = -p.body_force[k] * p.beta;
        S.check_lo[k] = p.check_lo[k];
        S.check_hi[k] = p.check_hi[k];
    }
    S.gamma = p.gamma;
    S.thermal = p.thermal;
    S.wall_pressure = p.solve != SPH_SOLVE_FLUID_WALL;
    S.uniform_gap = 0;
    S.check_enabled = p.check_enabled;
    S.nan_check = p.nan_check;
    S.dt = p.dt;
    S.dtdt = p.dt * p.dt;
    S.half_dtdt = S.dtdt * 0.5;
    S.reinit_interval = p.density_reinitialized_interval;
    S.check_interval = p.check_interval;

    for (int a = 0; a < 3; ++a) S.cell_f[a] = (float)S.cell_d[a];
    S.inv_cell_fx = 1.0f / S.cell_f[0];
    S.h_f = (float)p.h;
    S.rc2_f = (float)(rc * rc);
    S.rc2_prune = S.rc2_f * 1.00001f;
    S.prune = 1;
    S.hh001_f = (float)S.hh001;
    S.nu0_f = (float)p.nu_0;
    S.P_bg_f = (float)S.P_bg;
    S.kw_a_f = (float)S.kw_a;
    S.kg_a_f = (float)S.kg_a;
    S.inv_h_f = (float)(1.0 / p.h);
    S.c0_f = (float)p.c_0;
    S.rho0_f = (float)p.rho_0;
    S.inv_cp_f = (float)S.inv_cp_d;
    S.inv_rho0 = 1.0 / p.rho_0;
    S.inv_rho0_f = (float)(1.0 / p.rho_0);
    return true;
}

int32_t host_cell_key(const SceneDev& S, int dim, const double* x) {
    int32_t c[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a) {
        const double u = (x[a] - S.lo[a]) * S.inv_cell[a];
        if (!(u >= 0.0)) { c[a] = 0; continue; }
        const double f = std::floor(u);
        c[a] = f >= (double)(S.n[a] - 1) ? S.n[a] - 1 : (int32_t)f;
    }
    return S.cell_off + (c[2] * S.n[1] + c[1]) * S.n[0] + c[0];
}

}  // namespace

namespace sph {
// Shared with entry points defined in other translation units.
bool scene_from_params(const SphParams& p, SceneDev& S, std::string& err) { return build_scene(p, S, err); }
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace sph

namespace {

// One simulation = one scene of the scene table.  Its cells are the range
// [cell_off, cell_off + ncells] of the global cell space (the last cell is a sentinel
// that never holds a particle, so start[] of the scene's cells never runs into another
// scene's wall region), its walls the region [wall_off, wall_off + wall_n) of the wall
// arrays, sorted by (cell, upload index).
struct SceneRec {
    bool used = false;
    SceneDev dev{};
    int32_t cell_span = 0;  // ncells + 1
    int64_t wall_off = 0, wall_n = 0, wall_cap = 0;
    int64_t first_step = 1;
    int64_t step_host = 1;  // mirror of the scene's device step counter
    std::vector<double> wx, wn, wv, wgap, wT, wkappa;  // host copy of the walls
    std::vector<int32_t> wkind;
    std::vector<int64_t> wgroup_end;  // end of each sph_upload_walls group in the host copy
    double gap0 = 0.0;                // gap of the first uploaded fluid particle
    bool uniform_fluid = true;        // every uploaded fluid particle has gap0
    int32_t list_depth = 0;           // neighbour-list entries per particle this scene asks for
    int64_t n_uploaded = 0;           // fluid particles of the scene's upload (ids 0 .. n - 1)
};

// First-fit allocator of ranges in [0, cap).
struct RangeAlloc {
    std::map<int64_t, int64_t> free_;  // offset -> length
    void init(int64_t cap) {
        free_.clear();
        if (cap > 0) free_[0] = cap;
    }
    bool alloc(int64_t len, int64_t* off) {
        if (len == 0) {
            *off = 0;
            return true;
        }
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= len) {
                *off = it->first;
                const int64_t rest = it->second - len, at = it->first + len;
                free_.erase(it);
                if (rest > 0) free_[at] = rest;
                return true;
            }
        }
        return false;
    }
    void release(int64_t off, int64_t len) {
        if (len == 0) return;
        auto it = free_.emplace(off, len).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    int64_t largest() const {
        int64_t m = 0;
        for (auto& kv : free_) m = std::max(m, kv.second);
        return m;
    }
};

}  // namespace

struct SphHandle {
    SphParams prm{};  // prototype (single-scene handles: the scene's parameters)
    bool batch = false;
    int dim = 2, kernel = 0, mode = 0, thermal = 0, precision = 0;
    int64_t cap = 0, wcap = 0;
    int32_t total_cells = 0;  // cell capacity
    int32_t scan_cells = 1;   // end of the highest cell range in use: what the scan covers
    int64_t n_upper = 1;      // bound on the live particles (only deletions change it while stepping)
    int32_t scap = 1;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    SortedState S[2]{};
    NextState N{};
    WallState W{};
    SortScratch sc{};
    int32_t* nbuf = nullptr;
    SceneDev* d_scenes = nullptr;
    double* d_stat_partials = nullptr;
    double* d_stat_out = nullptr;
    unsigned long long* d_pair_counts = nullptr;
    int64_t* h_pinned = nullptr;  // [0]: step upload, [1]: status, [2..3]: ranges
    int par = 0;
    bool have_fluid = false;
    int64_t steps_done = 0;
    // FP32 launch shape: lanes per particle for continuity, momentum, Shepard; block size
    int tune[4] = {1, 1, 1, 128};  // the autotuner's most frequent pick on large 2D and 3D scenes
    // neighbour list of the FP32 form (momentum lanes code >= SPH_LANES_LIST - 1): grown
    // on demand to the per-particle grid and the deepest scene (ensure_list)
    NbrList nl{};
    // stencil pruning of the FP32 walks (sph_set_stencil_pruning); default on in 3D only:
    // measured on GB300, it saves 4-8% of a 3D step (25 neighbour rows, corner rows and
    // cells beyond r_cut skipped) and costs 0-7% in 2D (few cells to skip, per-row bounds)
    int prune = -1;  // -1: by dimension
    std::string err;
    std::vector<SceneRec> scenes;
    RangeAlloc cells, walls;
    // graph cache: key = (parity, pattern of Shepard steps) -> executable graph
    std::map<std::pair<int, std::vector<bool>>, cudaGraphExec_t> graphs;
    // inlet/outlet buffers (sph_upload_buffers)
    bool has_buffers = false;
    bool buffers_started = false;  // br.first_step fixed by the first step after the upload
    int64_t bcap = 0;
    BufferState B[2]{};
    BufferScratch bs{};
    BufferRules br{};
    int32_t* bn = nullptr;    // [2]: live buffer particles per parity
    int64_t n_uploaded = 0;   // fluid particles of the last upload (ids 0 .. n-1)
    std::vector<double> bgap_host;  // gaps of the uploaded buffer particles
    bool buffer_gap_uniform(double g) const {
        for (double v : bgap_host)
            if (v != g) return false;
        return true;
    }
    sph::VtpWriter* out = nullptr;  // VTP output (sph_output_open)
    double* probe_buf = nullptr;    // device points + results of sph_probe
    int64_t probe_cap = 0;          // doubles in probe_buf
    char* dl_buf = nullptr;         // device staging of downloads (row order + gathered fields)
    size_t dl_cap = 0;              // bytes in dl_buf
    int64_t out_walls = -1;         // wall groups the writer holds
};

namespace {

int fail(SphHandle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    else g_create_error = msg;
    return code;
}

int cuda_fail(SphHandle* h, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(h, e == cudaErrorMemoryAllocation ? SPH_ERR_OOM : SPH_ERR_CUDA, m);
}

#define SPH_CUDA(h, call)                                          \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return cuda_fail((h), _e, #call);   \
    } while (0)

template <typename T>
cudaError_t dalloc(SphHandle* h, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    h->allocs.push_back(q);
    *p = (T*)q;
    return cudaMemsetAsync(q, 0, std::max<size_t>(count, 1) * sizeof(T), h->stream);
}

size_t vec_bytes(int dim) { return dim == 2 ? sizeof(double2) : sizeof(double4_32a); }

cudaError_t alloc_vec(SphHandle* h, void** p, size_t n) {
    const size_t bytes = std::max<size_t>(n, 1) * vec_bytes(h->dim);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return e;
    h->allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes, h->stream);
}

cudaError_t alloc_sorted(SphHandle* h, SortedState& s) {
    const size_t n = (size_t)h->cap;
    cudaError_t e;
    if ((e = alloc_vec(h, &s.x, n)) != cudaSuccess) return e;
    if ((e = alloc_vec(h, &s.v, n)) != cudaSuccess) return e;
    double** d[] = {&s.rho, &s.rhoc, &s.p, &s.c, &s.P, &s.m, &s.gap};
    for (double** pp : d)
        if ((e = dalloc(h, pp, n)) != cudaSuccess) return e;
    if (h->thermal) {
        if ((e = dalloc(h, &s.T, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.kappa, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.cp, n)) != cudaSuccess) return e;
    }
    if ((e = dalloc(h, &s.id, n)) != cudaSuccess) return e;
    if ((e = dalloc(h, &s.scene, n)) != cudaSuccess) return e;
    if (h->precision == SPH_PRECISION_FP32_COMPENSATED) {  // FP32 shadows of the gathers
        if ((e = dalloc(h, &s.fa, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.fb, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.fc, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.fd, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.cell, n)) != cudaSuccess) return e;
        if ((e = dalloc(h, &s.vol, n)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Rows of the per-particle grids: the live bound, not the capacity (a served batch is
// sized for its memory budget and may hold far fewer particles); with inlet/outlet
// buffers the capacity, since fluid particles made from the inlet are appended behind
// the live ones.
int32_t grid_rows(const SphHandle* h) {
    if (h->has_buffers) return (int32_t)h->cap;
    return (int32_t)std::max<int64_t>(1, std::min<int64_t>(h->cap, h->n_upper));
}

bool uses_list(const SphHandle* h) {
    return h->precision == SPH_PRECISION_FP32_COMPENSATED && h->tune[1] >= SPH_LANES_LIST - 1;
}

// Neighbour-list entries a particle of spacing `gap` needs: the lattice points within
// r_cut of a lattice point, with a quarter of headroom for compression (a particle with
// more neighbours walks the cells instead).
int32_t list_depth_for(int dim, double rc2, double gap) {
    if (!(gap > 0.0) || !(rc2 > 0.0)) return 64;
    const double R2 = rc2 / (gap * gap) * (1.0 + 1e-9);
    const int R = (int)std::min(16.0, std::floor(std::sqrt(R2)));
    int64_t count = 0;
    for (int a = -R; a <= R; ++a)
        for (int b = -R; b <= R; ++b)
            for (int c = (dim == 3 ? -R : 0); c <= (dim == 3 ? R : 0); ++c)
                count += (double)(a * a + b * b + c * c) <= R2;
    const int64_t depth = ((int64_t)std::ceil(1.25 * (double)(count - 1)) + 8 + 7) / 8 * 8;
    return (int32_t)std::min<int64_t>(depth, 1024);
}

// Storage of the neighbour list for the current per-particle grid and scene depths;
// reallocating drops the captured graphs (they hold its address).
int32_t ensure_list(SphHandle* h) {
    if (!uses_list(h)) return SPH_OK;
    int32_t depth = 8;
    for (const SceneRec& R : h->scenes)
        if (R.used) depth = std::max(depth, R.list_depth);
    const int64_t rows = grid_rows(h);
    if (h->nl.e && rows <= h->nl.stride && depth <= h->nl.kmax) return SPH_OK;
    // rows grow by half again at least: a serving batch raises its live bound scene by scene
    int64_t stride = std::max<int64_t>(std::max<int64_t>(rows, h->nl.stride), 1);
    if (h->nl.e && rows > h->nl.stride)
        stride = std::max<int64_t>(stride, std::min<int64_t>(h->cap, h->nl.stride + h->nl.stride / 2));
    depth = std::max(depth, h->nl.kmax);
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->nl.e) cudaFree(h->nl.e);
    if (h->nl.n) cudaFree(h->nl.n);
    h->nl = NbrList{};
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    cudaError_t e = cudaMalloc((void**)&h->nl.e, (size_t)stride * (size_t)depth * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->nl.n, (size_t)stride * 4);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (h->nl.e) cudaFree(h->nl.e);
        h->nl = NbrList{};
        return fail(h, SPH_ERR_OOM, "no device memory for the neighbour list (" + std::to_string(stride) + " x " +
                                        std::to_string(depth) + " entries); use a cell-walk momentum lanes code");
    }
    h->nl.kmax = depth;
    h->nl.stride = stride;
    return SPH_OK;
}

LaunchCtx make_ctx(SphHandle* h) {
    LaunchCtx L{};
    L.stream = h->stream;
    L.dim = h->dim;
    L.kernel = h->kernel;
    L.mode = h->mode;
    L.thermal = h->thermal;
    L.precision = h->precision;
    L.cap = grid_rows(h);
    L.total_cells = h->scan_cells;
    L.nscenes = h->scap;
    L.scenes = h->d_scenes;
    L.st = h->S[h->par];
    L.st2 = h->S[h->par ^ 1];
    L.nx = h->N;
    L.wl = h->W;
    L.sc = h->sc;
    L.sc.n_live = h->nbuf + h->par;
    L.n_next = h->nbuf + (h->par ^ 1);
    L.shepard = 0;
    L.force_reinit = 0;
    L.skip_reinit = 0;
    L.block = h->tune[3];
    L.tpp_continuity = h->tune[0];
    L.tpp_momentum = h->tune[1];
    L.list_momentum = uses_list(h);
    if (L.list_momentum) L.tpp_momentum -= SPH_LANES_LIST;
    L.nl = h->nl;
    if (h->has_buffers) {
        L.bf = h->B[h->par];
        L.bf.n = h->bn + h->par;
        L.bf.start = h->bs.start;
        L.bf2 = h->B[h->par ^ 1];
        L.bf2.n = h->bn + (h->par ^ 1);
        L.bf2.start = h->bs.start;
        L.bs = h->bs;
        L.br = h->br;
        L.bn_next = h->bn + (h->par ^ 1);
    }
    return L;
}

void launch_physics(int stage, const LaunchCtx& L) {
    if (L.precision == SPH_PRECISION_FP64) launch_physics_fp64(stage, L);
    else launch_physics_fp32(stage, L);
}

// Enqueue one step (no synchronisation).  `reinit`: some running scene re-initialises
// its density at this step (the kernels decide per scene).
void enqueue_step(SphHandle* h, bool reinit) {
    LaunchCtx L = make_ctx(h);
    // count[] and the tile sums were zeroed by the previous placement (or the last re-sort);
    // with a tiled scan the momentum epilogue sums the arrivals per tile as well (not with
    // inlet/outlet buffers, whose transfers add arrivals after it)
    const bool tiles = !h->has_buffers && scan_uses_tiles(L.total_cells);
    if (tiles) L.sc.tile_acc = h->sc.block_sums;
    launch_physics(0, L);
    if (!reinit) {
        launch_physics(1, L);
    } else if (!h->batch) {  // the scene re-initialises: the momentum gather with the Shepard sums
        L.shepard = 1;
        launch_physics(1, L);
    } else {  // each particle through the momentum gather of its own scene's step kind
        L.skip_reinit = 1;
        launch_physics(1, L);
        L.shepard = 1;
        L.skip_reinit = 0;
        launch_physics(1, L);
    }
    if (h->has_buffers) launch_buffers(L);  // before the scan advances the step counter
    launch_scan(L, 1, tiles);
    // fluid made from inlet particles has no FP32 shadows yet: convert everything then
    launch_place(L, !h->has_buffers);
    h->par ^= 1;
}

// Sort the current state S[par] (n_live particles, possibly unsorted after an upload
// or with retired scenes to drop) into S[par^1] and swap.
int resort(SphHandle* h) {
    LaunchCtx L = make_ctx(h);
    L.nx.x = L.st.x;
    L.nx.v = L.st.v;
    L.nx.rho = L.st.rho;
    L.nx.T = L.st.T;
    SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->scan_cells, h->stream));
    launch_hash(L);
    launch_scan(L, 0);
    launch_place(L);
    SPH_CUDA(h, cudaGetLastError());
    h->par ^= 1;
    if (h->has_buffers) {  // the buffers follow the fluid's buffer parity
        const int from = h->par ^ 1, to = h->par;
        const size_t n = (size_t)h->bcap, vb = vec_bytes(h->dim);
        cudaStream_t st = h->stream;
        SPH_CUDA(h, cudaMemcpyAsync(h->B[to].x, h->B[from].x, n * vb, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->B[to].v, h->B[from].v, n * vb, cudaMemcpyDeviceToDevice, st));
        double* const src[5] = {h->B[from].rho, h->B[from].p, h->B[from].c, h->B[from].m, h->B[from].gap};
        double* const dst[5] = {h->B[to].rho, h->B[to].p, h->B[to].c, h->B[to].m, h->B[to].gap};
        for (int f = 0; f < 5; ++f) SPH_CUDA(h, cudaMemcpyAsync(dst[f], src[f], n * 8, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->B[to].order, h->B[from].order, n * 8, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->bn + to, h->bn + from, 4, cudaMemcpyDeviceToDevice, st));
    }
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

bool is_step_host(int64_t step, int64_t interval) { return interval > 0 && step % interval == 0; }

// New bound on the live particles; the captured step graphs bake the grid sizes.
void set_n_upper(SphHandle* h, int64_t n) {
    if (n != h->n_upper) {
        for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
        h->graphs.clear();
    }
    h->n_upper = n;
}

int32_t read_live(SphHandle* h, int32_t* n) {
    SPH_CUDA(h, cudaMemcpyAsync(&h->h_pinned[2], h->nbuf + h->par, 4, cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    std::memcpy(n, &h->h_pinned[2], 4);
    return SPH_OK;
}

// [begin, end) of scene s in the sorted arrays.
int32_t scene_range(SphHandle* h, int s, int32_t* b, int32_t* e) {
    const SceneRec& R = h->scenes[s];
    int32_t v[2];
    SPH_CUDA(h, cudaMemcpyAsync(&v[0], h->sc.start + R.dev.cell_off, 4, cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(h, cudaMemcpyAsync(&v[1], h->sc.start + R.dev.cell_off + R.dev.ncells, 4, cudaMemcpyDeviceToHost,
                                h->stream));
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    *b = v[0];
    *e = v[1];
    return SPH_OK;
}

int32_t upload_scene_const(SphHandle* h, int s) {
    SPH_CUDA(h, cudaMemcpyAsync(h->d_scenes + s, &h->scenes[s].dev, sizeof(SceneDev), cudaMemcpyHostToDevice,
                                h->stream));
    return SPH_OK;
}

int32_t set_scene_step(SphHandle* h, int s, int64_t step) {
    h->h_pinned[0] = step;
    SPH_CUDA(h, cudaMemcpyAsync(h->sc.scene_step + s, &h->h_pinned[0], 8, cudaMemcpyHostToDevice, h->stream));
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    h->scenes[s].step_host = step;
    return SPH_OK;
}

// Write the walls of scene s (host copy) into its region: sorted by (cell, upload
// index), with the scene's wall cell starts and FP32 shadows.
// Cells of a scene whose neighbour box (+-reach cells per axis, x wrapping on a periodic
// axis) holds a wall particle: the only cells whose particles need the wall walk.
// `start` is the scene's wall start array (ncells + 1 entries); the sentinel cell gets 0.
std::vector<uint8_t> wall_near_cells(const SceneDev& S, int dim, const std::vector<int32_t>& start) {
    const int64_t nx = S.n[0], ny = S.n[1], nz = dim == 3 ? S.n[2] : 1, m = S.reach;
    const int64_t ncells = nx * ny * nz;
    std::vector<uint8_t> a(ncells + 1, 0), b(ncells + 1, 0);
    for (int64_t c = 0; c < ncells; ++c) a[c] = start[c + 1] > start[c];
    // dilate by +-m along x, then y, then z
    for (int64_t row = 0; row < ny * nz; ++row)
        for (int64_t x = 0; x < nx; ++x) {
            uint8_t v = 0;
            for (int64_t d = -m; d <= m && !v; ++d) {
                int64_t q = x + d;
                if (S.periodic_x) q = (q % nx + nx) % nx;
                else if (q < 0 || q >= nx) continue;
                v = a[row * nx + q];
            }
            b[row * nx + x] = v;
        }
    for (int64_t z = 0; z < nz; ++z)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t x = 0; x < nx; ++x) {
                uint8_t v = 0;
                for (int64_t d = -m; d <= m && !v; ++d)
                    if (y + d >= 0 && y + d < ny) v = b[(z * ny + y + d) * nx + x];
                a[(z * ny + y) * nx + x] = v;
            }
    if (dim == 3) {
        for (int64_t z = 0; z < nz; ++z)
            for (int64_t c = 0; c < nx * ny; ++c) {
                uint8_t v = 0;
                for (int64_t d = -m; d <= m && !v; ++d)
                    if (z + d >= 0 && z + d < nz) v = a[(z + d) * nx * ny + c];
                b[z * nx * ny + c] = v;
            }
        a.swap(b);
    }
    a[ncells] = 0;
    return a;
}

int32_t write_scene_walls(SphHandle* h, int s) {
    SceneRec& R = h->scenes[s];
    const SceneDev& S = R.dev;
    const int dim = h->dim;
    const int64_t nw = (int64_t)R.wgap.size();
    std::vector<int32_t> key(nw);
    for (int64_t w = 0; w < nw; ++w) key[w] = host_cell_key(S, dim, &R.wx[w * dim]);
    std::vector<int64_t> order(nw);
    for (int64_t w = 0; w < nw; ++w) order[w] = w;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
    std::vector<int32_t> start(R.cell_span, 0);  // ncells + 1 entries
    for (int64_t w = 0; w < nw; ++w) start[key[w] - S.cell_off + 1]++;
    for (int32_t c = 0; c + 1 < R.cell_span; ++c) start[c + 1] += start[c];
    for (auto& v : start) v += (int32_t)R.wall_off;
    const size_t vb = vec_bytes(dim);
    std::vector<char> bx(nw * vb, 0), bn(nw * vb, 0), bv(nw * vb, 0);
    std::vector<double> bg(nw), bT(nw), bk(nw);
    std::vector<int32_t> bkind(nw);
    std::vector<float4> fa, fb, fc;
    const bool shadow = h->precision == SPH_PRECISION_FP32_COMPENSATED;
    if (shadow) {
        fa.resize(nw);
        fb.resize(nw);
        fc.resize(nw);
    }
    for (int64_t q = 0; q < nw; ++q) {
        const int64_t w = order[q];
        for (int k = 0; k < dim; ++k) {
            ((double*)(bx.data() + q * vb))[k] = R.wx[w * dim + k];
            ((double*)(bn.data() + q * vb))[k] = R.wn[w * dim + k];
            ((double*)(bv.data() + q * vb))[k] = R.wv[w * dim + k];
        }
        bg[q] = R.wgap[w];
        bT[q] = R.wT[w];
        bk[q] = R.wkappa[w];
        bkind[q] = R.wkind[w];
        if (shadow) {  // position relative to the origin of the wall's cell
            const int32_t k = key[w] - S.cell_off;
            const int32_t cc[3] = {k % S.n[0], (k / S.n[0]) % S.n[1], k / (S.n[0] * S.n[1])};
            float xr[3] = {0.f, 0.f, 0.f}, nr[3] = {0.f, 0.f, 0.f}, vr[3] = {0.f, 0.f, 0.f};
            for (int a = 0; a < dim; ++a) {
                xr[a] = (float)(R.wx[w * dim + a] - (S.lo[a] + (double)cc[a] * S.cell_d[a]));
                nr[a] = (float)R.wn[w * dim + a];
                vr[a] = (float)R.wv[w * dim + a];
            }
            const float g = (float)R.wgap[w], T = (float)R.wT[w], kap = (float)R.wkappa[w];
            const float thermo = R.wkind[w] == SPH_WALL_THERMOSTATIC ? 1.f : 0.f;
            if (dim == 2) {
                fa[q] = make_float4(xr[0], xr[1], nr[0], nr[1]);
                fb[q] = make_float4(vr[0], vr[1], g, T);
                fc[q] = make_float4(kap, thermo, 0.f, 0.f);
            } else {
                fa[q] = make_float4(xr[0], xr[1], xr[2], g);
                fb[q] = make_float4(nr[0], nr[1], nr[2], T);
                fc[q] = make_float4(vr[0], vr[1], vr[2], kap);
            }
        }
    }
    cudaStream_t st = h->stream;
    const int64_t o = R.wall_off;
    if (nw > 0) {
        SPH_CUDA(h, cudaMemcpyAsync((char*)h->W.x + o * vb, bx.data(), nw * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync((char*)h->W.nrm + o * vb, bn.data(), nw * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync((char*)h->W.v + o * vb, bv.data(), nw * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.gap + o, bg.data(), nw * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.T + o, bT.data(), nw * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.kappa + o, bk.data(), nw * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.kind + o, bkind.data(), nw * 4, cudaMemcpyHostToDevice, st));
        if (shadow) {
            SPH_CUDA(h, cudaMemcpyAsync(h->W.fa + o, fa.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(h->W.fb + o, fb.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(h->W.fc + o, fc.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, st));
        }
    }
    SPH_CUDA(h, cudaMemcpyAsync(h->W.start + S.cell_off, start.data(), start.size() * 4, cudaMemcpyHostToDevice, st));
    const std::vector<uint8_t> near = wall_near_cells(S, dim, start);
    SPH_CUDA(h, cudaMemcpyAsync(h->W.near + S.cell_off, near.data(), near.size(), cudaMemcpyHostToDevice, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    R.wall_n = nw;
    return SPH_OK;
}

// Append walls to the host copy of scene s.
int32_t add_walls_host(SphHandle* h, SceneRec& R, int32_t kind, int64_t n, const double* x, const double* normal,
                       const double* gap, const double* t, const double* kappa, const double* v) {
    const int dim = h->dim;
    if (kind < SPH_WALL_COMPULSIVE || kind > SPH_WALL_THERMOSTATIC) return fail(h, SPH_ERR_ARG, "unknown wall kind");
    if (n < 0) return fail(h, SPH_ERR_ARG, "negative wall count");
    if (n > 0 && (!x || !normal || !gap)) return fail(h, SPH_ERR_ARG, "wall x, normal, gap are required");
    if (n > 0 && kind == SPH_WALL_THERMOSTATIC && (!t || !kappa))
        return fail(h, SPH_ERR_ARG, "thermostatic walls need t and kappa");
    if (n > 0 && kind == SPH_WALL_STATIC_VELOCITY && !v) return fail(h, SPH_ERR_ARG, "velocity walls need v");
    for (int64_t i = 0; i < n; ++i) {
        for (int k = 0; k < dim; ++k) {
            R.wx.push_back(x[i * dim + k]);
            R.wn.push_back(normal[i * dim + k]);
            R.wv.push_back(kind == SPH_WALL_STATIC_VELOCITY ? v[i * dim + k] : 0.0);
        }
        R.wgap.push_back(gap[i]);
        R.wT.push_back(kind == SPH_WALL_THERMOSTATIC ? t[i] : 0.0);
        R.wkappa.push_back(kind == SPH_WALL_THERMOSTATIC ? kappa[i] : 0.0);
        R.wkind.push_back(kind);
    }
    return SPH_OK;
}

// Append n fluid particles of scene s at the end of the live range of S[par] (ids
// 0..n-1 within the scene), then re-sort.
// Device scratch of downloads and 3D uploads (h->dl_buf) of at least `need` bytes.
int32_t ensure_dl_buf(SphHandle* h, size_t need) {
    if (need <= h->dl_cap) return SPH_OK;
    if (h->dl_buf) cudaFree(h->dl_buf);
    h->dl_buf = nullptr;
    h->dl_cap = 0;
    SPH_CUDA(h, cudaMalloc((void**)&h->dl_buf, need));
    h->dl_cap = need;
    return SPH_OK;
}

int32_t append_fluid(SphHandle* h, int s, int32_t n_before, int64_t n, const double* x, const double* v,
                     const double* rho, const double* p, const double* c, const double* mass, const double* gap,
                     const double* t, const double* kappa, const double* cp) {
    const int dim = h->dim;
    const SceneDev& S = h->scenes[s].dev;
    if ((int64_t)n_before + n > h->cap) return fail(h, SPH_ERR_OOM, "fluid count exceeds the handle capacity");
    if (n > 0 && (!x || !v || !rho || !mass || !gap)) return fail(h, SPH_ERR_ARG, "x, v, rho, mass, gap are required");
    if (n > 0 && h->thermal && (!t || !kappa || !cp))
        return fail(h, SPH_ERR_ARG, "thermal particles need t, kappa and cp");
    const size_t vb = vec_bytes(dim);
    // p and c from the caller, or updatePressure! (UpdatePressure.jl:8-16) on the host
    std::vector<double> hp, hc;
    const double* pp = p;
    const double* cc = c;
    if (!(p && c)) {
        hp.resize(n);
        hc.resize(n);
        for (int64_t i = 0; i < n; ++i) {
            const double rr = rho[i] / S.rho0;
            hp[i] = S.b * (host_powi(rr, S.gamma) - 1.0) + S.p0;
            hc[i] = S.c0 * std::sqrt(host_powi(rr, S.gamma - 1));
        }
        pp = hp.data();
        cc = hc.data();
    }
    double gmin = 0.0;
    for (int64_t i = 0; i < n; ++i) gmin = (i == 0 || gap[i] < gmin) ? gap[i] : gmin;
    h->scenes[s].list_depth = n > 0 ? list_depth_for(dim, S.rc2, gmin) : 0;
    h->scenes[s].n_uploaded = n;
    SortedState& d = h->S[h->par];
    cudaStream_t st = h->stream;
    const size_t o = (size_t)n_before;
    // every field goes straight from the caller's array to the device (no host copy: on a
    // GB300 node a pageable copy of a few MB runs at >100 GB/s, a host-side repack at ~20);
    // 2D positions and velocities are already the state's double2 records, 3D ones are
    // widened to 32-byte records on the device
    if (n > 0) {
        if (dim == 2) {
            SPH_CUDA(h, cudaMemcpyAsync((char*)d.x + o * vb, x, n * 16, cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync((char*)d.v + o * vb, v, n * 16, cudaMemcpyHostToDevice, st));
        } else {
            if (int32_t rc = ensure_dl_buf(h, (size_t)n * 48); rc != SPH_OK) return rc;
            double* x3 = (double*)h->dl_buf;
            double* v3 = x3 + 3 * n;
            SPH_CUDA(h, cudaMemcpyAsync(x3, x, n * 24, cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(v3, v, n * 24, cudaMemcpyHostToDevice, st));
            launch_widen3(st, x3, v3, (char*)d.x + o * vb, (char*)d.v + o * vb, n);
        }
        SPH_CUDA(h, cudaMemcpyAsync(d.rho + o, rho, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(d.p + o, pp, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(d.c + o, cc, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(d.m + o, mass, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(d.gap + o, gap, n * 8, cudaMemcpyHostToDevice, st));
        launch_upload_ids(st, d.id + o, d.scene + o, n, s);
        SPH_CUDA(h, cudaGetLastError());
        if (h->thermal) {
            SPH_CUDA(h, cudaMemcpyAsync(d.T + o, t, n * 8, cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(d.kappa + o, kappa, n * 8, cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(d.cp + o, cp, n * 8, cudaMemcpyHostToDevice, st));
        }
    }
    h->h_pinned[2] = 0;
    const int32_t total = (int32_t)(n_before + n);
    set_n_upper(h, total);
    std::memcpy(&h->h_pinned[2], &total, 4);
    SPH_CUDA(h, cudaMemcpyAsync(h->nbuf + h->par, &h->h_pinned[2], 4, cudaMemcpyHostToDevice, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));  // host staging buffers die at return
    return resort(h);
}

// Row order of a download: positions of the sorted particles in ascending id (the
// caller's original order with deleted particles removed).  Ids are unique and small
// (upload indices, then inlet copies): a position table, linear in n; a sort otherwise.
void ascending_id_order(const std::vector<int32_t>& ids, std::vector<int32_t>& order) {
    const int64_t n = (int64_t)ids.size();
    order.resize(n);
    int32_t lo = INT32_MAX, hi = -1;
    for (int32_t id : ids) {
        lo = std::min(lo, id);
        hi = std::max(hi, id);
    }
    if (n > 0 && lo >= 0 && (int64_t)hi <= 8 * n + 1024) {
        std::vector<int32_t> pos((size_t)hi + 1, -1);
        for (int64_t k = 0; k < n; ++k) pos[ids[k]] = (int32_t)k;
        int64_t q = 0;
        for (int32_t id = 0; id <= hi; ++id)
            if (pos[id] >= 0) {
                if (q == n) break;
                order[q++] = pos[id];
            }
        if (q == n) return;  // unique ids: done
    }
    for (int64_t k = 0; k < n; ++k) order[k] = (int32_t)k;
    std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return ids[a] < ids[b]; });
}

// Download the live particles of scene s in ascending id: the rows are put in that order
// on the device (one gather launch into a staging buffer), then each requested array is
// copied straight into the caller's memory.
int32_t download_scene(SphHandle* h, int s, int64_t capacity, int64_t* n_out, double* x, double* v, double* rho,
                       double* p, double* c, double* mass, double* gap, double* t, double* kappa, double* cp,
                       int64_t* ids_out) {
    int32_t b = 0, e = 0;
    int32_t rc = scene_range(h, s, &b, &e);
    if (rc != SPH_OK) return rc;
    const int64_t n = e - b;
    *n_out = n;
    if (n > capacity) return fail(h, SPH_ERR_ARG, "caller arrays too small for the live fluid");
    if (n == 0) return SPH_OK;
    cudaStream_t st = h->stream;
    const int dim = h->dim;
    const SortedState& d = h->S[h->par];
    // with no particle deleted or created since the upload the ids are a permutation of
    // 0 .. n-1 and each particle's row is its id; otherwise the rows follow the ascending
    // ids, ordered on the host
    const bool permutation = n == h->scenes[s].n_uploaded && !h->has_buffers;
    std::vector<int32_t> ids, order;
    if (!permutation) {
        ids.resize(n);
        SPH_CUDA(h, cudaMemcpyAsync(ids.data(), d.id + b, n * 4, cudaMemcpyDeviceToHost, st));
        SPH_CUDA(h, cudaStreamSynchronize(st));
        ascending_id_order(ids, order);
    }
    if (ids_out)
        for (int64_t q = 0; q < n; ++q) ids_out[q] = permutation ? q : ids[order[q]];
    const double* srcs[8] = {d.rho, d.p, d.c, d.m, d.gap, d.T, d.kappa, d.cp};
    double* dsts[8] = {rho, p, c, mass, gap, t, kappa, cp};
    DownloadFields F{};
    F.x = x != nullptr;
    F.v = v != nullptr;
    double* out_of[8] = {};
    for (int f = 0; f < 8; ++f)
        if (dsts[f] && srcs[f]) {
            out_of[F.n] = dsts[f];
            F.src[F.n++] = srcs[f];
        }
    if (!F.x && !F.v && F.n == 0) return SPH_OK;
    const size_t cols = (size_t)(F.x + F.v) * dim + (size_t)F.n;
    const size_t need = (size_t)n * 4 + 16 + (size_t)n * cols * 8;
    if (int32_t rc = ensure_dl_buf(h, need); rc != SPH_OK) return rc;
    int32_t* d_order = (int32_t*)h->dl_buf;
    double* d_out = (double*)(h->dl_buf + (((size_t)n * 4 + 15) / 16) * 16);
    if (permutation) {
        launch_scatter_rows(st, dim, d.id, n, b, d.x, d.v, F, d_out);
    } else {
        SPH_CUDA(h, cudaMemcpyAsync(d_order, order.data(), n * 4, cudaMemcpyHostToDevice, st));
        launch_gather_rows(st, dim, d_order, n, b, d.x, d.v, F, d_out);
    }
    SPH_CUDA(h, cudaGetLastError());
    double* o = d_out;
    if (x) {
        SPH_CUDA(h, cudaMemcpyAsync(x, o, (size_t)n * dim * 8, cudaMemcpyDeviceToHost, st));
        o += n * dim;
    }
    if (v) {
        SPH_CUDA(h, cudaMemcpyAsync(v, o, (size_t)n * dim * 8, cudaMemcpyDeviceToHost, st));
        o += n * dim;
    }
    for (int f = 0; f < F.n; ++f) SPH_CUDA(h, cudaMemcpyAsync(out_of[f], o + (size_t)f * n, n * 8, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    return SPH_OK;
}

// Run nsteps steps of every scene (each at its own step number) as CUDA-graph bundles.
int32_t step_all_async(SphHandle* h, int64_t nsteps) {
    cudaStream_t st = h->stream;
    if (int32_t rc = ensure_list(h); rc != SPH_OK) return rc;
    const int64_t bundle = 10;
    int64_t done = 0;
    while (done < nsteps) {
        const int64_t nb = std::min(bundle, nsteps - done);
        std::vector<bool> pattern(nb, false);
        for (const SceneRec& R : h->scenes) {
            if (!R.used || !R.dev.active) continue;
            for (int64_t q = 0; q < nb; ++q) {
                const int64_t s = R.step_host + done + q;
                if (s <= R.dev.last_step && is_step_host(s, R.dev.reinit_interval)) pattern[q] = true;
            }
        }
        auto key = std::make_pair(h->par, pattern);
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            const int par0 = h->par;
            SPH_CUDA(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            for (int64_t q = 0; q < nb; ++q) enqueue_step(h, pattern[q]);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            h->par = par0;
            if (e != cudaSuccess) return cuda_fail(h, e, "graph capture");
            cudaGraphExec_t ge = nullptr;
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(h, e, "graph instantiate");
            if (h->graphs.size() > 64) {
                for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
                h->graphs.clear();
            }
            it = h->graphs.emplace(key, ge).first;
        }
        SPH_CUDA(h, cudaGraphLaunch(it->second, st));
        if (nb & 1) h->par ^= 1;
        done += nb;
    }
    for (SceneRec& R : h->scenes)
        if (R.used) R.step_host += nsteps;
    h->steps_done += nsteps;
    return SPH_OK;
}

int32_t allocate_handle(SphHandle* h, int64_t cells) {
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(nullptr, e, "stream");
    for (int b = 0; b < 2; ++b)
        if ((e = alloc_sorted(h, h->S[b])) != cudaSuccess) return cuda_fail(nullptr, e, "sorted state");
    if ((e = alloc_vec(h, &h->N.x, h->cap)) != cudaSuccess) return cuda_fail(nullptr, e, "next x");
    if ((e = alloc_vec(h, &h->N.v, h->cap)) != cudaSuccess) return cuda_fail(nullptr, e, "next v");
    if ((e = dalloc(h, &h->N.rho, h->cap)) != cudaSuccess) return cuda_fail(nullptr, e, "next rho");
    if (h->thermal && (e = dalloc(h, &h->N.T, h->cap)) != cudaSuccess) return cuda_fail(nullptr, e, "next T");
    const size_t ncell = (size_t)cells;
    const size_t wc = (size_t)std::max<int64_t>(h->wcap, 1);
    struct {
        int32_t** p;
        size_t n;
    } ints[] = {{&h->sc.key, (size_t)h->cap},        {&h->sc.slot, (size_t)h->cap},
                {&h->sc.tmp, (size_t)h->cap},        {&h->sc.count, ncell},
                {&h->sc.start, ncell + 1},           {&h->sc.block_sums, ncell / 1024 + 2},
                {&h->sc.status, 1},                  {&h->nbuf, 2},
                {&h->W.start, ncell + 1},            {&h->W.kind, wc}};
    for (auto& a : ints)
        if ((e = dalloc(h, a.p, a.n)) != cudaSuccess) return cuda_fail(nullptr, e, "scratch");
    if ((e = dalloc(h, &h->W.near, ncell + 1)) != cudaSuccess) return cuda_fail(nullptr, e, "scratch");
    if ((e = dalloc(h, &h->sc.scene_step, (size_t)h->scap)) != cudaSuccess) return cuda_fail(nullptr, e, "steps");
    if ((e = dalloc(h, &h->d_scenes, (size_t)h->scap)) != cudaSuccess) return cuda_fail(nullptr, e, "scenes");
    if ((e = alloc_vec(h, &h->W.x, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    if ((e = alloc_vec(h, &h->W.nrm, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    if ((e = alloc_vec(h, &h->W.v, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    if ((e = dalloc(h, &h->W.gap, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    if ((e = dalloc(h, &h->W.T, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    if ((e = dalloc(h, &h->W.kappa, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    if (h->precision == SPH_PRECISION_FP32_COMPENSATED) {
        if ((e = dalloc(h, &h->W.fa, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
        if ((e = dalloc(h, &h->W.fb, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
        if ((e = dalloc(h, &h->W.fc, wc)) != cudaSuccess) return cuda_fail(nullptr, e, "walls");
    }
    if ((e = dalloc(h, &h->d_stat_partials, 3 * 152)) != cudaSuccess) return cuda_fail(nullptr, e, "stats");
    if ((e = dalloc(h, &h->d_stat_out, 4)) != cudaSuccess) return cuda_fail(nullptr, e, "stats");
    if ((e = dalloc(h, &h->d_pair_counts, 2)) != cudaSuccess) return cuda_fail(nullptr, e, "pairs");
    if ((e = cudaMallocHost((void**)&h->h_pinned, sizeof(int64_t) * 4)) != cudaSuccess)
        return cuda_fail(nullptr, e, "pinned");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(nullptr, e, "create sync");
    h->total_cells = (int32_t)cells;
    h->cells.init(cells);
    h->walls.init(h->wcap);
    h->scenes.assign(h->scap, SceneRec());
    h->W.n = 1;  // wall walks read the (possibly empty) ranges of every scene
    return SPH_OK;
}

bool same_kind(const SphHandle* h, const SphParams& p) {
    return p.dim == h->dim && p.kernel == h->kernel && mode_of(p.solve) == h->mode && p.thermal == h->thermal &&
           p.precision == h->precision;
}

// The scan and the count clears cover cells [0, end of the highest range in use).
void update_scan_range(SphHandle* h) {
    int64_t hi = 1;
    for (const SceneRec& R : h->scenes)
        if (R.used) hi = std::max<int64_t>(hi, (int64_t)R.dev.cell_off + R.cell_span);
    if (hi != h->scan_cells) {  // the step graphs bake the scan length
        for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
        h->graphs.clear();
    }
    h->scan_cells = (int32_t)hi;
}

// Claim a scene slot and its cell range; walls are reserved with wall_cap entries.
int32_t open_scene(SphHandle* h, const SphParams& p, int64_t wall_cap, int64_t first_step, int64_t last_step,
                   int* out) {
    int s = -1;
    for (int k = 0; k < h->scap; ++k)
        if (!h->scenes[k].used) {
            s = k;
            break;
        }
    if (s < 0) return fail(h, SPH_ERR_OOM, "no free scene slot");
    SceneDev S;
    std::string err;
    if (!build_scene(p, S, err)) return fail(h, SPH_ERR_ARG, err);
    const int64_t span = (int64_t)S.ncells + 1;
    int64_t coff = 0, woff = 0;
    if (!h->cells.alloc(span, &coff)) return fail(h, SPH_ERR_OOM, "cell capacity exhausted");
    if (!h->walls.alloc(wall_cap, &woff)) {
        h->cells.release(coff, span);
        return fail(h, SPH_ERR_OOM, "wall capacity exhausted");
    }
    S.cell_off = (int32_t)coff;
    S.last_step = last_step;
    S.active = 1;
    S.prune = h->prune >= 0 ? h->prune : (p.dim == 3 ? 1 : 0);
    SceneRec& R = h->scenes[s];
    R = SceneRec();
    R.used = true;
    R.dev = S;
    R.cell_span = (int32_t)span;
    R.wall_off = woff;
    R.wall_cap = wall_cap;
    R.first_step = first_step;
    update_scan_range(h);
    int32_t rc = upload_scene_const(h, s);
    if (rc == SPH_OK) rc = set_scene_step(h, s, first_step);
    if (rc == SPH_OK) rc = write_scene_walls(h, s);  // empty cell starts
    if (rc != SPH_OK) return rc;
    *out = s;
    return SPH_OK;
}

}  // namespace

namespace {

// Device arrays of the buffers: both sorted sets, the sort scratch and the counters.
int32_t allocate_buffers(SphHandle* h, int64_t cap) {
    cudaError_t e;
    const size_t n = (size_t)cap, ncell = (size_t)h->total_cells;
    for (int b = 0; b < 2; ++b) {
        BufferState& B = h->B[b];
        double** d[5] = {&B.rho, &B.p, &B.c, &B.m, &B.gap};
        if ((e = alloc_vec(h, (void**)&B.x, n)) != cudaSuccess) return cuda_fail(h, e, "buffer x");
        if ((e = alloc_vec(h, (void**)&B.v, n)) != cudaSuccess) return cuda_fail(h, e, "buffer v");
        for (double** f : d)
            if ((e = dalloc(h, f, n)) != cudaSuccess) return cuda_fail(h, e, "buffer field");
        if ((e = dalloc(h, &B.order, n)) != cudaSuccess) return cuda_fail(h, e, "buffer order");
    }
    BufferScratch& S = h->bs;
    struct {
        int32_t** p;
        size_t n;
    } ints[] = {{&S.key, n}, {&S.slot, n}, {&S.count, ncell}, {&S.start, ncell + 1},
                {&S.block_sums, ncell / 1024 + 2}, {&S.pend, n}, {&S.npend, 1}, {&h->bn, 2}};
    for (auto& a : ints)
        if ((e = dalloc(h, a.p, a.n)) != cudaSuccess) return cuda_fail(h, e, "buffer scratch");
    if ((e = dalloc(h, &S.tmp, n)) != cudaSuccess) return cuda_fail(h, e, "buffer scratch");
    S.cap = (int32_t)cap;
    h->bcap = cap;
    return SPH_OK;
}

// The live buffer particles of the current parity, on the host (sorted order).
struct HostBuffers {
    int32_t n = 0;
    std::vector<char> x, v;
    std::vector<double> rho, p, c, m, gap;
    std::vector<int64_t> order;
};

int32_t read_buffers(SphHandle* h, HostBuffers& H) {
    cudaStream_t st = h->stream;
    SPH_CUDA(h, cudaMemcpyAsync(&H.n, h->bn + h->par, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    if (H.n < 0 || H.n > h->bcap) return fail(h, SPH_ERR_STATE, "buffer count out of range");
    const size_t n = (size_t)H.n, vb = vec_bytes(h->dim);
    const BufferState& B = h->B[h->par];
    H.x.resize(n * vb);
    H.v.resize(n * vb);
    H.order.resize(n);
    std::vector<double>* f[5] = {&H.rho, &H.p, &H.c, &H.m, &H.gap};
    const double* src[5] = {B.rho, B.p, B.c, B.m, B.gap};
    if (n > 0) {
        SPH_CUDA(h, cudaMemcpyAsync(H.x.data(), B.x, n * vb, cudaMemcpyDeviceToHost, st));
        SPH_CUDA(h, cudaMemcpyAsync(H.v.data(), B.v, n * vb, cudaMemcpyDeviceToHost, st));
        SPH_CUDA(h, cudaMemcpyAsync(H.order.data(), B.order, n * 8, cudaMemcpyDeviceToHost, st));
        for (int k = 0; k < 5; ++k) {
            f[k]->resize(n);
            SPH_CUDA(h, cudaMemcpyAsync(f[k]->data(), src[k], n * 8, cudaMemcpyDeviceToHost, st));
        }
    }
    SPH_CUDA(h, cudaStreamSynchronize(st));
    return SPH_OK;
}

// Sorted positions of the inlet (which = 0) or outlet (1) particles, in ascending order.
std::vector<int64_t> buffer_rank(const HostBuffers& H, int which) {
    std::vector<int64_t> sel;
    for (int64_t b = 0; b < H.n; ++b)
        if (((H.order[b] & kOutletBit) != 0) == (which == 1)) sel.push_back(b);
    std::sort(sel.begin(), sel.end(), [&](int64_t a, int64_t b) { return H.order[a] < H.order[b]; });
    return sel;
}

}  // namespace

extern "C" {

int32_t sph_version(void) { return SPH_ABI_VERSION; }

int32_t sph_create(const SphParams* params, int64_t fluid_capacity, int64_t wall_capacity, SphHandle** out) {
    if (!params || !out) return fail(nullptr, SPH_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(nullptr, SPH_ERR_NO_DEVICE, "no CUDA device");
    if (fluid_capacity < 1 || fluid_capacity > (int64_t)INT32_MAX / 8 || wall_capacity < 0 ||
        wall_capacity > (int64_t)INT32_MAX / 2)
        return fail(nullptr, SPH_ERR_ARG, "capacity out of range");
    SceneDev S;
    std::string err;
    if (!build_scene(*params, S, err)) return fail(nullptr, SPH_ERR_ARG, err);
    SphHandle* h = new SphHandle();
    h->prm = *params;
    h->dim = params->dim;
    h->kernel = params->kernel;
    h->mode = mode_of(params->solve);
    h->thermal = params->thermal;
    h->precision = params->precision;
    h->cap = fluid_capacity;
    h->wcap = wall_capacity;
    h->scap = 1;
    int32_t rc = allocate_handle(h, (int64_t)S.ncells + 1);
    int s = 0;
    if (rc == SPH_OK) rc = open_scene(h, *params, wall_capacity, 1, INT64_MAX, &s);
    if (rc != SPH_OK) {
        if (h->err.size()) g_create_error = h->err;
        sph_destroy(h);
        return rc;
    }
    *out = h;
    return SPH_OK;
}

int32_t sph_upload_fluid(SphHandle* h, int64_t n, const double* x, const double* v, const double* rho,
                         const double* p, const double* c, const double* mass, const double* gap, const double* t,
                         const double* kappa, const double* cp) {
    NvtxRange nvtx_range("sph_upload_fluid");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (h->batch) return fail(h, SPH_ERR_STATE, "batch handles take fluid through sph_batch_add_scene");
    if (n < 0 || n > h->cap) return fail(h, SPH_ERR_GRID_OVERFLOW, "fluid count exceeds the handle capacity");
    SceneRec& R = h->scenes[0];
    bool uniform = true;
    for (int64_t i = 1; i < n; ++i) uniform &= gap[i] == gap[0];
    R.gap0 = n > 0 ? gap[0] : 0.0;
    R.uniform_fluid = uniform;
    R.dev.uniform_gap = uniform && (!h->has_buffers || h->buffer_gap_uniform(R.gap0)) ? 1 : 0;
    int32_t rc = upload_scene_const(h, 0);
    if (rc != SPH_OK) return rc;
    rc = append_fluid(h, 0, 0, n, x, v, rho, p, c, mass, gap, t, kappa, cp);  // replaces the state
    if (rc != SPH_OK) return rc;
    h->have_fluid = true;
    h->n_uploaded = n;
    if (h->has_buffers) {  // fluid made from the inlet continues the ids of this upload
        h->br.id_base = n;
        for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
        h->graphs.clear();
    }
    return SPH_OK;
}

int32_t sph_upload_walls(SphHandle* h, int32_t kind, int64_t n, const double* x, const double* normal,
                         const double* gap, const double* t, const double* kappa, const double* v) {
    NvtxRange nvtx_range("sph_upload_walls");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (h->batch) return fail(h, SPH_ERR_STATE, "batch handles take walls through sph_batch_add_scene");
    SceneRec& R = h->scenes[0];
    if ((int64_t)R.wgap.size() + n > R.wall_cap) return fail(h, SPH_ERR_GRID_OVERFLOW, "wall count exceeds the handle capacity");
    int32_t rc = add_walls_host(h, R, kind, n, x, normal, gap, t, kappa, v);
    if (rc != SPH_OK) return rc;
    R.wgroup_end.push_back((int64_t)R.wgap.size());
    return write_scene_walls(h, 0);
}

int32_t sph_step_async(SphHandle* h, int64_t first_step, int64_t nsteps) {
    NvtxRange nvtx_range("sph_step_async");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (h->batch) return fail(h, SPH_ERR_STATE, "batch handles step with sph_batch_step");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "sph_step before sph_upload_fluid");
    if (nsteps < 0) return fail(h, SPH_ERR_ARG, "negative step count");
    if (nsteps == 0) return SPH_OK;
    if (h->has_buffers) {
        if (!h->buffers_started) {  // ids of inlet copies count steps from here
            h->br.first_step = first_step;
            h->buffers_started = true;
            for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
            h->graphs.clear();
        }
        if (first_step < h->br.first_step) return fail(h, SPH_ERR_ARG, "steps before the buffer upload");
        if (h->br.id_base + (first_step + nsteps - h->br.first_step) * h->br.n_inlet > INT32_MAX)
            return fail(h, SPH_ERR_ARG, "fluid ids of inlet copies would pass 2^31 - 1");
    }
    if (first_step != h->scenes[0].step_host) {  // the device counter only needs a reset on a jump
        int32_t rc = set_scene_step(h, 0, first_step);
        if (rc != SPH_OK) return rc;
    }
    return step_all_async(h, nsteps);
}

int32_t sph_synchronize(SphHandle* h) {
    NvtxRange nvtx_range("sph_synchronize");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    cudaStream_t st = h->stream;
    SPH_CUDA(h, cudaMemcpyAsync(&h->h_pinned[1], h->sc.status, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaMemsetAsync(h->sc.status, 0, 4, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    int32_t status = 0;
    std::memcpy(&status, &h->h_pinned[1], 4);
    bool nan_check = h->prm.nan_check;
    for (const SceneRec& R : h->scenes) nan_check |= R.used && R.dev.nan_check;
    if ((status & kStatusNonFinite) && nan_check)
        return fail(h, SPH_ERR_NAN, "non-finite fluid state (density, velocity or position)");
    if (status & kStatusBufferOverflow)
        return fail(h, SPH_ERR_GRID_OVERFLOW, "inlet/outlet transfers exceeded the fluid or buffer capacity");
    return SPH_OK;
}

int32_t sph_step(SphHandle* h, int64_t first_step, int64_t nsteps) {
    int32_t rc = sph_step_async(h, first_step, nsteps);
    if (rc != SPH_OK) return rc;
    return sph_synchronize(h);
}

int32_t sph_download_fluid(SphHandle* h, int64_t capacity, int64_t* n_out, double* x, double* v, double* rho,
                           double* p, double* c, double* mass, double* gap, double* t, double* kappa, double* cp) {
    NvtxRange nvtx_range("sph_download_fluid");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!n_out) return fail(h, SPH_ERR_ARG, "n_out is required");
    if (h->batch) return fail(h, SPH_ERR_STATE, "batch handles download with sph_batch_download_scene");
    if (!h->have_fluid) {
        *n_out = 0;
        return SPH_OK;
    }
    return download_scene(h, 0, capacity, n_out, x, v, rho, p, c, mass, gap, t, kappa, cp, nullptr);
}

int32_t sph_download_ids(SphHandle* h, int64_t capacity, int64_t* n_out, int64_t* ids_out) {
    NvtxRange nvtx_range("sph_download_ids");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!n_out) return fail(h, SPH_ERR_ARG, "n_out is required");
    if (h->batch) return fail(h, SPH_ERR_STATE, "batch handles download with sph_batch_download_scene");
    if (!h->have_fluid) {
        *n_out = 0;
        return SPH_OK;
    }
    return download_scene(h, 0, capacity, n_out, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                          nullptr, nullptr, nullptr, ids_out);
}

// ------------------------------------------------------------------ batch / serving
int32_t sph_batch_create(const SphParams* prototype, int64_t particle_capacity, int64_t cell_capacity,
                         int64_t wall_capacity, int32_t scene_capacity, SphHandle** out) {
    if (!prototype || !out) return fail(nullptr, SPH_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(nullptr, SPH_ERR_NO_DEVICE, "no CUDA device");
    if (particle_capacity < 1 || particle_capacity > (int64_t)INT32_MAX / 8 || cell_capacity < 2 ||
        cell_capacity > (int64_t)scan_max_cells() || wall_capacity < 0 || wall_capacity > (int64_t)INT32_MAX / 2 ||
        scene_capacity < 1 || scene_capacity > (1 << 20))
        return fail(nullptr, SPH_ERR_ARG, "capacity out of range");
    SceneDev S;
    std::string err;
    if (!build_scene(*prototype, S, err)) return fail(nullptr, SPH_ERR_ARG, err);
    SphHandle* h = new SphHandle();
    h->batch = true;
    h->prm = *prototype;
    h->dim = prototype->dim;
    h->kernel = prototype->kernel;
    h->mode = mode_of(prototype->solve);
    h->thermal = prototype->thermal;
    h->precision = prototype->precision;
    h->cap = particle_capacity;
    h->wcap = wall_capacity;
    h->scap = scene_capacity;
    int32_t rc = allocate_handle(h, cell_capacity);
    if (rc != SPH_OK) {
        sph_destroy(h);
        return rc;
    }
    h->have_fluid = true;
    *out = h;
    return SPH_OK;
}

int32_t sph_batch_add_scene(SphHandle* h, const SphParams* params, int64_t first_step, int64_t nsteps, int64_t n,
                            const double* x, const double* v, const double* rho, const double* p, const double* c,
                            const double* mass, const double* gap, const double* t, const double* kappa,
                            const double* cp, int64_t n_wall, const int32_t* wall_kind, const double* wall_x,
                            const double* wall_normal, const double* wall_gap, const double* wall_t,
                            const double* wall_kappa, const double* wall_v, int32_t* scene_id) {
    NvtxRange nvtx_range("sph_batch_add_scene");
    if (!h || !params || !scene_id) return fail(h, SPH_ERR_ARG, "null argument");
    if (!h->batch) return fail(h, SPH_ERR_STATE, "not a batch handle");
    if (!same_kind(h, *params)) return fail(h, SPH_ERR_ARG, "scene differs from the batch in dim/kernel/solve/form");
    if (n < 0 || n_wall < 0 || nsteps < 0) return fail(h, SPH_ERR_ARG, "negative count");
    if (n_wall > 0 && !wall_kind) return fail(h, SPH_ERR_ARG, "wall kinds are required");
    int32_t n_before = 0;
    int32_t rc = read_live(h, &n_before);
    if (rc != SPH_OK) return rc;
    if ((int64_t)n_before + n > h->cap) return fail(h, SPH_ERR_OOM, "particle capacity exhausted");
    int s = -1;
    rc = open_scene(h, *params, n_wall, first_step, first_step + nsteps - 1, &s);
    if (rc != SPH_OK) return rc;
    SceneRec& R = h->scenes[s];
    const int dim = h->dim;
    for (int64_t w = 0; w < n_wall && rc == SPH_OK; ++w)
        rc = add_walls_host(h, R, wall_kind[w], 1, wall_x + w * dim, wall_normal + w * dim, wall_gap + w,
                            wall_t ? wall_t + w : nullptr, wall_kappa ? wall_kappa + w : nullptr,
                            wall_v ? wall_v + w * dim : nullptr);
    bool uniform = true;
    for (int64_t i = 1; i < n; ++i) uniform &= gap[i] == gap[0];
    R.dev.uniform_gap = uniform ? 1 : 0;
    if (rc == SPH_OK) rc = upload_scene_const(h, s);
    if (rc == SPH_OK) rc = write_scene_walls(h, s);
    if (rc == SPH_OK) rc = append_fluid(h, s, n_before, n, x, v, rho, p, c, mass, gap, t, kappa, cp);
    if (rc != SPH_OK) {
        const std::string keep = h->err;
        R.dev.active = 0;
        upload_scene_const(h, s);
        h->cells.release(R.dev.cell_off, R.cell_span);
        h->walls.release(R.wall_off, R.wall_cap);
        R = SceneRec();
        update_scan_range(h);
        h->err = keep;
        return rc;
    }
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);  // Shepard patterns change
    h->graphs.clear();
    *scene_id = s;
    return SPH_OK;
}

int32_t sph_batch_step(SphHandle* h, int64_t nsteps) {
    NvtxRange nvtx_range("sph_batch_step");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->batch) return fail(h, SPH_ERR_STATE, "not a batch handle");
    if (nsteps < 0) return fail(h, SPH_ERR_ARG, "negative step count");
    if (nsteps == 0) return SPH_OK;
    return step_all_async(h, nsteps);
}

int32_t sph_batch_scene_info(SphHandle* h, int32_t scene_id, int64_t* info) {
    if (!h || !info) return fail(h, SPH_ERR_ARG, "null argument");
    if (scene_id < 0 || scene_id >= h->scap || !h->scenes[scene_id].used) return fail(h, SPH_ERR_ARG, "no such scene");
    const SceneRec& R = h->scenes[scene_id];
    int32_t b = 0, e = 0;
    int32_t rc = scene_range(h, scene_id, &b, &e);
    if (rc != SPH_OK) return rc;
    const int64_t total = R.dev.last_step - R.first_step + 1;
    const int64_t done = std::min<int64_t>(R.step_host - R.first_step, total);
    info[0] = e - b;
    info[1] = done;
    info[2] = done >= total ? 1 : 0;
    info[3] = R.step_host;
    return SPH_OK;
}

int32_t sph_batch_download_scene(SphHandle* h, int32_t scene_id, int64_t capacity, int64_t* n_out, double* x,
                                 double* v, double* rho, double* p, double* c, double* mass, double* gap, double* t,
                                 double* kappa, double* cp) {
    NvtxRange nvtx_range("sph_batch_download_scene");
    if (!h || !n_out) return fail(h, SPH_ERR_ARG, "null argument");
    if (scene_id < 0 || scene_id >= h->scap || !h->scenes[scene_id].used) return fail(h, SPH_ERR_ARG, "no such scene");
    return download_scene(h, scene_id, capacity, n_out, x, v, rho, p, c, mass, gap, t, kappa, cp, nullptr);
}

int32_t sph_batch_retire(SphHandle* h, int32_t scene_id) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->batch) return fail(h, SPH_ERR_STATE, "not a batch handle");
    if (scene_id < 0 || scene_id >= h->scap || !h->scenes[scene_id].used) return fail(h, SPH_ERR_ARG, "no such scene");
    SceneRec& R = h->scenes[scene_id];
    R.dev.active = 0;
    int32_t rc = upload_scene_const(h, scene_id);
    if (rc == SPH_OK) rc = resort(h);  // drops the scene's particles
    int32_t n_left = 0;
    if (rc == SPH_OK) rc = read_live(h, &n_left);
    if (rc == SPH_OK) set_n_upper(h, n_left);
    if (rc != SPH_OK) return rc;
    h->cells.release(R.dev.cell_off, R.cell_span);
    h->walls.release(R.wall_off, R.wall_cap);
    R = SceneRec();
    update_scan_range(h);
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SPH_OK;
}

int32_t sph_scene_footprint(const SphParams* params, int64_t n_fluid, int64_t n_wall, int64_t* out) {
    if (!params || !out || n_fluid < 0 || n_wall < 0) {
        set_global_error("sph_scene_footprint: invalid arguments");
        return SPH_ERR_ARG;
    }
    SceneDev S{};
    std::string err;
    if (!build_scene(*params, S, err)) {
        set_global_error(err);
        return SPH_ERR_ARG;
    }
    out[0] = n_fluid;
    out[1] = (int64_t)S.ncells + 1;
    out[2] = n_wall;
    return SPH_OK;
}

int32_t sph_batch_free(SphHandle* h, int64_t* out) {
    if (!h || !out) return fail(h, SPH_ERR_ARG, "null argument");
    int32_t n = 0;
    int32_t rc = read_live(h, &n);
    if (rc != SPH_OK) return rc;
    int64_t slots = 0;
    for (const SceneRec& R : h->scenes) slots += !R.used;
    out[0] = h->cap - n;
    out[1] = h->cells.largest();
    out[2] = h->walls.largest();
    out[3] = slots;
    return SPH_OK;
}


int32_t sph_stats(SphHandle* h, SphStats* out) {
    if (!h || !out) return fail(h, SPH_ERR_ARG, "null argument");
    std::memset(out, 0, sizeof(*out));
    LaunchCtx L = make_ctx(h);
    cudaStream_t st = h->stream;
    launch_stats(L, h->d_stat_partials, h->d_stat_out);
    SPH_CUDA(h, cudaGetLastError());
    double r[3];
    int32_t n32 = 0, status = 0;
    SPH_CUDA(h, cudaMemcpyAsync(r, h->d_stat_out, sizeof(r), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaMemcpyAsync(&n32, h->nbuf + h->par, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaMemcpyAsync(&status, h->sc.status, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    out->n_fluid = h->have_fluid ? n32 : 0;
    out->n_wall = 0;
    for (const SceneRec& R : h->scenes) out->n_wall += R.used ? R.wall_n : 0;
    out->steps_done = h->steps_done;
    out->total_mass = r[0];
    out->kinetic_energy = r[1];
    out->max_speed = r[2];
    out->status_flags = status;
    return SPH_OK;
}

int32_t sph_count_pairs(SphHandle* h, int64_t* fluid_pairs, int64_t* wall_pairs) {
    if (!h || !fluid_pairs || !wall_pairs) return fail(h, SPH_ERR_ARG, "null argument");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    cudaStream_t st = h->stream;
    SPH_CUDA(h, cudaMemsetAsync(h->d_pair_counts, 0, 16, st));
    LaunchCtx L = make_ctx(h);
    launch_count_pairs(L, h->d_pair_counts);
    SPH_CUDA(h, cudaGetLastError());
    unsigned long long r[2];
    SPH_CUDA(h, cudaMemcpyAsync(r, h->d_pair_counts, 16, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    *fluid_pairs = (int64_t)r[0];
    *wall_pairs = (int64_t)r[1];
    return SPH_OK;
}

int32_t sph_download_cell_keys(SphHandle* h, int64_t capacity, int64_t* n_out, int64_t* keys, int32_t* grid) {
    NvtxRange nvtx_range("sph_download_cell_keys");
    if (!h || !n_out) return fail(h, SPH_ERR_ARG, "null argument");
    if (h->batch) return fail(h, SPH_ERR_STATE, "cell keys are for single-scene handles");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    const SceneDev& S = h->scenes[0].dev;
    if (grid)
        for (int a = 0; a < 3; ++a) grid[a] = S.n[a];
    int32_t b = 0, e = 0;
    if (int32_t rc = scene_range(h, 0, &b, &e); rc != SPH_OK) return rc;
    const int64_t n = e - b;
    *n_out = n;
    if (!keys || n == 0) return SPH_OK;  // the count (and grid) only
    if (n > capacity) return fail(h, SPH_ERR_ARG, "caller array too small for the live fluid");
    cudaStream_t st = h->stream;
    std::vector<int32_t> ids(n), hk(n), order;
    int32_t* d_keys = nullptr;
    SPH_CUDA(h, cudaMalloc((void**)&d_keys, (size_t)n * 4));
    LaunchCtx L = make_ctx(h);
    launch_cell_keys(L, b, e, d_keys);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpyAsync(hk.data(), d_keys, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(ids.data(), h->S[h->par].id + b, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cudaFree(d_keys);
    if (err != cudaSuccess) return cuda_fail(h, err, "sph_download_cell_keys");
    ascending_id_order(ids, order);
    for (int64_t q = 0; q < n; ++q) keys[q] = hk[order[q]];
    return SPH_OK;
}

int32_t sph_download_neighbours(SphHandle* h, int64_t capacity, int64_t ids_capacity, int64_t* n_out,
                                int64_t* total_out, int64_t* offsets, int64_t* nbr_ids) {
    NvtxRange nvtx_range("sph_download_neighbours");
    if (!h || !n_out || !total_out || !offsets) return fail(h, SPH_ERR_ARG, "null argument");
    if (h->batch) return fail(h, SPH_ERR_STATE, "neighbour lists are for single-scene handles");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    int32_t b = 0, e = 0;
    if (int32_t rc = scene_range(h, 0, &b, &e); rc != SPH_OK) return rc;
    const int64_t n = e - b;
    *n_out = n;
    *total_out = 0;
    if (n + 1 > capacity) return fail(h, SPH_ERR_ARG, "offsets array too small (live fluid + 1)");
    offsets[0] = 0;
    if (n == 0) return SPH_OK;
    cudaStream_t st = h->stream;
    LaunchCtx L = make_ctx(h);
    std::vector<int32_t> ids(n), counts(n), order;
    int32_t* d_counts = nullptr;
    SPH_CUDA(h, cudaMalloc((void**)&d_counts, (size_t)n * 4));
    launch_neighbours(L, b, e, d_counts, nullptr, nullptr);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpyAsync(counts.data(), d_counts, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(ids.data(), h->S[h->par].id + b, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cudaFree(d_counts);
    if (err != cudaSuccess) return cuda_fail(h, err, "sph_download_neighbours (counts)");
    ascending_id_order(ids, order);
    std::vector<int64_t> rows(n);  // first entry of each sorted particle's row
    for (int64_t q = 0; q < n; ++q) {
        rows[order[q]] = offsets[q];
        offsets[q + 1] = offsets[q] + counts[order[q]];
    }
    const int64_t total = offsets[n];
    *total_out = total;
    if (!nbr_ids) return SPH_OK;
    if (total > ids_capacity) return fail(h, SPH_ERR_ARG, "ids array too small for the neighbour lists");
    if (total == 0) return SPH_OK;
    int64_t* d_rows = nullptr;
    int32_t* d_ids = nullptr;
    std::vector<int32_t> hid(total);
    err = cudaMalloc((void**)&d_rows, (size_t)n * 8);
    if (err == cudaSuccess) err = cudaMalloc((void**)&d_ids, (size_t)total * 4);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_rows, rows.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) {
        launch_neighbours(L, b, e, nullptr, d_rows, d_ids);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(hid.data(), d_ids, (size_t)total * 4, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (d_rows) cudaFree(d_rows);
    if (d_ids) cudaFree(d_ids);
    if (err != cudaSuccess) return cuda_fail(h, err, "sph_download_neighbours (ids)");
    for (int64_t q = 0; q < n; ++q) {
        std::sort(hid.begin() + offsets[q], hid.begin() + offsets[q + 1]);
        for (int64_t k = offsets[q]; k < offsets[q + 1]; ++k) nbr_ids[k] = hid[k];
    }
    return SPH_OK;
}

int32_t sph_get_stream(SphHandle* h, void** stream) {
    if (!h || !stream) return fail(h, SPH_ERR_ARG, "null argument");
    *stream = (void*)h->stream;
    return SPH_OK;
}

int32_t sph_time_stages(SphHandle* h, int32_t reps, double* ms_out) {
    if (!h || !ms_out || reps < 1) return fail(h, SPH_ERR_ARG, "bad argument");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    cudaStream_t st = h->stream;
    if (int32_t rc = ensure_list(h); rc != SPH_OK) return rc;
    cudaEvent_t e0, e1;
    SPH_CUDA(h, cudaEventCreate(&e0));
    SPH_CUDA(h, cudaEventCreate(&e1));
    LaunchCtx L = make_ctx(h);
    // the hash and placement stages read the current sorted positions as "next" ones
    LaunchCtx Lh = L;
    Lh.nx.x = L.st.x;
    Lh.nx.v = L.st.v;
    Lh.nx.rho = L.st.rho;
    Lh.nx.T = L.st.T;
    L.bs.npend = nullptr;  // timed momentum launches mark no particle for the outlet
    LaunchCtx Lr = L;      // the momentum gather of a re-initialisation step
    Lr.shepard = 1;
    Lr.force_reinit = 1;
    const int par = h->par;
    auto run = [&](int stage) {
        switch (stage) {
            case SPH_STAGE_CELL_COUNT:
                cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->scan_cells, st);
                launch_hash(Lh);
                break;
            case SPH_STAGE_SCAN: launch_scan(Lh, 0); break;
            case SPH_STAGE_SORT: launch_place(Lh); break;
            case SPH_STAGE_CONTINUITY: launch_physics(0, L); break;
            case SPH_STAGE_MOMENTUM: launch_physics(1, L); break;
            case SPH_STAGE_REINIT: launch_physics(1, Lr); break;
        }
    };
    for (int stage = 0; stage < SPH_NUM_STAGES; ++stage) {
        run(stage);  // warm-up
        SPH_CUDA(h, cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) run(stage);
        SPH_CUDA(h, cudaEventRecord(e1, st));
        SPH_CUDA(h, cudaEventSynchronize(e1));
        float ms = 0.f;
        SPH_CUDA(h, cudaEventElapsedTime(&ms, e0, e1));
        ms_out[stage] = (double)ms / reps;
        if (stage == SPH_STAGE_CELL_COUNT) {  // leave a consistent cell list for the later stages
            SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->scan_cells, st));
            launch_hash(Lh);
        }
    }
    // the momentum stage left arrivals in count[]: the next step expects it zeroed
    SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->scan_cells, st));
    // restore p and c (output-only fields) from the copy the placement stage wrote
    const size_t n = (size_t)h->cap;
    SPH_CUDA(h, cudaMemcpyAsync(h->S[par].p, h->S[par ^ 1].p, n * 8, cudaMemcpyDeviceToDevice, st));
    SPH_CUDA(h, cudaMemcpyAsync(h->S[par].c, h->S[par ^ 1].c, n * 8, cudaMemcpyDeviceToDevice, st));
    SPH_CUDA(h, cudaGetLastError());
    SPH_CUDA(h, cudaStreamSynchronize(st));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return SPH_OK;
}

int32_t sph_autotune(SphHandle* h, int32_t reps, int32_t* out) {
    NvtxRange nvtx_range("sph_autotune");
    if (!h || reps < 1) return fail(h, SPH_ERR_ARG, "bad argument");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    if (h->precision == SPH_PRECISION_FP32_COMPENSATED) {
        cudaStream_t st = h->stream;
        // storage for the list candidates (kept only when a list shape wins; released
        // with the handle)
        const int saved1 = h->tune[1];
        h->tune[1] = SPH_LANES_LIST + 1;
        const bool have_list = ensure_list(h) == SPH_OK;
        h->tune[1] = saved1;
        if (!have_list) h->err.clear();
        cudaEvent_t e0, e1;
        SPH_CUDA(h, cudaEventCreate(&e0));
        SPH_CUDA(h, cudaEventCreate(&e1));
        const int par = h->par;
        const size_t nbytes = (size_t)h->cap * 8;
        // p and c are output fields of the last step; the timed continuity launches
        // overwrite them, so park them in the idle sorted buffer meanwhile
        SPH_CUDA(h, cudaMemcpyAsync(h->S[par ^ 1].p, h->S[par].p, nbytes, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->S[par ^ 1].c, h->S[par].c, nbytes, cudaMemcpyDeviceToDevice, st));
        const int blocks[3] = {64, 128, 256};
        // time `reps` launches of one stage at one shape; list: continuity records the
        // neighbour list / momentum reads it
        auto trial = [&](int stage, int tpp, int block, bool list) -> float {
            LaunchCtx L = make_ctx(h);
            L.bs.npend = nullptr;  // trial launches mark no particle for the outlet
            L.block = block;
            L.tpp_continuity = L.tpp_momentum = tpp;
            L.list_momentum = list ? 1 : 0;
            L.nl = h->nl;
            launch_physics(stage, L);  // warm-up
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps; ++r) launch_physics(stage, L);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            return ms;
        };
        struct Best {
            float ms = 1e30f;
            int tpp = 1, block = 128;
        };
        auto search = [&](int stage, const int* tpps, int ntpp, bool list) {
            Best b;
            for (int q = 0; q < ntpp; ++q)
                for (int block : blocks) {
                    if (tpps[q] == -1 && stage == 1 && block > 256) continue;
                    const float ms = trial(stage, tpps[q], block, list);
                    if (ms < b.ms) b = Best{ms, tpps[q], block};
                }
            return b;
        };
        const int walk_tpps[5] = {-1, 1, 2, 4, 8};  // -1: one lane, software-pipelined loop
        const Best c_walk = search(0, walk_tpps, 5, false);
        const Best m_walk = search(1, walk_tpps, 5, false);
        Best c_list, m_list;
        if (have_list) {
            const int c_tpps[3] = {-1, 1, 2}, m_tpps[4] = {-1, 1, 2, 4};
            c_list = search(0, c_tpps, 3, true);
            // the momentum trials read the list the last continuity trial recorded
            trial(0, c_list.tpp, c_list.block, true);
            m_list = search(1, m_tpps, 4, true);
        }
        // the cell-walk pair against the list pair, each timed as it runs in a step
        // (continuity then momentum, at the momentum stage's block size)
        auto pair_ms = [&](const Best& c, const Best& m, bool list) -> float {
            LaunchCtx L = make_ctx(h);
            L.bs.npend = nullptr;
            L.block = m.block;
            L.tpp_continuity = c.tpp;
            L.tpp_momentum = m.tpp;
            L.list_momentum = list ? 1 : 0;
            L.nl = h->nl;
            launch_physics(0, L);
            launch_physics(1, L);
            const int n = std::max(reps, 5);
            cudaEventRecord(e0, st);
            for (int r = 0; r < n; ++r) {
                launch_physics(0, L);
                launch_physics(1, L);
            }
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            return ms;
        };
        const bool pick_list = have_list && pair_ms(c_list, m_list, true) < pair_ms(c_walk, m_walk, false);
        SPH_CUDA(h, cudaGetLastError());
        // one block size for all three stages: the momentum stage's (it dominates)
        if (pick_list) {
            h->tune[0] = c_list.tpp;
            h->tune[1] = SPH_LANES_LIST + m_list.tpp;
            h->tune[3] = m_list.block;
        } else {
            h->tune[0] = c_walk.tpp;
            h->tune[1] = m_walk.tpp;
            h->tune[3] = m_walk.block;
        }
        if (!pick_list && h->nl.e) {  // the list storage of the trials is not needed
            SPH_CUDA(h, cudaStreamSynchronize(st));
            cudaFree(h->nl.e);
            if (h->nl.n) cudaFree(h->nl.n);
            h->nl = NbrList{};
        }
        // restore what the timed launches touched: p and c, and the arrivals left in
        // count[]; every other field they wrote is rebuilt by the next step before use
        SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->scan_cells, st));
        if (h->has_buffers) SPH_CUDA(h, cudaMemsetAsync(h->bs.npend, 0, 4, st));  // outlet marks of the trials
        SPH_CUDA(h, cudaMemcpyAsync(h->S[par].p, h->S[par ^ 1].p, nbytes, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->S[par].c, h->S[par ^ 1].c, nbytes, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaGetLastError());
        SPH_CUDA(h, cudaStreamSynchronize(st));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
        h->graphs.clear();
    }
    if (out)
        for (int k = 0; k < 4; ++k) out[k] = h->tune[k];
    return SPH_OK;
}

int32_t sph_set_launch_shape(SphHandle* h, const int32_t* shape) {
    if (!h || !shape) return fail(h, SPH_ERR_ARG, "null argument");
    auto walk_code = [](int v) { return v == -1 || v == 1 || v == 2 || v == 4 || v == 8; };
    const bool list = shape[1] >= SPH_LANES_LIST - 1;
    if (!walk_code(shape[0]) || !walk_code(shape[2]))
        return fail(h, SPH_ERR_ARG, "lanes per particle must be 1, 2, 4, 8 or -1 (one pipelined lane)");
    if (list) {
        const int t = shape[1] - SPH_LANES_LIST;
        if (t != -1 && t != 1 && t != 2 && t != 4)
            return fail(h, SPH_ERR_ARG, "neighbour-list momentum lanes must be SPH_LANES_LIST + 1, 2, 4 or -1");
        if (shape[0] != 1 && shape[0] != -1 && shape[0] != 2)
            return fail(h, SPH_ERR_ARG, "the neighbour list is recorded by one or two continuity lanes (1, -1 or 2)");
    } else if (!walk_code(shape[1])) {
        return fail(h, SPH_ERR_ARG, "lanes per particle must be 1, 2, 4, 8 or -1 (one pipelined lane)");
    }
    if (shape[3] < 32 || shape[3] > 1024 || shape[3] % 32 != 0)
        return fail(h, SPH_ERR_ARG, "block size must be a multiple of 32 in [32, 1024]");
    if ((shape[1] == -1 || shape[1] == SPH_LANES_LIST - 1) && shape[3] > 256)
        return fail(h, SPH_ERR_ARG, "the pipelined momentum walk (-1) takes blocks of at most 256 threads");
    for (int k = 0; k < 4; ++k) h->tune[k] = shape[k];
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SPH_OK;
}

int32_t sph_set_stencil_pruning(SphHandle* h, int32_t on) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    h->prune = on ? 1 : 0;
    for (int s = 0; s < h->scap; ++s) {
        if (!h->scenes[s].used) continue;
        h->scenes[s].dev.prune = h->prune;
        if (int32_t rc = upload_scene_const(h, s); rc != SPH_OK) return rc;
    }
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

const char* sph_last_error(const SphHandle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int32_t sph_output_open(SphHandle* h, const char* dir_path, const char* file_name, const char* file_suffix,
                        int32_t step_digit, int32_t n_fields, const char* const* field_symbols,
                        const char* const* field_names, const char* wall_time) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (h->batch) return fail(h, SPH_ERR_STATE, "VTP output is for single-scene handles");
    int dev = 0;
    SPH_CUDA(h, cudaGetDevice(&dev));
    if (!h->out) h->out = new sph::VtpWriter();
    h->out_walls = -1;
    std::string err;
    int rc = h->out->open(dev, h->dim, h->thermal != 0, h->cap, dir_path, file_name, file_suffix, step_digit,
                          n_fields, field_symbols, field_names, wall_time, err);
    if (rc != SPH_OK) {
        delete h->out;
        h->out = nullptr;
        return fail(h, rc, err);
    }
    return SPH_OK;
}

int32_t sph_output_write(SphHandle* h, int64_t file_step, double time) {
    NvtxRange nvtx_range("sph_output_write");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->out || !h->out->is_open()) return fail(h, SPH_ERR_STATE, "sph_output_write before sph_output_open");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "sph_output_write before sph_upload_fluid");
    const SceneRec& R = h->scenes[0];
    std::string err;
    if (h->out_walls != (int64_t)R.wgroup_end.size()) {  // wall groups changed: hand the writer a copy
        std::vector<sph::WallGroupHost> groups;
        int64_t b = 0;
        const int dim = h->dim;
        for (int64_t e : R.wgroup_end) {
            sph::WallGroupHost g;
            g.kind = e > b ? R.wkind[b] : SPH_WALL_COMPULSIVE;
            g.n = e - b;
            g.x.assign(R.wx.begin() + b * dim, R.wx.begin() + e * dim);
            g.v.assign(R.wv.begin() + b * dim, R.wv.begin() + e * dim);
            g.gap.assign(R.wgap.begin() + b, R.wgap.begin() + e);
            g.T.assign(R.wT.begin() + b, R.wT.begin() + e);
            g.kappa.assign(R.wkappa.begin() + b, R.wkappa.begin() + e);
            groups.push_back(std::move(g));
            b = e;
        }
        int rc = h->out->set_walls(groups, err);
        if (rc != SPH_OK) return fail(h, rc, err);
        h->out_walls = (int64_t)R.wgroup_end.size();
    }
    const SortedState& d = h->S[h->par];
    sph::FluidSnapshotSrc src{};
    src.x = d.x;
    src.v = d.v;
    src.id = d.id;
    const double* f[sph::FF_COUNT] = {d.rho, d.p, d.c, d.m, d.gap, d.T, d.kappa, d.cp};
    for (int k = 0; k < sph::FF_COUNT; ++k) src.field[k] = f[k];
    src.start = h->sc.start;
    src.cell_lo = R.dev.cell_off;
    src.cell_hi = R.dev.cell_off + R.dev.ncells;
    src.n_upper = h->has_buffers ? h->cap : std::min<int64_t>(h->n_upper, h->cap);  // inlet copies append
    if (h->has_buffers) {
        const BufferState& B = h->B[h->par];
        src.bx = B.x;
        src.bv = B.v;
        const double* bf[5] = {B.rho, B.p, B.c, B.m, B.gap};
        for (int k = 0; k < 5; ++k) src.bfield[k] = bf[k];
        src.border = B.order;
        src.bn = h->bn + h->par;
        src.bcap = h->bcap;
    }
    int rc = h->out->enqueue(h->stream, src, file_step, time, err);
    if (rc != SPH_OK) return fail(h, rc, err);
    return SPH_OK;
}

int32_t sph_output_flush(SphHandle* h) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->out) return SPH_OK;
    std::string err;
    int rc = h->out->flush(err);
    if (rc != SPH_OK) return fail(h, rc, err);
    return SPH_OK;
}

int32_t sph_upload_buffers(SphHandle* h, const SphBufferRules* rules, int64_t capacity, int64_t n_inlet,
                           const double* x, const double* v, const double* rho, const double* p, const double* c,
                           const double* mass, const double* gap, int64_t n_outlet, const double* ox,
                           const double* ov, const double* orho, const double* op, const double* oc,
                           const double* omass, const double* ogap) {
    NvtxRange nvtx_range("sph_upload_buffers");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (h->batch) return fail(h, SPH_ERR_STATE, "inlet/outlet buffers are for single-scene handles");
    if (h->mode != 3) return fail(h, SPH_ERR_STATE, "buffers need solve = SPH_SOLVE_FLUID_INLET_OUTLET_WALL");
    if (!rules || n_inlet < 0 || n_outlet < 0 || capacity < n_inlet + n_outlet || capacity < 1 ||
        capacity > INT32_MAX / 2)
        return fail(h, SPH_ERR_ARG, "sph_upload_buffers: invalid counts or capacity");
    if ((n_inlet > 0 && (!x || !v || !rho || !p || !c || !mass || !gap)) ||
        (n_outlet > 0 && (!ox || !ov || !orho || !op || !oc || !omass || !ogap)))
        return fail(h, SPH_ERR_ARG, "sph_upload_buffers: missing arrays");
    const int dim = h->dim;
    if (capacity > h->bcap) {
        int32_t rc = allocate_buffers(h, capacity);
        if (rc != SPH_OK) return rc;
    }
    // rules
    BufferRules br{};
    for (int k = 0; k < 3; ++k) {
        br.in_n[k] = rules->inlet_normal[k];
        br.in_shift[k] = rules->inlet_shift[k];
        br.out_n[k] = rules->outlet_normal[k];
        br.drop_n[k] = rules->drop_normal[k];
    }
    br.in_d = rules->inlet_offset;
    br.out_d = rules->outlet_offset;
    br.drop_d = rules->drop_offset;
    br.n_inlet = n_inlet;
    br.id_base = h->n_uploaded;
    br.first_step = h->scenes[0].step_host;
    // host sort by (cell, order)
    const SceneRec& R = h->scenes[0];
    const int64_t n = n_inlet + n_outlet;
    std::vector<int64_t> order(n);
    std::vector<int32_t> key(n);
    auto xs = [&](int64_t b, int k) { return b < n_inlet ? x[b * dim + k] : ox[(b - n_inlet) * dim + k]; };
    for (int64_t b = 0; b < n; ++b) {
        order[b] = b < n_inlet ? b : (kOutletBit | (b - n_inlet));
        double xb[3] = {0, 0, 0};
        for (int k = 0; k < dim; ++k) xb[k] = xs(b, k);
        key[b] = host_cell_key(R.dev, dim, xb);
    }
    std::vector<int64_t> idx(n);
    for (int64_t b = 0; b < n; ++b) idx[b] = b;
    std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) {
        return key[a] != key[b] ? key[a] < key[b] : order[a] < order[b];
    });
    std::vector<int32_t> start((size_t)h->total_cells + 1, 0);
    for (int64_t b = 0; b < n; ++b) start[key[b] + 1]++;
    for (size_t q = 0; q + 1 < start.size(); ++q) start[q + 1] += start[q];
    const size_t vb = vec_bytes(dim);
    std::vector<char> hx(n * vb, 0), hv(n * vb, 0);
    std::vector<double> hf[5];
    for (auto& f : hf) f.resize(n);
    std::vector<int64_t> ho(n);
    h->bgap_host.assign(n, 0.0);
    for (int64_t q = 0; q < n; ++q) {
        const int64_t b = idx[q];
        const bool in = b < n_inlet;
        const int64_t j = in ? b : b - n_inlet;
        for (int k = 0; k < dim; ++k) {
            ((double*)(hx.data() + q * vb))[k] = in ? x[j * dim + k] : ox[j * dim + k];
            ((double*)(hv.data() + q * vb))[k] = in ? v[j * dim + k] : ov[j * dim + k];
        }
        hf[0][q] = in ? rho[j] : orho[j];
        hf[1][q] = in ? p[j] : op[j];
        hf[2][q] = in ? c[j] : oc[j];
        hf[3][q] = in ? mass[j] : omass[j];
        hf[4][q] = in ? gap[j] : ogap[j];
        h->bgap_host[q] = hf[4][q];
        ho[q] = order[b];
    }
    cudaStream_t st = h->stream;
    const BufferState& B = h->B[h->par];
    double* dst[5] = {B.rho, B.p, B.c, B.m, B.gap};
    if (n > 0) {
        SPH_CUDA(h, cudaMemcpyAsync(B.x, hx.data(), n * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(B.v, hv.data(), n * vb, cudaMemcpyHostToDevice, st));
        for (int f = 0; f < 5; ++f)
            SPH_CUDA(h, cudaMemcpyAsync(dst[f], hf[f].data(), n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(B.order, ho.data(), n * 8, cudaMemcpyHostToDevice, st));
    }
    SPH_CUDA(h, cudaMemcpyAsync(h->bs.start, start.data(), start.size() * 4, cudaMemcpyHostToDevice, st));
    const int32_t counts[2] = {(int32_t)n, (int32_t)n};
    SPH_CUDA(h, cudaMemcpyAsync(h->bn, counts, 8, cudaMemcpyHostToDevice, st));
    SPH_CUDA(h, cudaMemsetAsync(h->bs.count, 0, sizeof(int32_t) * (size_t)h->total_cells, st));
    SPH_CUDA(h, cudaMemsetAsync(h->bs.npend, 0, 4, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    h->br = br;
    h->has_buffers = true;
    h->buffers_started = false;
    // fluid made from the inlet (or a buffer with another gap) breaks the uniform-gap shortcut
    SceneRec& Rw = h->scenes[0];
    const bool uniform = Rw.uniform_fluid && h->buffer_gap_uniform(Rw.gap0);
    if ((Rw.dev.uniform_gap != 0) != uniform) {
        Rw.dev.uniform_gap = uniform ? 1 : 0;
        int32_t rc = upload_scene_const(h, 0);
        if (rc != SPH_OK) return rc;
    }
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SPH_OK;
}

int32_t sph_set_buffer_velocity(SphHandle* h, int32_t which, int64_t n, const double* v) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->has_buffers) return fail(h, SPH_ERR_STATE, "no inlet/outlet buffers");
    if ((which != 0 && which != 1) || n < 0 || (n > 0 && !v)) return fail(h, SPH_ERR_ARG, "bad arguments");
    HostBuffers H;
    int32_t rc = read_buffers(h, H);
    if (rc != SPH_OK) return rc;
    const std::vector<int64_t> sel = buffer_rank(H, which);
    if ((int64_t)sel.size() != n) return fail(h, SPH_ERR_ARG, "velocity count differs from the particle count");
    const int dim = h->dim;
    const size_t vb = vec_bytes(dim);
    for (int64_t q = 0; q < n; ++q)
        for (int k = 0; k < dim; ++k) ((double*)(H.v.data() + sel[q] * vb))[k] = v[q * dim + k];
    if (H.n > 0) {
        SPH_CUDA(h, cudaMemcpyAsync(h->B[h->par].v, H.v.data(), (size_t)H.n * vb, cudaMemcpyHostToDevice,
                                    h->stream));
        SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return SPH_OK;
}

int32_t sph_download_buffers(SphHandle* h, int32_t which, int64_t capacity, int64_t* n_out, double* x, double* v,
                             double* rho, double* p, double* c, double* mass, double* gap) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->has_buffers) return fail(h, SPH_ERR_STATE, "no inlet/outlet buffers");
    if ((which != 0 && which != 1) || !n_out) return fail(h, SPH_ERR_ARG, "bad arguments");
    HostBuffers H;
    int32_t rc = read_buffers(h, H);
    if (rc != SPH_OK) return rc;
    const std::vector<int64_t> sel = buffer_rank(H, which);
    *n_out = (int64_t)sel.size();
    if ((int64_t)sel.size() > capacity) return fail(h, SPH_ERR_ARG, "caller arrays too small for the buffers");
    const int dim = h->dim;
    const size_t vb = vec_bytes(dim);
    for (size_t q = 0; q < sel.size(); ++q) {
        const int64_t b = sel[q];
        for (int k = 0; k < dim; ++k) {
            if (x) x[q * dim + k] = ((const double*)(H.x.data() + b * vb))[k];
            if (v) v[q * dim + k] = ((const double*)(H.v.data() + b * vb))[k];
        }
        if (rho) rho[q] = H.rho[b];
        if (p) p[q] = H.p[b];
        if (c) c[q] = H.c[b];
        if (mass) mass[q] = H.m[b];
        if (gap) gap[q] = H.gap[b];
    }
    return SPH_OK;
}

int32_t sph_probe(SphHandle* h, int64_t n_points, const double* points, int32_t n_fields, const int32_t* fields,
                  double none_value, double* out) {
    NvtxRange nvtx_range("sph_probe");
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (h->batch) return fail(h, SPH_ERR_STATE, "probes are for single-scene handles");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "sph_probe before sph_upload_fluid");
    if (n_points < 0 || n_fields < 1 || n_fields > sph::kMaxProbeFields || !fields ||
        (n_points > 0 && (!points || !out)))
        return fail(h, SPH_ERR_ARG, "sph_probe: invalid arguments (1 to 8 fields)");
    sph::ProbeFields F{};
    F.n = n_fields;
    for (int f = 0; f < n_fields; ++f) {
        const int code = fields[f];
        if (code < SPH_PROBE_DENSITY || code > SPH_PROBE_MASS) return fail(h, SPH_ERR_ARG, "unknown probe field");
        if (code == SPH_PROBE_VELOCITY_Z && h->dim != 3) return fail(h, SPH_ERR_ARG, "VELOCITY_Z needs a 3D scene");
        if (code == SPH_PROBE_TEMPERATURE && !h->thermal)
            return fail(h, SPH_ERR_ARG, "TEMPERATURE needs a thermal model");
        F.code[f] = code;
    }
    if (n_points == 0) return SPH_OK;
    const int64_t need = n_points * (h->dim + n_fields);
    cudaStream_t st = h->stream;
    if (need > h->probe_cap) {
        if (h->probe_buf) {
            SPH_CUDA(h, cudaStreamSynchronize(st));
            cudaFree(h->probe_buf);
            h->probe_buf = nullptr;
            h->probe_cap = 0;
        }
        SPH_CUDA(h, cudaMalloc(&h->probe_buf, sizeof(double) * (size_t)need));
        h->probe_cap = need;
    }
    double* d_pts = h->probe_buf;
    double* d_out = h->probe_buf + n_points * h->dim;
    SPH_CUDA(h, cudaMemcpyAsync(d_pts, points, sizeof(double) * (size_t)(n_points * h->dim), cudaMemcpyHostToDevice,
                                st));
    LaunchCtx L = make_ctx(h);
    sph::launch_probe(L, n_points, d_pts, F, none_value, d_out);
    SPH_CUDA(h, cudaGetLastError());
    SPH_CUDA(h, cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)(n_points * n_fields), cudaMemcpyDeviceToHost,
                                st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    return SPH_OK;
}

int32_t sph_destroy(SphHandle* h) {
    if (!h) return SPH_OK;
    if (h->probe_buf) {
        if (h->stream) cudaStreamSynchronize(h->stream);
        cudaFree(h->probe_buf);
        h->probe_buf = nullptr;
    }
    if (h->dl_buf) {
        if (h->stream) cudaStreamSynchronize(h->stream);
        cudaFree(h->dl_buf);
        h->dl_buf = nullptr;
    }
    if (h->out) {
        std::string err;
        h->out->flush(err);
        delete h->out;
        h->out = nullptr;
    }
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    for (void* p : h->allocs) cudaFree(p);
    if (h->nl.e) cudaFree(h->nl.e);
    if (h->nl.n) cudaFree(h->nl.n);
    if (h->h_pinned) cudaFreeHost(h->h_pinned);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SPH_OK;
}

}  // extern "C"
