// sph_api.cu — host engine and C ABI (include/ethersph_gpu.h).
//
// One handle = one CUDA stream + the device state of one scene.  Step pipeline
// (FluidWallSolve.jl:8-83 and its siblings), all on the handle's stream:
//   memset(count) -> K4 continuity+EOS -> K5 momentum+integrate(+check, +next hash)
//   -> [K6 Shepard] -> scan -> fill+place (stable (cell, id) reorder into the other
//   buffer) -> swap.
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

#include "sph_kernels.h"

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
        default: return 2;
    }
}

// Parameter block -> per-scene device constants.  Grid: cell edge r_cut*(1+1e-9)
// (a periodic x axis is cut into floor(L/edge) equal cells), origin domain_lo.
bool build_scene(const SphParams& p, SceneDev& S, std::string& err) {
    std::memset(&S, 0, sizeof(S));
    if (p.dim != 2 && p.dim != 3) { err = "dim must be 2 or 3"; return false; }
    if (p.kernel < 0 || p.kernel > 3) { err = "unknown kernel"; return false; }
    if (p.solve < 0 || p.solve > 3) { err = "unknown solve variant"; return false; }
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
    const double edge = rc * (1.0 + 1e-9);
    int64_t ncells = 1;
    for (int a = 0; a < 3; ++a) {
        if (a >= p.dim) { S.n[a] = 1; S.lo[a] = 0.0; S.inv_cell[a] = 0.0; continue; }
        if (!(p.domain_hi[a] > p.domain_lo[a])) { err = "domain_hi must exceed domain_lo"; return false; }
        S.lo[a] = p.domain_lo[a];
        int64_t na;
        if (a == 0 && p.periodic_x) {
            const double L = p.domain_hi[0] - p.domain_lo[0];
            na = (int64_t)std::floor(L / edge);
            if (na < 3) { err = "a periodic axis needs at least 3 cells of edge r_cut"; return false; }
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
    S.reinit_interval = p.density_reinitialized_interval;
    S.check_interval = p.check_interval;

    for (int a = 0; a < 3; ++a) S.cell_f[a] = (float)S.cell_d[a];
    S.h_f = (float)p.h;
    S.rc2_f = (float)(rc * rc);
    S.hh001_f = (float)S.hh001;
    S.nu0_f = (float)p.nu_0;
    S.P_bg_f = (float)S.P_bg;
    S.kw_a_f = (float)S.kw_a;
    S.kg_a_f = (float)S.kg_a;
    S.inv_h_f = (float)(1.0 / p.h);
    S.c0_f = (float)p.c_0;
    S.rho0_f = (float)p.rho_0;
    S.inv_cp_f = (float)S.inv_cp_d;
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

struct SphHandle {
    SphParams prm{};
    SceneDev scene{};
    int dim = 2, kernel = 0, mode = 0, thermal = 0, precision = 0;
    int64_t cap = 0, wcap = 0;
    int32_t total_cells = 0;
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
    int64_t* h_pinned_step = nullptr;
    int par = 0;
    int64_t dev_step = INT64_MIN;  // value of the device step counter (host mirror)
    // FP32 launch shape: lanes per particle for continuity, momentum, Shepard; block size
    int tune[4] = {4, 4, 4, 128};
    bool have_fluid = false;
    int64_t steps_done = 0;
    std::string err;
    std::vector<double> hwx, hwn, hwv, hwgap, hwT, hwkappa;
    std::vector<int32_t> hwkind;
    // graph cache: key = (parity, pattern of reinit flags) -> executable graph
    std::map<std::pair<int, std::vector<bool>>, cudaGraphExec_t> graphs;
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

size_t vec_bytes(int dim) { return dim == 2 ? sizeof(double2) : sizeof(double4); }

cudaError_t alloc_sorted(SphHandle* h, SortedState& s) {
    const size_t n = (size_t)h->cap;
    cudaError_t e;
    void* q;
    if ((e = cudaMalloc(&q, n * vec_bytes(h->dim) + 16)) != cudaSuccess) return e;
    h->allocs.push_back(q);
    s.x = q;
    if ((e = cudaMalloc(&q, n * vec_bytes(h->dim) + 16)) != cudaSuccess) return e;
    h->allocs.push_back(q);
    s.v = q;
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

LaunchCtx make_ctx(SphHandle* h) {
    LaunchCtx L{};
    L.stream = h->stream;
    L.dim = h->dim;
    L.kernel = h->kernel;
    L.mode = h->mode;
    L.thermal = h->thermal;
    L.precision = h->precision;
    L.cap = (int32_t)h->cap;
    L.total_cells = h->total_cells;
    L.nscenes = 1;
    L.scenes = h->d_scenes;
    L.st = h->S[h->par];
    L.st2 = h->S[h->par ^ 1];
    L.nx = h->N;
    L.wl = h->W;
    L.sc = h->sc;
    L.sc.n_live = h->nbuf + h->par;
    L.n_next = h->nbuf + (h->par ^ 1);
    L.force_reinit = 0;
    L.block = h->tune[3];
    L.tpp_continuity = h->tune[0];
    L.tpp_momentum = h->tune[1];
    L.tpp_reinit = h->tune[2];
    return L;
}

void launch_physics(int stage, const LaunchCtx& L) {
    if (L.precision == SPH_PRECISION_FP64) launch_physics_fp64(stage, L);
    else launch_physics_fp32(stage, L);
}

// Enqueue one step (no synchronisation).  `reinit` must equal the device-side
// decision for the step (the kernel re-checks it per scene).
void enqueue_step(SphHandle* h, bool reinit) {
    LaunchCtx L = make_ctx(h);
    // count[] was zeroed by the previous placement (or by the upload)
    launch_physics(0, L);
    launch_physics(1, L);
    if (reinit) launch_physics(2, L);
    launch_scan(L, 1);
    launch_place(L);
    h->par ^= 1;
}

int sort_after_upload(SphHandle* h) {
    LaunchCtx L = make_ctx(h);
    SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->total_cells, h->stream));
    launch_hash(L);
    launch_scan(L, 0);
    launch_place(L);
    SPH_CUDA(h, cudaGetLastError());
    h->par ^= 1;
    SPH_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

bool is_step_host(int64_t step, int64_t interval) { return interval > 0 && step % interval == 0; }

}  // namespace

extern "C" {

int32_t sph_version(void) { return SPH_ABI_VERSION; }

int32_t sph_create(const SphParams* params, int64_t fluid_capacity, int64_t wall_capacity, SphHandle** out) {
    if (!params || !out) return fail(nullptr, SPH_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(nullptr, SPH_ERR_NO_DEVICE, "no CUDA device");
    if (fluid_capacity < 1 || fluid_capacity > (int64_t)INT32_MAX / 2 || wall_capacity < 0 ||
        wall_capacity > (int64_t)INT32_MAX / 2)
        return fail(nullptr, SPH_ERR_ARG, "capacity out of range");
    SceneDev S;
    std::string err;
    if (!build_scene(*params, S, err)) return fail(nullptr, SPH_ERR_ARG, err);

    SphHandle* h = new SphHandle();
    h->prm = *params;
    h->scene = S;
    h->dim = params->dim;
    h->kernel = params->kernel;
    h->mode = mode_of(params->solve);
    h->thermal = params->thermal;
    h->precision = params->precision;
    h->cap = fluid_capacity;
    h->wcap = wall_capacity;
    h->total_cells = S.ncells;
    int rc = SPH_OK;
    auto bail = [&](cudaError_t e, const char* what) {
        rc = cuda_fail(nullptr, e, what);
        sph_destroy(h);
        return rc;
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
    for (int b = 0; b < 2; ++b)
        if ((e = alloc_sorted(h, h->S[b])) != cudaSuccess) return bail(e, "sorted state");
    {
        void* q;
        if ((e = cudaMalloc(&q, (size_t)h->cap * vec_bytes(h->dim) + 16)) != cudaSuccess) return bail(e, "next x");
        h->allocs.push_back(q);
        h->N.x = q;
        if ((e = cudaMalloc(&q, (size_t)h->cap * vec_bytes(h->dim) + 16)) != cudaSuccess) return bail(e, "next v");
        h->allocs.push_back(q);
        h->N.v = q;
        if ((e = dalloc(h, &h->N.rho, h->cap)) != cudaSuccess) return bail(e, "next rho");
        if (h->thermal && (e = dalloc(h, &h->N.T, h->cap)) != cudaSuccess) return bail(e, "next T");
    }
    const size_t ncell = (size_t)h->total_cells;
    if ((e = dalloc(h, &h->sc.key, h->cap)) != cudaSuccess) return bail(e, "key");
    if ((e = dalloc(h, &h->sc.slot, h->cap)) != cudaSuccess) return bail(e, "slot");
    if ((e = dalloc(h, &h->sc.tmp, h->cap)) != cudaSuccess) return bail(e, "tmp");
    if ((e = dalloc(h, &h->sc.count, ncell)) != cudaSuccess) return bail(e, "count");
    if ((e = dalloc(h, &h->sc.start, ncell + 1)) != cudaSuccess) return bail(e, "start");
    if ((e = dalloc(h, &h->sc.block_sums, ncell / 4096 + 2)) != cudaSuccess) return bail(e, "block sums");
    if ((e = dalloc(h, &h->sc.status, 1)) != cudaSuccess) return bail(e, "status");
    if ((e = dalloc(h, &h->sc.scene_step, 1)) != cudaSuccess) return bail(e, "scene step");
    if ((e = dalloc(h, &h->nbuf, 2)) != cudaSuccess) return bail(e, "counters");
    if ((e = dalloc(h, &h->W.start, ncell + 1)) != cudaSuccess) return bail(e, "wall start");
    if ((e = dalloc(h, &h->d_scenes, 1)) != cudaSuccess) return bail(e, "scenes");
    if ((e = dalloc(h, &h->d_stat_partials, 3 * 152)) != cudaSuccess) return bail(e, "stats");
    if ((e = dalloc(h, &h->d_stat_out, 4)) != cudaSuccess) return bail(e, "stats");
    if ((e = dalloc(h, &h->d_pair_counts, 2)) != cudaSuccess) return bail(e, "pairs");
    if ((e = cudaMallocHost((void**)&h->h_pinned_step, sizeof(int64_t) * 2)) != cudaSuccess) return bail(e, "pinned");
    if ((e = cudaMemcpyAsync(h->d_scenes, &h->scene, sizeof(SceneDev), cudaMemcpyHostToDevice, h->stream)) !=
        cudaSuccess)
        return bail(e, "scene upload");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return bail(e, "create sync");
    *out = h;
    return SPH_OK;
}

int32_t sph_upload_fluid(SphHandle* h, int64_t n, const double* x, const double* v, const double* rho,
                         const double* p, const double* c, const double* mass, const double* gap, const double* t,
                         const double* kappa, const double* cp) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (n < 0 || n > h->cap) return fail(h, SPH_ERR_GRID_OVERFLOW, "fluid count exceeds the handle capacity");
    if (n > 0 && (!x || !v || !rho || !mass || !gap)) return fail(h, SPH_ERR_ARG, "x, v, rho, mass, gap are required");
    if (n > 0 && h->thermal && (!t || !kappa || !cp))
        return fail(h, SPH_ERR_ARG, "thermal particles need t, kappa and cp");
    const int dim = h->dim;
    const SceneDev& S = h->scene;
    // staging in the device layout
    const size_t vb = vec_bytes(dim);
    std::vector<char> hx(n * vb), hv(n * vb);
    for (int64_t i = 0; i < n; ++i) {
        double* px = (double*)(hx.data() + i * vb);
        double* pv = (double*)(hv.data() + i * vb);
        for (int k = 0; k < dim; ++k) {
            px[k] = x[i * dim + k];
            pv[k] = v[i * dim + k];
        }
        if (dim == 3) px[3] = pv[3] = 0.0;
    }
    std::vector<double> hp(n), hc(n);
    for (int64_t i = 0; i < n; ++i) {
        if (p && c) {
            hp[i] = p[i];
            hc[i] = c[i];
        } else {  // updatePressure! (UpdatePressure.jl:8-16)
            const double rr = rho[i] / S.rho0;
            hp[i] = S.b * (host_powi(rr, S.gamma) - 1.0) + S.p0;
            hc[i] = S.c0 * std::sqrt(host_powi(rr, S.gamma - 1));
        }
    }
    std::vector<int32_t> ids(n), scn(n, 0);
    for (int64_t i = 0; i < n; ++i) ids[i] = (int32_t)i;
    bool uniform = true;
    for (int64_t i = 1; i < n; ++i) uniform &= gap[i] == gap[0];
    h->scene.uniform_gap = uniform ? 1 : 0;

    SortedState& s = h->S[h->par];
    cudaStream_t st = h->stream;
    const int32_t n32 = (int32_t)n;
    SPH_CUDA(h, cudaMemcpyAsync(h->d_scenes, &h->scene, sizeof(SceneDev), cudaMemcpyHostToDevice, st));
    if (n > 0) {
        SPH_CUDA(h, cudaMemcpyAsync(h->N.x, hx.data(), n * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->N.v, hv.data(), n * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->N.rho, rho, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(s.p, hp.data(), n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(s.c, hc.data(), n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(s.m, mass, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(s.gap, gap, n * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(s.id, ids.data(), n * 4, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(s.scene, scn.data(), n * 4, cudaMemcpyHostToDevice, st));
        if (h->thermal) {
            SPH_CUDA(h, cudaMemcpyAsync(h->N.T, t, n * 8, cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(s.kappa, kappa, n * 8, cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(s.cp, cp, n * 8, cudaMemcpyHostToDevice, st));
        }
    }
    SPH_CUDA(h, cudaMemcpyAsync(h->nbuf + h->par, &n32, 4, cudaMemcpyHostToDevice, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));  // host staging buffers die at return
    int rc = sort_after_upload(h);
    if (rc != SPH_OK) return rc;
    h->have_fluid = true;
    return SPH_OK;
}

int32_t sph_upload_walls(SphHandle* h, int32_t kind, int64_t n, const double* x, const double* normal,
                         const double* gap, const double* t, const double* kappa, const double* v) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (kind < SPH_WALL_COMPULSIVE || kind > SPH_WALL_THERMOSTATIC) return fail(h, SPH_ERR_ARG, "unknown wall kind");
    if (n < 0) return fail(h, SPH_ERR_ARG, "negative wall count");
    if (n > 0 && (!x || !normal || !gap)) return fail(h, SPH_ERR_ARG, "x, normal, gap are required");
    if (n > 0 && kind == SPH_WALL_THERMOSTATIC && (!t || !kappa))
        return fail(h, SPH_ERR_ARG, "thermostatic walls need t and kappa");
    if (n > 0 && kind == SPH_WALL_STATIC_VELOCITY && !v) return fail(h, SPH_ERR_ARG, "velocity walls need v");
    const int dim = h->dim;
    const int64_t total = (int64_t)h->hwgap.size() + n;
    if (total > h->wcap) return fail(h, SPH_ERR_GRID_OVERFLOW, "wall count exceeds the handle capacity");
    for (int64_t i = 0; i < n; ++i) {
        for (int k = 0; k < dim; ++k) {
            h->hwx.push_back(x[i * dim + k]);
            h->hwn.push_back(normal[i * dim + k]);
            h->hwv.push_back(kind == SPH_WALL_STATIC_VELOCITY ? v[i * dim + k] : 0.0);
        }
        h->hwgap.push_back(gap[i]);
        h->hwT.push_back(kind == SPH_WALL_THERMOSTATIC ? t[i] : 0.0);
        h->hwkappa.push_back(kind == SPH_WALL_THERMOSTATIC ? kappa[i] : 0.0);
        h->hwkind.push_back(kind);
    }
    // sort all walls by (cell, upload index) and build the wall cell list on the host
    const int64_t nw = total;
    std::vector<int32_t> key(nw);
    for (int64_t w = 0; w < nw; ++w) key[w] = host_cell_key(h->scene, dim, &h->hwx[w * dim]);
    std::vector<int64_t> order(nw);
    for (int64_t w = 0; w < nw; ++w) order[w] = w;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
    std::vector<int32_t> start(h->total_cells + 1, 0);
    for (int64_t w = 0; w < nw; ++w) start[key[w] + 1]++;
    for (int32_t c = 0; c < h->total_cells; ++c) start[c + 1] += start[c];
    const size_t vb = vec_bytes(dim);
    std::vector<char> bx(nw * vb, 0), bn(nw * vb, 0), bv(nw * vb, 0);
    std::vector<double> bg(nw), bT(nw), bk(nw);
    std::vector<int32_t> bkind(nw);
    for (int64_t q = 0; q < nw; ++q) {
        const int64_t w = order[q];
        for (int k = 0; k < dim; ++k) {
            ((double*)(bx.data() + q * vb))[k] = h->hwx[w * dim + k];
            ((double*)(bn.data() + q * vb))[k] = h->hwn[w * dim + k];
            ((double*)(bv.data() + q * vb))[k] = h->hwv[w * dim + k];
        }
        bg[q] = h->hwgap[w];
        bT[q] = h->hwT[w];
        bk[q] = h->hwkappa[w];
        bkind[q] = h->hwkind[w];
    }
    // (re)allocate wall arrays to the full capacity once
    if (!h->W.x) {
        const size_t cap = (size_t)std::max<int64_t>(h->wcap, 1);
        void* q;
        SPH_CUDA(h, cudaMalloc(&q, cap * vb));
        h->allocs.push_back(q);
        h->W.x = q;
        SPH_CUDA(h, cudaMalloc(&q, cap * vb));
        h->allocs.push_back(q);
        h->W.nrm = q;
        SPH_CUDA(h, cudaMalloc(&q, cap * vb));
        h->allocs.push_back(q);
        h->W.v = q;
        SPH_CUDA(h, dalloc(h, &h->W.gap, cap));
        SPH_CUDA(h, dalloc(h, &h->W.T, cap));
        SPH_CUDA(h, dalloc(h, &h->W.kappa, cap));
        SPH_CUDA(h, dalloc(h, &h->W.kind, cap));
    }
    cudaStream_t st = h->stream;
    if (nw > 0) {
        SPH_CUDA(h, cudaMemcpyAsync(h->W.x, bx.data(), nw * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.nrm, bn.data(), nw * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.v, bv.data(), nw * vb, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.gap, bg.data(), nw * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.T, bT.data(), nw * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.kappa, bk.data(), nw * 8, cudaMemcpyHostToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->W.kind, bkind.data(), nw * 4, cudaMemcpyHostToDevice, st));
    }
    SPH_CUDA(h, cudaMemcpyAsync(h->W.start, start.data(), start.size() * 4, cudaMemcpyHostToDevice, st));
    std::vector<float4> fa, fb, fc;
    if (h->precision == SPH_PRECISION_FP32_COMPENSATED) {
        // FP32 wall shadows, positions relative to the origin of the wall's cell
        const SceneDev& S = h->scene;
        if (!h->W.fa) {
            const size_t cap = (size_t)std::max<int64_t>(h->wcap, 1);
            SPH_CUDA(h, dalloc(h, &h->W.fa, cap));
            SPH_CUDA(h, dalloc(h, &h->W.fb, cap));
            SPH_CUDA(h, dalloc(h, &h->W.fc, cap));
        }
        fa.resize(nw);
        fb.resize(nw);
        fc.resize(nw);
        for (int64_t q = 0; q < nw; ++q) {
            const int64_t w = order[q];
            const int32_t k = key[w] - S.cell_off;
            const int32_t cc[3] = {k % S.n[0], (k / S.n[0]) % S.n[1], k / (S.n[0] * S.n[1])};
            float xr[3] = {0.f, 0.f, 0.f}, nr[3] = {0.f, 0.f, 0.f}, vr[3] = {0.f, 0.f, 0.f};
            for (int a = 0; a < dim; ++a) {
                xr[a] = (float)(h->hwx[w * dim + a] - (S.lo[a] + (double)cc[a] * S.cell_d[a]));
                nr[a] = (float)h->hwn[w * dim + a];
                vr[a] = (float)h->hwv[w * dim + a];
            }
            const float g = (float)h->hwgap[w], T = (float)h->hwT[w], kap = (float)h->hwkappa[w];
            const float thermo = h->hwkind[w] == SPH_WALL_THERMOSTATIC ? 1.f : 0.f;
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
        if (nw > 0) {
            SPH_CUDA(h, cudaMemcpyAsync(h->W.fa, fa.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(h->W.fb, fb.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, st));
            SPH_CUDA(h, cudaMemcpyAsync(h->W.fc, fc.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, st));
        }
    }
    SPH_CUDA(h, cudaStreamSynchronize(st));
    h->W.n = nw;
    // the captured graphs hold the old wall state
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SPH_OK;
}

int32_t sph_step_async(SphHandle* h, int64_t first_step, int64_t nsteps) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "sph_step before sph_upload_fluid");
    if (nsteps < 0) return fail(h, SPH_ERR_ARG, "negative step count");
    if (nsteps == 0) return SPH_OK;
    cudaStream_t st = h->stream;
    if (first_step != h->dev_step) {  // the device step counter only needs a reset on a jump
        h->h_pinned_step[0] = first_step;
        SPH_CUDA(h, cudaMemcpyAsync(h->sc.scene_step, h->h_pinned_step, 8, cudaMemcpyHostToDevice, st));
    }
    const int64_t bundle = 10;
    int64_t s = first_step;
    const int64_t end = first_step + nsteps;
    while (s < end) {
        const int64_t nb = std::min(bundle, end - s);
        std::vector<bool> pattern(nb);
        for (int64_t q = 0; q < nb; ++q) pattern[q] = is_step_host(s + q, h->scene.reinit_interval);
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
        s += nb;
    }
    h->dev_step = end;
    h->steps_done += nsteps;
    return SPH_OK;
}

int32_t sph_synchronize(SphHandle* h) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    cudaStream_t st = h->stream;
    SPH_CUDA(h, cudaMemcpyAsync(&h->h_pinned_step[1], h->sc.status, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaMemsetAsync(h->sc.status, 0, 4, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    int32_t status = 0;
    std::memcpy(&status, &h->h_pinned_step[1], 4);
    if ((status & kStatusNonFinite) && h->prm.nan_check)
        return fail(h, SPH_ERR_NAN, "non-finite fluid state (density, velocity or position)");
    return SPH_OK;
}

int32_t sph_step(SphHandle* h, int64_t first_step, int64_t nsteps) {
    int32_t rc = sph_step_async(h, first_step, nsteps);
    if (rc != SPH_OK) return rc;
    return sph_synchronize(h);
}

int32_t sph_download_fluid(SphHandle* h, int64_t capacity, int64_t* n_out, double* x, double* v, double* rho,
                           double* p, double* c, double* mass, double* gap, double* t, double* kappa, double* cp) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!n_out) return fail(h, SPH_ERR_ARG, "n_out is required");
    cudaStream_t st = h->stream;
    int32_t n32 = 0;
    SPH_CUDA(h, cudaMemcpyAsync(&n32, h->nbuf + h->par, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    const int64_t n = h->have_fluid ? n32 : 0;
    *n_out = n;
    if (n > capacity) return fail(h, SPH_ERR_ARG, "caller arrays too small for the live fluid");
    if (n == 0) return SPH_OK;
    const int dim = h->dim;
    const SortedState& s = h->S[h->par];
    const size_t vb = vec_bytes(dim);
    std::vector<int32_t> ids(n);
    SPH_CUDA(h, cudaMemcpyAsync(ids.data(), s.id, n * 4, cudaMemcpyDeviceToHost, st));
    std::vector<char> bx, bv;
    std::vector<double> b1[8];
    const double* srcs[8] = {s.rho, s.p, s.c, s.m, s.gap, s.T, s.kappa, s.cp};
    double* dsts[8] = {rho, p, c, mass, gap, t, kappa, cp};
    if (x) {
        bx.resize(n * vb);
        SPH_CUDA(h, cudaMemcpyAsync(bx.data(), s.x, n * vb, cudaMemcpyDeviceToHost, st));
    }
    if (v) {
        bv.resize(n * vb);
        SPH_CUDA(h, cudaMemcpyAsync(bv.data(), s.v, n * vb, cudaMemcpyDeviceToHost, st));
    }
    for (int f = 0; f < 8; ++f) {
        if (!dsts[f] || !srcs[f]) continue;
        b1[f].resize(n);
        SPH_CUDA(h, cudaMemcpyAsync(b1[f].data(), srcs[f], n * 8, cudaMemcpyDeviceToHost, st));
    }
    SPH_CUDA(h, cudaStreamSynchronize(st));
    // ascending id = the caller's original order with deleted particles removed
    std::vector<int64_t> order(n);
    for (int64_t k = 0; k < n; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ids[a] < ids[b]; });
    for (int64_t q = 0; q < n; ++q) {
        const int64_t k = order[q];
        for (int d = 0; d < dim; ++d) {
            if (x) x[q * dim + d] = ((const double*)(bx.data() + k * vb))[d];
            if (v) v[q * dim + d] = ((const double*)(bv.data() + k * vb))[d];
        }
        for (int f = 0; f < 8; ++f)
            if (dsts[f] && srcs[f]) dsts[f][q] = b1[f][k];
    }
    return SPH_OK;
}

int32_t sph_download_ids(SphHandle* h, int64_t capacity, int64_t* n_out, int64_t* ids_out) {
    if (!h) return fail(nullptr, SPH_ERR_ARG, "null handle");
    if (!n_out) return fail(h, SPH_ERR_ARG, "n_out is required");
    cudaStream_t st = h->stream;
    int32_t n32 = 0;
    SPH_CUDA(h, cudaMemcpyAsync(&n32, h->nbuf + h->par, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    const int64_t n = h->have_fluid ? n32 : 0;
    *n_out = n;
    if (n > capacity) return fail(h, SPH_ERR_ARG, "caller array too small for the live fluid");
    if (n == 0 || !ids_out) return SPH_OK;
    std::vector<int32_t> ids(n);
    SPH_CUDA(h, cudaMemcpyAsync(ids.data(), h->S[h->par].id, n * 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(h, cudaStreamSynchronize(st));
    std::sort(ids.begin(), ids.end());
    for (int64_t k = 0; k < n; ++k) ids_out[k] = ids[k];
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
    out->n_wall = h->W.n;
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

int32_t sph_get_stream(SphHandle* h, void** stream) {
    if (!h || !stream) return fail(h, SPH_ERR_ARG, "null argument");
    *stream = (void*)h->stream;
    return SPH_OK;
}

int32_t sph_time_stages(SphHandle* h, int32_t reps, double* ms_out) {
    if (!h || !ms_out || reps < 1) return fail(h, SPH_ERR_ARG, "bad argument");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    cudaStream_t st = h->stream;
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
    L.force_reinit = 1;
    const int par = h->par;
    auto run = [&](int stage) {
        switch (stage) {
            case SPH_STAGE_CELL_COUNT:
                cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->total_cells, st);
                launch_hash(Lh);
                break;
            case SPH_STAGE_SCAN: launch_scan(Lh, 0); break;
            case SPH_STAGE_SORT: launch_place(Lh); break;
            case SPH_STAGE_CONTINUITY: launch_physics(0, L); break;
            case SPH_STAGE_MOMENTUM: launch_physics(1, L); break;
            case SPH_STAGE_REINIT: launch_physics(2, L); break;
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
            SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->total_cells, st));
            launch_hash(Lh);
        }
    }
    // the momentum stage left arrivals in count[]: the next step expects it zeroed
    SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->total_cells, st));
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
    if (!h || reps < 1) return fail(h, SPH_ERR_ARG, "bad argument");
    if (!h->have_fluid) return fail(h, SPH_ERR_STATE, "no fluid uploaded");
    if (h->precision == SPH_PRECISION_FP32_COMPENSATED) {
        cudaStream_t st = h->stream;
        cudaEvent_t e0, e1;
        SPH_CUDA(h, cudaEventCreate(&e0));
        SPH_CUDA(h, cudaEventCreate(&e1));
        const int par = h->par;
        const size_t nbytes = (size_t)h->cap * 8;
        // p and c are output fields of the last step; the timed continuity launches
        // overwrite them, so park them in the idle sorted buffer meanwhile
        SPH_CUDA(h, cudaMemcpyAsync(h->S[par ^ 1].p, h->S[par].p, nbytes, cudaMemcpyDeviceToDevice, st));
        SPH_CUDA(h, cudaMemcpyAsync(h->S[par ^ 1].c, h->S[par].c, nbytes, cudaMemcpyDeviceToDevice, st));
        const int tpps[4] = {1, 2, 4, 8};
        const int blocks[3] = {64, 128, 256};
        int best_tpp[3] = {4, 4, 4};
        int best_block[3] = {128, 128, 128};
        for (int stage = 0; stage < 3; ++stage) {
            float best = 1e30f;
            for (int tpp : tpps)
                for (int block : blocks) {
                    LaunchCtx L = make_ctx(h);
                    L.force_reinit = 1;
                    L.block = block;
                    L.tpp_continuity = L.tpp_momentum = L.tpp_reinit = tpp;
                    launch_physics(stage, L);  // warm-up
                    SPH_CUDA(h, cudaEventRecord(e0, st));
                    for (int r = 0; r < reps; ++r) launch_physics(stage, L);
                    SPH_CUDA(h, cudaEventRecord(e1, st));
                    SPH_CUDA(h, cudaEventSynchronize(e1));
                    float ms = 0.f;
                    SPH_CUDA(h, cudaEventElapsedTime(&ms, e0, e1));
                    if (ms < best) {
                        best = ms;
                        best_tpp[stage] = tpp;
                        best_block[stage] = block;
                    }
                }
        }
        // one block size for all three stages: the momentum stage's (it dominates)
        h->tune[0] = best_tpp[0];
        h->tune[1] = best_tpp[1];
        h->tune[2] = best_tpp[2];
        h->tune[3] = best_block[1];
        // restore what the timed launches touched: p and c, and the arrivals left in
        // count[]; every other field they wrote is rebuilt by the next step before use
        SPH_CUDA(h, cudaMemsetAsync(h->sc.count, 0, sizeof(int32_t) * (size_t)h->total_cells, st));
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
    for (int k = 0; k < 3; ++k)
        if (shape[k] != 1 && shape[k] != 2 && shape[k] != 4 && shape[k] != 8)
            return fail(h, SPH_ERR_ARG, "lanes per particle must be 1, 2, 4 or 8");
    if (shape[3] < 32 || shape[3] > 1024 || shape[3] % 32 != 0)
        return fail(h, SPH_ERR_ARG, "block size must be a multiple of 32 in [32, 1024]");
    for (int k = 0; k < 4; ++k) h->tune[k] = shape[k];
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return SPH_OK;
}

const char* sph_last_error(const SphHandle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int32_t sph_destroy(SphHandle* h) {
    if (!h) return SPH_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    for (void* p : h->allocs) cudaFree(p);
    if (h->h_pinned_step) cudaFreeHost(h->h_pinned_step);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SPH_OK;
}

}  // extern "C"
