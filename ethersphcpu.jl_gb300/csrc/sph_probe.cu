// sph_probe.cu — SPH interpolation of fluid fields at arbitrary points, on the device
// state.  Counterpart of kernelValueInterpolation (src/DataIO/VTPToDataFrame.jl:93-142),
// which the reference runs on VTP output for validation (e.g. velocity profiles across a
// Poiseuille channel):
//   kw_i = sum_j W(|x_i - x_j|) m_j / rho_j,   wv_i = sum_j W m_j / rho_j * f_j,
//   f(x_i) = wv_i / kw_i  (none_value where kw_i is not > 0),
// over the fluid particles j within r_cut of point i (CellListMap's neighborlist of the
// points against the particles, :108).  One thread per point walks the step's cell list;
// FP64 throughout, compiled without contraction like the plain step.
#include "sph_kernels.h"
#include "sph_physics.cuh"

namespace sph {

namespace {

template <int DIM>
__device__ __forceinline__ double probe_value(const SortedState& st, int code, int j) {
    switch (code) {
        case SPH_PROBE_DENSITY: return st.rho[j];
        case SPH_PROBE_PRESSURE: return st.p[j];
        case SPH_PROBE_SOUND_SPEED: return st.c[j];
        case SPH_PROBE_VELOCITY_X: return ((const typename VecT<DIM>::T*)st.v)[j].x;
        case SPH_PROBE_VELOCITY_Y: return ((const typename VecT<DIM>::T*)st.v)[j].y;
        case SPH_PROBE_VELOCITY_Z: return comp(((const typename VecT<DIM>::T*)st.v)[j], DIM - 1);
        case SPH_PROBE_TEMPERATURE: return st.T[j];
        default: return st.m[j];
    }
}

template <int DIM, int KK>
__global__ void __launch_bounds__(128) k_probe(const SceneDev* __restrict__ scenes, SortedState st, SortScratch sc,
                                               int64_t np, const double* __restrict__ pts, ProbeFields F,
                                               double none_value, double* __restrict__ out) {
    using V = typename VecT<DIM>::T;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const SceneDev& S = scenes[0];
    const V* __restrict__ x = (const V*)st.x;
    V xi{};
    xi.x = pts[i * DIM];
    xi.y = pts[i * DIM + 1];
    if constexpr (DIM == 3) xi.z = pts[i * DIM + 2];
    int32_t c[3];
    cell_of<DIM>(xi, S, c);
    double kw = 0.0;
    double wv[kMaxProbeFields];
#pragma unroll
    for (int f = 0; f < kMaxProbeFields; ++f) wv[f] = 0.0;
    walk_cells<DIM>(S, sc.start, c, [&](int jb, int je) {
        for (int j = jb; j < je; ++j) {
            double rv[DIM];
            make_rvec<DIM>(xi, x[j], S, rv);
            const double d2 = norm_sq<DIM>(rv);
            if (!(d2 <= S.rc2)) continue;
            const double t = kernel_w<KK>(sqrt(d2), S) * st.m[j] / st.rho[j];
            kw += t;
#pragma unroll
            for (int f = 0; f < kMaxProbeFields; ++f)
                if (f < F.n) wv[f] += t * probe_value<DIM>(st, F.code[f], j);
        }
    });
#pragma unroll
    for (int f = 0; f < kMaxProbeFields; ++f)
        if (f < F.n) out[f * np + i] = kw > 0.0 ? wv[f] / kw : none_value;
}

template <int DIM>
void launch_probe_dim(const LaunchCtx& L, int64_t np, const double* pts, const ProbeFields& F, double none_value,
                      double* out) {
    const int grid = (int)((np + 127) / 128);
    switch (L.kernel) {
        case SPH_KERNEL_CUBIC_SPLINE:
            k_probe<DIM, SPH_KERNEL_CUBIC_SPLINE><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.sc, np, pts, F,
                                                                              none_value, out);
            break;
        case SPH_KERNEL_GAUSSIAN:
            k_probe<DIM, SPH_KERNEL_GAUSSIAN><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.sc, np, pts, F,
                                                                          none_value, out);
            break;
        case SPH_KERNEL_WENDLAND_C2:
            k_probe<DIM, SPH_KERNEL_WENDLAND_C2><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.sc, np, pts, F,
                                                                             none_value, out);
            break;
        default:
            k_probe<DIM, SPH_KERNEL_WENDLAND_C4><<<grid, 128, 0, L.stream>>>(L.scenes, L.st, L.sc, np, pts, F,
                                                                             none_value, out);
    }
}

}  // namespace

void launch_probe(const LaunchCtx& L, int64_t np, const double* pts, const ProbeFields& F, double none_value,
                  double* out) {
    if (np <= 0) return;
    if (L.dim == 2) launch_probe_dim<2>(L, np, pts, F, none_value, out);
    else launch_probe_dim<3>(L, np, pts, F, none_value, out);
}

}  // namespace sph
