// sph_diag.cu — diagnostics of the per-step cell list: the cell key of every sorted
// particle, and the fluid neighbours each particle's gathers accept.
//
// They expose what the reference's neighbour search produces inside a step
// (CellListMap.update!/neighborlist! + findNeighbours!, FluidWallSolve.jl:21-35,
// Neighbour.jl:88-128) so that it can be compared particle by particle with a CPU
// restatement: the key is the one the step's sort uses, and the neighbour test is the
// one the gathers of the handle's form use (FP64: d^2 <= r_cut^2 in FP64 with the
// products and sums rounded one by one, as k_momentum_fp64; FP32-compensated: the same
// test in FP32 on cell-relative positions, as k_continuity_f32 records the neighbour
// list, stencil pruning included).
#include "sph_fp32.cuh"

namespace sph {

namespace {

template <int DIM>
__global__ void k_cell_keys(const SceneDev* __restrict__ scenes, SortedState st, int32_t b, int32_t e,
                            int32_t* __restrict__ keys) {
    using V = typename VecT<DIM>::T;
    const int i = b + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= e) return;
    const SceneDev& S = scenes[st.scene[i]];
    keys[i - b] = cell_key<DIM>(((const V*)st.x)[i], S) - S.cell_off;
}

// counts != null: the number of accepted neighbours of sorted particle i; ids != null:
// their ids (upload indices) from ids[rows[i - b]] on, in walk order.
template <int DIM>
__global__ void k_neighbours_fp64(const SceneDev* __restrict__ scenes, SortedState st, const int32_t* start,
                                  int32_t b, int32_t e, int32_t* __restrict__ counts, const int64_t* __restrict__ rows,
                                  int32_t* __restrict__ ids) {
    using V = typename VecT<DIM>::T;
    const int i = b + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= e) return;
    const SceneDev& S = scenes[st.scene[i]];
    const V* __restrict__ x = (const V*)st.x;
    const V xi = x[i];
    int32_t c[3];
    cell_of<DIM>(xi, S, c);
    int32_t* out = ids ? ids + rows[i - b] : nullptr;
    int32_t cnt = 0;
    float xd[3];
    cell_units<DIM>(xi, S, c, xd);
    walk_cells_pruned<DIM>(S, start, c, xd, [&](int jb, int je) {
        for (int j = jb; j < je; ++j) {
            if (j == i) continue;
            double rv[DIM];
            make_rvec<DIM>(xi, x[j], S, rv);
            if (!(norm_sq<DIM>(rv) <= S.rc2)) continue;
            if (out) out[cnt] = st.id[j];
            ++cnt;
        }
    });
    if (counts) counts[i - b] = cnt;
}

template <int DIM>
__global__ void k_neighbours_f32(const SceneDev* __restrict__ scenes, SortedState st, const int32_t* start,
                                 int32_t b, int32_t e, int32_t* __restrict__ counts, const int64_t* __restrict__ rows,
                                 int32_t* __restrict__ ids) {
    const int i = b + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= e) return;
    const SceneDev& S = scenes[st.scene[i]];
    const float4 ai = st.fa[i];
    const float xi[3] = {ai.x, ai.y, DIM == 3 ? ai.z : 0.f};
    int32_t c[3];
    decode_cell(st.cell[i], S, c);
    int32_t* out = ids ? ids + rows[i - b] : nullptr;
    int32_t cnt = 0;
    auto load = [&](int j) { return st.fa[j]; };
    walk<DIM, 1, false>(S, start, c, xi, 0, load, [&](int j, const float4& aj, float ox, float oy, float oz, int) {
        if (j == i) return;
        const float rx = xi[0] - ox - aj.x, ry = xi[1] - oy - aj.y;
        const float rz = DIM == 3 ? xi[2] - oz - aj.z : 0.f;
        if (!(dist2(rx, ry, rz) <= S.rc2_f)) return;
        if (out) out[cnt] = st.id[j];
        ++cnt;
    });
    if (counts) counts[i - b] = cnt;
}

}  // namespace

void launch_cell_keys(const LaunchCtx& L, int32_t b, int32_t e, int32_t* keys) {
    const int n = e - b, block = 128, grid = (n + block - 1) / block;
    if (n <= 0) return;
    if (L.dim == 2) k_cell_keys<2><<<grid, block, 0, L.stream>>>(L.scenes, L.st, b, e, keys);
    else k_cell_keys<3><<<grid, block, 0, L.stream>>>(L.scenes, L.st, b, e, keys);
}

void launch_neighbours(const LaunchCtx& L, int32_t b, int32_t e, int32_t* counts, const int64_t* rows,
                       int32_t* ids) {
    const int n = e - b, block = 128, grid = (n + block - 1) / block;
    if (n <= 0) return;
    const bool f32 = L.precision == SPH_PRECISION_FP32_COMPENSATED;
    if (L.dim == 2) {
        if (f32) k_neighbours_f32<2><<<grid, block, 0, L.stream>>>(L.scenes, L.st, L.sc.start, b, e, counts, rows, ids);
        else k_neighbours_fp64<2><<<grid, block, 0, L.stream>>>(L.scenes, L.st, L.sc.start, b, e, counts, rows, ids);
    } else {
        if (f32) k_neighbours_f32<3><<<grid, block, 0, L.stream>>>(L.scenes, L.st, L.sc.start, b, e, counts, rows, ids);
        else k_neighbours_fp64<3><<<grid, block, 0, L.stream>>>(L.scenes, L.st, L.sc.start, b, e, counts, rows, ids);
    }
}

}  // namespace sph
