// sph_buffer.cu — inlet/outlet buffer particles between the gathers and the sort
// (FluidInletOutletWallSolve.jl:160-262), compiled without contraction like the plain
// step so that every transfer decision matches the CPU restatement.
//
// Per step, after K4-K6 (which read the buffers as neighbours):
//   k_buf_move    buffer particles move (x += v dt, :171-186 with dv = 0); an inlet
//                 particle beyond the inlet plane is copied into the fluid (appended at
//                 the end of the unsorted fluid arrays with a new id and counted for the
//                 fluid's sort, :227-231) and shifted back (:251-255); an outlet particle
//                 beyond the drop plane is removed (:243-249).
//   k_buf_append  fluid particles that K5 marked beyond the outlet plane (and removed
//                 from the fluid) become outlet particles, with their end-of-step
//                 state (:232-236).
//   scan, k_buf_fill, k_buf_place: counting sort of the buffers by (cell, order) into
//                 the other buffer array set, as the fluid's (cell, id) sort.
#include "sph_kernels.h"
#include "sph_physics.cuh"

namespace sph {

namespace {

template <int DIM>
__global__ void k_buf_move(const SceneDev* __restrict__ scenes, BufferState cur, BufferScratch bs, BufferRules br,
                           SortedState st, NextState nx, SortScratch sc, int32_t fcap) {
    using V = typename VecT<DIM>::T;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs.cap || b >= *cur.n) return;
    const SceneDev& S = scenes[0];
    const int64_t step = sc.scene_step[0];
    const V x = ((const V*)cur.x)[b];
    const V v = ((const V*)cur.v)[b];
    double xn[DIM];
    xn[0] = x.x + v.x * S.dt;
    xn[1] = x.y + v.y * S.dt;
    if (DIM == 3) xn[DIM - 1] = comp(x, DIM - 1) + comp(v, DIM - 1) * S.dt;
    const int64_t order = cur.order[b];
    if (!(order & kOutletBit)) {
        if (beyond_plane<DIM>(br.in_n, br.in_d, xn)) {  // into the calculation domain: a fluid copy
            const int32_t a = atomicAdd(sc.n_live, 1);
            if (a < fcap) {
                V xo = x, vo = v;
                xo.x = xn[0];
                xo.y = xn[1];
                if constexpr (DIM == 3) xo.z = xn[2];
                ((V*)nx.x)[a] = xo;
                ((V*)nx.v)[a] = vo;
                nx.rho[a] = cur.rho[b];
                st.p[a] = cur.p[b];
                st.c[a] = cur.c[b];
                st.m[a] = cur.m[b];
                st.gap[a] = cur.gap[b];
                st.id[a] = (int32_t)(br.id_base + (step - br.first_step) * br.n_inlet + order);
                st.scene[a] = 0;
                cell_arrival(sc, a, cell_key<DIM>(xo, S));
            } else {
                atomicOr(sc.status, kStatusBufferOverflow);
            }
#pragma unroll
            for (int k = 0; k < DIM; ++k) xn[k] += br.in_shift[k];
        }
    } else if (beyond_plane<DIM>(br.drop_n, br.drop_d, xn)) {  // out of the outlet: removed
        bs.key[b] = kDeadKey;
        return;
    }
    V xo = x;
    xo.x = xn[0];
    xo.y = xn[1];
    if constexpr (DIM == 3) xo.z = xn[2];
    ((V*)cur.x)[b] = xo;
    const int32_t key = cell_key<DIM>(xo, S);
    bs.key[b] = key;
    bs.slot[b] = atomicAdd(bs.count + key, 1);
}

template <int DIM>
__global__ void k_buf_append(const SceneDev* __restrict__ scenes, BufferState cur, BufferScratch bs, BufferRules br,
                             SortedState st, NextState nx, SortScratch sc) {
    using V = typename VecT<DIM>::T;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= bs.cap || k >= *bs.npend) return;
    const SceneDev& S = scenes[0];
    const int64_t step = sc.scene_step[0];
    const int32_t i = bs.pend[k];
    const int32_t b = atomicAdd((int32_t*)cur.n, 1);
    if (b >= bs.cap) {
        atomicOr(sc.status, kStatusBufferOverflow);
        return;
    }
    const V x = ((const V*)nx.x)[i];
    ((V*)cur.x)[b] = x;
    ((V*)cur.v)[b] = ((const V*)nx.v)[i];
    cur.rho[b] = nx.rho[i];
    cur.p[b] = st.p[i];
    cur.c[b] = st.c[i];
    cur.m[b] = st.m[i];
    cur.gap[b] = st.gap[i];
    cur.order[b] = kOutletBit | ((step - br.first_step + 1) << 32) | (int64_t)st.id[i];
    const int32_t key = cell_key<DIM>(x, S);
    bs.key[b] = key;
    bs.slot[b] = atomicAdd(bs.count + key, 1);
}

__global__ void k_buf_fill(BufferState cur, BufferScratch bs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b == 0) *bs.npend = 0;  // consumed by k_buf_append
    if (b >= bs.cap || b >= *cur.n) return;
    const int32_t key = bs.key[b];
    if (key == kDeadKey) return;
    bs.tmp[bs.start[key] + bs.slot[b]] = cur.order[b];
}

template <int DIM>
__global__ void k_buf_place(BufferState cur, BufferState nxt, BufferScratch bs, int32_t ncells) {
    using V = typename VecT<DIM>::T;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    for (int k = b; k < ncells; k += gridDim.x * blockDim.x) bs.count[k] = 0;
    if (b >= bs.cap || b >= *cur.n) return;
    const int32_t key = bs.key[b];
    if (key == kDeadKey) return;
    const int32_t s0 = bs.start[key], s1 = bs.start[key + 1];
    const int64_t mine = cur.order[b];
    int32_t rank = 0;
    for (int32_t t = s0; t < s1; ++t) rank += bs.tmp[t] < mine;
    const int32_t d = s0 + rank;
    ((V*)nxt.x)[d] = ((const V*)cur.x)[b];
    ((V*)nxt.v)[d] = ((const V*)cur.v)[b];
    nxt.rho[d] = cur.rho[b];
    nxt.p[d] = cur.p[b];
    nxt.c[d] = cur.c[b];
    nxt.m[d] = cur.m[b];
    nxt.gap[d] = cur.gap[b];
    nxt.order[d] = mine;
}

template <int DIM>
void launch_buffers_dim(const LaunchCtx& L) {
    const int grid = (L.bs.cap + 127) / 128;
    k_buf_move<DIM><<<grid, 128, 0, L.stream>>>(L.scenes, L.bf, L.bs, L.br, L.st, L.nx, L.sc, L.cap);
    k_buf_append<DIM><<<grid, 128, 0, L.stream>>>(L.scenes, L.bf, L.bs, L.br, L.st, L.nx, L.sc);
    LaunchCtx B = L;  // the buffers' scan: their counts into the next step's cell starts
    B.sc.count = L.bs.count;
    B.sc.start = L.bs.start;
    B.sc.block_sums = L.bs.block_sums;
    B.n_next = L.bn_next;
    launch_scan(B, 0);
    k_buf_fill<<<grid, 128, 0, L.stream>>>(L.bf, L.bs);
    k_buf_place<DIM><<<grid, 128, 0, L.stream>>>(L.bf, L.bf2, L.bs, L.total_cells);
}

}  // namespace

void launch_buffers(const LaunchCtx& L) {
    if (!L.bf.n) return;
    if (L.dim == 2) launch_buffers_dim<2>(L);
    else launch_buffers_dim<3>(L);
}

}  // namespace sph
