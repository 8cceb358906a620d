// sph_fp32_list_2d.cu — the FP32-compensated continuity and momentum gathers
// (sph_fp32.cuh) for 2D scenes, with the neighbour list: continuity records it,
// momentum reads it.
#include "sph_fp32.cuh"

namespace sph {

void launch_physics_fp32_list_2d(int stage, const LaunchCtx& L) { dispatch<2, true, false>(stage, L); }

}  // namespace sph
