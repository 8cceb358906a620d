// sph_fp32_list_3d.cu — the FP32-compensated continuity and momentum gathers
// (sph_fp32.cuh) for 3D scenes, with the neighbour list.
#include "sph_fp32.cuh"

namespace sph {

void launch_physics_fp32_list_3d(int stage, const LaunchCtx& L) { dispatch<3, true, false>(stage, L); }

}  // namespace sph
