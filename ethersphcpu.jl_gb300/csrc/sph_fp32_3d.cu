// sph_fp32_3d.cu — the FP32-compensated gathers (sph_fp32.cuh) for 3D scenes with cell
// walks.
#include "sph_fp32.cuh"

namespace sph {

void launch_physics_fp32_3d(int stage, const LaunchCtx& L) { dispatch<3, false, false>(stage, L); }

}  // namespace sph
