// sph_fp32_2d.cu — the FP32-compensated gathers (sph_fp32.cuh) for 2D scenes, and the
// form's entry point.  2D and 3D are separate translation units so they compile in
// parallel.
#include "sph_fp32.cuh"

namespace sph {

void launch_physics_fp32_2d(int stage, const LaunchCtx& L) { dispatch<2>(stage, L); }

void launch_physics_fp32(int stage, const LaunchCtx& L) {
    if (L.dim == 2) launch_physics_fp32_2d(stage, L);
    else launch_physics_fp32_3d(stage, L);
}

}  // namespace sph
