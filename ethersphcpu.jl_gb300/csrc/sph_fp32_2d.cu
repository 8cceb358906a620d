// sph_fp32_2d.cu — the FP32-compensated gathers (sph_fp32.cuh) for 2D scenes with cell
// walks, and the form's entry point.  2D and 3D, cell walks and neighbour-list walks are
// separate translation units so they compile in parallel.
#include "sph_fp32.cuh"

namespace sph {

void launch_physics_fp32_2d(int stage, const LaunchCtx& L) { dispatch<2, false>(stage, L); }

void launch_physics_fp32(int stage, const LaunchCtx& L) {
    // the Shepard gather always walks the cells (it also counts coincident particles,
    // which the list leaves out)
    const bool list = L.list_momentum && stage != 2;
    if (L.dim == 2) list ? launch_physics_fp32_list_2d(stage, L) : launch_physics_fp32_2d(stage, L);
    else list ? launch_physics_fp32_list_3d(stage, L) : launch_physics_fp32_3d(stage, L);
}

}  // namespace sph
