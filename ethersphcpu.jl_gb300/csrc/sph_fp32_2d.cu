// sph_fp32_2d.cu — the FP32-compensated gathers (sph_fp32.cuh) for 2D scenes with cell
// walks, and the form's entry point.  2D and 3D, cell walks and neighbour-list walks, and
// the momentum gathers of re-initialisation steps (*_shep.cu) are separate translation
// units so they compile in parallel.
#include "sph_fp32.cuh"

namespace sph {

void launch_physics_fp32_2d(int stage, const LaunchCtx& L) { dispatch<2, false, false>(stage, L); }

void launch_physics_fp32(int stage, const LaunchCtx& L) {
    const bool list = L.list_momentum != 0;
    if (stage == 1 && L.shepard) {
        if (L.dim == 2) list ? launch_momentum_fp32_list_2d_shep(L) : launch_momentum_fp32_2d_shep(L);
        else list ? launch_momentum_fp32_list_3d_shep(L) : launch_momentum_fp32_3d_shep(L);
        return;
    }
    if (L.dim == 2) list ? launch_physics_fp32_list_2d(stage, L) : launch_physics_fp32_2d(stage, L);
    else list ? launch_physics_fp32_list_3d(stage, L) : launch_physics_fp32_3d(stage, L);
}

}  // namespace sph
