// sph_fp32_3d_shep.cu — the FP32-compensated momentum gather of density re-initialisation steps
// (momentum with the Shepard sums, sph_fp32.cuh) for 3D scenes with cell walks.
#include "sph_fp32.cuh"

namespace sph {

void launch_momentum_fp32_3d_shep(const LaunchCtx& L) { dispatch<3, false, true>(1, L); }

}  // namespace sph
