// sph_fp32_list_2d_shep.cu — the FP32-compensated momentum gather of density re-initialisation steps
// (momentum with the Shepard sums, sph_fp32.cuh) for 2D scenes with neighbour-list walks.
#include "sph_fp32.cuh"

namespace sph {

void launch_momentum_fp32_list_2d_shep(const LaunchCtx& L) { dispatch<2, true, true>(1, L); }

}  // namespace sph
