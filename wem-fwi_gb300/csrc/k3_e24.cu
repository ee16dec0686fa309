// 3D row and column passes (kernels3d.cuh) for transforms of 32 x 24 = 768 points.
#include "kernels3d.cuh"

namespace wg {
template void launch_k3_rows_e<24>(const Ctx3&, const Pass3&, int, cudaStream_t);
template void launch_k3_cols_e<24>(const Ctx3&, int, int, const float2*, float2*, cudaStream_t);
}  // namespace wg
