// Warp-per-row pass kernels instantiated for N = 32 x 8 = 256.
#include "kernels_w.cuh"

namespace wg {
template void launch_pass_w_e<8>(int, const DevCtx&, const Group*, int, const float2*, const float2*, float2*,
                                  float2*, float2*, float2*, float2*, int, cudaStream_t);
template size_t smem_w_e<8>(const DevCtx&, bool);
}  // namespace wg
