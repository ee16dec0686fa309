// Warp-per-row pass kernels instantiated for N = 32 x 12 = 384.
#include "kernels_w.cuh"

namespace wg {
template void launch_pass_w_e<12>(int, const DevCtx&, const Group*, int, const float2*, const float2*, float2*,
                                  float2*, float2*, float2*, float2*, int, cudaStream_t);
template size_t smem_w_e<12>(const DevCtx&, bool);
}  // namespace wg
