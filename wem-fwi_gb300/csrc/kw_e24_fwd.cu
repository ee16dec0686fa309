// Warp-per-row Born forward pass kernels for N = 32 x 24 = 768.
#include "kernels_w.cuh"

namespace wg {
template void launch_fwd_w<24>(const DevCtx&, const Group*, int, const float2*, const float2*, float2*, float2*,
                                float2*, cudaStream_t);
}  // namespace wg
