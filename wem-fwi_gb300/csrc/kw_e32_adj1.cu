// Warp-per-row Born adjoint with one-row CTAs for N = 32 x 32 = 1024.
#include "kernels_w.cuh"

namespace wg {
template void launch_adj2_one<32>(const DevCtx&, const Group*, int, float2*, float2*, float2*, float2*, float2*,
                                   float2*, int, cudaStream_t);
}  // namespace wg
