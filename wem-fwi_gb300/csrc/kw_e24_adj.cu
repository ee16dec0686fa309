// Warp-per-row Born adjoint pass kernels for N = 32 x 24 = 768.
#include "kernels_w.cuh"

namespace wg {
template void launch_adj_w<24>(const DevCtx&, const Group*, int, float2*, float2*, float2*, float2*, float2*,
                                float2*, int, cudaStream_t);
template bool adj_reuse_w<24>(const DevCtx&, int);
template int adj_rows_w<24>(const DevCtx&);
}  // namespace wg
