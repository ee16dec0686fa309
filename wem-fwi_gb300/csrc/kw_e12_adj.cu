// Warp-per-row Born adjoint pass kernels for N = 32 x 12 = 384.
#include "kernels_w.cuh"

namespace wg {
template void launch_adj_w<12>(const DevCtx&, const Group*, int, float2*, float2*, float2*, float2*, float2*,
                                float2*, int, cudaStream_t);
template bool adj_reuse_w<12>(const DevCtx&, int);
template int adj_rows_w<12>(const DevCtx&);
}  // namespace wg
