// Warp-per-row Born adjoint pass kernels for N = 32 x 12 = 384.
#include "kernels_w.cuh"

namespace wg {
// the one-row kernels are built in kw_e12_adj1.cu
extern template void launch_adj2_one<12>(const DevCtx&, const Group*, int, float2*, float2*, float2*, float2*,
                                          float2*, float2*, int, cudaStream_t);
template void launch_adj_w<12>(const DevCtx&, const Group*, int, float2*, float2*, float2*, float2*, float2*,
                                float2*, int, cudaStream_t);
template bool adj_reuse_w<12>(const DevCtx&, int);
template bool adj_split_w<12>(const DevCtx&);
template int adj_rows_w<12>(const DevCtx&);
}  // namespace wg
