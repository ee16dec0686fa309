// Warp-per-row WEM pass kernels for N = 32 x 16 = 512.
#include "kernels_w.cuh"

namespace wg {
template void launch_wem_w<16>(const DevCtx&, const Group*, int, float2*, float2*, cudaStream_t);
template size_t smem_w_e<16>(const DevCtx&, bool);
template int wem_rows_w<16>(const DevCtx&);
}  // namespace wg
