// Subsurface-offset Born sweep kernels (kernels_off.cuh) for N = 32 x 24 = 768.
#include "kernels_off.cuh"

namespace wg {
template void launch_off_w<24>(int, const OffCtx&, const OffGroup*, int, int, float2*, float2*, cudaStream_t);
template size_t off_smem_w<24>(int);
}  // namespace wg
