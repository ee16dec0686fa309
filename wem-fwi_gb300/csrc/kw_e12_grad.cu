// Exact modelling gradient kernels (kernels_wg.cuh) for N = 32 x 12 = 384.
#include "kernels_wg.cuh"

namespace wg {
template void launch_grad_w<12>(const DevCtx&, const Group*, int, const GradArgs&, cudaStream_t);
template bool grad_fits_w<12>(const DevCtx&);
}  // namespace wg
