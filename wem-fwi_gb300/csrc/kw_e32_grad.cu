// Exact modelling gradient kernels (kernels_wg.cuh) for N = 32 x 32 = 1024.
#include "kernels_wg.cuh"

namespace wg {
template void launch_grad_w<32>(const DevCtx&, const Group*, int, const GradArgs&, cudaStream_t);
template bool grad_fits_w<32>(const DevCtx&);
}  // namespace wg
