// Element-wise operators of the row-level API (include/wemgpu.h, wem_*
// and wemop_* per-operator entry points), the GPU side of the reference's
// py_wem_ops classes IC, Phshift, SplitStep and Reflect
// (propagator/src/python/py_wem_ops.cpp:24-208).  Each thread owns output
// elements, so results do not depend on the launch shape.
#include <cuda_runtime.h>

#include "kernels.h"

namespace wg {
namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // conj(a) b
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

int blocks_for(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? (b ? b : 1) : 152 * 32);
}

// out[r][k] = f[k] x in[r][k] (conj(f) with conj); with add the product is
// added, otherwise assigned
__global__ void k_diag_rows(const float2* __restrict__ in, const float2* __restrict__ f, float2* out, int n,
                            size_t total, int conj, int add) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const float2 a = f[i % n];
    const float2 v = conj ? cmulc(a, in[i]) : cmul(a, in[i]);
    out[i] = add ? make_float2(out[i].x + v.x, out[i].y + v.y) : v;
  }
}

// SplitStep on the listed points of each row (SplitStep.cpp:5-29): the
// points take m exp(-i w dz (s - s_ref) / sqrt(s_ref)) (adjoint:
// exp(+i w dz conj(...))); every other point is left as it is.  Evaluated
// in double, rounded once.
__global__ void k_splitstep(const float2* __restrict__ srow, const int* __restrict__ loc, int nloc, int nx,
                            int nrow, double wdz, double sr, double si, int adj, const float2* __restrict__ in,
                            float2* out) {
  const size_t total = (size_t)nrow * nloc;
  // 1 / sqrt(s_ref), principal root
  const double mod = sqrt(sr * sr + si * si);
  double qr = sqrt(0.5 * (mod + sr)), qi = sqrt(0.5 * (mod - sr));
  if (si < 0) qi = -qi;
  const double qn = qr * qr + qi * qi;
  const double ir = qr / qn, ii = -qi / qn;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / nloc);
    const int x = loc[t % nloc];
    const float2 s = srow[x];
    // (s - s_ref) / sqrt(s_ref)
    const double dr = s.x - sr, di = s.y - si;
    const double ur = dr * ir - di * ii, ui = dr * ii + di * ir;
    // forward -i wdz u, adjoint +i wdz conj(u): both have real part wdz ui
    const double er = wdz * ui;
    const double ph = adj ? wdz * ur : -wdz * ur;
    const double e = exp(er);
    const float2 fac = make_float2((float)(e * cos(ph)), (float)(e * sin(ph)));
    const size_t i = (size_t)r * nx + x;
    out[i] = cmul(in[i], fac);
  }
}

}  // namespace

void launch_diag_rows(const float2* in, const float2* f, float2* out, int n, int nrow, int conj, int add,
                      cudaStream_t st) {
  const size_t total = (size_t)n * nrow;
  if (!total) return;
  k_diag_rows<<<blocks_for(total), 256, 0, st>>>(in, f, out, n, total, conj, add);
  note_launch();
}

void launch_splitstep(const float2* srow, const int* loc, int nloc, int nx, int nrow, double wdz, double sr,
                      double si, int adj, const float2* in, float2* out, cudaStream_t st) {
  const size_t total = (size_t)nrow * nloc;
  if (!total) return;
  k_splitstep<<<blocks_for(total), 256, 0, st>>>(srow, loc, nloc, nx, nrow, wdz, sr, si, adj, in, out);
  note_launch();
}

}  // namespace wg
