// Element-wise operators of the row-level API (include/wemgpu.h, wem_*
// and wemop_* per-operator entry points), the GPU side of the reference's
// py_wem_ops classes IC, Phshift, SplitStep, Reflect and Injection
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

// Injection forward (Injection.cpp:8-19, 52-62): data[z][x] = (or +=) the sum
// over the points i at depth z with |x - tap - ix[i]| <= ng of
// g[x - tap - ix[i] + ng] m_i, m_i = model[off0 + i stride]; one thread per
// data element, the points in order
__global__ void k_inject_fwd(const int* __restrict__ iz, const int* __restrict__ ix, int npt,
                             const float* __restrict__ g, int ng, int tap, int nx, size_t total,
                             const float2* __restrict__ model, size_t off0, size_t stride, float2* data, int add) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(t / nx), x = (int)(t % nx);
    float2 acc = make_float2(0.f, 0.f);
    for (int i = 0; i < npt; ++i) {
      const int ig = x - tap - ix[i];
      if (iz[i] != z || ig < -ng || ig > ng) continue;
      const float w = g[ig + ng];
      const float2 m = model[off0 + (size_t)i * stride];
      // the reference's roundings: the product, then the sum
      acc = make_float2(__fadd_rn(acc.x, __fmul_rn(w, m.x)), __fadd_rn(acc.y, __fmul_rn(w, m.y)));
    }
    data[t] = add ? make_float2(data[t].x + acc.x, data[t].y + acc.y) : acc;
  }
}

// the gathered value of point i (Injection.cpp:21-33, 64-75): the sum over
// its window of g[ig + ng] data[iz[i]][ix[i] + ig + tap], inside the row
__device__ __forceinline__ float2 inject_gather(const int* iz, const int* ix, int i, const float* g, int ng,
                                                int tap, int nx, const float2* data) {
  float2 acc = make_float2(0.f, 0.f);
  for (int ig = -ng; ig <= ng; ++ig) {
    const int off = ix[i] + ig + tap;
    if (off < 0 || off >= nx) continue;
    const float w = g[ig + ng];
    const float2 d = data[(size_t)iz[i] * nx + off];
    acc = make_float2(__fadd_rn(acc.x, __fmul_rn(w, d.x)), __fadd_rn(acc.y, __fmul_rn(w, d.y)));
  }
  return acc;
}

// Injection adjoint, one value per point: model[off0 + i stride] +=
// gather(i) (the model was cleared beforehand unless adding)
__global__ void k_inject_adj_points(const int* __restrict__ iz, const int* __restrict__ ix, int npt,
                                    const float* __restrict__ g, int ng, int tap, int nx,
                                    const float2* __restrict__ data, float2* model, size_t off0, size_t stride) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npt; i += gridDim.x * blockDim.x) {
    const float2 v = inject_gather(iz, ix, i, g, ng, tap, nx, data);
    float2& m = model[off0 + (size_t)i * stride];
    m = make_float2(m.x + v.x, m.y + v.y);
  }
}

// Injection adjoint into one model sample (the 1D form): model[off0] += the
// sum over every point of gather(i); one CTA of 256 threads, each summing
// the points i = t (mod 256) in order, then a fixed tree
__global__ void k_inject_adj_sum(const int* __restrict__ iz, const int* __restrict__ ix, int npt,
                                 const float* __restrict__ g, int ng, int tap, int nx,
                                 const float2* __restrict__ data, float2* model, size_t off0) {
  __shared__ float2 part[256];
  float2 acc = make_float2(0.f, 0.f);
  for (int i = threadIdx.x; i < npt; i += 256) {
    const float2 v = inject_gather(iz, ix, i, g, ng, tap, nx, data);
    acc = make_float2(acc.x + v.x, acc.y + v.y);
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      part[threadIdx.x] = make_float2(part[threadIdx.x].x + part[threadIdx.x + w].x,
                                      part[threadIdx.x].y + part[threadIdx.x + w].y);
    __syncthreads();
  }
  if (threadIdx.x == 0) model[off0] = make_float2(model[off0].x + part[0].x, model[off0].y + part[0].y);
}

}  // namespace

void launch_inject(const int* iz, const int* ix, int npt, const float* g, int ng, int tap, int nx, int nz, int adj,
                   float2* model, size_t off0, size_t stride, float2* data, int add, cudaStream_t st) {
  if (!adj) {
    const size_t total = (size_t)nx * nz;
    if (!total) return;
    k_inject_fwd<<<blocks_for(total), 256, 0, st>>>(iz, ix, npt, g, ng, tap, nx, total, model, off0, stride, data,
                                                    add);
  } else if (stride == 0) {
    k_inject_adj_sum<<<1, 256, 0, st>>>(iz, ix, npt, g, ng, tap, nx, data, model, off0);
  } else {
    if (!npt) return;
    k_inject_adj_points<<<blocks_for((size_t)npt), 256, 0, st>>>(iz, ix, npt, g, ng, tap, nx, data, model, off0,
                                                                 stride);
  }
  note_launch();
}

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
