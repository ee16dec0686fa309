// Subsurface-offset extended imaging condition: the lag sums of the
// extended reflectivity Born (no reference counterpart; at one lag these are
// IC::forward / IC::adjoint, propagator/src/ic.cpp:5-29, as BornRefl uses
// them, ext_born_refl.cpp:45,98), and the dispatch of the sweep kernels.
//
// Lags l = -hm .. hm (hm = (nh - 1) / 2) are horizontal grid offsets; the
// model r is [nh][nz][nx] with r_l at index l + hm.  On a shot's aperture
// (padded coordinates x in [0, nxg), model cells [pad, pad + w)):
//   forward  sc(x) = sum_l r_l(x - l) bg(x - 2 l)
//   adjoint  I_l(y) += conj(bg(y - l)) a(y + l)      (y a model cell)
// with r zero off the aperture's model cells and bg, a zero off [0, nxg), so
// the two are exact transposes.  Both run in fixed order (no atomics): the
// image sums shots in order and a shot's frequencies in order.
#include <algorithm>

#include "fft.cuh"
#include "kernels.h"
#include "phase.cuh"

namespace wg {

template <int E>
void launch_off_w(int, const OffCtx&, const OffGroup*, int, int, float2*, float2*, cudaStream_t);
template <int E>
size_t off_smem_w(int);

namespace {

constexpr int kSrcChunk = 256;  // aperture points per CTA of the source kernel
constexpr int kSrcBatch = 8;    // frequencies staged per barrier in the source kernel
constexpr int kImgChunk = 128;  // model columns per CTA of the image kernel
constexpr int kImgBatch = 16;   // frequencies staged per barrier in the image kernel

// grid (nz, ns, chunks); thread t: padded aperture point x = chunk * 256 + t.
// The lag values r_l(x - l) stay in registers for all frequencies of the
// shot; the bg segments [x_lo - 2 hm, x_hi + 2 hm] of kSrcBatch frequencies
// go through shared memory per barrier, so each thread has that many loads
// in flight.
template <int NL>
__global__ void __launch_bounds__(kSrcChunk) k_off_source(OffCtx c, const float2* model, const float2* bg,
                                                          float2* sc) {
  extern __shared__ float2 seg[];  // [kSrcBatch][len]
  const int z = blockIdx.x, s = blockIdx.y;
  const int x0 = c.x0[s], w = c.w[s], pad = c.pad, nxg = w + 2 * pad, hm = (c.nh - 1) / 2;
  const int xlo = blockIdx.z * kSrcChunk;
  if (xlo >= nxg) return;
  const int x = xlo + threadIdx.x;
  const bool on = x < nxg;
  float2 rv[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    rv[k] = make_float2(0.f, 0.f);
    const int l = k - hm, y = x - l;
    if (k < c.nh && on && y >= pad && y < pad + w) rv[k] = model[((size_t)k * c.nz + z) * c.nx + x0 + y - pad];
  }
  const int lo = xlo - 2 * hm, len = kSrcChunk + 4 * hm;
  const size_t r0 = (size_t)c.rowbase[s];
  for (int f0 = 0; f0 < c.nfreq; f0 += kSrcBatch) {
    const int nb = min(kSrcBatch, c.nfreq - f0);
    __syncthreads();
    for (int i = threadIdx.x; i < nb * len; i += blockDim.x) {
      const int b = i / len, xb = lo + i % len;
      const float2* src = bg + c.roff[r0 + f0 + b] + (size_t)z * nxg;
      seg[i] = (xb >= 0 && xb < nxg) ? src[xb] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (!on) continue;
    for (int b = 0; b < nb; ++b) {
      const float2* g = seg + (size_t)b * len + (x - lo);
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < NL; ++k)
        if (k < c.nh) acc = c_fma(acc, rv[k], g[-2 * (k - hm)]);
      sc[c.roff[r0 + f0 + b] + (size_t)z * nxg + x] = acc;
    }
  }
}

// grid (nz, chunks of model columns); thread t: model column m.  For every
// shot whose aperture meets the chunk (in order) and each of its
// frequencies (in order, kImgBatch per barrier), the bg and a segments of the
// chunk (halo hm) go through shared memory and every lag accumulates in a
// register.
template <int NL>
__global__ void __launch_bounds__(kImgChunk) k_off_image(OffCtx c, const float2* bg, const float2* a, float2* img,
                                                         int add) {
  extern __shared__ float2 sh[];
  const int z = blockIdx.x, hm = (c.nh - 1) / 2, pad = c.pad;
  const int m0 = blockIdx.y * kImgChunk, m = m0 + threadIdx.x;
  const int len = kImgChunk + 2 * hm;
  float2* sbg = sh;                                  // [kImgBatch][len]
  float2* sa = sh + (size_t)kImgBatch * len;         // [kImgBatch][len]
  float2 acc[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) acc[k] = make_float2(0.f, 0.f);
  for (int s = 0; s < c.ns; ++s) {
    const int x0 = c.x0[s], w = c.w[s], nxg = w + 2 * pad;
    if (x0 >= m0 + kImgChunk || x0 + w <= m0) continue;
    const bool on = m < c.nx && m >= x0 && m < x0 + w;
    const int y = m - x0 + pad;                      // padded aperture point of column m
    const int lo = m0 - x0 + pad - hm;               // first staged point
    for (int f0 = 0; f0 < c.nfreq; f0 += kImgBatch) {
      const int nb = min(kImgBatch, c.nfreq - f0);
      __syncthreads();
      for (int i = threadIdx.x; i < nb * len; i += blockDim.x) {
        const int b = i / len, xi = lo + i % len;
        const size_t o = c.roff[(size_t)c.rowbase[s] + f0 + b] + (size_t)z * nxg;
        const bool in = xi >= 0 && xi < nxg;
        sbg[i] = in ? bg[o + xi] : make_float2(0.f, 0.f);
        sa[i] = in ? a[o + xi] : make_float2(0.f, 0.f);
      }
      __syncthreads();
      if (!on) continue;
      for (int b = 0; b < nb; ++b) {
        const float2* gb = sbg + (size_t)b * len + (y - lo);
        const float2* ga = sa + (size_t)b * len + (y - lo);
#pragma unroll
        for (int k = 0; k < NL; ++k)
          if (k < c.nh) acc[k] = c_fmac(acc[k], ga[k - hm], gb[-(k - hm)]);  // + conj(bg(y - l)) a(y + l)
      }
    }
  }
  if (m >= c.nx) return;
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    if (k >= c.nh) break;
    float2* o = img + ((size_t)k * c.nz + z) * c.nx + m;
    *o = add ? c_add(*o, acc[k]) : acc[k];
  }
}

// grid (nz, rows): the phase-shift factors of row `row0 + blockIdx.y` at
// depth z over the k grid of its length, and its split-step factors (taper
// over N included) over the aperture; the formulas of the table builders
// (phase.cuh), from the aperture's reference slowness and split-step
// exponents
__global__ void k_off_tables(OffCtx c, int row0, int N) {
  const int z = blockIdx.x;
  const int row = row0 + blockIdx.y, s = c.rowshot[row], f = row - c.rowbase[s];
  const int nxg = c.w[s] + 2 * c.pad;
  const float w = c.omega[f];
  const float2 sr = c.sref[(size_t)s * c.nz + z];
  float2* ph = const_cast<float2*>(c.tph) + c.poff[row] + (size_t)z * N;
  for (int k = threadIdx.x; k < N; k += blockDim.x) ph[k] = phase_factor(w * w, sr, c.kx[k], c.eps, c.dz, c.phase_law);
  const float2* q = c.q + c.toff[s] + (size_t)z * nxg;
  const float* tp = c.taperN + c.tpo[s];
  float2* fa = const_cast<float2*>(c.tfac) + c.roff[row] + (size_t)z * nxg;
  for (int x = threadIdx.x; x < nxg; x += blockDim.x) fa[x] = ssf_factor(q[x], w, c.dz, tp[x]);
}

template <class K>
void set_smem(K kern, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

void launch_off_tables(const OffCtx& c, int row0, int nrows, int N, cudaStream_t st) {
  if (nrows <= 0) return;
  k_off_tables<<<dim3(c.nz, nrows), 256, 0, st>>>(c, row0, N);
  note_launch();
}

int off_row_length(int min_n) {
  for (int e : {8, 12, 16, 24, 32})
    if (32 * e >= min_n) return 32 * e;
  return 0;
}

size_t off_smem_bytes(int E, int nxg_max) {
  switch (E) {
    case 8: return off_smem_w<8>(nxg_max);
    case 12: return off_smem_w<12>(nxg_max);
    case 16: return off_smem_w<16>(nxg_max);
    case 24: return off_smem_w<24>(nxg_max);
    case 32: return off_smem_w<32>(nxg_max);
  }
  return 0;
}

void launch_off_sweep(int mode, int E, const OffCtx& c, const OffGroup* g, int ng, int nxg_max, float2* store,
                      float2* bins, cudaStream_t st) {
  switch (E) {
    case 8: launch_off_w<8>(mode, c, g, ng, nxg_max, store, bins, st); break;
    case 12: launch_off_w<12>(mode, c, g, ng, nxg_max, store, bins, st); break;
    case 16: launch_off_w<16>(mode, c, g, ng, nxg_max, store, bins, st); break;
    case 24: launch_off_w<24>(mode, c, g, ng, nxg_max, store, bins, st); break;
    case 32: launch_off_w<32>(mode, c, g, ng, nxg_max, store, bins, st); break;
  }
}

// lag register bound of the lag kernels: nh <= 41
static int lag_bound(int nh) { return nh <= 1 ? 1 : (nh <= 21 ? 21 : 41); }

void launch_off_source(const OffCtx& c, const float2* model, const float2* bg, float2* sc, int nxg_max,
                       cudaStream_t st) {
  const int hm = (c.nh - 1) / 2;
  const dim3 grid(c.nz, c.ns, (nxg_max + kSrcChunk - 1) / kSrcChunk);
  const size_t sm = (size_t)kSrcBatch * (kSrcChunk + 4 * hm) * 8;
  auto go = [&](auto kern) {
    set_smem(kern, sm);
    kern<<<grid, kSrcChunk, sm, st>>>(c, model, bg, sc);
    note_launch();
  };
  switch (lag_bound(c.nh)) {
    case 1: go(k_off_source<1>); break;
    case 21: go(k_off_source<21>); break;
    default: go(k_off_source<41>); break;
  }
}

void launch_off_image(const OffCtx& c, const float2* bg, const float2* a, float2* img, int add, cudaStream_t st) {
  const int hm = (c.nh - 1) / 2;
  const dim3 grid(c.nz, (c.nx + kImgChunk - 1) / kImgChunk);
  const size_t sm = (size_t)2 * kImgBatch * (kImgChunk + 2 * hm) * 8;
  auto go = [&](auto kern) {
    set_smem(kern, sm);
    kern<<<grid, kImgChunk, sm, st>>>(c, bg, a, img, add);
    note_launch();
  };
  switch (lag_bound(c.nh)) {
    case 1: go(k_off_image<1>); break;
    case 21: go(k_off_image<21>); break;
    default: go(k_off_image<41>); break;
  }
}

}  // namespace wg
