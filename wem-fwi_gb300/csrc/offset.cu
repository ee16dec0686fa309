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
constexpr int kSrcBatch = 8;    // frequencies per stage of the source kernel
constexpr int kImgCols = 2;     // model columns per thread of the image kernel
constexpr int kImgThreads = 128;
constexpr int kImgChunk = kImgCols * kImgThreads;  // model columns per CTA of the image kernel
constexpr int kImgBatch = 4;    // frequencies per stage of the image kernel

// 8-byte asynchronous copy global -> shared; ok = false writes zeros
// (src-size 0) and reads nothing
__device__ __forceinline__ void cp8(float2* dst, const float2* src, bool ok) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src), "r"(ok ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit8() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait8_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// grid (nz, ns, chunks); thread t: padded aperture point x = chunk * 256 + t.
// The lag values r_l(x - l) stay in registers for all frequencies of the
// shot; the bg segments [x_lo - 2 hm, x_hi + 2 hm] of kSrcBatch frequencies
// stream through two shared-memory stages with cp.async, the next batch in
// flight while the current one is summed.
template <int NL>
__global__ void __launch_bounds__(kSrcChunk) k_off_source(OffCtx c, const float2* model, const float2* bg,
                                                          float2* sc) {
  extern __shared__ float2 seg[];  // [2][kSrcBatch][len]
  const int z = blockIdx.x, s = blockIdx.y;
  const int x0 = c.x0[s], w = c.w[s], pad = c.pad, nxg = w + 2 * pad, hm = (c.nh - 1) / 2;
  const int xlo = blockIdx.z * kSrcChunk;
  if (xlo >= nxg) return;
  const int x = xlo + threadIdx.x;
  const bool on = x < nxg;
  const int lo = xlo - 2 * hm, len = kSrcChunk + 4 * hm;
  const size_t r0 = (size_t)c.rowbase[s], zo = (size_t)z * nxg;
  const int nbatch = (c.nfreq + kSrcBatch - 1) / kSrcBatch;
  auto issue = [&](int bt) {
    if (bt < nbatch) {
      float2* dst = seg + (size_t)(bt & 1) * kSrcBatch * len;
      for (int b = 0; b < kSrcBatch; ++b) {
        const int f = bt * kSrcBatch + b;
        if (f >= c.nfreq) break;
        const float2* src = bg + c.roff[r0 + f] + zo;
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
          const int xb = lo + i;
          const bool ok = xb >= 0 && xb < nxg;
          cp8(dst + b * len + i, ok ? src + xb : src, ok);
        }
      }
    }
    cp_commit8();
  };
  issue(0);
  float2 rv[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    rv[k] = make_float2(0.f, 0.f);
    const int l = k - hm, y = x - l;
    if (k < c.nh && on && y >= pad && y < pad + w) rv[k] = model[((size_t)k * c.nz + z) * c.nx + x0 + y - pad];
  }
  for (int bt = 0; bt < nbatch; ++bt) {
    issue(bt + 1);
    cp_wait8_1();
    __syncthreads();
    if (on) {
      const float2* buf = seg + (size_t)(bt & 1) * kSrcBatch * len;
      const int nb = min(kSrcBatch, c.nfreq - bt * kSrcBatch);
      for (int b = 0; b < nb; ++b) {
        const float2* g = buf + (size_t)b * len + (x - lo);
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NL; ++k)
          if (k < c.nh) acc = c_fma(acc, rv[k], g[-2 * (k - hm)]);
        sc[c.roff[r0 + bt * kSrcBatch + b] + zo + x] = acc;
      }
    }
    __syncthreads();  // the stage is free for batch bt + 2
  }
}

// grid (nz, chunks of kImgChunk model columns); thread t: model columns
// m, m + 1 (m = chunk start + 2 t).  The batches (a shot whose aperture meets
// the chunk, kImgBatch of its frequencies; shots and frequencies in order)
// stream their bg and a segments (the chunk with a halo of hm + 1) through
// two shared-memory stages with cp.async.  Lags run as a sliding window:
// from lag l to l + 1 the two columns need one new bg and one new a value.
template <int NL>
__global__ void __launch_bounds__(kImgThreads) k_off_image(OffCtx c, const float2* bg, const float2* a, float2* img,
                                                           int add) {
  extern __shared__ float2 sh[];  // [2][2][kImgBatch][len]
  const int z = blockIdx.x, hm = (c.nh - 1) / 2, pad = c.pad;
  const int m0 = blockIdx.y * kImgChunk, m = m0 + kImgCols * threadIdx.x;
  const int len = kImgChunk + 2 * hm + 3;
  const size_t stage = (size_t)2 * kImgBatch * len;
  float2 acc0[NL], acc1[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) acc0[k] = acc1[k] = make_float2(0.f, 0.f);
  auto meets = [&](int s) { return c.x0[s] < m0 + kImgChunk && c.x0[s] + c.w[s] > m0; };
  // batch cursor: shot s (meeting the chunk) and first frequency f0
  auto advance = [&](int& s, int& f0) {
    f0 += kImgBatch;
    if (f0 >= c.nfreq) {
      f0 = 0;
      for (++s; s < c.ns && !meets(s); ++s) {
      }
    }
  };
  auto issue = [&](int s, int f0, int buf) {
    if (s < c.ns) {
      const int nxg = c.w[s] + 2 * pad;
      const int lo = m0 - c.x0[s] + pad - hm - 1;
      const size_t r0 = (size_t)c.rowbase[s], zo = (size_t)z * nxg;
      float2* sb = sh + (size_t)buf * stage;
      for (int b = 0; b < kImgBatch; ++b) {
        const int f = f0 + b;
        if (f >= c.nfreq) break;
        const size_t o = c.roff[r0 + f] + zo;
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
          const int xi = lo + i;
          const bool ok = xi >= 0 && xi < nxg;
          cp8(sb + b * len + i, bg + o + (ok ? xi : 0), ok);
          cp8(sb + (kImgBatch + b) * len + i, a + o + (ok ? xi : 0), ok);
        }
      }
    }
    cp_commit8();
  };
  int s = 0, f0 = 0;
  while (s < c.ns && !meets(s)) ++s;
  int sn = s, fn = f0;
  issue(s, f0, 0);
  for (int bt = 0; s < c.ns; ++bt) {
    advance(sn, fn);
    issue(sn, fn, (bt + 1) & 1);
    cp_wait8_1();
    __syncthreads();
    const int x0 = c.x0[s], w = c.w[s];
    const bool on0 = m < c.nx && m >= x0 && m < x0 + w;
    const bool on1 = m + 1 < c.nx && m + 1 >= x0 && m + 1 < x0 + w;
    if (on0 || on1) {
      const int y = m - x0 + pad, lo = m0 - x0 + pad - hm - 1;
      const float2* sb = sh + (size_t)(bt & 1) * stage;
      const int nb = min(kImgBatch, c.nfreq - f0);
      for (int b = 0; b < nb; ++b) {
        const float2* gb = sb + (size_t)b * len + (y - lo);  // gb[d] = bg(y + d)
        const float2* ga = sb + (size_t)(kImgBatch + b) * len + (y - lo);
        // lag l = k - hm: column y takes conj(bg(y - l)) a(y + l), column
        // y + 1 conj(bg(y + 1 - l)) a(y + 1 + l)
        float2 b0 = gb[hm], b1 = gb[hm + 1], a0 = ga[-hm], a1 = ga[1 - hm];
#pragma unroll
        for (int k = 0; k < NL; ++k) {
          if (k < c.nh) {
            acc0[k] = c_fmac(acc0[k], a0, b0);
            acc1[k] = c_fmac(acc1[k], a1, b1);
            const int l = k - hm;
            b1 = b0;
            b0 = gb[-(l + 1)];
            a0 = a1;
            a1 = ga[l + 2];
          }
        }
      }
    }
    __syncthreads();  // the stage is free for the batch after next
    s = sn;
    f0 = fn;
  }
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    if (k >= c.nh) break;
    float2* o = img + ((size_t)k * c.nz + z) * c.nx + m;
    if (m < c.nx) o[0] = add ? c_add(o[0], acc0[k]) : acc0[k];
    if (m + 1 < c.nx) o[1] = add ? c_add(o[1], acc1[k]) : acc1[k];
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
  const size_t sm = (size_t)2 * kSrcBatch * (kSrcChunk + 4 * hm) * 8;
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
  const size_t sm = (size_t)2 * 2 * kImgBatch * (kImgChunk + 2 * hm + 3) * 8;
  auto go = [&](auto kern) {
    set_smem(kern, sm);
    kern<<<grid, kImgThreads, sm, st>>>(c, bg, a, img, add);
    note_launch();
  };
  switch (lag_bound(c.nh)) {
    case 1: go(k_off_image<1>); break;
    case 21: go(k_off_image<21>); break;
    default: go(k_off_image<41>); break;
  }
}

}  // namespace wg
