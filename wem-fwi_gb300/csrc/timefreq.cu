// Time <-> frequency transforms of the traces, sm_103a.
//
// The reference moves data between real time traces [nt] and complex bins
// with FFT1_r (operator/src/FFT1_r.cpp:74-96): the trace is zero-padded to
// n = nt + tpad samples, transformed by the complex FFT (FFTW_FORWARD) and
// scaled by 1/sqrt(n); the inverse takes the complex inverse transform of the
// bins, scales it by 1/sqrt(n) and keeps the real part of the first nt
// samples.  The propagated frequencies are the consecutive bins
// [b0, b0 + nf) (PropParam.h:75-78), so the library keeps only those
// ("compact" bins [trace][nf]).
//
// Two ways to the same numbers, picked by the trace length:
//  * n whose prime factors are all <= 7: the whole row is transformed in
//    shared memory by a Stockham FFT whose stages are compiled per radix
//    (16, 12, 8, 6 as in-register DFTs with the W_96 table of wfft.cuh, and
//    4, 3, 2, 5, 7), largest radices first so that few passes go through
//    shared memory, with per-stage twiddle tables laid out [r - 1][l] so that
//    consecutive butterflies read consecutive twiddles, the row and
//    butterfly indices from precomputed multiply-high divisions, and rows
//    padded by one slot every 16 points (the first stage writes with stride
//    R);
//  * any other n (a large prime factor makes an FFT stage cost O(p) per
//    point): the DFT restricted to the nf propagated bins, as sums over the
//    bins (bins -> time) or over the samples (time -> bins), with the
//    twiddles carried by a complex-rotation recurrence re-seeded from the
//    table of exp(-2 pi i j / n) every 32 steps.
// The FWI residual (BornFull.cpp:80-102 with the solver's data misfit) runs
// as one pass over the traces: modelled bins -> time, minus the observed
// trace, the sum of squares (the loss), and the residual's bins back in
// place of the modelled ones.  Every rounding of the residual is written
// out and the transform is one non-inlined function per direction, so the
// fused residual equals the residual of separate calls bit for bit.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "fft.cuh"
#include "kernels.h"
#include "wfft.cuh"

namespace wg {
namespace {

constexpr int kTfThreads = 256;
constexpr int kReseed = 32;  // twiddle recurrence steps between exact table values

// q = a / d with m = ceil(2^32 / d), exact while a d < 2^32 (rows of at most
// 16384 points, at most 8 rows)
__device__ __forceinline__ unsigned fdiv(unsigned a, unsigned m) { return __umulhi(a, m); }

// padded index of a row's point: one slot every 16 points
__device__ __forceinline__ int pd(int i) { return i + (i >> 4); }
__host__ __device__ inline int padded_len(int n) { return n + (n >> 4) + 1; }

// one Stockham stage of radix R over `rows` rows of n points (padded row
// stride ld): butterfly b (l = b mod L) reads x[b + r nb], multiplies by the
// stage twiddle tw[(r - 1) L + l] = W_n^(r l n / (L R)), takes the R-point
// DFT and writes y[(b - l) R + l + q L]
template <int R, bool INV>
__device__ __forceinline__ void tf_stage(const float2* __restrict__ x, float2* __restrict__ y, int rows,
                                         const TfStage& S, const float2* __restrict__ tw) {
  const int nb = S.nb, L = S.L, ld = S.ld;
  const int total = rows * nb;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int row = nb == 1 ? idx : (int)fdiv((unsigned)idx, S.mag_nb);
    const int b = idx - row * nb;
    const int l = L == 1 ? 0 : b - L * (int)fdiv((unsigned)b, S.mag_L);
    const float2* xr = x + (size_t)row * ld;
    float2* yr = y + (size_t)row * ld;
    const int o = (b - l) * R + l;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float2 a = xr[pd(b + r * nb)];
      if (r > 0) {
        const float2 w = tw[(r - 1) * L + l];
        a = INV ? c_mulc(a, w) : c_mul(a, w);
      }
      v[r] = a;
    }
    if constexpr (R == 16 || R == 12 || R == 8 || R == 6) {
      Dft<R, INV>::run(v);
    } else if constexpr (R == 2) {
      dft2(v);
    } else if constexpr (R == 3) {
      dft3(v, INV);
    } else if constexpr (R == 4) {
      dft4(v, INV);
    } else if constexpr (R == 5) {
      dft5(v, INV);
    } else {
      // 7: direct, with the powers of W_7 carried in the stage descriptor
      float2 u[R];
#pragma unroll
      for (int q = 0; q < R; ++q) {
        float2 acc = v[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float2 w = S.w7[(r * q) % R];
          acc = c_add(acc, INV ? c_mulc(v[r], w) : c_mul(v[r], w));
        }
        u[q] = acc;
      }
#pragma unroll
      for (int q = 0; q < R; ++q) v[q] = u[q];
    }
#pragma unroll
    for (int q = 0; q < R; ++q) yr[pd(o + q * L)] = v[q];
  }
}

// the transform of every mode, compiled once per direction (the modelled
// traces, the residual's bins and the bins of caller traces then come from
// the same instructions); returns the buffer holding the result, ends
// synchronised
template <bool INV>
__device__ __noinline__ float2* tf_fft(float2* a, float2* b, int rows, const TimeFreq& t, const float2* tws) {
  for (int s = 0; s < t.plan.nstage; ++s) {
    const TfStage& S = t.st[s];
    const float2* tw = tws + S.twoff;
    switch (S.R) {
      case 16: tf_stage<16, INV>(a, b, rows, S, tw); break;
      case 12: tf_stage<12, INV>(a, b, rows, S, tw); break;
      case 8: tf_stage<8, INV>(a, b, rows, S, tw); break;
      case 6: tf_stage<6, INV>(a, b, rows, S, tw); break;
      case 4: tf_stage<4, INV>(a, b, rows, S, tw); break;
      case 2: tf_stage<2, INV>(a, b, rows, S, tw); break;
      case 3: tf_stage<3, INV>(a, b, rows, S, tw); break;
      case 5: tf_stage<5, INV>(a, b, rows, S, tw); break;
      default: tf_stage<7, INV>(a, b, rows, S, tw); break;
    }
    __syncthreads();
    float2* tmp = a;
    a = b;
    b = tmp;
  }
  return a;
}

// FFT path.  mode 0: bins -> time (time = or += Re IFFT), 1: time -> bins,
// 2: bins <- FFT(Re IFFT(bins) - obs) and the sum of squares of the residual
template <int MODE>
__global__ void __launch_bounds__(kTfThreads) k_tf_fft(TimeFreq t, float2* __restrict__ bins,
                                                       float* __restrict__ time, const float* __restrict__ obs,
                                                       int ntr, int R, int add, double* __restrict__ part) {
  extern __shared__ float2 sm[];
  const int n = t.n, nt = t.nt, nf = t.nf, b0 = t.b0;
  const float sc = t.sc;
  const int ld = padded_len(n);
  float2* tws = sm;
  float2* X = sm + t.tw_len;
  float2* Y = X + (size_t)R * ld;
  for (int i = threadIdx.x; i < t.tw_len; i += blockDim.x) tws[i] = t.tws[i];
  double loss = 0;
  const int nblk = (ntr + R - 1) / R;
  const int rn = R * n;
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int tr0 = blk * R;
    for (int i = threadIdx.x; i < rn; i += blockDim.x) {
      const int r = i / n, k = i - r * n, tr = tr0 + r;
      float2 v = make_float2(0.f, 0.f);
      if (tr < ntr) {
        if (MODE == 1) {
          if (k < nt) v.x = time[(size_t)tr * nt + k];
        } else {
          const int f = k - b0;
          if (f >= 0 && f < nf) v = bins[(size_t)tr * nf + f];
        }
      }
      X[r * ld + pd(k)] = v;
    }
    __syncthreads();
    float2* A = MODE == 1 ? tf_fft<false>(X, Y, R, t, tws) : tf_fft<true>(X, Y, R, t, tws);
    if (MODE == 0) {
      for (int i = threadIdx.x; i < R * nt; i += blockDim.x) {
        const int r = i / nt, k = i - r * nt, tr = tr0 + r;
        if (tr < ntr) {
          const float v = __fmul_rn(A[(size_t)r * ld + pd(k)].x, sc);
          float* dst = time + (size_t)tr * nt + k;
          *dst = add ? __fadd_rn(*dst, v) : v;
        }
      }
    } else {
      if (MODE == 2) {
        float2* B = (A == X) ? Y : X;
        for (int i = threadIdx.x; i < rn; i += blockDim.x) {
          const int r = i / n, k = i - r * n, tr = tr0 + r;
          float v = 0.f;
          const int pi = r * ld + pd(k);
          if (k < nt && tr < ntr) {
            v = __fsub_rn(__fmul_rn(A[pi].x, sc), obs[(size_t)tr * nt + k]);
            loss += (double)v * v;
          }
          B[pi] = make_float2(v, 0.f);
        }
        __syncthreads();
        A = tf_fft<false>(B, A, R, t, tws);
      }
      for (int i = threadIdx.x; i < R * nf; i += blockDim.x) {
        const int r = i / nf, f = i - r * nf, tr = tr0 + r;
        if (tr < ntr) bins[(size_t)tr * nf + f] = c_scale(A[(size_t)r * ld + pd(b0 + f)], sc);
      }
    }
    __syncthreads();
  }
  if (MODE == 2) {
    __shared__ double red[kTfThreads];
    red[threadIdx.x] = loss;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
  }
}

// ---------------------------------------------------------- DFT path
// exp(-2 pi i (j mod n) / n) from the table
__device__ __forceinline__ float2 wn_at(const float2* wn, long long j, int n) { return wn[(int)(j % n)]; }

// Re(sum_f B_f exp(2 pi i (b0 + f) k / n)) at sample k for TT traces held
// in shared memory Bs[TT][nf]
template <int TT>
__device__ __forceinline__ void dft_b2t_point(const TimeFreq& t, const float2* Bs, int k, float (&acc)[TT]) {
  const int n = t.n, nf = t.nf;
#pragma unroll
  for (int r = 0; r < TT; ++r) acc[r] = 0.f;
  // exp(+2 pi i k / n): the conjugate of table entry k
  const float2 stepc = t.wn[k % n];
  const float2 step = make_float2(stepc.x, -stepc.y);
  float2 w = make_float2(1.f, 0.f);
  for (int f = 0; f < nf; ++f) {
    if (f % kReseed == 0) {
      const float2 e = wn_at(t.wn, (long long)(t.b0 + f) * k, n);
      w = make_float2(e.x, -e.y);
    }
#pragma unroll
    for (int r = 0; r < TT; ++r) {
      const float2 b = Bs[r * nf + f];
      acc[r] = fmaf(b.x, w.x, fmaf(-b.y, w.y, acc[r]));
    }
    w = c_mul(w, step);
  }
}

// sum over the samples k in [k0, k1) of TT traces Ts[TT][ldt] against
// exp(-2 pi i (b0 + f) k / n)
template <int TT>
__device__ __forceinline__ void dft_t2b_bin(const TimeFreq& t, const float* Ts, int ldt, int f, int k0, int k1,
                                            float2 (&acc)[TT]) {
  const int n = t.n, bf = t.b0 + f;
#pragma unroll
  for (int r = 0; r < TT; ++r) acc[r] = make_float2(0.f, 0.f);
  const float2 step = t.wn[bf % n];
  float2 w = make_float2(1.f, 0.f);
  for (int k = k0; k < k1; ++k) {
    if ((k - k0) % kReseed == 0) w = wn_at(t.wn, (long long)bf * k, n);
#pragma unroll
    for (int r = 0; r < TT; ++r) {
      const float v = Ts[r * ldt + k];
      acc[r].x = fmaf(v, w.x, acc[r].x);
      acc[r].y = fmaf(v, w.y, acc[r].y);
    }
    w = c_mul(w, step);
  }
}

constexpr int kTT = 8;  // traces per CTA of the DFT path

// mode 0: time (+)= Re(sum_f B exp(..)) sc; one CTA per kTT traces and
// blockDim samples
__global__ void __launch_bounds__(kTfThreads) k_dft_b2t(TimeFreq t, const float2* __restrict__ bins,
                                                        float* __restrict__ time, int ntr, int add) {
  extern __shared__ float2 sm[];
  const int nf = t.nf, nt = t.nt, tr0 = blockIdx.x * kTT;
  for (int i = threadIdx.x; i < kTT * nf; i += blockDim.x) {
    const int r = i / nf, tr = tr0 + r;
    sm[i] = tr < ntr ? bins[(size_t)tr * nf + (i - r * nf)] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  float acc[kTT];
  dft_b2t_point<kTT>(t, sm, k, acc);
#pragma unroll
  for (int r = 0; r < kTT; ++r) {
    if (tr0 + r >= ntr) break;
    float* dst = time + (size_t)(tr0 + r) * nt + k;
    const float v = __fmul_rn(acc[r], t.sc);
    *dst = add ? __fadd_rn(*dst, v) : v;
  }
}

// modes 1 and 2 for kTT traces per CTA, over chunks of kChunk samples: the
// chunk of the traces (mode 2: the residual of the modelled traces, from
// the bins, against the observed ones) in shared memory, then every bin by
// groups of threads over contiguous sample ranges of the chunk; each
// thread's sums run on over the chunks, and the groups' partial sums are
// added in group order at the end
constexpr int kChunk = 2048;
template <int MODE>
__global__ void __launch_bounds__(kTfThreads) k_dft_t2b(TimeFreq t, float2* __restrict__ bins,
                                                        const float* __restrict__ time, const float* __restrict__ obs,
                                                        int ntr, double* __restrict__ part) {
  extern __shared__ float2 sm[];
  const int nf = t.nf, nt = t.nt, tr0 = blockIdx.x * kTT;
  const int kc = nt < kChunk ? nt : kChunk;
  float* Ts = reinterpret_cast<float*>(sm);                              // [kTT][kc]
  float2* Bs = reinterpret_cast<float2*>(Ts + ((kTT * kc + 1) & ~1));    // mode 2: [kTT][nf]
  float2* P = Bs + (MODE == 2 ? (size_t)kTT * nf : 0);                   // [G][kTT][nf] partial sums
  double loss = 0;
  if (MODE == 2) {
    for (int i = threadIdx.x; i < kTT * nf; i += blockDim.x) {
      const int r = i / nf, tr = tr0 + r;
      Bs[i] = tr < ntr ? bins[(size_t)tr * nf + (i - r * nf)] : make_float2(0.f, 0.f);
    }
  }
  // group g of G takes the chunk's samples [g len / G, (g + 1) len / G)
  const int G = nf >= (int)blockDim.x ? 1 : (int)blockDim.x / nf;
  const int nu = (G * nf + blockDim.x - 1) / blockDim.x;  // (group, bin) units per thread
  float2 acc[2][kTT];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int r = 0; r < kTT; ++r) acc[a][r] = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < nt; k0 += kc) {
    const int len = nt - k0 < kc ? nt - k0 : kc;
    __syncthreads();  // the previous chunk is consumed (mode 2: Bs is in place)
    if (MODE == 1) {
      for (int i = threadIdx.x; i < kTT * len; i += blockDim.x) {
        const int r = i / len, tr = tr0 + r;
        Ts[r * kc + (i - r * len)] = tr < ntr ? time[(size_t)tr * nt + k0 + (i - r * len)] : 0.f;
      }
    } else {
      for (int k = threadIdx.x; k < len; k += blockDim.x) {
        float syn[kTT];
        dft_b2t_point<kTT>(t, Bs, k0 + k, syn);
#pragma unroll
        for (int r = 0; r < kTT; ++r) {
          float v = 0.f;
          if (tr0 + r < ntr) {
            v = __fsub_rn(__fmul_rn(syn[r], t.sc), obs[(size_t)(tr0 + r) * nt + k0 + k]);
            loss += (double)v * v;
          }
          Ts[r * kc + k] = v;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int u = threadIdx.x + a * blockDim.x;
      if (a < nu && u < G * nf) {
        const int g = u / nf, f = u - g * nf;
        float2 c[kTT];
        dft_t2b_bin<kTT>(t, Ts - k0, kc, f, k0 + (int)((long long)g * len / G),
                         k0 + (int)((long long)(g + 1) * len / G), c);
#pragma unroll
        for (int r = 0; r < kTT; ++r) acc[a][r] = c_add(acc[a][r], c[r]);
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const int u = threadIdx.x + a * blockDim.x;
    if (a < nu && u < G * nf) {
      const int g = u / nf, f = u - g * nf;
#pragma unroll
      for (int r = 0; r < kTT; ++r) P[((size_t)g * kTT + r) * nf + f] = acc[a][r];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kTT * nf; i += blockDim.x) {
    const int r = i / nf, f = i - r * nf;
    if (tr0 + r >= ntr) continue;
    float2 a = make_float2(0.f, 0.f);
    for (int g = 0; g < G; ++g) a = c_add(a, P[((size_t)g * kTT + r) * nf + f]);
    bins[(size_t)(tr0 + r) * nf + f] = c_scale(a, t.sc);
  }
  if (MODE == 2) {
    __shared__ double red[kTfThreads];
    red[threadIdx.x] = loss;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
  }
}

// out[0] = 1/2 sum of part[0..n), in a fixed order
__global__ void k_half_sum(const double* part, int n, double* out) {
  __shared__ double red[kTfThreads];
  double a = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a += part[i];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = 0.5 * red[0];
}

// the largest dynamic shared size a kernel can take: the device's opt-in
// bound less the kernel's static shared memory
template <class K>
void set_dyn_smem(K kern) {
  cudaFuncAttributes a{};
  size_t stat = 0;
  if (cudaFuncGetAttributes(&a, kern) == cudaSuccess) stat = a.sharedSizeBytes;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_per_block() - (int)stat);
}

size_t dft_t2b_smem(int nt, int nf) {
  const int kc = nt < kChunk ? nt : kChunk;
  const int G = nf >= kTfThreads ? 1 : kTfThreads / nf;
  const size_t ts = (size_t)((kTT * kc + 1) & ~1) * 4;
  return ts + (size_t)kTT * nf * 8 + (size_t)G * kTT * nf * 8;
}

}  // namespace

TfShape timefreq_shape(const TimeFreq& t, int ntr) {
  TfShape s{};
  // the bound of the kernels with static shared memory (mode 2)
  const size_t lim = (size_t)max_smem_per_block() - kTfThreads * sizeof(double);
  s.ok = 1;
  if (t.fft) {
    const size_t tw = (size_t)t.tw_len * 8;
    const long long ld = padded_len(t.n);
    // two CTAs per SM where the rows allow, one otherwise
    size_t cap = (lim / 2) & ~size_t(127);
    long long R = ((long long)cap - (long long)tw) / (16LL * ld);
    if (R < 1) {
      cap = lim;
      R = ((long long)cap - (long long)tw) / (16LL * ld);
    }
    if (R >= 1) {
      s.R = (int)(R > 8 ? 8 : R);
      s.smem = tw + (size_t)2 * s.R * ld * 8;
      s.grid = (ntr + s.R - 1) / s.R;
      if (s.grid > 152 * 8) s.grid = 152 * 8;
      if (s.grid < 1) s.grid = 1;
      s.use_fft = 1;
      return s;
    }
  }
  // restricted DFT: kTT traces per CTA
  s.use_fft = 0;
  s.R = kTT;
  s.grid = (ntr + kTT - 1) / kTT;
  if (s.grid < 1) s.grid = 1;
  s.smem = dft_t2b_smem(t.nt, t.nf);
  s.ok = s.smem <= lim ? 1 : 0;
  return s;
}

void launch_timefreq(int mode, const TimeFreq& t, const TfShape& s, float2* bins, float* time, const float* obs,
                     int ntr, int add, double* part, cudaStream_t st) {
  if (ntr <= 0) return;
  // this unit's copy of the W_96 table of the in-register DFTs
  static std::once_flag once;
  std::call_once(once, [] {
    float2 h[96];
    for (int k = 0; k < 96; ++k) {
      const long double a = -2.0L * 3.14159265358979323846264338327950288L * k / 96;
      h[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    cudaMemcpyToSymbol(c_w96, h, sizeof(h));
  });
  if (s.use_fft) {
    switch (mode) {
      case 0:
        set_dyn_smem(k_tf_fft<0>);
        k_tf_fft<0><<<s.grid, kTfThreads, s.smem, st>>>(t, bins, time, obs, ntr, s.R, add, part);
        break;
      case 1:
        set_dyn_smem(k_tf_fft<1>);
        k_tf_fft<1><<<s.grid, kTfThreads, s.smem, st>>>(t, bins, time, obs, ntr, s.R, add, part);
        break;
      default:
        set_dyn_smem(k_tf_fft<2>);
        k_tf_fft<2><<<s.grid, kTfThreads, s.smem, st>>>(t, bins, time, obs, ntr, s.R, add, part);
        break;
    }
  } else if (mode == 0) {
    const size_t sm = (size_t)kTT * t.nf * 8;
    set_dyn_smem(k_dft_b2t);
    const dim3 grid(s.grid, (t.nt + kTfThreads - 1) / kTfThreads);
    k_dft_b2t<<<grid, kTfThreads, sm, st>>>(t, bins, time, ntr, add);
  } else if (mode == 1) {
    set_dyn_smem(k_dft_t2b<1>);
    k_dft_t2b<1><<<s.grid, kTfThreads, s.smem, st>>>(t, bins, time, obs, ntr, part);
  } else {
    set_dyn_smem(k_dft_t2b<2>);
    k_dft_t2b<2><<<s.grid, kTfThreads, s.smem, st>>>(t, bins, time, obs, ntr, part);
  }
  note_launch();
}

void launch_half_sum(const double* part, int n, double* out, cudaStream_t st) {
  k_half_sum<<<1, kTfThreads, 0, st>>>(part, n, out);
  note_launch();
}

}  // namespace wg
