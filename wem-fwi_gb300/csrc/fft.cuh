// Shared-memory mixed-radix Stockham FFT for batches of rows, sm_103a.
//
// The depth step (propagator/src/SSF.cpp:8-60) transforms each padded
// wavefield row, applies a diagonal k-domain operator and transforms back;
// rows of one CTA are transformed together.  A plan is the radix sequence of
// the row length n (radix 4/2/3/5/7 butterflies are written out; any other
// prime runs a direct DFT, O(p) per point).  Twiddles come from a table of n
// values w[t] = exp(-2 pi i t / n) computed in double on the host and staged
// in shared memory once per CTA.
//
// Stage s with radix R and L = product of earlier radices (Stockham,
// decimation in time): butterfly b in [0, n/R) with l = b mod L reads
// x[b + r n/R] (r < R), multiplies by w^(r l n/(L R)), takes the R-point DFT
// and writes y[(b/L) L R + l + q L] (q < R).  Output is in natural order.
#pragma once
#include <cuda_runtime.h>

#include "fft_plan.h"

namespace wg {

// Complex add and subtract issue as one paired FP32 instruction on sm_100 and
// later (add/sub .f32x2: both components in one instruction, each rounded as
// the scalar operation), halving the issue slots of the transforms'
// butterflies.
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
#define WG_F32X2 1
#endif
__host__ __device__ inline float2 c_add(float2 a, float2 b) {
#ifdef WG_F32X2
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__host__ __device__ inline float2 c_sub(float2 a, float2 b) {
#ifdef WG_F32X2
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
// Complex products with their roundings written out (one product rounded,
// the other fused into it), so that every inlined copy of a transform or a
// depth step computes the same bits whatever the surrounding code: a
// checkpointed recompute reproduces the stored wavefields exactly.
#ifdef __CUDA_ARCH__
__device__ inline float2 c_mul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
// a * conj(b)
__device__ inline float2 c_mulc(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, __fmul_rn(a.y, b.y)), __fmaf_rn(a.y, b.x, -__fmul_rn(a.x, b.y)));
}
#else
inline float2 c_mul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
inline float2 c_mulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
#endif
// acc + a b and acc + a conj(b) as four fused multiply-adds (the paired add
// above would otherwise stop the accumulation from contracting)
__host__ __device__ inline float2 c_fma(float2 acc, float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y)));
}
__host__ __device__ inline float2 c_fmac(float2 acc, float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x)), fmaf(a.y, b.x, fmaf(-a.x, b.y, acc.y)));
}
__host__ __device__ inline float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
#ifdef __CUDA_ARCH__
__device__ inline float2 c_scale(float2 a, float s) { return make_float2(__fmul_rn(a.x, s), __fmul_rn(a.y, s)); }
#else
inline float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
#endif
// multiply by -i (fwd) or +i (inv)
__device__ inline float2 c_rot(float2 a, bool inv) {
  return inv ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---- small DFT kernels; inv selects the sign of the exponent
__device__ inline void dft2(float2* v) {
  float2 a = v[0];
  v[0] = c_add(a, v[1]);
  v[1] = c_sub(a, v[1]);
}

__device__ inline void dft4(float2* v, bool inv) {
  float2 s0 = c_add(v[0], v[2]), d0 = c_sub(v[0], v[2]);
  // d1 = -i (v1 - v3) (fwd) or +i (v1 - v3) (inv), formed from two scalar
  // differences so that it lands as a pair for the paired adds below
  float2 s1 = c_add(v[1], v[3]);
  float2 d1 = inv ? make_float2(v[3].y - v[1].y, v[1].x - v[3].x) : make_float2(v[1].y - v[3].y, v[3].x - v[1].x);
  v[0] = c_add(s0, s1);
  v[2] = c_sub(s0, s1);
  v[1] = c_add(d0, d1);
  v[3] = c_sub(d0, d1);
}

__device__ inline void dft3(float2* v, bool inv) {
  const float c = -0.5f, s = inv ? 0.86602540378443864676f : -0.86602540378443864676f;
  float2 t = c_add(v[1], v[2]);
  float2 d = c_sub(v[1], v[2]);
  float2 y0 = c_add(v[0], t);
#ifdef WG_F32X2
  float2 m = __ffma2_rn(t, make_float2(c, c), v[0]);
#else
  float2 m = make_float2(v[0].x + c * t.x, v[0].y + c * t.y);
#endif
  // s * i * d
  float2 r = make_float2(-s * d.y, s * d.x);
  v[0] = y0;
  v[1] = c_add(m, r);
  v[2] = c_sub(m, r);
}

__device__ inline void dft5(float2* v, bool inv) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  const float s1 = inv ? 0.95105651629515357212f : -0.95105651629515357212f;
  const float s2 = inv ? 0.58778525229247312917f : -0.58778525229247312917f;
  float2 a1 = c_add(v[1], v[4]), b1 = c_sub(v[1], v[4]);
  float2 a2 = c_add(v[2], v[3]), b2 = c_sub(v[2], v[3]);
  float2 y0 = make_float2(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
  float2 m1 = make_float2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
  float2 m2 = make_float2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
  // i*(s1 b1 + s2 b2) and i*(s2 b1 - s1 b2)
  float2 n1 = make_float2(-(s1 * b1.y + s2 * b2.y), s1 * b1.x + s2 * b2.x);
  float2 n2 = make_float2(-(s2 * b1.y - s1 * b2.y), s2 * b1.x - s1 * b2.x);
  v[0] = y0;
  v[1] = c_add(m1, n1);
  v[4] = c_sub(m1, n1);
  v[2] = c_add(m2, n2);
  v[3] = c_sub(m2, n2);
}

// One Stockham stage over `nrow` rows of length n (row stride ld) for the
// threads of the CTA.  Generic primes use the twiddle table for W_R.
__device__ inline void fft_stage(const float2* __restrict__ in, float2* __restrict__ out, int nrow, int ld,
                                 int n, int R, int L, const float2* __restrict__ tw, bool inv) {
  const int nb = n / R;
  const int Lp = L * R;
  const int tws = n / Lp;
  const int total = nrow * nb;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int row = idx / nb;
    const int b = idx - row * nb;
    const int l = b % L;
    const float2* x = in + (size_t)row * ld + b;
    float2* y = out + (size_t)row * ld + (b - l) * R + l;
    if (R <= 8 && R != 6) {
      float2 v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r)
        if (r < R) {
          float2 a = x[r * nb];
          if (r && l) {
            float2 w = tw[r * l * tws];
            a = inv ? c_mulc(a, w) : c_mul(a, w);
          }
          v[r] = a;
        }
      switch (R) {
        case 2: dft2(v); break;
        case 3: dft3(v, inv); break;
        case 4: dft4(v, inv); break;
        case 5: dft5(v, inv); break;
        default: {  // 7 (and 8 is never planned): direct DFT from the table
          float2 u[8];
          const int step = n / R;
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (q < R) {
              float2 acc = v[0];
              for (int r = 1; r < R; ++r) {
                float2 w = tw[((r * q) % R) * step];
                acc = c_add(acc, inv ? c_mulc(v[r], w) : c_mul(v[r], w));
              }
              u[q] = acc;
            }
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (q < R) v[q] = u[q];
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < R) y[q * L] = v[q];
    } else {
      // large prime: direct DFT, inputs re-read from shared memory
      const int step = n / R;
      for (int q = 0; q < R; ++q) {
        float2 acc = make_float2(0.f, 0.f);
        for (int r = 0; r < R; ++r) {
          float2 a = x[r * nb];
          if (r && l) {
            float2 w = tw[r * l * tws];
            a = inv ? c_mulc(a, w) : c_mul(a, w);
          }
          float2 w2 = tw[((r * q) % R) * step];
          acc = c_add(acc, inv ? c_mulc(a, w2) : c_mul(a, w2));
        }
        y[q * L] = acc;
      }
    }
  }
}

// Transform `nrow` rows held in buffer a (stride ld), using b as the second
// buffer; returns the buffer holding the result.  Unnormalised; inv selects
// FFTW_BACKWARD.  Ends with __syncthreads().
__device__ inline float2* smem_fft(float2* a, float2* b, int nrow, int ld, const FftPlan& P,
                                   const float2* __restrict__ tw, bool inv) {
  int L = 1;
  for (int s = 0; s < P.nstage; ++s) {
    const int R = P.radix[s];
    fft_stage(a, b, nrow, ld, P.n, R, L, tw, inv);
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    L *= R;
  }
  return a;
}

}  // namespace wg
