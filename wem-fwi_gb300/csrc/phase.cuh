// Point formulas of the depth step's two diagonal operators, shared by the
// table builders (kernels.cu k_phase, k_fac) and the kernels that evaluate
// them per row (kernels_off.cuh), so both give the same numbers.
#pragma once
#include <cuda_runtime.h>

#include "wemgpu.h"

namespace wg {

// phase_shift.ispc:2-16: a = w^2 s_re - k^2, b = w^2 (s_im - eps s_re),
// c = |a + ib|, re = sqrt((c+a)/2), im = -sqrt((c-a)/2),
// factor = exp(im dz) exp(-i re dz).
// FP32 with the cancellation-free form of the complex square root: the part
// whose square root is taken of c + |a| comes first, the other is |b| / (2
// that part), so neither c - a (a > 0) nor c + a (a < 0) is formed.
// EXACT_KZ law (extPropagator/src/Phshift.cpp:59,81): kz = sqrt(a + i (w^2
// s_im + 1e-5)), factor exp(-i dz conj(kz)) = exp(-dz Im kz - i dz Re kz);
// Im kz >= 0 for b >= 0, the principal root's sign otherwise.
// k2: the squared wavenumber (kx^2 + ky^2 in 3D)
__device__ __forceinline__ float2 phase_factor_k2(float w2, float2 s, float k2, float eps, float dz, int law) {
  const float a = fmaf(w2, s.x, -k2);
  const bool exact = law == WEM_PHASE_EXACT_KZ;
  const float b = exact ? fmaf(w2, s.y, 1e-5f) : w2 * fmaf(-eps, s.x, s.y);
  const float cc = sqrtf(fmaf(a, a, b * b));
  float re, im;  // real part and non-positive imaginary part of the root
  if (a >= 0.f) {
    re = sqrtf(0.5f * (cc + a));
    im = re > 0.f ? -fabsf(b) / (2.f * re) : 0.f;
  } else {
    const float q = sqrtf(0.5f * (cc - a));
    im = -q;
    re = fabsf(b) / (2.f * q);
  }
  if (exact && b < 0.f) im = -im;  // principal root: Im kz takes the sign of b
  const float e = expf(im * dz);
  float sn, cs;
  sincosf(re * dz, &sn, &cs);
  return make_float2(e * cs, -e * sn);
}
__device__ __forceinline__ float2 phase_factor(float w2, float2 s, float k, float eps, float dz, int law) {
  return phase_factor_k2(w2, s, __fmul_rn(k, k), eps, dz, law);
}

// SSF per-point factor: tp * exp(-i w dz q) (SplitStep.cpp:13-14), tp the
// taper over N.  w dz is carried as an unevaluated float pair hi + lo (lo the
// FMA-exact error of the float product), so the phase w dz q is the float
// rounding of the exact product with FP32 operations only.
__device__ __forceinline__ float2 ssf_factor(float2 qq, float w, float dz, float tp) {
  const float hi = w * dz, lo = fmaf(w, dz, -hi);
  const float amp = expf(fmaf(hi, qq.y, lo * qq.y)) * tp;
  float sn, cs;
  sincosf(fmaf(hi, qq.x, lo * qq.x), &sn, &cs);
  return make_float2(amp * cs, -amp * sn);
}

}  // namespace wg
