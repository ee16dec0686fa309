// Warp-per-row register FFT for row lengths N = 32 E (sm_103a).
//
// Lane t of a warp holds the E points n = t + 32 j (j < E) of one row in
// registers: the "natural layout".  A transform is a short Stockham sequence
// whose first radix is E (a DFT held entirely in one lane's registers) and
// whose later radices divide E, so every butterfly of a stage reads its R
// inputs from the lane's own registers; between stages the row is
// redistributed through a per-warp shared buffer (write scattered, read
// natural, __syncwarp only).  The last stage of a Stockham sequence writes
// natural order, so it needs no exchange: a transform costs (stages - 1)
// exchanges, e.g. one for N = 1024 (32 x 32) and two for N = 768 (24 x 8 x 4).
//
// In-register DFTs are unrolled mixed-radix decompositions with compile-time
// indices; their twiddles W_R^k (R | 96) come from a 96-entry table in
// constant memory, computed in double on the host.  Inter-stage twiddles
// W_N^(r l N/(L R)) come from a table in shared memory laid out per stage as
// [r - 1][l] (stage s >= 1 holds (R_s - 1) L_s entries; all stages together
// N - E), so the 32 lanes of a twiddle load read consecutive l.
//
// Shared-memory banks: the exchange buffer pads one slot every 2^k points
// (k = 4 for E = 8, 16; k = 5 for E = 12, 32), chosen by counting the
// wavefronts of every exchange write and read of each plan; the natural-order
// reads stay conflict-free and fold the padding into immediate offsets.
// E = 24 uses blocks of two 24-point rows padded by one slot (rows_layout).
#pragma once
#include <cuda_runtime.h>

#include "fft.cuh"

namespace wg {

// W_96^k = exp(-2 pi i k / 96); one copy per translation unit, filled by
// that unit's launcher
static __constant__ float2 c_w96[96];

template <int R>
__device__ __forceinline__ float2 wr(int k, bool inv) {
  float2 w = c_w96[(k % R) * (96 / R)];
  return inv ? make_float2(w.x, -w.y) : w;
}

// x W_R^k (conjugate twiddle for INV): the powers -1 and -+i are a negation
// or a swap, with no multiplication; the others come from the table.  k is a
// compile-time constant after unrolling, so the switch folds away.
template <int R, bool INV>
__device__ __forceinline__ float2 tw_mul(float2 x, int k) {
  int e = (k % R) * (96 / R);  // exponent in units of 2 pi / 96
  if (INV) e = (96 - e) % 96;
  switch (e) {
    case 0: return x;
    case 24: return make_float2(x.y, -x.x);   // -i
    case 48: return make_float2(-x.x, -x.y);  // -1
    case 72: return make_float2(-x.y, x.x);   // +i
    default: return c_mul(x, wr<R>(k, INV));
  }
}

// ------------------------------------------------ in-register small DFTs
template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<1, INV> {
  __device__ __forceinline__ static void run(float2*) {}
};
template <bool INV>
struct Dft<2, INV> {
  __device__ __forceinline__ static void run(float2* v) { dft2(v); }
};
template <bool INV>
struct Dft<3, INV> {
  __device__ __forceinline__ static void run(float2* v) { dft3(v, INV); }
};
template <bool INV>
struct Dft<4, INV> {
  __device__ __forceinline__ static void run(float2* v) { dft4(v, INV); }
};

// composite size: R = P M, decimation in time, P in {4, 2, 3}
template <int R, bool INV>
struct Dft {
  static constexpr int P = (R % 4 == 0 && R != 8) ? 4 : ((R % 2 == 0) ? 2 : 3);
  static constexpr int M = R / P;
  __device__ __forceinline__ static void run(float2* v) {
    float2 sub[P][M];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
      for (int i = 0; i < M; ++i) sub[q][i] = v[q + P * i];
#pragma unroll
    for (int q = 0; q < P; ++q) Dft<M, INV>::run(sub[q]);
#pragma unroll
    for (int k = 0; k < M; ++k) {
      float2 a[P];
#pragma unroll
      for (int q = 0; q < P; ++q) a[q] = tw_mul<R, INV>(sub[q][k], q * k);
      Dft<P, INV>::run(a);
#pragma unroll
      for (int r = 0; r < P; ++r) v[k + M * r] = a[r];
    }
  }
};

// ------------------------------------------------ stage plans
// radices of N = 32 E: first E, then factors of 32 that divide E
template <int E>
struct WPlan;
template <>
struct WPlan<8> {
  static constexpr int n = 3;
  __host__ __device__ static constexpr int r(int s) { return s == 0 ? 8 : (s == 1 ? 8 : 4); }
};
template <>
struct WPlan<12> {
  static constexpr int n = 4;
  __host__ __device__ static constexpr int r(int s) { return s == 0 ? 12 : (s == 3 ? 2 : 4); }
};
template <>
struct WPlan<16> {
  static constexpr int n = 3;
  __host__ __device__ static constexpr int r(int s) { return s == 2 ? 2 : 16; }
};
template <>
struct WPlan<24> {
  static constexpr int n = 3;
  __host__ __device__ static constexpr int r(int s) { return s == 0 ? 24 : (s == 1 ? 8 : 4); }
};
template <>
struct WPlan<32> {
  static constexpr int n = 2;
  __host__ __device__ static constexpr int r(int) { return 32; }
};

// padded index of the exchange buffer: one pad slot per 2^k points
template <int E>
__host__ __device__ constexpr int swz_shift() {
  return (E == 8 || E == 16) ? 4 : 5;
}
template <int E>
__device__ __forceinline__ int swz(int i) {
  return i + (i >> swz_shift<E>());
}
// E = 24 lays the exchange out instead in blocks of two rows of E points
// (2 E = 48) padded by one slot: every exchange address is a per-butterfly
// base plus compile-time offsets; the stage-0 writes (a lane's row starts
// E slots after the previous lane's, or E + 1 across a block) are free of
// bank conflicts, and so are the natural-order reads, whose 16-lane halves
// never cross a block (48 is a multiple of 16).  Counting wavefronts of every
// exchange access of a transform: 208 against 192 without conflicts (224 with
// one pad slot per row of 24).
template <int E>
__host__ __device__ constexpr bool rows_layout() {
  return E == 24;
}
template <int E>
__device__ __forceinline__ int xaddr(int i) {
  if constexpr (rows_layout<E>()) return (i / (2 * E)) * (2 * E + 1) + i % (2 * E);
  else return swz<E>(i);
}
// the buffer also holds a row in the swz layout (receiver records)
template <int E>
__host__ __device__ constexpr int wbuf_len() {
  return (rows_layout<E>() ? 32 * (E + 1) : 32 * E + ((32 * E) >> swz_shift<E>())) + 2;
}

// offset of stage S's twiddles in the per-stage table: sum over 1 <= s < S of
// (R_s - 1) L_s, with L_s the product of the radices before s
template <int E>
__host__ __device__ constexpr int tw_offset(int S) {
  int off = 0, L = WPlan<E>::r(0);
  for (int s = 1; s < S; ++s) {
    off += (WPlan<E>::r(s) - 1) * L;
    L *= WPlan<E>::r(s);
  }
  return off;
}
template <int E>
__host__ __device__ constexpr int tw_entries() {
  return tw_offset<E>(WPlan<E>::n);
}

template <int E, bool INV, int S, int L>
__device__ __forceinline__ void wfft_stage(float2 (&v)[E], float2* sb, const float2* tw, int lane) {
  constexpr int R = WPlan<E>::r(S);
  constexpr int M = E / R;
  constexpr bool LAST = (S == WPlan<E>::n - 1);
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int b = lane + 32 * m;
    const int l = (L == 1) ? 0 : (b % L);
    float2 a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float2 x = v[m + r * M];
      if (L > 1 && r > 0) {
        float2 w = tw[tw_offset<E>(S) + (r - 1) * L + l];
        x = INV ? c_mulc(x, w) : c_mul(x, w);
      }
      a[r] = x;
    }
    Dft<R, INV>::run(a);
    if constexpr (LAST) {
#pragma unroll
      for (int q = 0; q < R; ++q) v[m + q * M] = a[q];
    } else if constexpr (rows_layout<E>()) {
      // positions o + q L, o = (b - l) R + l: one row (L = 1; o is a
      // multiple of E) or one point of each of R rows (L = E; o = l modulo
      // 2 E, as (b - l) R is a multiple of 2 E), so position q lies
      // q L + floor(q L / 2 E) slots after o's
      static_assert(L == 1 || (L == E && ((E * R) % (2 * E)) == 0), "block layout: L = 1, or L = E with R even");
      const int a0 = xaddr<E>((b - l) * R + l);
#pragma unroll
      for (int q = 0; q < R; ++q) sb[a0 + q * L + (q * L) / (2 * E)] = a[q];
    } else {
      const int o = (b - l) * R + l;
#pragma unroll
      for (int q = 0; q < R; ++q) sb[swz<E>(o + q * L)] = a[q];
    }
  }
  if constexpr (!LAST) {
    __syncwarp();
    if constexpr (rows_layout<E>()) {
      // natural order, read per butterfly of the next stage: positions
      // lane + 32 m + r 32 M2 lie 32 M2 / 2 E whole blocks apart
      constexpr int R2 = WPlan<E>::r(S + 1), M2 = E / R2;
      static_assert((32 * M2) % (2 * E) == 0, "block layout needs 32 M2 to be a multiple of 2 E");
      constexpr int RSTEP = 32 * M2 + (32 * M2) / (2 * E);
#pragma unroll
      for (int m = 0; m < M2; ++m) {
        const int base = xaddr<E>(lane + 32 * m);
#pragma unroll
        for (int r = 0; r < R2; ++r) v[m + r * M2] = sb[base + r * RSTEP];
      }
    } else {
#pragma unroll
      for (int j = 0; j < E; ++j) v[j] = sb[swz<E>(lane + 32 * j)];
    }
    __syncwarp();
    wfft_stage<E, INV, S + 1, L * R>(v, sb, tw, lane);
  }
}

// unnormalised DFT of the row held by this warp, natural layout in and out
template <int E, bool INV>
__device__ __forceinline__ void wfft(float2 (&v)[E], float2* sb, const float2* tw, int lane) {
  wfft_stage<E, INV, 0, 1>(v, sb, tw, lane);
}

}  // namespace wg
