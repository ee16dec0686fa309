// 3D one-way depth step on planes (no reference counterpart: the
// reference's propagators are 2D; at ny = 1 these passes are its SSF / PSPI
// step, propagator/src/SSF.cpp:8-60 and PSPI.cpp:8-53, with the 2D FFT of
// a depth slice in place of FFT1_c).  The step of depth d:
//   forward  W' = sum_j select_j( taper x IFFT2( ph_j(d) FFT2(W) ) [x split step_j] )
//   adjoint  W' = IFFT2( sum_j conj(ph_j(d)) FFT2( select_j( taper x W ) [x conj split step_j] ) )
// runs as two batched passes over all (shot, frequency) rows:
//   row pass     one warp per line y of a row: the transforms along x (the
//                register FFT of wfft.cuh) and every point operation
//                (selection, taper, split step, injection, recording,
//                Reflect, stores);
//   column pass  one CTA per 8 columns of a row: the tile goes through
//                shared memory (coalesced 64-byte segments), one warp per
//                column transforms along y in registers and applies each
//                reference's phase shift, read from the quadrant table of
//                |kx|, |ky| built once per background.
// The 1/(Nx Ny) of the transform pair is folded into the taper.
#pragma once
#include "kernels_w.cuh"
#include "phase.cuh"

namespace wg {
namespace {

constexpr int kWarps3 = 8;

// twiddles of a length-32E transform in wfft.cuh's per-stage layout from the
// natural table
template <int E>
__device__ __forceinline__ void stage_tw(const float2* nat, float2* out) {
  constexpr int N = 32 * E;
  for (int i = threadIdx.x; i < tw_entries<E>(); i += blockDim.x) {
    int S = 1, L = WPlan<E>::r(0), off = 0;
    while (S < WPlan<E>::n - 1 && i >= off + (WPlan<E>::r(S) - 1) * L) {
      off += (WPlan<E>::r(S) - 1) * L;
      L *= WPlan<E>::r(S);
      ++S;
    }
    const int R = WPlan<E>::r(S), r = (i - off) / L + 1, l = (i - off) % L;
    out[i] = nat[r * l * (N / (L * R))];
  }
}

__device__ __forceinline__ int quad(int i, int n) { return i < n / 2 ? i : (i == n / 2 ? 0 : n - i); }

template <int E>
__host__ __device__ constexpr size_t rows3_smem() {
  return ((size_t)tw_entries<E>() * 8 + 15) / 16 * 16 + (size_t)kWarps3 * wbuf_len<E>() * 8;
}

// row pass: line gl = blockIdx.x * 8 + warp of the rows x Ny lines
template <int EX, bool ADJ>
__global__ void __launch_bounds__(kWarps3 * 32) k3_rows(Ctx3 c, Pass3 a) {
  constexpr int N = 32 * EX;
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* sb0 = tw + ((size_t)tw_entries<EX>() * 8 + 15) / 16 * 2;
  stage_tw<EX>(c.twx, tw);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long gl = (long long)blockIdx.x * kWarps3 + warp;
  if (gl >= (long long)c.rows * c.Ny) return;  // no barrier below
  const int r = (int)(gl / c.Ny), y = (int)(gl % c.Ny);
  const int f = r / c.ns, s = r % c.ns;
  const int yg = y - c.tapy, nxg = c.nxg;
  const bool yin = (unsigned)yg < (unsigned)c.nyg;
  float2* sb = sb0 + warp * wbuf_len<EX>();
  const float om = c.omega[f];
  const float2 zero = make_float2(0.f, 0.f);
  const size_t plane = (size_t)c.Ny * N, rowoff = (size_t)r * plane + (size_t)y * N;
  const size_t fplane = (size_t)c.nyg * nxg;
  const size_t frow = ((size_t)r * c.nyg + (yin ? yg : 0)) * nxg;  // this line in [rows][nyg][nxg]
  auto xat = [&](int j, bool& in) {
    const int x = lane + 32 * j - c.tapx;
    in = yin && (unsigned)x < (unsigned)nxg;
    return in ? x : 0;
  };
  const size_t tz = a.zt >= 0 ? ((size_t)a.zt * c.nyg + (yin ? yg : 0)) * nxg : 0;
  const float* tp = c.taper + (size_t)(yin ? yg : 0) * nxg;
  float2 W[EX], X[EX];
#pragma unroll
  for (int j = 0; j < EX; ++j) W[j] = zero;

  if (yin) {
    // ---- the field of depth z
    if (a.init == 0) {
      if (!ADJ) {
#pragma unroll 1
        for (int jr = 0; jr < c.nref; ++jr) {
          const float2* in = a.tin + (size_t)jr * c.rows * plane + rowoff;
#pragma unroll
          for (int j = 0; j < EX; ++j) X[j] = in[lane + 32 * j];
          wfft<EX, true>(X, sb, tw, lane);
#pragma unroll
          for (int j = 0; j < EX; ++j) {
            bool in_;
            const int x = xat(j, in_);
            const int rf = c.ref[tz + x];
            if (in_ && rf == jr) W[j] = c.q ? c_mul(X[j], ssf_factor(c.q[tz + x], om, c.dz, tp[x])) : c_scale(X[j], tp[x]);
          }
        }
      } else {
        const float2* in = a.tin + rowoff;
#pragma unroll
        for (int j = 0; j < EX; ++j) X[j] = in[lane + 32 * j];
        wfft<EX, true>(X, sb, tw, lane);
#pragma unroll
        for (int j = 0; j < EX; ++j) {
          bool in_;
          xat(j, in_);
          W[j] = in_ ? X[j] : zero;
        }
      }
    } else if (a.init == 2) {
#pragma unroll
      for (int j = 0; j < EX; ++j) {
        bool in_;
        const int x = xat(j, in_);
        const float2 v = a.load[frow + x];
        W[j] = in_ ? v : zero;
      }
    }
    // ---- point operations at depth z
    const size_t rz = ((size_t)a.z * c.nyg + yg) * nxg;
    if (a.add) {
#pragma unroll
      for (int j = 0; j < EX; ++j) {
        bool in_;
        const int x = xat(j, in_);
        if (!in_) continue;
        float2 v = a.add[frow + x];
        if (a.add_rw) v = c_mul(c.rc[rz + x], v);
        if (a.refl) {
          const int xm = x - c.pad, ym = yg - c.pady;
          const bool m = (unsigned)xm < (unsigned)c.nx && (unsigned)ym < (unsigned)c.ny;
          v = m ? c_mul(a.refl[((size_t)a.z * c.ny + ym) * c.nx + xm], v) : zero;
        }
        W[j] = c_add(W[j], v);
      }
    }
    if (a.src && c.sz[s] == a.z && c.sy[s] + c.pady == yg) {
      const float2 wv = c.wave[f];
      for (int g = -c.ngs; g <= c.ngs; ++g) {
        const int x = c.sx[s] + g + c.pad;
        if (x < 0 || x >= nxg) continue;
        const int n = x + c.tapx;
        if ((n & 31) != lane) continue;
        const int jn = n >> 5;
        const float2 v = c_scale(wv, c.gs[g + c.ngs]);
#pragma unroll
        for (int j = 0; j < EX; ++j)
          if (j == jn) W[j] = c_add(W[j], v);
      }
    }
    const int k0 = c.rptr[a.z * c.nyg + yg], k1 = c.rptr[a.z * c.nyg + yg + 1];
    if (a.rec_in && k0 < k1) {
#pragma unroll
      for (int j = 0; j < EX; ++j) {
        bool in_;
        const int x = xat(j, in_);
        if (!in_) continue;
        const int lo = x - c.pad - c.ngr, hi = x - c.pad + c.ngr;
        int lo_k = k0, hi_k = k1;
        while (lo_k < hi_k) {
          const int mid = (lo_k + hi_k) >> 1;
          if (c.rxs[mid] < lo) lo_k = mid + 1; else hi_k = mid;
        }
        float2 acc = zero;
        for (int k = lo_k; k < k1 && c.rxs[k] <= hi; ++k) {
          const int g = x - c.pad - c.rxs[k];
          acc = c_add(acc, c_scale(a.bins[((size_t)s * c.nr + c.rid[k]) * c.nfreq + f], c.gr[g + c.ngr]));
        }
        W[j] = c_add(W[j], acc);
      }
    }
    if (a.record && k0 < k1) {
      __syncwarp();
#pragma unroll
      for (int j = 0; j < EX; ++j) sb[swz<EX>(lane + 32 * j)] = W[j];
      __syncwarp();
      for (int k = k0 + lane; k < k1; k += 32) {
        const int xr = c.rxs[k] + c.pad;
        float2 acc = zero;
        for (int g = -c.ngr; g <= c.ngr; ++g) {
          const int x = xr + g;
          if (x >= 0 && x < nxg) acc = c_add(acc, c_scale(sb[swz<EX>(x + c.tapx)], c.gr[g + c.ngr]));
        }
        float2* d = a.bins + ((size_t)s * c.nr + c.rid[k]) * c.nfreq + f;
        *d = c_add(*d, acc);
      }
      __syncwarp();
    }
    if (a.store || a.spatial) {
#pragma unroll
      for (int j = 0; j < EX; ++j) {
        bool in_;
        const int x = xat(j, in_);
        if (!in_) continue;
        if (a.store) a.store[frow + x] = a.store_rw ? c_mul(c.rc[rz + x], W[j]) : W[j];
        if (a.spatial) a.spatial[frow + x] = W[j];
      }
    }
  }
  (void)fplane;
  if (a.last) return;
  // ---- the transform output
  if (!ADJ) {
    float2* out = a.tout + rowoff;
#pragma unroll
    for (int j = 0; j < EX; ++j) X[j] = W[j];
    if (yin) wfft<EX, false>(X, sb, tw, lane);
#pragma unroll
    for (int j = 0; j < EX; ++j) out[lane + 32 * j] = X[j];
  } else {
#pragma unroll 1
    for (int jr = 0; jr < c.nref; ++jr) {
      float2* out = a.tout + (size_t)jr * c.rows * plane + rowoff;
#pragma unroll
      for (int j = 0; j < EX; ++j) {
        bool in_;
        const int x = xat(j, in_);
        const int rf = yin ? c.ref[tz + x] : -1;
        X[j] = (in_ && rf == jr) ? (c.q ? c_mulc(W[j], ssf_factor(c.q[tz + x], om, c.dz, tp[x])) : c_scale(W[j], tp[x]))
                                 : zero;
      }
      if (yin) wfft<EX, false>(X, sb, tw, lane);
#pragma unroll
      for (int j = 0; j < EX; ++j) out[lane + 32 * j] = X[j];
    }
  }
}

template <int E>
__host__ __device__ constexpr size_t cols3_smem(int Ny) {
  return ((size_t)tw_entries<E>() * 8 + 15) / 16 * 16 + ((size_t)Ny * 9 * 8 + 15) / 16 * 16 +
         (size_t)kWarps3 * wbuf_len<E>() * 8;
}

// column pass: CTA = (row, 8 columns); warp w transforms column xb + w
template <int EY, bool ADJ>
__global__ void __launch_bounds__(kWarps3 * 32) k3_cols(Ctx3 c, int z, const float2* in, float2* out) {
  constexpr int N = 32 * EY;  // == c.Ny
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  float2* tile = tw + ((size_t)tw_entries<EY>() * 8 + 15) / 16 * 2;           // [N][9]
  float2* sb0 = tile + ((size_t)N * 9 * 8 + 15) / 16 * 2;
  stage_tw<EY>(c.twy, tw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nb = c.Nx / 8;
  const int r = blockIdx.x / nb, xb = (blockIdx.x % nb) * 8, f = r / c.ns;
  const size_t plane = (size_t)N * c.Nx, rp = (size_t)r * plane;
  float2* sb = sb0 + warp * wbuf_len<EY>();
  const int ix = quad(xb + warp, c.Nx);
  const size_t tab = ((size_t)f * c.nz + z) * c.nref;
  const size_t qsz = (size_t)c.Qy * c.Qx;
  auto load_tile = [&](const float2* src) {
    for (int i = threadIdx.x; i < N * 8; i += blockDim.x) tile[(i >> 3) * 9 + (i & 7)] = src[rp + (size_t)(i >> 3) * c.Nx + xb + (i & 7)];
  };
  auto store_tile = [&](float2* dst) {
    for (int i = threadIdx.x; i < N * 8; i += blockDim.x) dst[rp + (size_t)(i >> 3) * c.Nx + xb + (i & 7)] = tile[(i >> 3) * 9 + (i & 7)];
  };
  float2 X[EY], Y[EY];
  if (!ADJ) {
    load_tile(in);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < EY; ++j) X[j] = tile[(lane + 32 * j) * 9 + warp];
    wfft<EY, false>(X, sb, tw, lane);
#pragma unroll 1
    for (int jr = 0; jr < c.nref; ++jr) {
      const float2* ph = c.ph + (tab + jr) * qsz + ix;
#pragma unroll
      for (int j = 0; j < EY; ++j) Y[j] = c_mul(X[j], ph[(size_t)quad(lane + 32 * j, N) * c.Qx]);
      wfft<EY, true>(Y, sb, tw, lane);
      __syncthreads();  // the tile's previous contents are read or stored
#pragma unroll
      for (int j = 0; j < EY; ++j) tile[(lane + 32 * j) * 9 + warp] = Y[j];
      __syncthreads();
      store_tile(out + (size_t)jr * c.rows * plane);
    }
  } else {
#pragma unroll
    for (int j = 0; j < EY; ++j) Y[j] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int jr = 0; jr < c.nref; ++jr) {
      __syncthreads();
      load_tile(in + (size_t)jr * c.rows * plane);
      __syncthreads();
#pragma unroll
      for (int j = 0; j < EY; ++j) X[j] = tile[(lane + 32 * j) * 9 + warp];
      wfft<EY, false>(X, sb, tw, lane);
      const float2* ph = c.ph + (tab + jr) * qsz + ix;
#pragma unroll
      for (int j = 0; j < EY; ++j) Y[j] = c_add(Y[j], c_mulc(X[j], ph[(size_t)quad(lane + 32 * j, N) * c.Qx]));
    }
    wfft<EY, true>(Y, sb, tw, lane);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < EY; ++j) tile[(lane + 32 * j) * 9 + warp] = Y[j];
    __syncthreads();
    store_tile(out);
  }
}

}  // namespace

template <int E>
void launch_k3_rows_e(const Ctx3& c, const Pass3& a, int adj, cudaStream_t st) {
  init_w96();
  const long long lines = (long long)c.rows * c.Ny;
  const unsigned grid = (unsigned)((lines + kWarps3 - 1) / kWarps3);
  const size_t sm = rows3_smem<E>();
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<grid, kWarps3 * 32, sm, st>>>(c, a);
    note_launch();
  };
  if (adj) go(k3_rows<E, true>);
  else go(k3_rows<E, false>);
}

template <int E>
void launch_k3_cols_e(const Ctx3& c, int z, int adj, const float2* in, float2* out, cudaStream_t st) {
  init_w96();
  const unsigned grid = (unsigned)((long long)c.rows * (c.Nx / 8));
  const size_t sm = cols3_smem<E>(c.Ny);
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<grid, kWarps3 * 32, sm, st>>>(c, z, in, out);
    note_launch();
  };
  if (adj) go(k3_cols<E, true>);
  else go(k3_cols<E, false>);
}

}  // namespace wg
