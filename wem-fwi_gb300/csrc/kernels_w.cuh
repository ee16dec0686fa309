// Warp-per-row pass kernels for row lengths N = 32 E, E in {8,12,16,24,32}
// (N = 256, 384, 512, 768, 1024).  Same passes as kernels.cu (WEM forward,
// two-sweep Born forward and adjoint), but every (shot, frequency) row is
// owned by one warp and lives in that warp's registers in the natural
// layout of wfft.cuh (lane t holds padded-row points t + 32 j).  Rows of a
// CTA share one frequency, so the per-(frequency, depth) tables they read
// hit L1; the WEM and Born-forward kernels need no block barrier at all, the
// Born adjoint one per image row for its fixed-order cross-row reduction.
//
// Invariant: points of the padded row outside the model grid (the FFT zero
// pad of width tap on each side) are zero in every state array.
#pragma once
#include <cmath>

#include "kernels.h"
#include "wfft.cuh"

namespace wg {
namespace {

constexpr int kW = 8;  // warps (rows) per CTA

struct WRow {
  const DevCtx& c;
  const float2* tw;  // [N] shared
  float2* sb;        // warp exchange buffer
  int lane;
};

template <int E>
__device__ __forceinline__ bool in_grid(const DevCtx& c, int lane, int j, int& x) {
  x = lane + 32 * j - c.tap;
  return x >= 0 && x < c.nxg;
}

// clamped grid index of register j: loads through it are issued without a
// branch (so a lane's E loads are all in flight together) and the result is
// selected with `in` afterwards
__device__ __forceinline__ int xclamp(const DevCtx& c, int lane, int j, bool& in) {
  const int x = lane + 32 * j - c.tap;
  in = (unsigned)x < (unsigned)c.nxg;
  return in ? x : 0;
}

template <int E>
__device__ __forceinline__ void w_load(const DevCtx& c, int lane, const float2* row, float2 (&v)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const float2 a = row[xclamp(c, lane, j, in)];
    v[j] = in ? a : make_float2(0.f, 0.f);
  }
}

template <int E>
__device__ __forceinline__ void w_store(const DevCtx& c, int lane, float2* row, const float2 (&v)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) {
    int x;
    if (in_grid<E>(c, lane, j, x)) row[x] = v[j];
  }
}

// o = P_z u  (SSF.cpp:8-32, PSPI.cpp:8-29); u and o may be the same array.
// SSF: the split-step table is zero where a point has no reference, so the
// reference index is only read for PSPI with several references.
template <int E>
__device__ void w_step_fwd(const WRow& w, int f, int z, const float2 (&u)[E], float2 (&o)[E]) {
  const DevCtx& c = w.c;
  constexpr int N = 32 * E;
  const int m = c.ext ? f : 0;
  const signed char* ref = c.ref + ((size_t)m * c.nz + z) * c.nxg;
  const float2* fac = c.fac ? c.fac + ((size_t)f * c.nz + z) * c.nxg : nullptr;
  const float2* ph = c.ph + ((size_t)f * c.nz + z) * c.nref * N;
  float2 X[E];
#pragma unroll
  for (int j = 0; j < E; ++j) X[j] = u[j];
  wfft<E, false>(X, w.sb, w.tw, w.lane);
  if (c.nref == 1) {
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = c_mul(X[j], ph[w.lane + 32 * j]);
    wfft<E, true>(X, w.sb, w.tw, w.lane);
    if (fac) {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const float2 fx = fac[xclamp(c, w.lane, j, in)];
        o[j] = in ? c_mul(X[j], fx) : make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, w.lane, j, in);
        const float tp = c.taperN[x];
        const int r = ref[x];
        o[j] = (in && r == 0) ? c_scale(X[j], tp) : make_float2(0.f, 0.f);
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < E; ++j) o[j] = make_float2(0.f, 0.f);
    for (int jr = 0; jr < c.nref; ++jr) {
      float2 Y[E];
      const float2* pj = ph + (size_t)jr * N;
#pragma unroll
      for (int j = 0; j < E; ++j) Y[j] = c_mul(X[j], pj[w.lane + 32 * j]);
      wfft<E, true>(Y, w.sb, w.tw, w.lane);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, w.lane, j, in);
        const int r = ref[x];
        const float2 v = fac ? c_mul(Y[j], fac[x]) : c_scale(Y[j], c.taperN[x]);
        if (in && r == jr) o[j] = v;
      }
    }
  }
}

// o = P^H_z d  (SSF.cpp:34-60, PSPI.cpp:31-53); d and o may be the same array
template <int E>
__device__ void w_step_adj(const WRow& w, int f, int z, const float2 (&d)[E], float2 (&o)[E]) {
  const DevCtx& c = w.c;
  constexpr int N = 32 * E;
  const int m = c.ext ? f : 0;
  const signed char* ref = c.ref + ((size_t)m * c.nz + z) * c.nxg;
  const float2* fac = c.fac ? c.fac + ((size_t)f * c.nz + z) * c.nxg : nullptr;
  const float2* ph = c.ph + ((size_t)f * c.nz + z) * c.nref * N;
  float2 A[E];
  if (c.nref == 1) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, w.lane, j, in);
      if (fac) {
        const float2 fx = fac[x];
        A[j] = in ? c_mulc(d[j], fx) : make_float2(0.f, 0.f);
      } else {
        const float tp = c.taperN[x];
        const int r = ref[x];
        A[j] = (in && r == 0) ? c_scale(d[j], tp) : make_float2(0.f, 0.f);
      }
    }
    wfft<E, false>(A, w.sb, w.tw, w.lane);
#pragma unroll
    for (int j = 0; j < E; ++j) A[j] = c_mulc(A[j], ph[w.lane + 32 * j]);
  } else {
    float2 acc[E];
#pragma unroll
    for (int j = 0; j < E; ++j) acc[j] = make_float2(0.f, 0.f);
    for (int jr = 0; jr < c.nref; ++jr) {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, w.lane, j, in);
        const int r = ref[x];
        const float2 v = fac ? c_mulc(d[j], fac[x]) : c_scale(d[j], c.taperN[x]);
        A[j] = (in && r == jr) ? v : make_float2(0.f, 0.f);
      }
      wfft<E, false>(A, w.sb, w.tw, w.lane);
      const float2* pj = ph + (size_t)jr * N;
#pragma unroll
      for (int j = 0; j < E; ++j) acc[j] = c_add(acc[j], c_mulc(A[j], pj[w.lane + 32 * j]));
    }
#pragma unroll
    for (int j = 0; j < E; ++j) A[j] = acc[j];
  }
  wfft<E, true>(A, w.sb, w.tw, w.lane);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    xclamp(c, w.lane, j, in);
    o[j] = in ? A[j] : make_float2(0.f, 0.f);
  }
}

// Taylor Born scatter (Scatter.cpp:35-111) for ntaylor <= 1 (the warp path
// serves ntaylor 0 and 1; larger orders run on the shared-memory kernels).
// mode 0 forward, 1 adjoint as coded (filter before scaling), 2 exact
// adjoint.  o = Sc u (overwrite); u and o may be the same array.
template <int E>
__device__ void w_scatter(const WRow& w, int f, int z, int mode, const float2 (&u)[E], float2 (&o)[E]) {
  const DevCtx& c = w.c;
  const int m = c.ext ? f : 0;
  const float om = c.omega[f];
  const float wdz = om * c.dz;
  const float2 iw = make_float2(0.f, mode == 0 ? -wdz : wdz);
  const size_t plane = (size_t)c.nz * c.nxg;
  const float2* c0 = c.sc + (size_t)m * (c.ntaylor + 1) * plane + (size_t)z * c.nxg;
  const float2* c1 = c0 + plane;
  const bool t1 = c.ntaylor >= 1;
  float2 X[E];
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(c, w.lane, j, in);
    const float2 k0 = c0[x];
    const float2 k1 = t1 ? c1[x] : make_float2(0.f, 0.f);
    // transform input: u, or conj(c_1) u for the exact adjoint
    X[j] = (mode == 2 && t1) ? (in ? c_mulc(u[j], k1) : make_float2(0.f, 0.f)) : u[j];
    o[j] = in ? c_mul(iw, mode == 0 ? c_mul(k0, u[j]) : c_mulc(u[j], k0)) : make_float2(0.f, 0.f);
  }
  if (!t1) return;
  wfft<E, false>(X, w.sb, w.tw, w.lane);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    float kw = c.kx[w.lane + 32 * j] / om;
    X[j] = c_scale(X[j], kw * kw * c.invN);
  }
  wfft<E, true>(X, w.sb, w.tw, w.lane);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(c, w.lane, j, in);
    const float2 k1 = c1[x];
    float2 y = X[j];
    if (mode == 0) y = c_mul(k1, y);
    else if (mode == 1) y = c_mulc(y, k1);
    if (in) o[j] = c_add(o[j], c_mul(iw, y));
  }
}

// add gs[g] wavelet into the row of shot s at depth z (Injection.cpp:8-19)
template <int E>
__device__ __forceinline__ void w_inject_src(const WRow& w, float2 (&v)[E], int s, int f, int z) {
  const DevCtx& c = w.c;
  if (c.sz[s] != z) return;
  const float2 wv = c.wave[f];
  for (int g = -c.ngs; g <= c.ngs; ++g) {
    int x = c.sx[s] + g + c.pad;
    if (x < 0 || x >= c.nxg) continue;
    int n = x + c.tap;
    if ((n & 31) != w.lane) continue;
    const int jn = n >> 5;
    const float2 add = c_scale(wv, c.gs[g + c.ngs]);
#pragma unroll
    for (int j = 0; j < E; ++j)
      if (j == jn) v[j] = c_add(v[j], add);
  }
}

// data[s][i][bin] += sum_g gr[g] v[rx_i + g] for receivers at depth z
// (Injection.cpp:69-80); goes through the warp buffer
template <int E>
__device__ __forceinline__ void w_record(const WRow& w, const float2 (&v)[E], int s, int bin, int z, float2* bins) {
  const DevCtx& c = w.c;
  const int k0 = c.rptr[z], k1 = c.rptr[z + 1];
  if (k0 == k1) return;
#pragma unroll
  for (int j = 0; j < E; ++j) w.sb[swz(w.lane + 32 * j)] = v[j];
  __syncwarp();
  for (int k = k0 + w.lane; k < k1; k += 32) {
    const int x0 = c.rxs[k] + c.pad;
    float2 acc = make_float2(0.f, 0.f);
    for (int g = -c.ngr; g <= c.ngr; ++g) {
      int x = x0 + g;
      if (x >= 0 && x < c.nxg) acc = c_add(acc, c_scale(w.sb[swz(x + c.tap)], c.gr[g + c.ngr]));
    }
    float2* d = bins + ((size_t)s * c.nr + c.rid[k]) * c.nbin + bin;
    *d = c_add(*d, acc);
  }
  __syncwarp();
}

// v += receivers of depth z spreading data[s][.][bin] (Injection.cpp:56-67)
template <int E>
__device__ __forceinline__ void w_inject_rec(const WRow& w, float2 (&v)[E], int s, int bin, int z,
                                             const float2* bins) {
  const DevCtx& c = w.c;
  const int k0 = c.rptr[z], k1 = c.rptr[z + 1];
  if (k0 == k1) return;
#pragma unroll
  for (int j = 0; j < E; ++j) {
    int x;
    if (!in_grid<E>(c, w.lane, j, x)) continue;
    int lo = x - c.pad - c.ngr, hi = x - c.pad + c.ngr;
    int a = k0, b = k1;
    while (a < b) {
      int mid = (a + b) >> 1;
      if (c.rxs[mid] < lo) a = mid + 1; else b = mid;
    }
    float2 acc = make_float2(0.f, 0.f);
    for (int k = a; k < k1 && c.rxs[k] <= hi; ++k) {
      int g = x - c.pad - c.rxs[k];
      acc = c_add(acc, c_scale(bins[((size_t)s * c.nr + c.rid[k]) * c.nbin + bin], c.gr[g + c.ngr]));
    }
    v[j] = c_add(v[j], acc);
  }
}

template <int E>
__device__ __forceinline__ void stage_tw(const DevCtx& c, float2* tw) {
  for (int i = threadIdx.x; i < 32 * E; i += blockDim.x) tw[i] = c.tw[i];
}

// =============================================================== passes
// nonlinear modelling, as k_wem (kernels.cu)
template <int E>
__global__ void __launch_bounds__(kW * 32, 1) kw_wem(DevCtx c, const Group* groups, float2* store, float2* bins) {
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* sb = tw + 32 * E + warp * wbuf_len<E>();
  stage_tw<E>(c, tw);
  __syncthreads();
  const Group gp = groups[blockIdx.x];
  if (warp >= gp.n) return;
  const WRow w{c, tw, sb, lane};
  const int f = gp.f, s = gp.s0 + warp, bin = c.bin[f], m = c.ext ? f : 0, nz = c.nz, nxg = c.nxg;
  const size_t plane = (size_t)nz * nxg;
  float2* A = store + (size_t)(gp.row0 + warp) * plane;
  float2 W[E];
#pragma unroll
  for (int j = 0; j < E; ++j) W[j] = make_float2(0.f, 0.f);
  w_inject_src<E>(w, W, s, f, 0);
  for (int z = 0; z < nz; ++z) {
    w_record<E>(w, W, s, bin, z, bins);
    const float2* rc = c.rc + ((size_t)m * nz + z) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 r = rc[x];
      if (in) A[(size_t)z * nxg + x] = c_mul(r, W[j]);
    }
    if (z == nz - 1) break;
    w_step_fwd<E>(w, f, z, W, W);
    w_inject_src<E>(w, W, s, f, z + 1);
  }
  w_load<E>(c, lane, A + (size_t)(nz - 1) * nxg, W);
  for (int z = nz - 1; z >= 0; --z) {
    w_record<E>(w, W, s, bin, z, bins);
    if (z == 0) break;
    w_step_fwd<E>(w, f, z, W, W);
    const float2* a = A + (size_t)(z - 1) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 v = a[xclamp(c, lane, j, in)];
      if (in) W[j] = c_add(W[j], v);
    }
  }
}

// Born forward, two sweeps per row (see k_born_fwd in kernels.cu)
template <int E>
__global__ void __launch_bounds__(kW * 32, 1) kw_born_fwd(DevCtx c, const Group* groups, const float2* dm,
                                                          const float2* drm, float2* storeA, float2* storeB,
                                                          float2* bins) {
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* sb = tw + 32 * E + warp * wbuf_len<E>();
  stage_tw<E>(c, tw);
  __syncthreads();
  const Group gp = groups[blockIdx.x];
  if (warp >= gp.n) return;
  const WRow w{c, tw, sb, lane};
  const int f = gp.f, s = gp.s0 + warp, bin = c.bin[f], m = c.ext ? f : 0, nz = c.nz, nxg = c.nxg;
  const size_t plane = (size_t)nz * nxg;
  float2* A = storeA + (size_t)(gp.row0 + warp) * plane;
  float2* B = storeB + (size_t)(gp.row0 + warp) * plane;
  float2 bg[E], sd[E], t[E];
#pragma unroll
  for (int j = 0; j < E; ++j) bg[j] = sd[j] = make_float2(0.f, 0.f);
  w_inject_src<E>(w, bg, s, f, 0);
  for (int z = 0; z < nz; ++z) {
    w_record<E>(w, sd, s, bin, z, bins);
    const size_t zo = ((size_t)m * nz + z) * nxg;
    const float2 *rc = c.rc + zo, *dr = drm + zo, *dmz = dm + zo;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 r = rc[x], d = dr[x], q = dmz[x];
      t[j] = in ? c_mul(bg[j], q) : make_float2(0.f, 0.f);
      if (in) {
        A[(size_t)z * nxg + x] = c_mul(r, bg[j]);
        B[(size_t)z * nxg + x] = c_add(c_mul(bg[j], d), c_mul(r, sd[j]));
      }
    }
    if (z == nz - 1) break;
    w_scatter<E>(w, f, z, 0, t, t);
#pragma unroll
    for (int j = 0; j < E; ++j) sd[j] = c_add(sd[j], t[j]);
    w_step_fwd<E>(w, f, z, sd, sd);
    w_step_fwd<E>(w, f, z, bg, bg);
    w_inject_src<E>(w, bg, s, f, z + 1);
  }
  w_load<E>(c, lane, A + (size_t)(nz - 1) * nxg, bg);
  w_load<E>(c, lane, B + (size_t)(nz - 1) * nxg, sd);
  for (int z = nz - 1; z >= 0; --z) {
    w_record<E>(w, sd, s, bin, z, bins);
    if (z == 0) break;
    const float2* dmz = dm + ((size_t)m * nz + z) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 q = dmz[xclamp(c, lane, j, in)];
      t[j] = in ? c_mul(bg[j], q) : make_float2(0.f, 0.f);
    }
    w_scatter<E>(w, f, z, 0, t, t);
#pragma unroll
    for (int j = 0; j < E; ++j) sd[j] = c_add(sd[j], t[j]);
    w_step_fwd<E>(w, f, z, sd, sd);
    w_step_fwd<E>(w, f, z, bg, bg);
    const float2* a = A + (size_t)(z - 1) * nxg;
    const float2* b = B + (size_t)(z - 1) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 va = a[x], vb = b[x];
      if (in) {
        bg[j] = c_add(bg[j], va);
        sd[j] = c_add(sd[j], vb);
      }
    }
  }
}

// image row z of the group = sum over the CTA's rows of each warp's slot,
// in warp order (deterministic)
__device__ __forceinline__ void reduce_slots(const float2* slots, int nxg, int nw, float2* out) {
  for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
    float2 a = make_float2(0.f, 0.f);
    for (int k = 0; k < nw; ++k) a = c_add(a, slots[k * nxg + x]);
    out[x] = a;
  }
}

// Born adjoint, two sweeps per row (see k_born_adj in kernels.cu)
template <int E>
__global__ void __launch_bounds__(kW * 32, 1) kw_born_adj(DevCtx c, const Group* groups, float2* storeBG,
                                                          float2* storeT, const float2* bins, float2* imgR,
                                                          float2* imgS, int compat) {
  extern __shared__ float4 smem4[];
  float2* tw = reinterpret_cast<float2*>(smem4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* sb = tw + 32 * E + warp * wbuf_len<E>();
  float2* slots = tw + 32 * E + kW * wbuf_len<E>();
  const int nxg = c.nxg, nz = c.nz;
  float2* slot = slots + warp * nxg;
  stage_tw<E>(c, tw);
  __syncthreads();
  const Group gp = groups[blockIdx.x];
  const bool act = warp < gp.n;
  const WRow w{c, tw, sb, lane};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f], m = c.ext ? f : 0;
  const size_t plane = (size_t)nz * nxg;
  float2* SBG = storeBG + (size_t)(gp.row0 + warp) * plane;
  float2* ST = storeT + (size_t)(gp.row0 + warp) * plane;
  float2* IR = imgR + (size_t)blockIdx.x * plane;
  float2* IS = imgS + (size_t)blockIdx.x * plane;
  const int scmode = compat ? 1 : 2;
  const float2 zero = make_float2(0.f, 0.f);
  // ---------------- down sweep: bg (Down of the source) and wu (Up^H of the data)
  float2 bg[E], wu[E];
#pragma unroll
  for (int j = 0; j < E; ++j) bg[j] = wu[j] = zero;
  if (act) {
    w_inject_src<E>(w, bg, s, f, 0);
    w_inject_rec<E>(w, wu, s, bin, 0, bins);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      int x;
      if (in_grid<E>(c, lane, j, x)) ST[x] = zero;
    }
  }
  for (int z = 0; z < nz; ++z) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      int x;
      if (in_grid<E>(c, lane, j, x)) slot[x] = act ? c_mulc(wu[j], bg[j]) : zero;
    }
    __syncthreads();
    reduce_slots(slots, nxg, kW, IR + (size_t)z * nxg);
    __syncthreads();
    if (!act) continue;
    w_store<E>(c, lane, SBG + (size_t)z * nxg, bg);
    if (z == nz - 1) continue;
    w_step_fwd<E>(w, f, z, bg, bg);
    w_inject_src<E>(w, bg, s, f, z + 1);
    w_step_adj<E>(w, f, z + 1, wu, wu);  // T[z+1]
    w_store<E>(c, lane, ST + (size_t)(z + 1) * nxg, wu);
    w_inject_rec<E>(w, wu, s, bin, z + 1, bins);
  }
  // ---------------- up sweep: bu (Up of R bg) and wd (Down^H of rec + conj(R) wu)
  float2 bu[E], wd[E], t[E];
  const bool keep_last = !compat || (c.ext ? (s == c.ns - 1) : (f == c.nfreq - 1));
  if (act) {
    const float2* rc = c.rc + ((size_t)m * nz + nz - 1) * nxg;
    w_load<E>(c, lane, SBG + (size_t)(nz - 1) * nxg, bu);
    w_load<E>(c, lane, ST + (size_t)(nz - 1) * nxg, t);
    w_inject_rec<E>(w, t, s, bin, nz - 1, bins);  // wu[nz-1]
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 r = rc[xclamp(c, lane, j, in)];
      bu[j] = in ? c_mul(r, bu[j]) : zero;
      wd[j] = in ? c_mulc(t[j], r) : zero;
    }
    w_inject_rec<E>(w, wd, s, bin, nz - 1, bins);
  }
#pragma unroll
  for (int j = 0; j < E; ++j) {
    int x;
    if (in_grid<E>(c, lane, j, x)) slot[x] = zero;
  }
  for (int z = nz - 1; z >= 0; --z) {
    // LinUp^H at depth z: conj(bu) Sc^H_z T[z]
    if (act && z >= 1 && (z < nz - 1 || keep_last)) {
      w_load<E>(c, lane, ST + (size_t)z * nxg, t);
      w_scatter<E>(w, f, z, scmode, t, t);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        int x;
        if (in_grid<E>(c, lane, j, x)) slot[x] = c_add(slot[x], c_mulc(t[j], bu[j]));
      }
    }
    __syncthreads();
    reduce_slots(slots, nxg, kW, IS + (size_t)z * nxg);
    __syncthreads();
    if (z == 0) break;
    if (!act) continue;  // the slot of an idle warp stays zero
    // q = P^H_{z-1} wd;  LinDown^H: conj(bg[z-1]) Sc^H_{z-1} q
    w_step_adj<E>(w, f, z - 1, wd, wd);  // wd holds q
    w_scatter<E>(w, f, z - 1, scmode, wd, t);
    const float2* bgp = SBG + (size_t)(z - 1) * nxg;
    const float2* tp = ST + (size_t)(z - 1) * nxg;
    const float2* rc = c.rc + ((size_t)m * nz + z - 1) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 b = bgp[x];
      if (in) slot[x] = c_mulc(t[j], b);
    }
    // wd[z-1] = q + rec + conj(R) (T[z-1] + rec)
    w_load<E>(c, lane, tp, t);
    w_inject_rec<E>(w, t, s, bin, z - 1, bins);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 r = rc[xclamp(c, lane, j, in)];
      if (in) wd[j] = c_add(wd[j], c_mulc(t[j], r));
    }
    w_inject_rec<E>(w, wd, s, bin, z - 1, bins);
    // bu[z-1] = P_z bu + R[z-1] bg[z-1]
    w_step_fwd<E>(w, f, z, bu, bu);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 r = rc[x], b = bgp[x];
      if (in) bu[j] = c_add(bu[j], c_mul(r, b));
    }
  }
}

template <int E>
size_t smem_w(const DevCtx& c, bool slots) {
  return 8 * ((size_t)32 * E + (size_t)kW * wbuf_len<E>() + (slots ? (size_t)kW * c.nxg : 0));
}

template <int E>
void launch_pass_w(int which, const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm,
                   float2* s1, float2* s2, float2* bins, float2* ir, float2* is, int compat, cudaStream_t st) {
  if (which == 0) {
    size_t sm = smem_w<E>(c, false);
    cudaFuncSetAttribute(kw_wem<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kw_wem<E><<<ng, kW * 32, sm, st>>>(c, g, s1, bins);
  } else if (which == 1) {
    size_t sm = smem_w<E>(c, false);
    cudaFuncSetAttribute(kw_born_fwd<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kw_born_fwd<E><<<ng, kW * 32, sm, st>>>(c, g, dm, drm, s1, s2, bins);
  } else {
    size_t sm = smem_w<E>(c, true);
    cudaFuncSetAttribute(kw_born_adj<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kw_born_adj<E><<<ng, kW * 32, sm, st>>>(c, g, s1, s2, bins, ir, is, compat);
  }
}

}  // namespace

// one instantiation per translation unit (kw_e*.cu)
template <int E>
void launch_pass_w_e(int which, const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm,
                     float2* s1, float2* s2, float2* bins, float2* ir, float2* is, int compat, cudaStream_t st) {
  static bool init = false;
  if (!init) {
    float2 h[96];
    for (int k = 0; k < 96; ++k) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * k / 96;
      h[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    cudaMemcpyToSymbol(c_w96, h, sizeof(h));
    init = true;
  }
  launch_pass_w<E>(which, c, g, ng, dm, drm, s1, s2, bins, ir, is, compat, st);
}

template <int E>
size_t smem_w_e(const DevCtx& c, bool slots) {
  return smem_w<E>(c, slots);
}

}  // namespace wg
