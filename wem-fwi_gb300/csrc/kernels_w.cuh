// Warp-per-row pass kernels for row lengths N = 32 E, E in {8,12,16,24,32}
// (N = 256, 384, 512, 768, 1024).  Same passes as kernels.cu (WEM forward,
// two-sweep Born forward and adjoint), but every (shot, frequency) row is
// owned by one warp and lives in that warp's registers in the natural
// layout of wfft.cuh (lane t holds padded-row points t + 32 j).
//
// The rows of a CTA share one frequency and march through the depths
// together.  Each depth's tables (phase row, split-step row, Reflect and
// Scatter rows, perturbation rows) are copied into a three-slot ring in
// shared memory two depths ahead with cp.async, so the steps read them at
// shared-memory latency; where the budget allows, each warp also prefetches
// the stored field row it needs next.  Barriers: two __syncthreads per depth
// for the ring (the Born adjoint adds two around its fixed-order cross-row
// image reduction); the transforms themselves synchronise warps only.
//
// Invariant: points of the padded row outside the model grid (the FFT zero
// pad of width tap on each side) are zero in every state array.
#pragma once
#include <cmath>

#include "kernels.h"
#include "wfft.cuh"

namespace wg {

// byte offsets of one depth's tables inside a ring slot (-1: read from global)
struct SlotLayout {
  int ph, fac, ref, rc, c0, c1, dm, dr;
  int bytes;      // slot size (multiple of 16)
  int nslots;     // 0 (no ring) or 3
  int row_bytes;  // per-warp prefetched row, 0 if none
};

namespace {

constexpr int kW = 8;  // warps (rows) per CTA

// ------------------------------------------------------- async copies
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
// CTA-cooperative copy; bytes a multiple of 16, both ends 16-byte aligned
__device__ __forceinline__ void cta_copy(void* dst, const void* src, int bytes) {
  for (int i = threadIdx.x * 16; i < bytes; i += blockDim.x * 16)
    cp16(static_cast<char*>(dst) + i, static_cast<const char*>(src) + i);
}
// bring a row into L2 ahead of its loads (bulk prefetch; bytes multiple of 16)
__device__ __forceinline__ void l2_prefetch(const void* src, int bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void warp_copy(void* dst, const void* src, int bytes, int lane) {
  for (int i = lane * 16; i < bytes; i += 32 * 16)
    cp16(static_cast<char*>(dst) + i, static_cast<const char*>(src) + i);
}

// ------------------------------------------------------- per-depth tables
struct Tabs {
  const float2* ph;        // [nref][N]
  const float2* fac;       // [nxg] taper * split step / N (SSF), or null
  const signed char* ref;  // [nxg] reference index
  const float2* rc;        // [nxg] Reflect
  const float2* c0;        // [nxg] Scatter coefficient it = 0
  const float2* c1;        // [nxg] Scatter coefficient it = 1
  const float2* dm;        // [nxg] padded slowness perturbation (Born forward)
  const float2* dr;        // [nxg] dR(dm) (Born forward)
};

struct Src {  // global sources of the perturbation rows
  const float2* dm;
  const float2* drm;
};

__device__ __forceinline__ Tabs global_tabs(const DevCtx& c, const Src& s, int f, int z) {
  const int m = c.ext ? f : 0;
  const size_t zo = ((size_t)m * c.nz + z) * c.nxg;
  const size_t plane = (size_t)c.nz * c.nxg;
  Tabs t;
  t.ph = c.ph + ((size_t)f * c.nz + z) * c.nref * c.N;
  t.fac = c.fac ? c.fac + ((size_t)f * c.nz + z) * c.nxg : nullptr;
  t.ref = c.ref + zo;
  t.rc = c.rc + zo;
  t.c0 = c.sc ? c.sc + (size_t)m * (c.ntaylor + 1) * plane + (size_t)z * c.nxg : nullptr;
  t.c1 = (c.sc && c.ntaylor >= 1) ? t.c0 + plane : nullptr;
  t.dm = s.dm ? s.dm + zo : nullptr;
  t.dr = s.drm ? s.drm + zo : nullptr;
  return t;
}

// copy depth z's tables into a slot (CTA-cooperative, asynchronous)
__device__ __forceinline__ void stage_tabs(const DevCtx& c, const SlotLayout& L, char* slot, const Tabs& g) {
  const int rowb = c.nxg * 8;
  if (L.ph >= 0) cta_copy(slot + L.ph, g.ph, c.nref * c.N * 8);
  if (L.fac >= 0) cta_copy(slot + L.fac, g.fac, rowb);
  if (L.ref >= 0) cta_copy(slot + L.ref, g.ref, c.nxg);
  if (L.rc >= 0) cta_copy(slot + L.rc, g.rc, rowb);
  if (L.c0 >= 0) cta_copy(slot + L.c0, g.c0, rowb);
  if (L.c1 >= 0) cta_copy(slot + L.c1, g.c1, rowb);
  if (L.dm >= 0) cta_copy(slot + L.dm, g.dm, rowb);
  if (L.dr >= 0) cta_copy(slot + L.dr, g.dr, rowb);
}

__device__ __forceinline__ Tabs slot_tabs(const SlotLayout& L, const char* slot, Tabs g) {
  if (L.ph >= 0) g.ph = reinterpret_cast<const float2*>(slot + L.ph);
  if (L.fac >= 0) g.fac = reinterpret_cast<const float2*>(slot + L.fac);
  if (L.ref >= 0) g.ref = reinterpret_cast<const signed char*>(slot + L.ref);
  if (L.rc >= 0) g.rc = reinterpret_cast<const float2*>(slot + L.rc);
  if (L.c0 >= 0) g.c0 = reinterpret_cast<const float2*>(slot + L.c0);
  if (L.c1 >= 0) g.c1 = reinterpret_cast<const float2*>(slot + L.c1);
  if (L.dm >= 0) g.dm = reinterpret_cast<const float2*>(slot + L.dm);
  if (L.dr >= 0) g.dr = reinterpret_cast<const float2*>(slot + L.dr);
  return g;
}

// The ring: depth d lives in slot d mod 3; at iteration z the tables of
// depths z and z + dir are ready while z + 2 dir is in flight.
struct Ring {
  const DevCtx& c;
  const SlotLayout& L;
  char* base;
  Src src;
  int f;
  __device__ char* slot(int d) const { return base + (size_t)(d % 3) * L.bytes; }
  __device__ void issue(int d) const {
    if (L.nslots && d >= 0 && d < c.nz) stage_tabs(c, L, slot(d), global_tabs(c, src, f, d));
  }
  __device__ Tabs tabs(int d) const {
    Tabs g = global_tabs(c, src, f, d);
    return L.nslots ? slot_tabs(L, slot(d), g) : g;
  }
};

struct WRow {
  const DevCtx& c;
  const float2* tw;  // [N] shared
  float2* sb;        // warp exchange buffer
  const float* taperN;
  const float* kx;
  int lane;
};

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
    bool in;
    const int x = xclamp(c, lane, j, in);
    if (in) row[x] = v[j];
  }
}

template <int E>
__device__ __forceinline__ void w_zero(float2 (&v)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) v[j] = make_float2(0.f, 0.f);
}

// o = P_z u  (SSF.cpp:8-32, PSPI.cpp:8-29); u and o may be the same array.
// SSF: the split-step table is zero where a point has no reference, so the
// reference index is only read for PSPI or several references.
template <int E>
__device__ void w_step_fwd(const WRow& w, const Tabs& T, const float2 (&u)[E], float2 (&o)[E]) {
  const DevCtx& c = w.c;
  constexpr int N = 32 * E;
  float2 X[E];
#pragma unroll
  for (int j = 0; j < E; ++j) X[j] = u[j];
  wfft<E, false>(X, w.sb, w.tw, w.lane);
  if (c.nref == 1) {
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = c_mul(X[j], T.ph[w.lane + 32 * j]);
    wfft<E, true>(X, w.sb, w.tw, w.lane);
    if (T.fac) {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const float2 fx = T.fac[xclamp(c, w.lane, j, in)];
        o[j] = in ? c_mul(X[j], fx) : make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, w.lane, j, in);
        const float tp = w.taperN[x];
        const int r = T.ref[x];
        o[j] = (in && r == 0) ? c_scale(X[j], tp) : make_float2(0.f, 0.f);
      }
    }
  } else {
    w_zero<E>(o);
    for (int jr = 0; jr < c.nref; ++jr) {
      float2 Y[E];
      const float2* pj = T.ph + (size_t)jr * N;
#pragma unroll
      for (int j = 0; j < E; ++j) Y[j] = c_mul(X[j], pj[w.lane + 32 * j]);
      wfft<E, true>(Y, w.sb, w.tw, w.lane);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, w.lane, j, in);
        const int r = T.ref[x];
        const float2 v = T.fac ? c_mul(Y[j], T.fac[x]) : c_scale(Y[j], w.taperN[x]);
        if (in && r == jr) o[j] = v;
      }
    }
  }
}

// o = P^H_z d  (SSF.cpp:34-60, PSPI.cpp:31-53); d and o may be the same array
template <int E>
__device__ void w_step_adj(const WRow& w, const Tabs& T, const float2 (&d)[E], float2 (&o)[E]) {
  const DevCtx& c = w.c;
  constexpr int N = 32 * E;
  float2 A[E];
  if (c.nref == 1) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, w.lane, j, in);
      if (T.fac) {
        const float2 fx = T.fac[x];
        A[j] = in ? c_mulc(d[j], fx) : make_float2(0.f, 0.f);
      } else {
        const float tp = w.taperN[x];
        const int r = T.ref[x];
        A[j] = (in && r == 0) ? c_scale(d[j], tp) : make_float2(0.f, 0.f);
      }
    }
    wfft<E, false>(A, w.sb, w.tw, w.lane);
#pragma unroll
    for (int j = 0; j < E; ++j) A[j] = c_mulc(A[j], T.ph[w.lane + 32 * j]);
  } else {
    float2 acc[E];
    w_zero<E>(acc);
    for (int jr = 0; jr < c.nref; ++jr) {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, w.lane, j, in);
        const int r = T.ref[x];
        const float2 v = T.fac ? c_mulc(d[j], T.fac[x]) : c_scale(d[j], w.taperN[x]);
        A[j] = (in && r == jr) ? v : make_float2(0.f, 0.f);
      }
      wfft<E, false>(A, w.sb, w.tw, w.lane);
      const float2* pj = T.ph + (size_t)jr * N;
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
__device__ void w_scatter(const WRow& w, const Tabs& T, float om, int mode, const float2 (&u)[E],
                          float2 (&o)[E]) {
  const DevCtx& c = w.c;
  const float wdz = om * c.dz;
  const float2 iw = make_float2(0.f, mode == 0 ? -wdz : wdz);
  const bool t1 = c.ntaylor >= 1;
  float2 X[E];
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(c, w.lane, j, in);
    const float2 k0 = T.c0[x];
    const float2 k1 = t1 ? T.c1[x] : make_float2(0.f, 0.f);
    // transform input: u, or conj(c_1) u for the exact adjoint
    X[j] = (mode == 2 && t1) ? (in ? c_mulc(u[j], k1) : make_float2(0.f, 0.f)) : u[j];
    o[j] = in ? c_mul(iw, mode == 0 ? c_mul(k0, u[j]) : c_mulc(u[j], k0)) : make_float2(0.f, 0.f);
  }
  if (!t1) return;
  wfft<E, false>(X, w.sb, w.tw, w.lane);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    float kw = w.kx[w.lane + 32 * j] / om;
    X[j] = c_scale(X[j], kw * kw * c.invN);
  }
  wfft<E, true>(X, w.sb, w.tw, w.lane);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(c, w.lane, j, in);
    const float2 k1 = T.c1[x];
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
    bool in;
    const int x = xclamp(c, w.lane, j, in);
    if (!in) continue;
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

// shared-memory carve-up common to the pass kernels:
// [tw: N][kx: N][taper: nxg][exchange: kW x wbuf][ring][rows][image slots]
template <int E>
struct Carve {
  float2* tw;
  float* kx;
  float* taperN;
  float2* sb0;
  char* ring;
  char* rows;
  float2* slots;
  __device__ Carve(const DevCtx& c, const SlotLayout& L, bool with_slots) {
    extern __shared__ float4 smem4[];
    char* p = reinterpret_cast<char*>(smem4);
    auto take = [&](size_t bytes) {
      char* r = p;
      p += (bytes + 15) & ~size_t(15);
      return r;
    };
    tw = reinterpret_cast<float2*>(take((size_t)32 * E * 8));
    kx = reinterpret_cast<float*>(take((size_t)32 * E * 4));
    taperN = reinterpret_cast<float*>(take((size_t)c.nxg * 4));
    sb0 = reinterpret_cast<float2*>(take((size_t)kW * wbuf_len<E>() * 8));
    ring = take((size_t)L.nslots * L.bytes);
    rows = take((size_t)2 * kW * L.row_bytes);
    slots = reinterpret_cast<float2*>(take(with_slots ? (size_t)kW * c.nxg * 8 : 0));
  }
};

template <int E>
__device__ __forceinline__ void stage_static(const DevCtx& c, const Carve<E>& sm) {
  for (int i = threadIdx.x; i < 32 * E; i += blockDim.x) {
    sm.tw[i] = c.tw[i];
    sm.kx[i] = c.kx[i];
  }
  for (int i = threadIdx.x; i < c.nxg; i += blockDim.x) sm.taperN[i] = c.taperN[i];
}

// =============================================================== passes
// nonlinear modelling (wem_prop.cpp:52-74), as k_wem in kernels.cu
template <int E>
__global__ void __launch_bounds__(kW * 32, 1) kw_wem(DevCtx c, SlotLayout L, const Group* groups, float2* store,
                                                     float2* bins) {
  const Carve<E> sm(c, L, false);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  stage_static<E>(c, sm);
  const Group gp = groups[blockIdx.x];
  const bool act = warp < gp.n;
  const WRow w{c, sm.tw, sm.sb0 + warp * wbuf_len<E>(), sm.taperN, sm.kx, lane};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f], nz = c.nz, nxg = c.nxg;
  const size_t plane = (size_t)nz * nxg;
  float2* A = store + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  float2* wrow = reinterpret_cast<float2*>(sm.rows + (size_t)warp * 2 * L.row_bytes);
  float2 W[E];
  w_zero<E>(W);
  if (act) w_inject_src<E>(w, W, s, f, 0);
  ring.issue(0);
  cp_commit();
  ring.issue(1);
  cp_commit();
  for (int z = 0; z < nz; ++z) {
    __syncthreads();
    ring.issue(z + 2);
    cp_commit();
    cp_wait1();
    __syncthreads();
    if (!act) continue;
    const Tabs T = ring.tabs(z);
    w_record<E>(w, W, s, bin, z, bins);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 r = T.rc[x];
      if (in) A[(size_t)z * nxg + x] = c_mul(r, W[j]);
    }
    if (z == nz - 1) break;
    w_step_fwd<E>(w, T, W, W);
    w_inject_src<E>(w, W, s, f, z + 1);
  }
  // up sweep; each warp prefetches its stored row one depth ahead
  cp_wait0();
  __syncthreads();  // the stores of A are visible to the copies below; the ring is idle
  auto issue_row = [&](int d) {
    if (L.row_bytes && act && d >= 0) warp_copy(wrow + (size_t)(d & 1) * nxg, A + (size_t)d * nxg, nxg * 8, lane);
  };
  if (act) w_load<E>(c, lane, A + (size_t)(nz - 1) * nxg, W);
  ring.issue(nz - 1);
  issue_row(nz - 2);
  cp_commit();
  ring.issue(nz - 2);
  cp_commit();
  for (int z = nz - 1; z >= 0; --z) {
    __syncthreads();
    ring.issue(z - 2);
    issue_row(z - 2);
    cp_commit();
    cp_wait1();
    __syncthreads();
    if (!act) continue;
    w_record<E>(w, W, s, bin, z, bins);
    if (z == 0) break;
    const Tabs T = ring.tabs(z);
    w_step_fwd<E>(w, T, W, W);
    const float2* a = L.row_bytes ? wrow + (size_t)((z - 1) & 1) * nxg : A + (size_t)(z - 1) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 v = a[xclamp(c, lane, j, in)];
      if (in) W[j] = c_add(W[j], v);
    }
  }
  cp_wait0();
}

// Born forward, two sweeps per row (born_prop.cpp:75-113; k_born_fwd in kernels.cu)
template <int E>
__global__ void __launch_bounds__(kW * 32, 1) kw_born_fwd(DevCtx c, SlotLayout L, const Group* groups,
                                                          const float2* dm, const float2* drm, float2* storeA,
                                                          float2* storeB, float2* bins) {
  const Carve<E> sm(c, L, false);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  stage_static<E>(c, sm);
  const Group gp = groups[blockIdx.x];
  const bool act = warp < gp.n;
  const WRow w{c, sm.tw, sm.sb0 + warp * wbuf_len<E>(), sm.taperN, sm.kx, lane};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f], nz = c.nz, nxg = c.nxg;
  const size_t plane = (size_t)nz * nxg;
  float2* A = storeA + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* B = storeB + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  const float om = c.omega[f];
  const Ring ring{c, L, sm.ring, Src{dm, drm}, f};
  float2 bg[E], sd[E], t[E];
  w_zero<E>(bg);
  w_zero<E>(sd);
  if (act) w_inject_src<E>(w, bg, s, f, 0);
  ring.issue(0);
  cp_commit();
  ring.issue(1);
  cp_commit();
  for (int z = 0; z < nz; ++z) {
    __syncthreads();
    ring.issue(z + 2);
    cp_commit();
    cp_wait1();
    __syncthreads();
    if (!act) continue;
    const Tabs T = ring.tabs(z);
    w_record<E>(w, sd, s, bin, z, bins);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 r = T.rc[x], d = T.dr[x], q = T.dm[x];
      t[j] = in ? c_mul(bg[j], q) : make_float2(0.f, 0.f);
      if (in) {
        A[(size_t)z * nxg + x] = c_mul(r, bg[j]);
        B[(size_t)z * nxg + x] = c_add(c_mul(bg[j], d), c_mul(r, sd[j]));
      }
    }
    if (z == nz - 1) break;
    w_scatter<E>(w, T, om, 0, t, t);
#pragma unroll
    for (int j = 0; j < E; ++j) sd[j] = c_add(sd[j], t[j]);
    w_step_fwd<E>(w, T, sd, sd);
    w_step_fwd<E>(w, T, bg, bg);
    w_inject_src<E>(w, bg, s, f, z + 1);
  }
  cp_wait0();
  __syncthreads();
  if (act) {
    w_load<E>(c, lane, A + (size_t)(nz - 1) * nxg, bg);
    w_load<E>(c, lane, B + (size_t)(nz - 1) * nxg, sd);
  }
  ring.issue(nz - 1);
  cp_commit();
  ring.issue(nz - 2);
  cp_commit();
  for (int z = nz - 1; z >= 0; --z) {
    __syncthreads();
    ring.issue(z - 2);
    cp_commit();
    cp_wait1();
    __syncthreads();
    if (!act) continue;
    w_record<E>(w, sd, s, bin, z, bins);
    if (z == 0) break;
    if (lane == 0 && z >= 2) {
      l2_prefetch(A + (size_t)(z - 2) * nxg, nxg * 8);
      l2_prefetch(B + (size_t)(z - 2) * nxg, nxg * 8);
    }
    const Tabs T = ring.tabs(z);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 q = T.dm[xclamp(c, lane, j, in)];
      t[j] = in ? c_mul(bg[j], q) : make_float2(0.f, 0.f);
    }
    w_scatter<E>(w, T, om, 0, t, t);
#pragma unroll
    for (int j = 0; j < E; ++j) sd[j] = c_add(sd[j], t[j]);
    w_step_fwd<E>(w, T, sd, sd);
    w_step_fwd<E>(w, T, bg, bg);
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
  cp_wait0();
}

// image row of the group = sum over the CTA's rows of each warp's slot, in
// warp order (deterministic)
__device__ __forceinline__ void reduce_slots(const float2* slots, int nxg, int nw, float2* out) {
  for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
    float2 a = make_float2(0.f, 0.f);
    for (int k = 0; k < nw; ++k) a = c_add(a, slots[k * nxg + x]);
    out[x] = a;
  }
}

// Born adjoint, two sweeps per row (born_prop.cpp:178-216; k_born_adj in kernels.cu)
template <int E>
__global__ void __launch_bounds__(kW * 32, 1) kw_born_adj(DevCtx c, SlotLayout L, const Group* groups,
                                                          float2* storeBG, float2* storeT, const float2* bins,
                                                          float2* imgR, float2* imgS, int compat) {
  const Carve<E> sm(c, L, true);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  stage_static<E>(c, sm);
  const int nxg = c.nxg, nz = c.nz;
  float2* slot = sm.slots + warp * nxg;
  const Group gp = groups[blockIdx.x];
  const bool act = warp < gp.n;
  const WRow w{c, sm.tw, sm.sb0 + warp * wbuf_len<E>(), sm.taperN, sm.kx, lane};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg;
  float2* SBG = storeBG + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* ST = storeT + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* IR = imgR + (size_t)blockIdx.x * plane;
  float2* IS = imgS + (size_t)blockIdx.x * plane;
  const int scmode = compat ? 1 : 2;
  const float om = c.omega[f];
  const float2 zero = make_float2(0.f, 0.f);
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  // ---------------- down sweep: bg (Down of the source) and wu (Up^H of the data)
  float2 bg[E], wu[E];
  w_zero<E>(bg);
  w_zero<E>(wu);
  if (act) {
    w_inject_src<E>(w, bg, s, f, 0);
    w_inject_rec<E>(w, wu, s, bin, 0, bins);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      if (in) ST[x] = zero;
    }
  }
  ring.issue(0);
  cp_commit();
  ring.issue(1);
  cp_commit();
  for (int z = 0; z < nz; ++z) {
    __syncthreads();
    ring.issue(z + 2);
    cp_commit();
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      if (in) slot[x] = act ? c_mulc(wu[j], bg[j]) : zero;
    }
    cp_wait1();
    __syncthreads();
    reduce_slots(sm.slots, nxg, kW, IR + (size_t)z * nxg);
    if (!act) continue;
    w_store<E>(c, lane, SBG + (size_t)z * nxg, bg);
    if (z == nz - 1) continue;
    w_step_fwd<E>(w, ring.tabs(z), bg, bg);
    w_inject_src<E>(w, bg, s, f, z + 1);
    w_step_adj<E>(w, ring.tabs(z + 1), wu, wu);  // T[z+1]
    w_store<E>(c, lane, ST + (size_t)(z + 1) * nxg, wu);
    w_inject_rec<E>(w, wu, s, bin, z + 1, bins);
  }
  cp_wait0();
  __syncthreads();  // the down sweep's images are out of the slots; the ring is idle
  // ---------------- up sweep: bu (Up of R bg) and wd (Down^H of rec + conj(R) wu)
  float2 bu[E], wd[E], t[E];
  const bool keep_last = !compat || (c.ext ? (s == c.ns - 1) : (f == c.nfreq - 1));
  ring.issue(nz - 1);
  cp_commit();
  ring.issue(nz - 2);
  cp_commit();
  if (act && lane == 0) {
    l2_prefetch(SBG + (size_t)(nz - 2) * nxg, nxg * 8);
    l2_prefetch(ST + (size_t)(nz - 2) * nxg, nxg * 8);
  }
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(c, lane, j, in);
    if (in) slot[x] = zero;
  }
  for (int z = nz - 1; z >= 0; --z) {
    __syncthreads();
    ring.issue(z - 2);
    cp_commit();
    cp_wait1();
    __syncthreads();
    if (act && z == nz - 1) {
      const float2* rc = ring.tabs(nz - 1).rc;
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
    // LinUp^H at depth z: conj(bu) Sc^H_z T[z]
    if (act && z >= 1 && (z < nz - 1 || keep_last)) {
      w_load<E>(c, lane, ST + (size_t)z * nxg, t);
      w_scatter<E>(w, ring.tabs(z), om, scmode, t, t);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(c, lane, j, in);
        if (in) slot[x] = c_add(slot[x], c_mulc(t[j], bu[j]));
      }
    }
    __syncthreads();
    reduce_slots(sm.slots, nxg, kW, IS + (size_t)z * nxg);
    __syncthreads();
    if (z == 0) break;
    if (!act) continue;  // the slot of an idle warp stays zero
    if (lane == 0 && z >= 2) {
      l2_prefetch(SBG + (size_t)(z - 2) * nxg, nxg * 8);
      l2_prefetch(ST + (size_t)(z - 2) * nxg, nxg * 8);
    }
    const Tabs Tz = ring.tabs(z), Tp = ring.tabs(z - 1);
    // q = P^H_{z-1} wd;  LinDown^H: conj(bg[z-1]) Sc^H_{z-1} q
    w_step_adj<E>(w, Tp, wd, wd);  // wd holds q
    w_scatter<E>(w, Tp, om, scmode, wd, t);
    const float2* bgp = SBG + (size_t)(z - 1) * nxg;
    const float2* tp = ST + (size_t)(z - 1) * nxg;
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
      const float2 r = Tp.rc[xclamp(c, lane, j, in)];
      if (in) wd[j] = c_add(wd[j], c_mulc(t[j], r));
    }
    w_inject_rec<E>(w, wd, s, bin, z - 1, bins);
    // bu[z-1] = P_z bu + R[z-1] bg[z-1]
    w_step_fwd<E>(w, Tz, bu, bu);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(c, lane, j, in);
      const float2 r = Tp.rc[x], b = bgp[x];
      if (in) bu[j] = c_add(bu[j], c_mul(r, b));
    }
  }
  cp_wait0();
}

// ------------------------------------------------------ host side
template <int E>
size_t base_bytes(const DevCtx& c, bool slots) {
  auto r16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  return r16((size_t)32 * E * 8) + r16((size_t)32 * E * 4) + r16((size_t)c.nxg * 4) +
         r16((size_t)kW * wbuf_len<E>() * 8) + (slots ? r16((size_t)kW * c.nxg * 8) : 0);
}

// which: 0 WEM, 1 Born forward, 2 Born adjoint.  Lays out the ring (and the
// per-warp rows for WEM) and drops them when the shared memory does not fit.
template <int E>
SlotLayout slot_layout(const DevCtx& c, int which, int limit) {
  SlotLayout L{};
  int off = 0;
  auto put = [&](int bytes) {
    int o = off;
    off += (bytes + 15) & ~15;
    return o;
  };
  const int rowb = c.nxg * 8;
  L.ph = put(c.nref * c.N * 8);
  L.fac = c.fac ? put(rowb) : -1;
  const bool need_ref = (!c.fac || c.nref > 1);
  L.ref = (need_ref && c.nxg % 16 == 0) ? put(c.nxg) : -1;
  L.rc = put(rowb);
  L.c0 = which != 0 ? put(rowb) : -1;
  L.c1 = (which != 0 && c.ntaylor >= 1) ? put(rowb) : -1;
  L.dm = which == 1 ? put(rowb) : -1;
  L.dr = which == 1 ? put(rowb) : -1;
  L.bytes = off;
  L.nslots = 3;
  L.row_bytes = which == 0 ? rowb : 0;
  const bool slots = which == 2;
  auto total = [&]() { return base_bytes<E>(c, slots) + (size_t)L.nslots * L.bytes + (size_t)2 * kW * L.row_bytes; };
  if (total() > (size_t)limit) L.row_bytes = 0;
  if (total() > (size_t)limit) {
    L = SlotLayout{};
    L.ph = L.fac = L.ref = L.rc = L.c0 = L.c1 = L.dm = L.dr = -1;
  }
  return L;
}

template <int E>
size_t smem_w(const DevCtx& c, int which, const SlotLayout& L) {
  return base_bytes<E>(c, which == 2) + (size_t)L.nslots * L.bytes + (size_t)2 * kW * L.row_bytes;
}

template <int E>
void launch_pass_w(int which, const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm,
                   float2* s1, float2* s2, float2* bins, float2* ir, float2* is, int compat, cudaStream_t st) {
  const int limit = max_smem_per_block();
  const SlotLayout L = slot_layout<E>(c, which, limit);
  const size_t sm = smem_w<E>(c, which, L);
  if (which == 0) {
    cudaFuncSetAttribute(kw_wem<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kw_wem<E><<<ng, kW * 32, sm, st>>>(c, L, g, s1, bins);
    note_launch();
  } else if (which == 1) {
    cudaFuncSetAttribute(kw_born_fwd<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kw_born_fwd<E><<<ng, kW * 32, sm, st>>>(c, L, g, dm, drm, s1, s2, bins);
    note_launch();
  } else {
    cudaFuncSetAttribute(kw_born_adj<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kw_born_adj<E><<<ng, kW * 32, sm, st>>>(c, L, g, s1, s2, bins, ir, is, compat);
    note_launch();
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
  const int which = slots ? 2 : 0;
  return smem_w<E>(c, which, slot_layout<E>(c, which, max_smem_per_block()));
}

}  // namespace wg
