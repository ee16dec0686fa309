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
#include <mutex>
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
  bool has_fac;            // SSF split-step table present
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
  t.has_fac = c.fac != nullptr;
  t.ph = c.ph + ((size_t)f * c.nz + z) * c.nref * c.N;
  t.fac = c.fac ? c.fac + ((size_t)f * c.nz + z) * c.nxg : nullptr;
  t.ref = c.ref + zo;
  t.rc = rc_row(c, f, z);
  t.c0 = c.sc ? c.sc + (size_t)m * (c.ntaylor + 1) * plane + (size_t)z * c.nxg : nullptr;
  t.c1 = (c.sc && c.ntaylor >= 1) ? t.c0 + plane : nullptr;
  t.dm = s.dm ? s.dm + pert_off(c, f, z) : nullptr;
  t.dr = s.drm ? s.drm + pert_off(c, f, z) : nullptr;
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
  // every table of the depth from its slot (the caller guarantees that the
  // layout holds all tables it reads); pointers stay in the shared window
  __device__ Tabs stabs(int d) const {
    const char* p = slot(d);
    Tabs t;
    t.has_fac = c.fac != nullptr;
    t.ph = reinterpret_cast<const float2*>(p + L.ph);
    t.fac = reinterpret_cast<const float2*>(p + L.fac);
    t.ref = reinterpret_cast<const signed char*>(p + L.ref);
    t.rc = reinterpret_cast<const float2*>(p + L.rc);
    t.c0 = reinterpret_cast<const float2*>(p + L.c0);
    t.c1 = reinterpret_cast<const float2*>(p + L.c1);
    t.dm = reinterpret_cast<const float2*>(p + L.dm);
    t.dr = reinterpret_cast<const float2*>(p + L.dr);
    return t;
  }
};

struct WRow {
  const DevCtx& c;
  const float2* tw;  // [N] shared
  float2* sb;        // warp exchange buffer
  const float* taperN;
  const float* kx;
  int lane;
  // FFT zero pad and grid width of the row; kernels built for tap = 0 pass
  // the constants 0 and N, so every point is known to be on the grid
  int tap, nxg;
};

// clamped grid index of register j: loads through it are issued without a
// branch (so a lane's E loads are all in flight together) and the result is
// selected with `in` afterwards
__device__ __forceinline__ int xclamp(const WRow& w, int j, bool& in) {
  const int x = w.lane + 32 * j - w.tap;
  in = (unsigned)x < (unsigned)w.nxg;
  return in ? x : 0;
}

template <int E>
__device__ __forceinline__ void w_load(const WRow& w, const float2* row, float2 (&v)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const float2 a = row[xclamp(w, j, in)];
    v[j] = in ? a : make_float2(0.f, 0.f);
  }
}

template <int E>
__device__ __forceinline__ void w_store(const WRow& w, float2* row, const float2 (&v)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(w, j, in);
    if (in) row[x] = v[j];
  }
}

template <int E>
__device__ __forceinline__ void w_zero(float2 (&v)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) v[j] = make_float2(0.f, 0.f);
}

// ---------------------------------------------------------------- row ops
// Every transform of a depth step is one "op": X <- pre(X); X <- FFT(X);
// X <- mid(X); X <- IFFT(X); post(X).  A pass kernel runs the ops of a depth
// in a loop that is not unrolled, so the kernel holds one forward and one
// inverse transform per sweep whatever the number of ops, and only the state
// rows plus the op's X are live in registers.  MR (several references) runs
// the reference loop of SSF.cpp / PSPI.cpp around the transform pair; the
// single-reference kernels are instantiated without it.

// A row of 32 E points in shared memory in the registers' layout (lane t
// holds points t + 32 j): the several-reference kernels keep the sum over
// references here instead of in registers.  Each lane reads and writes only
// its own points, so no synchronisation is needed.
struct SRow {
  float2* p;  // this lane's point j = 0
  __device__ __forceinline__ float2& operator[](int j) const { return p[32 * j]; }
};

// forward step, mid: X *= phase row of reference jr (SSF.cpp:18-23, PSPI.cpp:15-20)
template <int E>
__device__ __forceinline__ void fwd_mid(const WRow& w, const Tabs& T, int jr, float2 (&X)[E]) {
  const float2* pj = T.ph + (size_t)jr * 32 * E;
#pragma unroll
  for (int j = 0; j < E; ++j) X[j] = c_mul(X[j], pj[w.lane + 32 * j]);
}

// forward step, post: o = split step x taper x X / N at the points whose
// reference is jr (SSF.cpp:24-31, PSPI.cpp:21-28).  Single reference: the
// split-step table is zero where a point has no reference, so the index is
// only read without it (PSPI).  MR: o keeps its value at other points and is
// cleared at jr = 0.
template <int E, bool MR, class O>
__device__ __forceinline__ void fwd_post(const WRow& w, const Tabs& T, int jr, const float2 (&X)[E], O&& o) {
  const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(w, j, in);
    if (!MR) {
      if (T.has_fac) {
        const float2 fx = T.fac[x];
        o[j] = in ? c_mul(X[j], fx) : zero;
      } else {
        const float tp = w.taperN[x];
        const int r = T.ref[x];
        o[j] = (in && r == 0) ? c_scale(X[j], tp) : zero;
      }
    } else {
      const int r = T.ref[x];
      const float2 v = T.has_fac ? c_mul(X[j], T.fac[x]) : c_scale(X[j], w.taperN[x]);
      o[j] = (in && r == jr) ? v : (jr == 0 ? zero : o[j]);
    }
  }
}

// adjoint step, pre: X = conj(split step) x taper x d / N at the points of
// reference jr (SSF.cpp:36-45, PSPI.cpp:33-41)
template <int E, bool MR>
__device__ __forceinline__ void adj_pre(const WRow& w, const Tabs& T, int jr, const float2 (&d)[E], float2 (&X)[E]) {
  const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(w, j, in);
    if (!MR) {
      if (T.has_fac) {
        const float2 fx = T.fac[x];
        X[j] = in ? c_mulc(d[j], fx) : zero;
      } else {
        const float tp = w.taperN[x];
        const int r = T.ref[x];
        X[j] = (in && r == 0) ? c_scale(d[j], tp) : zero;
      }
    } else {
      const int r = T.ref[x];
      const float2 v = T.has_fac ? c_mulc(d[j], T.fac[x]) : c_scale(d[j], w.taperN[x]);
      X[j] = (in && r == jr) ? v : zero;
    }
  }
}

// adjoint step, mid: X *= conj(phase row jr); MR sums the references'
// spectra in Y and returns true once X holds the sum (the inverse transform
// runs after the last reference only)
template <int E, bool MR, class YR>
__device__ __forceinline__ bool adj_mid(const WRow& w, const Tabs& T, int jr, float2 (&X)[E], YR&& Y) {
  const float2* pj = T.ph + (size_t)jr * 32 * E;
  if constexpr (!MR) {
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = c_mulc(X[j], pj[w.lane + 32 * j]);
    return true;
  } else {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const float2 v = c_mulc(X[j], pj[w.lane + 32 * j]);
      Y[j] = jr == 0 ? v : c_add(Y[j], v);
    }
    if (jr + 1 < w.c.nref) return false;
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = Y[j];
    return true;
  }
}

// adjoint step, post: o = X on the model grid, zero in the FFT pad
template <int E>
__device__ __forceinline__ void adj_post(const WRow& w, const float2 (&X)[E], float2 (&o)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    xclamp(w, j, in);
    o[j] = in ? X[j] : make_float2(0.f, 0.f);
  }
}

// Forward step with several references (SSF.cpp:14-31, PSPI.cpp:11-28):
// the padded row is transformed once and every reference's field is the
// inverse transform of that spectrum times its phase row, selected into Y.
// X holds the row on entry; the caller's state row is dead meanwhile.
template <int E, class O>
__device__ __forceinline__ void fwd_step_mr(const WRow& w, const Tabs& T, int nref, float2 (&X)[E], O&& Y) {
  wfft<E, false>(X, w.sb, w.tw, w.lane);
#pragma unroll 1
  for (int jr = 0; jr < nref; ++jr) {
    float2 Z[E];
#pragma unroll
    for (int j = 0; j < E; ++j) Z[j] = X[j];
    fwd_mid<E>(w, T, jr, Z);
    wfft<E, true>(Z, w.sb, w.tw, w.lane);
    fwd_post<E, true>(w, T, jr, Z, Y);
  }
}

// Taylor Born scatter (Scatter.cpp:35-111) for ntaylor <= 1; mode 0 forward,
// 1 adjoint as coded (filter before scaling), 2 exact adjoint.
// pre: the filter's input, u or conj(c_1) u (exact adjoint)
template <int E>
__device__ __forceinline__ void sc_pre(const WRow& w, const Tabs& T, int mode, const float2 (&u)[E], float2 (&X)[E]) {
#pragma unroll
  for (int j = 0; j < E; ++j) {
    if (mode == 2) {
      bool in;
      const float2 k1 = T.c1[xclamp(w, j, in)];
      X[j] = in ? c_mulc(u[j], k1) : make_float2(0.f, 0.f);
    } else {
      X[j] = u[j];
    }
  }
}
// mid: the (k / omega)^2 filter, with the 1/N of the inverse transform
// (one division per call: k^2 times 1 / omega^2)
template <int E>
__device__ __forceinline__ void sc_mid(const WRow& w, float om, float2 (&X)[E]) {
  const float s = w.c.invN / (om * om);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const float k = w.kx[w.lane + 32 * j];
    X[j] = c_scale(X[j], k * k * s);
  }
}
// (k / omega)^2 X: the filtered spectrum of a row whose transform is X / N
// away (the inverse transform and the filter's forward one cancel when no
// point is masked between them)
template <int E>
__device__ __forceinline__ void sc_spec(const WRow& w, float om, const float2 (&X)[E], float2 (&Y)[E]) {
  const float s = 1.f / (om * om);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const float k = w.kx[w.lane + 32 * j];
    Y[j] = c_scale(X[j], k * k * s);
  }
}
// post, one point: i w dz (c_0 u + c_1 filtered) with the mode's conjugations;
// x is the filtered value (ignored when ntaylor = 0).  iw = (0, +-w dz)
// (sc_iw): the product by it is the scaled swap, two multiplies (the
// complex product's fused terms with the zero real part give the same
// values, up to the sign of a zero)
__device__ __forceinline__ float2 sc_val(float2 iw, int mode, bool t1, float2 k0, float2 k1, float2 u, float2 x) {
  float2 y = mode == 0 ? c_mul(k0, u) : c_mulc(u, k0);
  if (t1) y = c_add(y, mode == 0 ? c_mul(k1, x) : (mode == 1 ? c_mulc(x, k1) : x));
  return make_float2(-__fmul_rn(iw.y, y.y), __fmul_rn(iw.y, y.x));
}
__device__ __forceinline__ float2 sc_iw(const DevCtx& c, float om, int mode) {
  const float wdz = om * c.dz;
  return make_float2(0.f, mode == 0 ? -wdz : wdz);
}

// add gs[g] wavelet into the row of shot s at depth z for every source
// point of the shot (Injection.cpp:8-19)
template <int E>
__device__ __forceinline__ void w_inject_src(const WRow& w, float2 (&v)[E], int s, int f, int z) {
  const DevCtx& c = w.c;
  if (c.sz[s] != z) return;
  const float2 wv = c.wave[f];
  const int p0 = c.sptr ? c.sptr[s] : s, p1 = c.sptr ? c.sptr[s + 1] : s + 1;
  for (int pt = p0; pt < p1; ++pt)
    for (int g = -c.ngs; g <= c.ngs; ++g) {
      int x = c.sx[pt] + g + c.pad;
      if (x < 0 || x >= c.nxg) continue;
      int n = x + w.tap;
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
  for (int j = 0; j < E; ++j) w.sb[swz<E>(w.lane + 32 * j)] = v[j];
  __syncwarp();
  for (int k = k0 + w.lane; k < k1; k += 32) {
    const int x0 = c.rxs[k] + c.pad;
    float2 acc = make_float2(0.f, 0.f);
    for (int g = -c.ngr; g <= c.ngr; ++g) {
      int x = x0 + g;
      if (x >= 0 && x < c.nxg) acc = c_add(acc, c_scale(w.sb[swz<E>(x + w.tap)], c.gr[g + c.ngr]));
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
    const int x = xclamp(w, j, in);
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
// [tw: N][kx: N][taper: nxg][exchange: nbuf x wbuf][ring][rows][image slots]
template <int E>
struct Carve {
  float2* tw;
  float* kx;
  float* taperN;
  float2* sb0;
  char* ring;
  char* rows;
  float2* slots;
  float2* yrow;  // several references: one row per warp for the sum over references
  __device__ Carve(const DevCtx& c, const SlotLayout& L, bool with_slots, int nbuf = kW, bool with_taper = true) {
    extern __shared__ float4 smem4[];
    char* p = reinterpret_cast<char*>(smem4);
    auto take = [&](size_t bytes) {
      char* r = p;
      p += (bytes + 15) & ~size_t(15);
      return r;
    };
    tw = reinterpret_cast<float2*>(take((size_t)32 * E * 8));
    kx = reinterpret_cast<float*>(take((size_t)32 * E * 4));
    taperN = with_taper ? reinterpret_cast<float*>(take((size_t)c.nxg * 4)) : nullptr;
    sb0 = reinterpret_cast<float2*>(take((size_t)nbuf * wbuf_len<E>() * 8));
    ring = take((size_t)L.nslots * L.bytes);
    rows = take((size_t)2 * nbuf * L.row_bytes);
    slots = reinterpret_cast<float2*>(take(with_slots ? (size_t)kW * c.nxg * 8 : 0));
    yrow = reinterpret_cast<float2*>(take(ysum_rows(c, with_slots) * 32 * E * 8));
  }
  // rows of reference sums in shared memory: the several-reference modelling
  // and Born forward; the Born adjoint (with image slots) keeps its sum in
  // registers, since its shared memory is taken by the slots and the table
  // ring (with the sum there too the ring no longer fits for N = 1024 and the
  // pass ran 35 % slower)
  __device__ static size_t ysum_rows(const DevCtx& c, bool with_slots) { return c.nref > 1 && !with_slots ? kW : 0; }
  // this lane's view of warp `warp`'s reference-sum row
  __device__ SRow ysum(int warp, int lane) const { return SRow{yrow + (size_t)warp * 32 * E + lane}; }
};

// twiddles in the per-stage layout of wfft.cuh (gathered from the natural
// table W_N^t), k grid and taper
template <int E>
__device__ __forceinline__ void stage_static(const DevCtx& c, const Carve<E>& sm) {
  constexpr int N = 32 * E;
  for (int i = threadIdx.x; i < tw_entries<E>(); i += blockDim.x) {
    int S = 1, L = WPlan<E>::r(0), off = 0;
    while (S < WPlan<E>::n - 1 && i >= off + (WPlan<E>::r(S) - 1) * L) {
      off += (WPlan<E>::r(S) - 1) * L;
      L *= WPlan<E>::r(S);
      ++S;
    }
    const int R = WPlan<E>::r(S), r = (i - off) / L + 1, l = (i - off) % L;
    sm.tw[i] = c.tw[r * l * (N / (L * R))];
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) sm.kx[i] = c.kx[i];
  if (sm.taperN)
    for (int i = threadIdx.x; i < c.nxg; i += blockDim.x) sm.taperN[i] = c.taperN[i];
}

// =============================================================== passes
// nonlinear modelling (wem_prop.cpp:52-74), as k_wem in kernels.cu
template <int E, bool MR, bool NT, int R>
__global__ void __launch_bounds__(R * 32, 1) kw_wem(DevCtx c, SlotLayout L, const Group* groups, float2* store,
                                                    float2* bins) {
  const Carve<E> sm(c, L, false, R, R > 1 || !c.fac);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  stage_static<E>(c, sm);
  const Group gp = groups[blockIdx.x];
  const bool act = warp < gp.n;
  const WRow w{c, sm.tw, sm.sb0 + warp * wbuf_len<E>(), sm.taperN, sm.kx, lane, NT ? 0 : c.tap, NT ? 32 * E : c.nxg};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f], nz = c.nz, nxg = c.nxg;
  const int nj = MR ? c.nref : 1;
  const size_t plane = (size_t)nz * nxg;
  float2* A = store + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* BG = c.bg_store ? c.bg_store + (size_t)(gp.row0 + (act ? warp : 0)) * plane : nullptr;
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  float2* wrow = reinterpret_cast<float2*>(sm.rows + (size_t)warp * 2 * L.row_bytes);
  float2 W[E], X[E];
  const SRow Y = sm.ysum(warp, lane);  // used by the several-reference instantiation only
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
      const int x = xclamp(w, j, in);
      const float2 r = T.rc[x];
      if (in) A[(size_t)z * nxg + x] = c_mul(r, W[j]);
    }
    // the down field itself for the Born adjoint of the FWI gradient
    if (BG) w_store<E>(w, BG + (size_t)z * nxg, W);
    if (z == nz - 1) break;
    // W = P_z W
    if constexpr (MR) {
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = W[j];
      fwd_step_mr<E>(w, T, nj, X, Y);
#pragma unroll
      for (int j = 0; j < E; ++j) W[j] = Y[j];
    } else {
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = W[j];
      wfft<E, false>(X, w.sb, w.tw, lane);
      fwd_mid<E>(w, T, 0, X);
      wfft<E, true>(X, w.sb, w.tw, lane);
      fwd_post<E, false>(w, T, 0, X, W);
    }
    w_inject_src<E>(w, W, s, f, z + 1);
  }
  // up sweep; each warp prefetches its stored row one depth ahead
  cp_wait0();
  __syncthreads();  // the stores of A are visible to the copies below; the ring is idle
  auto issue_row = [&](int d) {
    if (L.row_bytes && act && d >= 0) warp_copy(wrow + (size_t)(d & 1) * nxg, A + (size_t)d * nxg, nxg * 8, lane);
  };
  if (act) w_load<E>(w, A + (size_t)(nz - 1) * nxg, W);
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
    // without the shared-memory row, bring the row of the next depth into L2
    if (!L.row_bytes && lane == 0 && z >= 2) l2_prefetch(A + (size_t)(z - 2) * nxg, nxg * 8);
    const Tabs T = ring.tabs(z);
    // W = P_z W + R[z-1] down[z-1]
    if constexpr (MR) {
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = W[j];
      fwd_step_mr<E>(w, T, nj, X, Y);
#pragma unroll
      for (int j = 0; j < E; ++j) W[j] = Y[j];
    } else {
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = W[j];
      wfft<E, false>(X, w.sb, w.tw, lane);
      fwd_mid<E>(w, T, 0, X);
      wfft<E, true>(X, w.sb, w.tw, lane);
      fwd_post<E, false>(w, T, 0, X, W);
    }
    const float2* a = L.row_bytes ? wrow + (size_t)((z - 1) & 1) * nxg : A + (size_t)(z - 1) * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const float2 v = a[xclamp(w, j, in)];
      if (in) W[j] = c_add(W[j], v);
    }
  }
  cp_wait0();
}

// Born forward, two sweeps per row (born_prop.cpp:75-113; k_born_fwd in kernels.cu).
// Ops of a depth: 0 scatter of bg dm into sd, 1 sd = P sd, 2 bg = P bg.
template <int E, bool MR>
__global__ void __launch_bounds__(kW * 32, 1) kw_born_fwd(DevCtx c, SlotLayout L, const Group* groups,
                                                          const float2* dm, const float2* drm, float2* storeA,
                                                          float2* storeB, float2* bins) {
  const Carve<E> sm(c, L, false);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  stage_static<E>(c, sm);
  const Group gp = groups[blockIdx.x];
  const bool act = warp < gp.n;
  const WRow w{c, sm.tw, sm.sb0 + warp * wbuf_len<E>(), sm.taperN, sm.kx, lane, c.tap, c.nxg};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f], nz = c.nz, nxg = c.nxg;
  const size_t plane = (size_t)nz * nxg;
  float2* A = storeA + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* B = storeB + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  const float om = c.omega[f];
  const float2 iw = sc_iw(c, om, 0);
  const bool t1 = c.ntaylor >= 1;
  const Ring ring{c, L, sm.ring, Src{dm, drm}, f};
  const float2 zero = make_float2(0.f, 0.f);
  float2 bg[E], sd[E], X[E];
  const SRow Y = sm.ysum(warp, lane);  // used by the several-reference instantiation only
  w_zero<E>(bg);
  w_zero<E>(sd);
  if (act) w_inject_src<E>(w, bg, s, f, 0);

  // the three ops of one depth with tables T; up adds the stored rows
  // (a: A[z-1], b: B[z-1]) after the steps, down injects the source
  auto depth_ops = [&](const Tabs& T, int znext, const float2* a, const float2* b) {
    // several references: ops 1 and 2 follow the loop, written out so that
    // the stepped row is dead while its spectrum and transform are live
#pragma unroll 1
    for (int k = 0; k < (MR ? 1 : 3); ++k) {
      const int nj = 1;
#pragma unroll 1
      for (int jr = 0; jr < nj; ++jr) {
        if (k == 0) {
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const float2 q = T.dm[xclamp(w, j, in)];
            X[j] = in ? c_mul(bg[j], q) : zero;
          }
        } else if (k == 1) {
#pragma unroll
          for (int j = 0; j < E; ++j) X[j] = sd[j];
        } else {
#pragma unroll
          for (int j = 0; j < E; ++j) X[j] = bg[j];
        }
        if (k > 0 || t1) {
          wfft<E, false>(X, w.sb, w.tw, lane);
          if (k == 0) sc_mid<E>(w, om, X);
          else fwd_mid<E>(w, T, jr, X);
          wfft<E, true>(X, w.sb, w.tw, lane);
        }
        if (k == 0) {
          // sd += Sc_z (bg dm)
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const int x = xclamp(w, j, in);
            const float2 q = T.dm[x], k0 = T.c0[x], k1 = t1 ? T.c1[x] : zero;
            const float2 v = sc_val(iw, 0, t1, k0, k1, c_mul(bg[j], q), X[j]);
            if (in) sd[j] = c_add(sd[j], v);
          }
        } else if constexpr (!MR) {
          if (k == 1) fwd_post<E, false>(w, T, jr, X, sd);
          else fwd_post<E, false>(w, T, jr, X, bg);
        }
      }
    }
    if constexpr (MR) {
      // sd = P sd, then bg = P bg
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = sd[j];
      fwd_step_mr<E>(w, T, c.nref, X, Y);
#pragma unroll
      for (int j = 0; j < E; ++j) sd[j] = Y[j];
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = bg[j];
      fwd_step_mr<E>(w, T, c.nref, X, Y);
#pragma unroll
      for (int j = 0; j < E; ++j) bg[j] = Y[j];
    }
    if (a) {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xclamp(w, j, in);
        const float2 va = a[x], vb = b[x];
        if (in) {
          bg[j] = c_add(bg[j], va);
          sd[j] = c_add(sd[j], vb);
        }
      }
    } else {
      w_inject_src<E>(w, bg, s, f, znext);
    }
  };

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
    if (!c.no_fwd_record) w_record<E>(w, sd, s, bin, z, bins);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(w, j, in);
      const float2 r = T.rc[x], d = T.dr[x];
      if (in) {
        A[(size_t)z * nxg + x] = c_mul(r, bg[j]);
        B[(size_t)z * nxg + x] = c_add(c_mul(bg[j], d), c_mul(r, sd[j]));
      }
    }
    if (z == nz - 1) break;
    depth_ops(T, z + 1, nullptr, nullptr);
  }
  cp_wait0();
  __syncthreads();
  if (act) {
    w_load<E>(w, A + (size_t)(nz - 1) * nxg, bg);
    w_load<E>(w, B + (size_t)(nz - 1) * nxg, sd);
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
    depth_ops(ring.tabs(z), z - 1, A + (size_t)(z - 1) * nxg, B + (size_t)(z - 1) * nxg);
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

// Born adjoint, two sweeps per row (born_prop.cpp:178-216; k_born_adj in kernels.cu).
// Down sweep, depth z: image IR[z] += conj(wu) bg, then ops bg = P_z bg and
// wu = P^H_{z+1} wu (= T[z+1], stored).  Up sweep, iteration z = nz .. 1
// accumulates image row z - 1: ops q = P^H_{z-1} wd (B), LinDown^H
// conj(bg[z-1]) Sc^H_{z-1} q (C), bu = P_z bu + R[z-1] bg[z-1] (D), LinUp^H
// conj(bu[z-1]) Sc^H_{z-1} T[z-1] (A).
template <int E, bool MR>
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
  const WRow w{c, sm.tw, sm.sb0 + warp * wbuf_len<E>(), sm.taperN, sm.kx, lane, c.tap, c.nxg};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg;
  float2* SBG = storeBG + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* ST = storeT + (size_t)(gp.row0 + (act ? warp : 0)) * plane;
  float2* IR = imgR + (size_t)blockIdx.x * plane;
  float2* IS = imgS + (size_t)blockIdx.x * plane;
  const int scmode = compat ? 1 : 2;
  const float om = c.omega[f];
  const float2 iw = sc_iw(c, om, scmode);
  const bool t1 = c.ntaylor >= 1;
  const int nj_step = MR ? c.nref : 1;
  const float2 zero = make_float2(0.f, 0.f);
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  float2 X[E];
  float2 Y[MR ? E : 1];  // the sum over references (in registers: see Carve::ysum_rows)
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
      const int x = xclamp(w, j, in);
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
      const int x = xclamp(w, j, in);
      if (in) slot[x] = act ? c_mulc(wu[j], bg[j]) : zero;
    }
    cp_wait1();
    __syncthreads();
    reduce_slots(sm.slots, nxg, kW, IR + (size_t)z * nxg);
    if (!act) continue;
    w_store<E>(w, SBG + (size_t)z * nxg, bg);
    if (z == nz - 1) continue;
    if constexpr (MR) {
      // bg = P bg: one forward transform for all references; the bg row
      // is dead until the references' sum replaces it
#pragma unroll
      for (int j = 0; j < E; ++j) X[j] = bg[j];
      fwd_step_mr<E>(w, ring.tabs(z), nj_step, X, Y);
#pragma unroll
      for (int j = 0; j < E; ++j) bg[j] = Y[j];
      w_inject_src<E>(w, bg, s, f, z + 1);
    }
#pragma unroll 1
    for (int k = MR ? 1 : 0; k < 2; ++k) {
      const Tabs T = ring.tabs(z + k);
      const int nj = nj_step;
#pragma unroll 1
      for (int jr = 0; jr < nj; ++jr) {
        if (k == 0) {
#pragma unroll
          for (int j = 0; j < E; ++j) X[j] = bg[j];
        } else {
          adj_pre<E, MR>(w, T, jr, wu, X);
        }
        wfft<E, false>(X, w.sb, w.tw, lane);
        if (k == 0) fwd_mid<E>(w, T, jr, X);
        else if (!adj_mid<E, MR>(w, T, jr, X, Y)) continue;
        wfft<E, true>(X, w.sb, w.tw, lane);
        if (k == 0) {
          if constexpr (MR) fwd_post<E, true>(w, T, jr, X, Y);
          else fwd_post<E, false>(w, T, jr, X, bg);
        } else {
          adj_post<E>(w, X, wu);
        }
      }
      if (k == 0) {
        if constexpr (MR) {
#pragma unroll
          for (int j = 0; j < E; ++j) bg[j] = Y[j];
        }
        w_inject_src<E>(w, bg, s, f, z + 1);
      } else {
        w_store<E>(w, ST + (size_t)(z + 1) * nxg, wu);  // T[z+1]
        w_inject_rec<E>(w, wu, s, bin, z + 1, bins);
      }
    }
  }
  cp_wait0();
  __syncthreads();  // the down sweep's images are out of the slots; the ring is idle
  // ---------------- up sweep: bu (Up of R bg) and wd (Down^H of rec + conj(R) wu)
  float2 bu[E], wd[E];
  const bool keep_last = keep_last_row(c, compat, f, s);
#pragma unroll
  for (int j = 0; j < E; ++j) {
    bool in;
    const int x = xclamp(w, j, in);
    if (in) slot[x] = zero;
  }
  ring.issue(nz - 1);
  cp_commit();
  for (int z = nz; z >= 1; --z) {
    __syncthreads();
    ring.issue(z - 2);
    cp_commit();
    cp_wait1();
    __syncthreads();
    if (act) {
      const Tabs Tp = ring.tabs(z - 1);
      const float2* bgp = SBG + (size_t)(z - 1) * nxg;
      const float2* tp = ST + (size_t)(z - 1) * nxg;
      if (lane == 0 && z >= 2) {
        l2_prefetch(SBG + (size_t)(z - 2) * nxg, nxg * 8);
        l2_prefetch(ST + (size_t)(z - 2) * nxg, nxg * 8);
      }
      if (z == nz) {
        // bu[nz-1] = R bg[nz-1]; wd[nz-1] = conj(R) (T[nz-1] + rec) + rec
        w_load<E>(w, bgp, bu);
        w_load<E>(w, tp, X);
        w_inject_rec<E>(w, X, s, bin, nz - 1, bins);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          bool in;
          const float2 r = Tp.rc[xclamp(w, j, in)];
          bu[j] = in ? c_mul(r, bu[j]) : zero;
          wd[j] = in ? c_mulc(X[j], r) : zero;
        }
        if (!c.no_fwd_record) w_inject_rec<E>(w, wd, s, bin, nz - 1, bins);
      }
      if constexpr (MR) {
        // D first (it is independent of B and C): bu[z-1] = P_z bu +
        // R[z-1] bg[z-1], one forward transform for all references
        if (z < nz && z >= 2) {
#pragma unroll
          for (int j = 0; j < E; ++j) X[j] = bu[j];
          fwd_step_mr<E>(w, ring.tabs(z), nj_step, X, Y);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const int x = xclamp(w, j, in);
            const float2 r = Tp.rc[x], b = bgp[x];
            bu[j] = in ? c_fma(Y[j], r, b) : Y[j];
          }
        }
      }
#pragma unroll 1
      for (int k = 0; k < 4; ++k) {
        // k: 0 B, 1 C, 2 D, 3 A
        if (MR && k == 2) continue;
        const bool on = k < 2 ? (z < nz) : (k == 2 ? (z < nz && z >= 2) : (z >= 2 && (z < nz || keep_last)));
        if (!on) continue;
        const bool step = (k == 0 || k == 2);
        const Tabs T = k == 2 ? ring.tabs(z) : Tp;
        const int nj = step ? nj_step : 1;
#pragma unroll 1
        for (int jr = 0; jr < nj; ++jr) {
          // pre
          if (k == 0) {
            adj_pre<E, MR>(w, T, jr, wd, X);
          } else if (k == 2) {
#pragma unroll
            for (int j = 0; j < E; ++j) X[j] = bu[j];
          } else if (t1) {
            if (k == 1) {
              sc_pre<E>(w, T, scmode, wd, X);
            } else {
              w_load<E>(w, tp, X);
              if (scmode == 2) sc_pre<E>(w, T, scmode, X, X);
            }
          }
          if (step || t1) {
            wfft<E, false>(X, w.sb, w.tw, lane);
            if (k == 0) {
              if (!adj_mid<E, MR>(w, T, jr, X, Y)) continue;
            } else if (k == 2) {
              fwd_mid<E>(w, T, jr, X);
            } else {
              sc_mid<E>(w, om, X);
            }
            wfft<E, true>(X, w.sb, w.tw, lane);
          }
          // post
          if (k == 0) {
            adj_post<E>(w, X, wd);  // wd holds q
          } else if (k == 2) {
            if constexpr (MR) fwd_post<E, true>(w, T, jr, X, Y);
            else fwd_post<E, false>(w, T, jr, X, bu);
          } else if (k == 1) {
            // LinDown^H: slot = conj(bg[z-1]) Sc^H_{z-1} q
#pragma unroll
            for (int j = 0; j < E; ++j) {
              bool in;
              const int x = xclamp(w, j, in);
              const float2 k0 = T.c0[x], k1 = t1 ? T.c1[x] : zero, b = bgp[x];
              const float2 v = sc_val(iw, scmode, t1, k0, k1, wd[j], X[j]);
              if (in) slot[x] = c_mulc(v, b);
            }
          } else {
            // LinUp^H: slot += conj(bu[z-1]) Sc^H_{z-1} T[z-1]
#pragma unroll
            for (int j = 0; j < E; ++j) {
              bool in;
              const int x = xclamp(w, j, in);
              const float2 k0 = T.c0[x], k1 = t1 ? T.c1[x] : zero, u = tp[x];
              const float2 v = sc_val(iw, scmode, t1, k0, k1, u, X[j]);
              if (in) slot[x] = c_fmac(slot[x], v, bu[j]);
            }
          }
        }
        if (k == 1 && z >= 2) {
          // wd[z-1] = q + rec + conj(R[z-1]) (T[z-1] + rec)
          w_load<E>(w, tp, X);
          w_inject_rec<E>(w, X, s, bin, z - 1, bins);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const float2 r = T.rc[xclamp(w, j, in)];
            if (in) wd[j] = c_fmac(wd[j], X[j], r);
          }
          if (!c.no_fwd_record) w_inject_rec<E>(w, wd, s, bin, z - 1, bins);
        } else if (k == 2) {
          // bu[z-1] = P_z bu + R[z-1] bg[z-1]
          if constexpr (MR) {
#pragma unroll
            for (int j = 0; j < E; ++j) bu[j] = Y[j];
          }
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const int x = xclamp(w, j, in);
            const float2 r = Tp.rc[x], b = bgp[x];
            if (in) bu[j] = c_fma(bu[j], r, b);
          }
        }
      }
    }
    __syncthreads();
    reduce_slots(sm.slots, nxg, kW, IS + (size_t)(z - 1) * nxg);
  }
  cp_wait0();
}

// Born adjoint with the two chains of a row on two warps (single reference).
// Warp 2r is the source side of row r (down: bg; up: bu and LinUp^H), warp
// 2r + 1 the receiver side (down: wu, whose steps are the stored T; up: wd
// and LinDown^H).  Within a depth the chains meet only in the image, so each
// warp holds one state row plus the register row of its transform, and the
// CTA runs 16 warps.  A warp writes its image contribution into its own
// exchange buffer after its last transform of the depth; after the depth's
// barrier the CTA sums the buffers of its rows in row order (deterministic).
// Two barriers per depth: the ring's copies are issued at the top of a depth
// and waited for at its end.
// an int the compiler cannot see through: values derived from it after this
// point are recomputed there instead of being kept live across the code
// before it
__device__ __forceinline__ int launder(int v) {
  int r;
  asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(v));
  return r;
}

template <int E, bool NT, int R, bool MR = false>
__global__ void __launch_bounds__(2 * R * 32, 1) kw_born_adj2(DevCtx c, SlotLayout L, const Group* groups,
                                                              float2* storeBG, float2* storeT, float2* storeG,
                                                              const float2* bins, float2* imgR, float2* imgS,
                                                              int compat) {
  const Carve<E> sm(c, L, false, 2 * R, R > 1 || !c.fac);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row = warp >> 1;
  const bool recv = warp & 1;
  stage_static<E>(c, sm);
  const int nxg = c.nxg, nz = c.nz;
  const Group gp = groups[blockIdx.x];
  const int nrows = gp.n;
  const bool act = row < nrows;
  float2* xb = sm.sb0 + warp * wbuf_len<E>();
  const WRow w{c, sm.tw, xb, sm.taperN, sm.kx, lane, NT ? 0 : c.tap, NT ? 32 * E : c.nxg};
  const int f = gp.f, s = gp.s0 + (act ? row : 0), bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg;
  float2* SBG = storeBG + (size_t)(gp.row0 + (act ? row : 0)) * plane;
  float2* ST = storeT + (size_t)(gp.row0 + (act ? row : 0)) * plane;
  float2* IR = imgR + (size_t)blockIdx.x * plane;
  float2* IS = imgS + (size_t)blockIdx.x * plane;
  const int scmode = compat ? 1 : 2;
  const float om = c.omega[f];
  const float2 iw = sc_iw(c, om, scmode);
  const bool t1 = c.ntaylor >= 1;
  // Spectral reuse (tap 0, as-coded scatter adjoint, one Taylor term): no
  // point is masked between a step's inverse transform and the scatter's
  // forward one, so the scatter filters the step's spectrum directly.  The
  // receiver side keeps it in registers; for LinUp^H the down sweep stores
  // the filtered spectrum of T (storeG) next to T.
  const bool reuse = NT && compat && t1 && storeG != nullptr;
  float2* SG = reuse ? storeG + (size_t)(gp.row0 + (act ? row : 0)) * plane : nullptr;
  const float2 zero = make_float2(0.f, 0.f);
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  const float2* xb0 = sm.sb0;
  constexpr int WB = wbuf_len<E>();
  // Y: several references, the receiver side's sum of the references'
  // spectra (PSPI adjoint step); one reference, unused
  float2 S[E], X[E], Y[MR ? E : 1];
  // a depth's tables: from the ring (one reference: every table fits), or,
  // several references, from the ring where it fits and the global tables
  // otherwise
  auto tabs_at = [&](int d) {
    if constexpr (MR) return ring.tabs(d);
    else return ring.stabs(d);
  };

  // this warp's row into its buffer (grid points)
  auto put = [&](const float2 (&v)[E]) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(w, j, in);
      if (in) xb[x] = v[j];
    }
  };
  auto put_zero = [&]() {
    for (int x = lane; x < nxg; x += 32) xb[x] = zero;
  };

  // ---------------- down sweep: bg (source side), wu (receiver side); with
  // c.adj_split the modelling pass stored bg and kw_adj_down ran this sweep
  // for the receiver side (T, its filtered spectra and the image IR)
  if (!c.adj_split) {
  w_zero<E>(S);
  if (act) {
    if (!recv) {
      w_inject_src<E>(w, S, s, f, 0);
      w_store<E>(w, SBG, S);
    } else {
      w_inject_rec<E>(w, S, s, bin, 0, bins);
      for (int x = lane; x < nxg; x += 32) ST[x] = zero;  // T[0] = 0
    }
    put(S);
  }
  ring.issue(0);
  ring.issue(1);
  cp_commit();
  cp_wait0();
  __syncthreads();
  // IR[z] = sum over rows of wu[z] conj(bg[z])
  auto reduce_down = [&](float2* out) {
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      float2 a = zero;
      for (int r = 0; r < nrows; ++r) a = c_add(a, c_mulc(xb0[(2 * r + 1) * WB + x], xb0[2 * r * WB + x]));
      out[x] = a;
    }
  };
  reduce_down(IR);
  for (int z = 0; z + 1 < nz; ++z) {
    __syncthreads();  // the buffers are summed; slot (z + 2) % 3 is free
    ring.issue(z + 2);
    cp_commit();
    if (act) {
      // source side: bg[z+1] = P_z bg + src; receiver side: T[z+1] = P^H_{z+1} wu
      const Tabs T = tabs_at(recv ? z + 1 : z);
      if constexpr (MR) {
        if (!recv) {
          // one forward transform, one inverse per reference, selected into bg
#pragma unroll
          for (int j = 0; j < E; ++j) X[j] = S[j];
          fwd_step_mr<E>(w, T, c.nref, X, S);
          w_inject_src<E>(w, S, s, f, z + 1);
          w_store<E>(w, SBG + (size_t)(z + 1) * nxg, S);
        } else {
          // the references' spectra summed, one inverse transform
#pragma unroll 1
          for (int jr = 0; jr < c.nref; ++jr) {
            adj_pre<E, true>(w, T, jr, S, X);
            wfft<E, false>(X, w.sb, w.tw, lane);
            if (!adj_mid<E, true>(w, T, jr, X, Y)) continue;
            wfft<E, true>(X, w.sb, w.tw, lane);
          }
          adj_post<E>(w, X, S);
          w_store<E>(w, ST + (size_t)(z + 1) * nxg, S);
          w_inject_rec<E>(w, S, s, bin, z + 1, bins);
        }
        put(S);
      } else {
      if (!recv) {
#pragma unroll
        for (int j = 0; j < E; ++j) X[j] = S[j];
      } else {
        adj_pre<E, false>(w, T, 0, S, X);
      }
      wfft<E, false>(X, w.sb, w.tw, lane);
      if (!recv) {
        fwd_mid<E>(w, T, 0, X);
      } else {
        adj_mid<E, false>(w, T, 0, X, Y);
        if (reuse) {
          // filtered spectrum of T[z+1], every point (tap 0: N = nxg)
          float2* g = SG + (size_t)(z + 1) * nxg;
          const float s2 = 1.f / (om * om);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            const float k = w.kx[lane + 32 * j];
            g[lane + 32 * j] = c_scale(X[j], k * k * s2);
          }
        }
      }
      wfft<E, true>(X, w.sb, w.tw, lane);
      if (!recv) {
        fwd_post<E, false>(w, T, 0, X, S);
        w_inject_src<E>(w, S, s, f, z + 1);
        w_store<E>(w, SBG + (size_t)(z + 1) * nxg, S);
      } else {
        adj_post<E>(w, X, S);
        w_store<E>(w, ST + (size_t)(z + 1) * nxg, S);
        w_inject_rec<E>(w, S, s, bin, z + 1, bins);
      }
      put(S);
      }  // one reference
    }
    cp_wait0();
    __syncthreads();
    reduce_down(IR + (size_t)(z + 1) * nxg);
  }
  }  // down sweep

  // ---------------- up sweep, iteration z = nz .. 1 builds image row z - 1
  // source side: bu[z-1] = P_z bu + R[z-1] bg[z-1] (op 0), LinUp^H
  // conj(bu[z-1]) Sc^H_{z-1} T[z-1] (op 1); receiver side: q = P^H_{z-1} wd
  // (op 0), LinDown^H conj(bg[z-1]) Sc^H_{z-1} q (op 1), then
  // wd[z-1] = q + rec + conj(R[z-1]) (T[z-1] + rec)
  const bool keep_last = keep_last_row(c, compat, f, s);
  __syncthreads();  // the down sweep's buffers are summed; the ring is idle
  ring.issue(nz - 1);
  cp_commit();
  cp_wait0();
  __syncthreads();
  auto reduce_up = [&](float2* out) {
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      float2 a = zero;
      for (int r = 0; r < nrows; ++r) a = c_add(a, c_add(xb0[2 * r * WB + x], xb0[(2 * r + 1) * WB + x]));
      out[x] = a;
    }
  };
  for (int z = nz; z >= 1; --z) {
    if (z < nz) __syncthreads();  // the buffers are summed; slot (z - 2) % 3 is free
    ring.issue(z - 2);
    cp_commit();
    if (act) {
      const Tabs Tp = tabs_at(z - 1);
      const float2* bgp = SBG + (size_t)(z - 1) * nxg;
      const float2* tp = ST + (size_t)(z - 1) * nxg;
      if (z == nz) {
        if (!recv) {
          // bu[nz-1] = R bg[nz-1]
          w_load<E>(w, bgp, S);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const float2 r = Tp.rc[xclamp(w, j, in)];
            S[j] = in ? c_mul(r, S[j]) : zero;
          }
        } else {
          // wd[nz-1] = conj(R) (T[nz-1] + rec) + rec
          w_load<E>(w, tp, X);
          w_inject_rec<E>(w, X, s, bin, nz - 1, bins);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const float2 r = Tp.rc[xclamp(w, j, in)];
            S[j] = in ? c_mulc(X[j], r) : zero;
          }
          if (!c.no_fwd_record) w_inject_rec<E>(w, S, s, bin, nz - 1, bins);
        }
      } else if (lane == 0 && !recv && z >= 2) {
        l2_prefetch(SBG + (size_t)(z - 2) * nxg, nxg * 8);
        l2_prefetch(ST + (size_t)(z - 2) * nxg, nxg * 8);
        if (reuse) l2_prefetch(SG + (size_t)(z - 2) * nxg, nxg * 8);
      }
      bool wrote = false;
#pragma unroll 1
      for (int k = 0; k < 2; ++k) {
        const bool on = recv ? (z < nz) : (k == 0 ? (z < nz && z >= 2) : (z >= 2 && (z < nz || keep_last)));
        if (!on) continue;
        const bool step = k == 0;
        const Tabs T = (step && !recv) ? tabs_at(z) : Tp;
        // pre
        bool done = false;  // several references: the step ran whole here
        if constexpr (MR) {
          if (step) {
            if (!recv) {
              // bu: one forward transform, one inverse per reference,
              // selected into bu (R bg added below)
#pragma unroll
              for (int j = 0; j < E; ++j) X[j] = S[j];
              fwd_step_mr<E>(w, T, c.nref, X, S);
            } else {
              // q: the references' spectra summed, one inverse transform
#pragma unroll 1
              for (int jr = 0; jr < c.nref; ++jr) {
                adj_pre<E, true>(w, T, jr, S, X);
                wfft<E, false>(X, w.sb, w.tw, lane);
                if (!adj_mid<E, true>(w, T, jr, X, Y)) continue;
                wfft<E, true>(X, w.sb, w.tw, lane);
              }
            }
            done = true;
          }
        }
        if (done) {
        } else if (step) {
          if (!recv) {
#pragma unroll
            for (int j = 0; j < E; ++j) X[j] = S[j];
          } else {
            adj_pre<E, false>(w, T, 0, S, X);
          }
        } else if (reuse) {
          if (!recv) {
            w_load<E>(w, SG + (size_t)(z - 1) * nxg, X);  // filtered spectrum of T[z-1]
          } else {
            // X holds q, S the filtered spectrum of q (see the step's post)
#pragma unroll
            for (int j = 0; j < E; ++j) {
              const float2 t = X[j];
              X[j] = S[j];
              S[j] = t;
            }
          }
        } else if (t1) {
          if (!recv) {
            w_load<E>(w, tp, X);
            if (scmode == 2) sc_pre<E>(w, T, 2, X, X);
          } else {
            sc_pre<E>(w, T, scmode, S, X);
          }
        }
        if (!done && (step || t1)) {
          if (step || !reuse) {
            wfft<E, false>(X, w.sb, w.tw, lane);
            if (!step) {
              sc_mid<E>(w, om, X);
            } else if (!recv) {
              fwd_mid<E>(w, T, 0, X);
            } else {
              adj_mid<E, false>(w, T, 0, X, Y);
              if (reuse) sc_spec<E>(w, om, X, S);  // wd is spent
            }
          }
          wfft<E, true>(X, w.sb, w.tw, lane);
        }
        // post: the depth's tables and rows again from a laundered depth
        const int zl = launder(z);
        const Tabs Tq = tabs_at(zl - 1);
        const float2* bgq = SBG + (size_t)(zl - 1) * nxg;
        const float2* tq = ST + (size_t)(zl - 1) * nxg;
        if (step) {
          if (!recv) {
            if constexpr (!MR) fwd_post<E, false>(w, ring.stabs(zl), 0, X, S);
#pragma unroll
            for (int j = 0; j < E; ++j) {
              bool in;
              const int x = xclamp(w, j, in);
              const float2 r = Tq.rc[x], b = bgq[x];
              if (in) S[j] = c_add(S[j], c_mul(r, b));
            }
          } else if (!reuse) {
            adj_post<E>(w, X, S);  // S holds q
          }  // with reuse X holds q (tap 0: no point to mask)
        } else {
          if (recv) {
#pragma unroll
            for (int j = 0; j < E; ++j) {
              bool in;
              const int x = xclamp(w, j, in);
              const float2 k0 = Tq.c0[x], k1 = t1 ? Tq.c1[x] : zero, b = bgq[x];
              const float2 v = sc_val(iw, scmode, t1, k0, k1, S[j], X[j]);
              if (in) xb[x] = c_mulc(v, b);
            }
          } else {
#pragma unroll
            for (int j = 0; j < E; ++j) {
              bool in;
              const int x = xclamp(w, j, in);
              const float2 k0 = Tq.c0[x], k1 = t1 ? Tq.c1[x] : zero, u = tq[x];
              const float2 v = sc_val(iw, scmode, t1, k0, k1, u, X[j]);
              if (in) xb[x] = c_mulc(v, S[j]);
            }
          }
          wrote = true;
          if (recv && z >= 2) {
            w_load<E>(w, tq, X);
            w_inject_rec<E>(w, X, s, bin, z - 1, bins);
#pragma unroll
            for (int j = 0; j < E; ++j) {
              bool in;
              const float2 r = Tq.rc[xclamp(w, j, in)];
              if (in) S[j] = c_add(S[j], c_mulc(X[j], r));
            }
            if (!c.no_fwd_record) w_inject_rec<E>(w, S, s, bin, z - 1, bins);
          }
        }
      }
      if (!wrote) put_zero();
    }
    cp_wait0();
    __syncthreads();
    reduce_up(IS + (size_t)(z - 1) * nxg);
  }
}

// Down sweep of the Born adjoint's receiver side alone, one warp per row,
// for the FWI gradient, whose modelling pass has already stored the source
// field bg of every depth (c.bg_store): wu[0] = the injected data;
// T[z+1] = P^H_{z+1} wu (stored, with its filtered spectrum for the
// scatter's spectral reuse), wu[z+1] = T[z+1] + the data injected at z + 1;
// IR[z] = sum over the CTA's rows, in row order, of wu[z] conj(bg[z]).  The
// arithmetic of each row is that of kw_born_adj2's receiver warp; the
// source warp's recomputation of bg is what this saves.  Two barriers per
// depth, as there: the ring's copies are issued at the top of a depth and
// waited for at its end; the products wait for the previous sum.
template <int E, bool NT, int R>
__global__ void __launch_bounds__(R * 32, 2) kw_adj_down(DevCtx c, SlotLayout L, const Group* groups,
                                                         const float2* storeBG, float2* storeT, float2* storeG,
                                                         const float2* bins, float2* imgR) {
  const Carve<E> sm(c, L, false, R, true);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  stage_static<E>(c, sm);
  const int nxg = c.nxg, nz = c.nz;
  const Group gp = groups[blockIdx.x];
  const int nrows = gp.n;
  const bool act = warp < nrows;
  float2* xb = sm.sb0 + warp * wbuf_len<E>();
  const WRow w{c, sm.tw, xb, sm.taperN, sm.kx, lane, NT ? 0 : c.tap, NT ? 32 * E : c.nxg};
  const int f = gp.f, s = gp.s0 + (act ? warp : 0), bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg, row = (size_t)gp.row0 + (act ? warp : 0);
  const float2* SBG = storeBG + row * plane;
  float2* ST = storeT + row * plane;
  float2* SG = storeG ? storeG + row * plane : nullptr;
  float2* IR = imgR + (size_t)blockIdx.x * plane;
  const float om = c.omega[f];
  const float2 zero = make_float2(0.f, 0.f);
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  const float2* xb0 = sm.sb0;
  constexpr int WB = wbuf_len<E>();
  float2 S[E], X[E], Yd[1];
  // this row's products wu[z] conj(bg[z]) into its buffer
  auto put_products = [&](int z) {
    const float2* b = SBG + (size_t)z * nxg;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(w, j, in);
      const float2 v = b[x];
      if (in) xb[x] = c_mulc(S[j], v);
    }
  };
  auto reduce_down = [&](float2* out) {
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      float2 a = zero;
      for (int r = 0; r < nrows; ++r) a = c_add(a, xb0[r * WB + x]);
      out[x] = a;
    }
  };
  w_zero<E>(S);
  if (act) {
    w_inject_rec<E>(w, S, s, bin, 0, bins);
    for (int x = lane; x < nxg; x += 32) ST[x] = zero;  // T[0] = 0
    put_products(0);
  }
  ring.issue(0);
  ring.issue(1);
  cp_commit();
  cp_wait0();
  __syncthreads();
  reduce_down(IR);
  for (int z = 0; z + 1 < nz; ++z) {
    __syncthreads();  // the buffers are summed; slot (z + 2) % 3 is free
    ring.issue(z + 2);
    cp_commit();
    if (act) {
      if (lane == 0 && z + 2 < nz) l2_prefetch(SBG + (size_t)(z + 2) * nxg, nxg * 8);
      // T[z+1] = P^H_{z+1} wu
      const Tabs T = ring.stabs(z + 1);
      adj_pre<E, false>(w, T, 0, S, X);
      wfft<E, false>(X, w.sb, w.tw, lane);
      adj_mid<E, false>(w, T, 0, X, Yd);
      if (SG) {
        // filtered spectrum of T[z+1], every point (tap 0: N = nxg)
        float2* g = SG + (size_t)(z + 1) * nxg;
        const float s2 = 1.f / (om * om);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const float k = w.kx[lane + 32 * j];
          g[lane + 32 * j] = c_scale(X[j], k * k * s2);
        }
      }
      wfft<E, true>(X, w.sb, w.tw, lane);
      adj_post<E>(w, X, S);
      w_store<E>(w, ST + (size_t)(z + 1) * nxg, S);
      w_inject_rec<E>(w, S, s, bin, z + 1, bins);
      put_products(z + 1);
    }
    cp_wait0();
    __syncthreads();
    reduce_down(IR + (size_t)(z + 1) * nxg);
  }
  cp_wait0();
}

// ------------------------------------------------------ host side
// which: 0 WEM, 1 Born forward, 2 Born adjoint (one warp per row), 3 Born
// adjoint with the two chains of a row on two warps (kw_born_adj2)
// rows per CTA of kw_born_adj2 (two warps per row: 16 warps at 128
// registers; 8 rows measured faster than 6 rows at 168 registers)
constexpr int kRowsAdj2 = 8;
// rows per CTA of the several-reference two-warp Born adjoint: a warp's
// rows (state, transform and the references' spectrum or sum) take up to
// 255 registers, so 8 warps per SM
constexpr int kRowsAdj2Mr = 4;
// rows per CTA of the single-reference WEM kernel when its buffers fit
// (16 warps at 128 registers)
constexpr int kRowsWem = 16;

// which: 4 is WEM with kRowsWem rows per CTA, 5 WEM with one row, 6 the
// two-warp Born adjoint with one row, 7 the exact modelling gradient
// (kernels_wg.cuh); exchange buffers per CTA
inline int nbuf_of(int which) {
  switch (which) {
    case 8: return kRowsAdj2;
    case 9: return 2 * kRowsAdj2Mr;
    case 3: return 2 * kRowsAdj2;
    case 7: return 2 * kRowsAdj2;
    case 4: return kRowsWem;
    case 5: return 1;
    case 6: return 2;
    default: return kW;
  }
}
// the tables a pass reads: as WEM (0), Born forward (1) or Born adjoint (2)
inline int tables_of(int which) {
  if (which == 8) return 3;  // the adjoint step alone: phase and split-step rows
  return (which == 4 || which == 5 || which == 7) ? 0 : ((which == 3 || which == 6 || which == 9) ? 2 : which);
}
// one-row CTAs leave the taper out of shared memory when the split-step table
// carries it (SSF)
inline bool taper_of(const DevCtx& c, int which) { return !((which == 5 || which == 6) && c.fac); }

template <int E>
size_t base_bytes(const DevCtx& c, int which) {
  auto r16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  const int nbuf = nbuf_of(which);
  return r16((size_t)32 * E * 8) + r16((size_t)32 * E * 4) + (taper_of(c, which) ? r16((size_t)c.nxg * 4) : 0) +
         r16((size_t)nbuf * wbuf_len<E>() * 8) + (which == 2 ? r16((size_t)kW * c.nxg * 8) : 0) +
         (c.nref > 1 && which != 2 ? r16((size_t)kW * 32 * E * 8) : 0);
}

// Lays out the ring (and the per-warp rows for WEM) and drops them when the
// shared memory does not fit.
template <int E>
SlotLayout slot_layout(const DevCtx& c, int pass, int limit) {
  const int which = tables_of(pass);
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
  L.rc = which != 3 ? put(rowb) : -1;
  L.c0 = (which != 0 && which != 3) ? put(rowb) : -1;
  L.c1 = (which != 0 && which != 3 && c.ntaylor >= 1) ? put(rowb) : -1;
  L.dm = which == 1 ? put(rowb) : -1;
  L.dr = which == 1 ? put(rowb) : -1;
  L.bytes = off;
  L.nslots = 3;
  // one-row WEM CTAs read the stored row through L2 (prefetched a depth
  // ahead) so that three of them fit on an SM
  L.row_bytes = (which == 0 && pass != 5 && pass != 7) ? rowb : 0;
  auto total = [&]() {
    return base_bytes<E>(c, pass) + (size_t)L.nslots * L.bytes + (size_t)2 * nbuf_of(pass) * L.row_bytes;
  };
  if (total() > (size_t)limit) L.row_bytes = 0;
  if (total() > (size_t)limit) {
    L = SlotLayout{};
    L.ph = L.fac = L.ref = L.rc = L.c0 = L.c1 = L.dm = L.dr = -1;
  }
  return L;
}

template <int E>
size_t smem_w(const DevCtx& c, int which, const SlotLayout& L) {
  return base_bytes<E>(c, which) + (size_t)L.nslots * L.bytes + (size_t)2 * nbuf_of(which) * L.row_bytes;
}

// the 16-row WEM kernel serves this context: one reference, and its buffers
// and the full ring fit in shared memory
template <int E>
bool wem16_fits(const DevCtx& c) {
  if (c.nref != 1) return false;
  return slot_layout<E>(c, 4, max_smem_per_block()).nslots == 3;
}

// kw_born_adj2 serves this context: one reference, and its buffers, the
// full ring and every table of a depth fit in shared memory
// the several-reference two-warp form (pass 9): grouped CTAs, its buffers
// in shared memory (the tables where the ring does not fit come from L2)
template <int E>
bool adj2mr_fits(const DevCtx& c) {
  if (c.nref < 2 || c.one_row) return false;
  return base_bytes<E>(c, 9) <= (size_t)max_smem_per_block();
}
template <int E>
bool adj2_fits(const DevCtx& c) {
  if (c.nref != 1) return false;
  const SlotLayout L3 = slot_layout<E>(c, 3, max_smem_per_block());
  return L3.nslots == 3 && (c.fac || L3.ref >= 0);
}
// a kernel may take up to the device's opt-in shared memory per block; set
// once to that bound (not to one launch's size), so launches of the same
// kernel from several host threads never see a smaller bound set by another
template <class K>
void set_max_smem(K kern) {
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_per_block());
}
// W_96 twiddles of this translation unit's copy of c_w96
inline void init_w96() {
  static std::once_flag once;
  std::call_once(once, [] {
    float2 h[96];
    for (int k = 0; k < 96; ++k) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * k / 96;
      h[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    cudaMemcpyToSymbol(c_w96, h, sizeof(h));
  });
}

}  // namespace

// one kernel family per translation unit (kw_e<E>_<pass>.cu); each unit
// fills its own copy of the W_96 table before its first launch
template <int E>
void launch_wem_w(const DevCtx& c, const Group* g, int ng, float2* store, float2* bins, cudaStream_t st) {
  init_w96();
  const bool one = c.one_row && c.nref == 1;
  const int pass = one ? 5 : (wem16_fits<E>(c) ? 4 : 0);
  const SlotLayout L = slot_layout<E>(c, pass, max_smem_per_block());
  const size_t sm = smem_w<E>(c, pass, L);
  const int threads = (pass == 5 ? 1 : (pass == 4 ? kRowsWem : kW)) * 32;
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<ng, threads, sm, st>>>(c, L, g, store, bins);
    note_launch();
  };
  if (c.nref > 1) go(kw_wem<E, true, false, kW>);
  else if (pass == 5 && c.tap == 0) go(kw_wem<E, false, true, 1>);
  else if (pass == 5) go(kw_wem<E, false, false, 1>);
  else if (pass == 4 && c.tap == 0) go(kw_wem<E, false, true, kRowsWem>);
  else if (pass == 4) go(kw_wem<E, false, false, kRowsWem>);
  else if (c.tap == 0) go(kw_wem<E, false, true, kW>);
  else go(kw_wem<E, false, false, kW>);
}

// rows per CTA the WEM launcher expects
template <int E>
int wem_rows_w(const DevCtx& c) {
  if (c.one_row && c.nref == 1) return 1;
  return wem16_fits<E>(c) ? kRowsWem : kW;
}

template <int E>
void launch_fwd_w(const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm, float2* sA,
                  float2* sB, float2* bins, cudaStream_t st) {
  init_w96();
  const SlotLayout L = slot_layout<E>(c, 1, max_smem_per_block());
  const size_t sm = smem_w<E>(c, 1, L);
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<ng, kW * 32, sm, st>>>(c, L, g, dm, drm, sA, sB, bins);
    note_launch();
  };
  if (c.nref > 1) go(kw_born_fwd<E, true>);
  else go(kw_born_fwd<E, false>);
}

// the two-warp Born adjoint with one-row CTAs (every group holds one row);
// instantiated in its own translation unit (kw_e<E>_adj1.cu)
template <int E>
void launch_adj2_one(const DevCtx& c, const Group* g, int ng, float2* sBG, float2* sT, float2* sG, float2* bins,
                     float2* ir, float2* is, int compat, cudaStream_t st) {
  init_w96();
  const SlotLayout L6 = slot_layout<E>(c, 6, max_smem_per_block());
  const size_t sm6 = smem_w<E>(c, 6, L6);
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<ng, 2 * 32, sm6, st>>>(c, L6, g, sBG, sT, sG, bins, ir, is, compat);
    note_launch();
  };
  if (c.tap == 0) go(kw_born_adj2<E, true, 1>);
  else go(kw_born_adj2<E, false, 1>);
}

template <int E>
void launch_adj_w(const DevCtx& c, const Group* g, int ng, float2* sBG, float2* sT, float2* sG, float2* bins,
                  float2* ir, float2* is, int compat, cudaStream_t st) {
  init_w96();
  const int limit = max_smem_per_block();
  if (adj2_fits<E>(c)) {
    // the two chains of a row on two warps, when their buffers, the full
    // ring and every table of a depth fit
    if (c.one_row) {
      launch_adj2_one<E>(c, g, ng, sBG, sT, sG, bins, ir, is, compat, st);
      return;
    }
    if (c.adj_split) {
      // the receiver side's down sweep on its own (bg stored by the modelling)
      const SlotLayout L8 = slot_layout<E>(c, 8, limit);
      const size_t sm8 = smem_w<E>(c, 8, L8);
      auto down = [&](auto kern) {
        set_max_smem(kern);
        kern<<<ng, kRowsAdj2 * 32, sm8, st>>>(c, L8, g, sBG, sT, sG, bins, ir);
        note_launch();
      };
      if (c.tap == 0) down(kw_adj_down<E, true, kRowsAdj2>);
      else down(kw_adj_down<E, false, kRowsAdj2>);
    }
    const SlotLayout L3 = slot_layout<E>(c, 3, limit);
    const size_t sm3 = smem_w<E>(c, 3, L3);
    auto go = [&](auto kern) {
      set_max_smem(kern);
      kern<<<ng, 2 * kRowsAdj2 * 32, sm3, st>>>(c, L3, g, sBG, sT, sG, bins, ir, is, compat);
      note_launch();
    };
    if (c.tap == 0) go(kw_born_adj2<E, true, kRowsAdj2>);
    else go(kw_born_adj2<E, false, kRowsAdj2>);
    return;
  }
  if (adj2mr_fits<E>(c)) {
    // several references: the two chains of a row on two warps
    const SlotLayout L9 = slot_layout<E>(c, 9, limit);
    const size_t sm9 = smem_w<E>(c, 9, L9);
    auto go = [&](auto kern) {
      set_max_smem(kern);
      kern<<<ng, 2 * kRowsAdj2Mr * 32, sm9, st>>>(c, L9, g, sBG, sT, nullptr, bins, ir, is, compat);
      note_launch();
    };
    if (c.tap == 0) go(kw_born_adj2<E, true, kRowsAdj2Mr, true>);
    else go(kw_born_adj2<E, false, kRowsAdj2Mr, true>);
    return;
  }
  const SlotLayout L = slot_layout<E>(c, 2, limit);
  const size_t sm = smem_w<E>(c, 2, L);
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<ng, kW * 32, sm, st>>>(c, L, g, sBG, sT, bins, ir, is, compat);
    note_launch();
  };
  if (c.nref > 1) go(kw_born_adj<E, true>);
  else go(kw_born_adj<E, false>);
}

// the FWI gradient may split the Born adjoint's down sweep off
// (c.adj_split): one reference, the two-warp kernel with grouped CTAs, and
// the receiver side's tables ring in shared memory
template <int E>
bool adj_split_w(const DevCtx& c) {
  if (!adj2_fits<E>(c) || c.one_row) return false;
  const SlotLayout L8 = slot_layout<E>(c, 8, max_smem_per_block());
  return L8.nslots == 3 && (c.fac || L8.ref >= 0);
}

// rows per CTA the Born adjoint launcher expects
template <int E>
int adj_rows_w(const DevCtx& c) {
  if (adj2mr_fits<E>(c)) return kRowsAdj2Mr;
  if (!adj2_fits<E>(c)) return kW;
  return c.one_row ? 1 : kRowsAdj2;
}
// the Born adjoint reuses step spectra in its scatters (and then needs the
// third stored field of filtered spectra)
template <int E>
bool adj_reuse_w(const DevCtx& c, int compat) {
  return adj2_fits<E>(c) && c.tap == 0 && compat && c.ntaylor == 1;
}

template <int E>
size_t smem_w_e(const DevCtx& c, bool slots) {
  const int which = slots ? 2 : 0;
  return smem_w<E>(c, which, slot_layout<E>(c, which, max_smem_per_block()));
}

}  // namespace wg
