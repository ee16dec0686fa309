// GB300 kernels of the one-way depth-continuation path (sm_103a).
//
// Every pass kernel runs one group of rows (shots of one frequency) through
// all depth steps with the rows in shared memory.  The reference performs
// the same arithmetic one (shot, frequency) row at a time on the CPU
// (propagator/src/wem_prop.cpp:52-74, born_prop.cpp:75-113, 178-216); the
// Born passes here use the linearity of the one-way operators to merge the
// reference's seven one-way sweeps per row into two (see the pass comments).
#include <algorithm>
#include <atomic>
#include <cmath>

#include "fft.cuh"
#include "kernels.h"
#include "phase.cuh"
#include "wemgpu.h"

namespace wg {
namespace {

struct Carve {
  float2* p;
  __device__ float2* take(size_t n) {
    float2* r = p;
    p += (n + 1) & ~size_t(1);  // keep 16-byte alignment
    return r;
  }
};

__device__ __forceinline__ float2 zero2() { return make_float2(0.f, 0.f); }

__device__ void load_tw(const DevCtx& c, float2* tw) {
  for (int i = threadIdx.x; i < c.N; i += blockDim.x) tw[i] = c.tw[i];
}

// ------------------------------------------------------------ depth step
// o_r = P_z u_r for nrow rows of frequency f: pad -> FFT -> per reference:
// phase shift -> IFFT -> unpad -> taper (and split step) -> select
// (SSF.cpp:8-32, PSPI.cpp:8-29).  add follows SSF::forward(add=true): the
// selected points are assigned and the others keep their value.
// X, Y (and Z when nref > 1) hold nrow*N values each.  Ends synchronised.
__device__ void step_fwd(const DevCtx& c, const float2* tw, int f, int z, const float2* u, int ldu, float2* o,
                         int ldo, int nrow, float2* X, float2* Y, float2* Z, bool add) {
  const int N = c.N, nxg = c.nxg, tap = c.tap, T = blockDim.x;
  const int m = c.ext ? f : 0;
  const signed char* ref = c.ref + ((size_t)m * c.nz + z) * nxg;
  const float2* fac = c.fac ? c.fac + ((size_t)f * c.nz + z) * nxg : nullptr;
  for (int i = threadIdx.x; i < nrow * N; i += T) {
    int r = i / N, x = i - r * N - tap;
    X[i] = (x >= 0 && x < nxg) ? u[(size_t)r * ldu + x] : zero2();
  }
  __syncthreads();
  float2* Xf = smem_fft(X, Y, nrow, N, c.plan, tw, false);
  float2* spare = (Xf == X) ? Y : X;
  for (int j = 0; j < c.nref; ++j) {
    const float2* ph = c.ph + (((size_t)f * c.nz + z) * c.nref + j) * N;
    float2* Wb = (c.nref == 1) ? Xf : Z;
    for (int i = threadIdx.x; i < nrow * N; i += T) Wb[i] = c_mul(Xf[i], ph[i % N]);
    __syncthreads();
    float2* Rr = smem_fft(Wb, spare, nrow, N, c.plan, tw, true);
    for (int i = threadIdx.x; i < nrow * nxg; i += T) {
      int r = i / nxg, x = i - r * nxg;
      int jr = ref[x];
      float2* dst = o + (size_t)r * ldo + x;
      if (jr == j) {
        float2 y = Rr[r * N + x + tap];
        *dst = fac ? c_mul(y, fac[x]) : c_scale(y, c.taperN[x]);
      } else if (j == 0 && jr < 0 && !add) {
        *dst = zero2();
      }
    }
    __syncthreads();
  }
}

// o_r (+)= P^H_z d_r (SSF.cpp:34-60, PSPI.cpp:31-53).  Ends synchronised.
__device__ void step_adj(const DevCtx& c, const float2* tw, int f, int z, const float2* d, int ldd, float2* o,
                         int ldo, int nrow, float2* X, float2* Y, float2* Z, bool add) {
  const int N = c.N, nxg = c.nxg, tap = c.tap, T = blockDim.x;
  const int m = c.ext ? f : 0;
  const signed char* ref = c.ref + ((size_t)m * c.nz + z) * nxg;
  const float2* fac = c.fac ? c.fac + ((size_t)f * c.nz + z) * nxg : nullptr;
  float2* acc = nullptr;
  for (int j = 0; j < c.nref; ++j) {
    for (int i = threadIdx.x; i < nrow * N; i += T) {
      int r = i / N, x = i - r * N - tap;
      float2 v = zero2();
      if (x >= 0 && x < nxg && ref[x] == j) {
        float2 dv = d[(size_t)r * ldd + x];
        v = fac ? c_mulc(dv, fac[x]) : c_scale(dv, c.taperN[x]);
      }
      X[i] = v;
    }
    __syncthreads();
    float2* Af = smem_fft(X, Y, nrow, N, c.plan, tw, false);
    const float2* ph = c.ph + (((size_t)f * c.nz + z) * c.nref + j) * N;
    if (c.nref == 1) {
      for (int i = threadIdx.x; i < nrow * N; i += T) Af[i] = c_mulc(Af[i], ph[i % N]);
      acc = Af;
    } else {
      for (int i = threadIdx.x; i < nrow * N; i += T) {
        float2 v = c_mulc(Af[i], ph[i % N]);
        Z[i] = j ? c_add(Z[i], v) : v;
      }
      acc = Z;
    }
    __syncthreads();
  }
  float2* spare = (acc == X) ? Y : X;
  float2* Rr = smem_fft(acc, spare, nrow, N, c.plan, tw, true);
  for (int i = threadIdx.x; i < nrow * nxg; i += T) {
    int r = i / nxg, x = i - r * nxg;
    float2 v = Rr[r * N + x + tap];
    float2* dst = o + (size_t)r * ldo + x;
    *dst = add ? c_add(*dst, v) : v;
  }
  __syncthreads();
}

// ------------------------------------------------------------- Scatter
// mode 0: forward  o += sum_it -i w dz c_it unpad(IFFT(K_it FFT(pad u)))
// mode 1: adjoint as coded (k filter before the conj(c_it) scaling)
// mode 2: exact adjoint (Scatter.cpp:35-111).  it = 0 has K = 1 and needs no
// transform.  Ends synchronised.
__device__ void scatter_rows(const DevCtx& c, const float2* tw, int f, int z, int mode, const float2* in, int ldi,
                             float2* o, int ldo, int nrow, float2* X, float2* Y, float2* Z, bool add) {
  const int N = c.N, nxg = c.nxg, tap = c.tap, T = blockDim.x, nz = c.nz;
  const int m = c.ext ? f : 0;
  const int nt = c.ntaylor;
  const float w = c.omega[f];
  const float wdz = w * c.dz;
  const float2 iw = make_float2(0.f, mode == 0 ? -wdz : wdz);  // -i w dz or +i w dz
  auto coef = [&](int it) { return c.sc + (((size_t)m * (nt + 1) + it) * nz + z) * nxg; };
  const float2* c0 = coef(0);
  for (int i = threadIdx.x; i < nrow * nxg; i += T) {
    int r = i / nxg, x = i - r * nxg;
    float2 u = in[(size_t)r * ldi + x];
    float2 v = c_mul(iw, mode == 0 ? c_mul(c0[x], u) : c_mulc(u, c0[x]));
    float2* dst = o + (size_t)r * ldo + x;
    *dst = add ? c_add(*dst, v) : v;
  }
  __syncthreads();
  if (nt == 0) return;
  auto kfilt = [&](int n, int it) {
    float kw = c.kx[n] / w;
    float q = kw * kw, p = q;
    for (int e = 1; e < it; ++e) p *= q;
    return p;
  };
  if (mode != 2) {
    for (int i = threadIdx.x; i < nrow * N; i += T) {
      int r = i / N, x = i - r * N - tap;
      X[i] = (x >= 0 && x < nxg) ? in[(size_t)r * ldi + x] : zero2();
    }
    __syncthreads();
    float2* Xf = smem_fft(X, Y, nrow, N, c.plan, tw, false);
    float2* spare = (Xf == X) ? Y : X;
    for (int it = 1; it <= nt; ++it) {
      float2* Wb = (nt == 1) ? Xf : Z;
      for (int i = threadIdx.x; i < nrow * N; i += T) Wb[i] = c_scale(Xf[i], kfilt(i % N, it));
      __syncthreads();
      float2* Rr = smem_fft(Wb, spare, nrow, N, c.plan, tw, true);
      const float2* ci = coef(it);
      for (int i = threadIdx.x; i < nrow * nxg; i += T) {
        int r = i / nxg, x = i - r * nxg;
        float2 y = c_scale(Rr[r * N + x + tap], c.invN);
        float2 v = c_mul(iw, mode == 0 ? c_mul(ci[x], y) : c_mulc(y, ci[x]));
        float2* dst = o + (size_t)r * ldo + x;
        *dst = c_add(*dst, v);
      }
      __syncthreads();
    }
  } else {
    float2* acc = nullptr;
    for (int it = 1; it <= nt; ++it) {
      const float2* ci = coef(it);
      for (int i = threadIdx.x; i < nrow * N; i += T) {
        int r = i / N, x = i - r * N - tap;
        X[i] = (x >= 0 && x < nxg) ? c_mulc(in[(size_t)r * ldi + x], ci[x]) : zero2();
      }
      __syncthreads();
      float2* Af = smem_fft(X, Y, nrow, N, c.plan, tw, false);
      if (nt == 1) {
        for (int i = threadIdx.x; i < nrow * N; i += T) Af[i] = c_scale(Af[i], kfilt(i % N, it));
        acc = Af;
      } else {
        for (int i = threadIdx.x; i < nrow * N; i += T) {
          float2 v = c_scale(Af[i], kfilt(i % N, it));
          Z[i] = it > 1 ? c_add(Z[i], v) : v;
        }
        acc = Z;
      }
      __syncthreads();
    }
    float2* spare = (acc == X) ? Y : X;
    float2* Rr = smem_fft(acc, spare, nrow, N, c.plan, tw, true);
    for (int i = threadIdx.x; i < nrow * nxg; i += T) {
      int r = i / nxg, x = i - r * nxg;
      float2 v = c_mul(iw, c_scale(Rr[r * N + x + tap], c.invN));
      float2* dst = o + (size_t)r * ldo + x;
      *dst = c_add(*dst, v);
    }
    __syncthreads();
  }
}

// ------------------------------------------------- injection / recording
// Injection.cpp:8-19 (source of shot s0 + r at depth z): one thread per
// row, points and window taps in order (the windows of several points of a
// shot may overlap)
__device__ void inject_src(const DevCtx& c, float2* W, int ldw, int nrow, int s0, int f, int z) {
  const float2 wv = c.wave[f];
  for (int r = threadIdx.x; r < nrow; r += blockDim.x) {
    const int s = s0 + r;
    if (c.sz[s] != z) continue;
    const int p0 = c.sptr ? c.sptr[s] : s, p1 = c.sptr ? c.sptr[s + 1] : s + 1;
    for (int pt = p0; pt < p1; ++pt)
      for (int g = 0; g <= 2 * c.ngs; ++g) {
        const int x = c.sx[pt] + g - c.ngs + c.pad;
        if (x >= 0 && x < c.nxg) W[(size_t)r * ldw + x] = c_add(W[(size_t)r * ldw + x], c_scale(wv, c.gs[g]));
      }
  }
}

// Injection.cpp:69-80: bins[s][i][bin] += sum_g gr[g] W[rx_i + g + pad]
__device__ void record(const DevCtx& c, const float2* W, int ldw, int nrow, int s0, int bin, int z, float2* bins) {
  const int k0 = c.rptr[z], nk = c.rptr[z + 1] - k0;
  if (nk == 0) return;
  for (int i = threadIdx.x; i < nrow * nk; i += blockDim.x) {
    int r = i / nk, k = k0 + i - r * nk;
    int x0 = c.rxs[k] + c.pad;
    float2 acc = zero2();
    for (int g = -c.ngr; g <= c.ngr; ++g) {
      int x = x0 + g;
      if (x >= 0 && x < c.nxg) acc = c_add(acc, c_scale(W[(size_t)r * ldw + x], c.gr[g + c.ngr]));
    }
    float2* d = bins + ((size_t)(s0 + r) * c.nr + c.rid[k]) * c.nbin + bin;
    *d = c_add(*d, acc);
  }
}

// Injection.cpp:56-67 (receivers as sources), gathered per point so that
// overlapping windows add in a fixed order
__device__ void inject_rec(const DevCtx& c, float2* W, int ldw, int nrow, int s0, int bin, int z,
                           const float2* bins) {
  const int k0 = c.rptr[z], k1 = c.rptr[z + 1];
  if (k0 == k1) return;
  for (int i = threadIdx.x; i < nrow * c.nxg; i += blockDim.x) {
    int r = i / c.nxg, x = i - r * c.nxg;
    int lo = x - c.pad - c.ngr, hi = x - c.pad + c.ngr;
    int a = k0, b = k1;
    while (a < b) {
      int mid = (a + b) >> 1;
      if (c.rxs[mid] < lo) a = mid + 1; else b = mid;
    }
    float2 acc = zero2();
    for (int k = a; k < k1 && c.rxs[k] <= hi; ++k) {
      int g = x - c.pad - c.rxs[k];
      const float2 dv = bins[((size_t)(s0 + r) * c.nr + c.rid[k]) * c.nbin + bin];
      acc = c_add(acc, c_scale(dv, c.gr[g + c.ngr]));
    }
    if (k0 != k1) W[(size_t)r * ldw + x] = c_add(W[(size_t)r * ldw + x], acc);
  }
}

// ================================================================ passes
// Nonlinear modelling, WEM::full_fwd (wem_prop.cpp:52-74) for one group:
//   down: W[0] = src, W[z+1] = P_z W[z] + src[z+1]; record W; keep A = R W
//   up:   V[nz-1] = A[nz-1], V[z-1] = P_z V[z] + A[z-1]; record V
__global__ void __launch_bounds__(kThreads) k_wem(DevCtx c, const Group* groups, int G, float2* store,
                                                  float2* bins) {
  extern __shared__ float4 smem4[];
  Carve sm{reinterpret_cast<float2*>(smem4)};
  const int N = c.N, nxg = c.nxg, nz = c.nz;
  float2* tw = sm.take(N);
  float2* X = sm.take((size_t)G * N);
  float2* Y = sm.take((size_t)G * N);
  float2* Z = c.nref > 1 ? sm.take((size_t)G * N) : nullptr;
  float2* W = sm.take((size_t)G * nxg);
  float2* V = sm.take((size_t)G * nxg);
  const Group gp = groups[blockIdx.x];
  const int nrow = gp.n, f = gp.f, s0 = gp.s0, bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg;
  float2* A = store + (size_t)gp.row0 * plane;
  load_tw(c, tw);
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) W[i] = zero2();
  __syncthreads();
  inject_src(c, W, nxg, nrow, s0, f, 0);
  __syncthreads();
  for (int z = 0; z < nz; ++z) {
    record(c, W, nxg, nrow, s0, bin, z, bins);
    const float2* rc = rc_row(c, f, z);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      A[r * plane + (size_t)z * nxg + x] = c_mul(rc[x], W[i]);
    }
    if (z == nz - 1) break;
    step_fwd(c, tw, f, z, W, nxg, V, nxg, nrow, X, Y, Z, false);
    float2* t = W; W = V; V = t;
    inject_src(c, W, nxg, nrow, s0, f, z + 1);
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
    int r = i / nxg, x = i - r * nxg;
    W[i] = A[r * plane + (size_t)(nz - 1) * nxg + x];
  }
  __syncthreads();
  for (int z = nz - 1; z >= 0; --z) {
    record(c, W, nxg, nrow, s0, bin, z, bins);
    if (z == 0) break;
    step_fwd(c, tw, f, z, W, nxg, V, nxg, nrow, X, Y, Z, false);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      V[i] = c_add(V[i], A[r * plane + (size_t)(z - 1) * nxg + x]);
    }
    float2* t = W; W = V; V = t;
    __syncthreads();
  }
}

// Born forward, BornFull::full_fwd (born_prop.cpp:75-113) merged by
// linearity into two sweeps per row:
//   down: bg[z+1] = P_z bg[z] + src;  sd[z+1] = P_z(sd[z] + Sc_z(bg[z] dm[z]))
//         record sd; keep A = R bg and B = bg dR(dm) + R sd
//   up:   bu[z-1] = P_z bu[z] + A[z-1]
//         su[z-1] = P_z(su[z] + Sc_z(bu[z] dm[z])) + B[z-1];  record su
// (sd is the reference's forward-scattering field, recorded and reused for
// its down-scattering term; su sums its reflectivity, down-scattering and
// up-scattering up-going sweeps.)  bg and sd rows share one depth step call.
__global__ void __launch_bounds__(kThreads) k_born_fwd(DevCtx c, const Group* groups, int G, const float2* dm,
                                                       const float2* drm, float2* storeA, float2* storeB,
                                                       float2* bins) {
  extern __shared__ float4 smem4[];
  Carve sm{reinterpret_cast<float2*>(smem4)};
  const int N = c.N, nxg = c.nxg, nz = c.nz;
  float2* tw = sm.take(N);
  float2* X = sm.take((size_t)2 * G * N);
  float2* Y = sm.take((size_t)2 * G * N);
  float2* Z = (c.nref > 1 || c.ntaylor > 1) ? sm.take((size_t)2 * G * N) : nullptr;
  float2* P = sm.take((size_t)2 * G * nxg);
  float2* Q = sm.take((size_t)2 * G * nxg);
  float2* T1 = sm.take((size_t)G * nxg);
  float2* T2 = sm.take((size_t)G * nxg);
  const Group gp = groups[blockIdx.x];
  const int nrow = gp.n, f = gp.f, s0 = gp.s0, bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg;
  const size_t half = (size_t)nrow * nxg;
  float2* A = storeA + (size_t)gp.row0 * plane;
  float2* B = storeB + (size_t)gp.row0 * plane;
  load_tw(c, tw);
  for (int i = threadIdx.x; i < 2 * nrow * nxg; i += blockDim.x) P[i] = zero2();
  __syncthreads();
  inject_src(c, P, nxg, nrow, s0, f, 0);
  __syncthreads();
  for (int z = 0; z < nz; ++z) {
    float2* bg = P;
    float2* sd = P + half;
    if (!c.no_fwd_record) record(c, sd, nxg, nrow, s0, bin, z, bins);
    const float2* rc = rc_row(c, f, z);
    const float2* dr = drm + pert_off(c, f, z);
    const float2* dmz = dm + pert_off(c, f, z);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      size_t o = r * plane + (size_t)z * nxg + x;
      A[o] = c_mul(rc[x], bg[i]);
      B[o] = c_add(c_mul(bg[i], dr[x]), c_mul(rc[x], sd[i]));
      T1[i] = c_mul(bg[i], dmz[x]);
    }
    if (z == nz - 1) break;
    __syncthreads();
    scatter_rows(c, tw, f, z, 0, T1, nxg, T2, nxg, nrow, X, Y, Z, false);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) sd[i] = c_add(sd[i], T2[i]);
    __syncthreads();
    step_fwd(c, tw, f, z, P, nxg, Q, nxg, 2 * nrow, X, Y, Z, false);
    float2* t = P; P = Q; Q = t;
    inject_src(c, P, nxg, nrow, s0, f, z + 1);
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
    int r = i / nxg, x = i - r * nxg;
    size_t o = r * plane + (size_t)(nz - 1) * nxg + x;
    P[i] = A[o];
    P[half + i] = B[o];
  }
  __syncthreads();
  for (int z = nz - 1; z >= 0; --z) {
    float2* bu = P;
    float2* su = P + half;
    record(c, su, nxg, nrow, s0, bin, z, bins);
    if (z == 0) break;
    const float2* dmz = dm + pert_off(c, f, z);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) T1[i] = c_mul(bu[i], dmz[i % nxg]);
    __syncthreads();
    scatter_rows(c, tw, f, z, 0, T1, nxg, T2, nxg, nrow, X, Y, Z, false);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) su[i] = c_add(su[i], T2[i]);
    __syncthreads();
    step_fwd(c, tw, f, z, P, nxg, Q, nxg, 2 * nrow, X, Y, Z, false);
    float2* t = P; P = Q; Q = t;
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      size_t o = r * plane + (size_t)(z - 1) * nxg + x;
      P[i] = c_add(P[i], A[o]);
      P[half + i] = c_add(P[half + i], B[o]);
    }
    __syncthreads();
  }
}

// Born adjoint, BornFull::full_adj (born_prop.cpp:178-216) in two sweeps:
//   down: bg[z+1] = P_z bg[z] + src;  wu[z+1] = P^H_{z+1} wu[z] + rec[z+1]
//         (wu is the reference's Up^H of the injected data, computed once
//         for its three uses); image IR[z] += conj(bg) wu (Born_refl^H)
//         keep bg and T[z] = P^H_z wu[z-1]
//   up:   bu[z-1] = P_z bu[z] + R bg[z-1]
//         wd[z-1] = q + S[z-1], q = P^H_{z-1} wd[z],
//           S = rec + conj(R) wu   (Down^H of the data and of conj(R) wu)
//         IS[z-1] += conj(bg[z-1]) Sc^H_{z-1} q         (LinDown^H)
//         IS[z]   += conj(bu[z])   Sc^H_z T[z]           (LinUp^H)
// Images are per group and summed afterwards in a fixed order.
__global__ void __launch_bounds__(kThreads) k_born_adj(DevCtx c, const Group* groups, int G, float2* storeBG,
                                                       float2* storeT, const float2* bins, float2* imgR,
                                                       float2* imgS, int compat) {
  extern __shared__ float4 smem4[];
  Carve sm{reinterpret_cast<float2*>(smem4)};
  const int N = c.N, nxg = c.nxg, nz = c.nz;
  float2* tw = sm.take(N);
  float2* X = sm.take((size_t)G * N);
  float2* Y = sm.take((size_t)G * N);
  float2* Z = (c.nref > 1 || c.ntaylor > 1) ? sm.take((size_t)G * N) : nullptr;
  float2* S0 = sm.take((size_t)G * nxg);
  float2* S1 = sm.take((size_t)G * nxg);
  float2* S2 = sm.take((size_t)G * nxg);
  float2* S3 = sm.take((size_t)G * nxg);
  float2* S4 = sm.take((size_t)G * nxg);
  float2* ACC = sm.take(nxg);
  const Group gp = groups[blockIdx.x];
  const int nrow = gp.n, f = gp.f, s0 = gp.s0, bin = c.bin[f];
  const size_t plane = (size_t)nz * nxg;
  float2* SBG = storeBG + (size_t)gp.row0 * plane;
  float2* ST = storeT + (size_t)gp.row0 * plane;
  float2* IR = imgR + (size_t)blockIdx.x * plane;
  float2* IS = imgS + (size_t)blockIdx.x * plane;
  const int scmode = compat ? 1 : 2;
  load_tw(c, tw);
  // ---------------- down sweep
  float2* BG = S0;
  float2* O1 = S1;
  float2* WU = S2;
  float2* TT = S3;
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
    BG[i] = zero2();
    WU[i] = zero2();
    TT[i] = zero2();
  }
  __syncthreads();
  inject_src(c, BG, nxg, nrow, s0, f, 0);
  inject_rec(c, WU, nxg, nrow, s0, bin, 0, bins);
  __syncthreads();
  for (int z = 0; z < nz; ++z) {
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      float2 a = zero2();
      for (int r = 0; r < nrow; ++r) a = c_add(a, c_mulc(WU[r * nxg + x], BG[r * nxg + x]));
      IR[(size_t)z * nxg + x] = a;
    }
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      size_t o = r * plane + (size_t)z * nxg + x;
      SBG[o] = BG[i];
      ST[o] = TT[i];
    }
    if (z == nz - 1) break;
    step_fwd(c, tw, f, z, BG, nxg, O1, nxg, nrow, X, Y, Z, false);
    float2* t = BG; BG = O1; O1 = t;
    inject_src(c, BG, nxg, nrow, s0, f, z + 1);
    step_adj(c, tw, f, z + 1, WU, nxg, TT, nxg, nrow, X, Y, Z, false);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) WU[i] = TT[i];
    __syncthreads();
    inject_rec(c, WU, nxg, nrow, s0, bin, z + 1, bins);
    __syncthreads();
  }
  __syncthreads();
  // ---------------- up sweep
  float2* BU = S0;
  float2* WD = S1;
  float2* Q1 = S2;
  float2* Q2 = S3;
  float2* T1 = S4;
  auto source_S = [&](int z) {  // WD = conj(R[z]) (T[z] + rec[z]) + rec[z] + WD_in (in Q1)
    const float2* rc = rc_row(c, f, z);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      T1[i] = ST[r * plane + (size_t)z * nxg + x];
    }
    __syncthreads();
    inject_rec(c, T1, nxg, nrow, s0, bin, z, bins);
    __syncthreads();
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int x = i % nxg;
      WD[i] = c_add(Q1[i], c_mulc(T1[i], rc[x]));
    }
    __syncthreads();
    if (!c.no_fwd_record) inject_rec(c, WD, nxg, nrow, s0, bin, z, bins);  // adjoint of the forward-scattering record
    __syncthreads();
  };
  {
    const float2* rc = rc_row(c, f, nz - 1);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      BU[i] = c_mul(rc[x], SBG[r * plane + (size_t)(nz - 1) * nxg + x]);
      Q1[i] = zero2();
    }
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) ACC[x] = zero2();
    __syncthreads();
    source_S(nz - 1);
  }
  for (int z = nz - 1; z >= 0; --z) {
    if (z >= 1) {
      // LinUp^H at depth z; the compat rule keeps only one frequency's
      // (or, extended, one shot's) contribution in the last row
      scatter_rows(c, tw, f, z, scmode, ST + (size_t)z * nxg, (int)plane, T1, nxg, nrow, X, Y, Z, false);
      for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
        float2 a = ACC[x];
        for (int r = 0; r < nrow; ++r) {
          bool keep = z != nz - 1 || keep_last_row(c, compat, f, s0 + r);
          if (keep) a = c_add(a, c_mulc(T1[r * nxg + x], BU[r * nxg + x]));
        }
        ACC[x] = a;
      }
    }
    __syncthreads();
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) IS[(size_t)z * nxg + x] = ACC[x];
    if (z == 0) break;
    // q = P^H_{z-1} wd[z]; LinDown^H into row z-1
    step_adj(c, tw, f, z - 1, WD, nxg, Q1, nxg, nrow, X, Y, Z, false);
    scatter_rows(c, tw, f, z - 1, scmode, Q1, nxg, T1, nxg, nrow, X, Y, Z, false);
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      float2 a = zero2();
      for (int r = 0; r < nrow; ++r)
        a = c_add(a, c_mulc(T1[r * nxg + x], SBG[r * plane + (size_t)(z - 1) * nxg + x]));
      ACC[x] = a;
    }
    __syncthreads();
    source_S(z - 1);  // WD = q + S[z-1]
    // bu[z-1] = P_z bu[z] + R[z-1] bg[z-1]
    step_fwd(c, tw, f, z, BU, nxg, Q2, nxg, nrow, X, Y, Z, false);
    const float2* rc = rc_row(c, f, z - 1);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      BU[i] = c_add(Q2[i], c_mul(rc[x], SBG[r * plane + (size_t)(z - 1) * nxg + x]));
    }
    __syncthreads();
  }
}

// ------------------------------------------------- row-level operators
__global__ void __launch_bounds__(kThreads) k_onestep(DevCtx c, int f, int z, int adj, const float2* in,
                                                      float2* out, int nrow_total, int add, int G) {
  extern __shared__ float4 smem4[];
  Carve sm{reinterpret_cast<float2*>(smem4)};
  const int N = c.N, nxg = c.nxg;
  float2* tw = sm.take(N);
  float2* X = sm.take((size_t)G * N);
  float2* Y = sm.take((size_t)G * N);
  float2* Z = sm.take((size_t)G * N);
  float2* U = sm.take((size_t)G * nxg);
  float2* O = sm.take((size_t)G * nxg);
  const int r0 = blockIdx.x * G, nrow = min(G, nrow_total - r0);
  load_tw(c, tw);
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
    U[i] = in[(size_t)r0 * nxg + i];
    O[i] = add ? out[(size_t)r0 * nxg + i] : zero2();
  }
  __syncthreads();
  if (!adj) step_fwd(c, tw, f, z, U, nxg, O, nxg, nrow, X, Y, Z, add != 0);
  else step_adj(c, tw, f, z, U, nxg, O, nxg, nrow, X, Y, Z, add != 0);
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) out[(size_t)r0 * nxg + i] = O[i];
}

__global__ void __launch_bounds__(kThreads) k_scatter(DevCtx c, int f, int z, int mode, const float2* in,
                                                      float2* out, int nrow_total, int add, int G) {
  extern __shared__ float4 smem4[];
  Carve sm{reinterpret_cast<float2*>(smem4)};
  const int N = c.N, nxg = c.nxg;
  float2* tw = sm.take(N);
  float2* X = sm.take((size_t)G * N);
  float2* Y = sm.take((size_t)G * N);
  float2* Z = sm.take((size_t)G * N);
  float2* U = sm.take((size_t)G * nxg);
  float2* O = sm.take((size_t)G * nxg);
  const int r0 = blockIdx.x * G, nrow = min(G, nrow_total - r0);
  load_tw(c, tw);
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
    U[i] = in[(size_t)r0 * nxg + i];
    O[i] = add ? out[(size_t)r0 * nxg + i] : zero2();
  }
  __syncthreads();
  scatter_rows(c, tw, f, z, mode, U, nxg, O, nxg, nrow, X, Y, Z, true);
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) out[(size_t)r0 * nxg + i] = O[i];
}

// Down/Up forward/adjoint (OneWay.cpp:32-109) over whole fields.  With
// recursive set the propagated row is the previous output (in-place use);
// otherwise it is the input row (out-of-place single steps).
__global__ void __launch_bounds__(kThreads) k_oneway(DevCtx c, int f, int up, int adj, int recursive,
                                                     const float2* in, float2* out, int nrow_total, int add,
                                                     int G) {
  extern __shared__ float4 smem4[];
  Carve sm{reinterpret_cast<float2*>(smem4)};
  const int N = c.N, nxg = c.nxg, nz = c.nz;
  float2* tw = sm.take(N);
  float2* X = sm.take((size_t)G * N);
  float2* Y = sm.take((size_t)G * N);
  float2* Z = sm.take((size_t)G * N);
  float2* U = sm.take((size_t)G * nxg);
  float2* O = sm.take((size_t)G * nxg);
  const int r0 = blockIdx.x * G, nrow = min(G, nrow_total - r0);
  const size_t plane = (size_t)nz * nxg;
  const float2* I = in + (size_t)r0 * plane;
  float2* D = out + (size_t)r0 * plane;
  load_tw(c, tw);
  if (recursive && !add) {  // the reference zeroes its own input first
    for (size_t i = threadIdx.x; i < (size_t)nrow * plane; i += blockDim.x) D[i] = zero2();
    return;
  }
  // direction: forward Down walks z up, forward Up walks z down; the
  // adjoints walk the other way
  const bool zup = (up == 0) != (adj != 0);
  const int zs = zup ? 0 : nz - 1;
  for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
    int r = i / nxg, x = i - r * nxg;
    float2 v = I[r * plane + (size_t)zs * nxg + x];
    U[i] = v;
    D[r * plane + (size_t)zs * nxg + x] = v;
  }
  __syncthreads();
  for (int k = 0; k < nz - 1; ++k) {
    const int zc = zup ? k : nz - 1 - k;   // row propagated
    const int zn = zup ? zc + 1 : zc - 1;  // row written
    if (!recursive) {
      for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
        int r = i / nxg, x = i - r * nxg;
        U[i] = I[r * plane + (size_t)zc * nxg + x];
      }
      __syncthreads();
    }
    // depth of the operator: forward uses the propagated row's depth;
    // Down^H uses zc-1 = zn, Up^H uses zc+1 = zn
    const int zop = adj ? zn : zc;
    if (!adj) step_fwd(c, tw, f, zop, U, nxg, O, nxg, nrow, X, Y, Z, false);
    else step_adj(c, tw, f, zop, U, nxg, O, nxg, nrow, X, Y, Z, false);
    for (int i = threadIdx.x; i < nrow * nxg; i += blockDim.x) {
      int r = i / nxg, x = i - r * nxg;
      float2 v = c_add(O[i], I[r * plane + (size_t)zn * nxg + x]);
      D[r * plane + (size_t)zn * nxg + x] = v;
      U[i] = v;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- tables
// Phase-shift factors (phase_factor, phase.cuh): one CTA row per
// (frequency, depth, reference) table row, threads over the N points.
__global__ void k_phase(DevCtx c, const float2* sref, float eps, float2* ph) {
  const int nrow = c.nfreq * c.nz * c.nref;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= c.N) return;
  const float k = c.kx[n];
  for (int r = blockIdx.y; r < nrow; r += gridDim.y) {
    const int j = r % c.nref, z = (r / c.nref) % c.nz, f = r / (c.nref * c.nz);
    const int m = c.ext ? f : 0;
    const float2 s = sref[((size_t)m * c.nz + z) * c.nref + j];
    const float w = c.omega[f];
    ph[(size_t)r * c.N + n] = phase_factor(w * w, s, k, eps, c.dz, c.phase_law);
  }
}

// SSF per-point factor taper / N * exp(-i w dz q) (ssf_factor, phase.cuh),
// zero at points without a reference.  One CTA row per (frequency, depth)
// table row, threads over the points.
__global__ void k_fac(DevCtx c, const float2* q, float2* fac) {
  const int nrow = c.nfreq * c.nz;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= c.nxg) return;
  const float tp = c.taperN[x];
  for (int r = blockIdx.y; r < nrow; r += gridDim.y) {
    const int z = r % c.nz, f = r / c.nz;
    const int m = c.ext ? f : 0;
    const size_t qi = ((size_t)m * c.nz + z) * c.nxg + x;
    fac[(size_t)r * c.nxg + x] = c.ref[qi] >= 0 ? ssf_factor(q[qi], c.omega[f], c.dz, tp) : zero2();
  }
}

// ------------------------------------------------------------- helpers
__global__ void k_pad_model(const float2* in, float2* out, int M, int nz, int nx, int pad) {
  const int nxg = nx + 2 * pad;
  const size_t total = (size_t)M * nz * nxg;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % nxg) - pad;
    size_t rz = i / nxg;
    out[i] = (x >= 0 && x < nx) ? in[rz * nx + x] : zero2();
  }
}

// dReflect forward (dReflect.h:29-49), rows 1..nz-2
__global__ void k_drefl_fwd(int M, int nz, int nxg, const float2* a0, const float2* b0, const float2* a1,
                            const float2* b1, const float2* dm0, const float2* dm1, float2* out) {
  const size_t total = (size_t)M * nz * nxg;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int z = (int)((i / nxg) % nz);
    float2 v = zero2();
    if (z >= 1 && z <= nz - 2) {
      v = c_sub(c_mul(a0[i], dm0[i - nxg]), c_mul(b0[i], dm0[i]));
      v = c_add(v, c_sub(c_mul(a1[i], dm1[i]), c_mul(b1[i], dm1[i - nxg])));
    }
    out[i] = v;
  }
}

// out[m] += sum over groups g in [beg[m], beg[m+1]) of parts[g], in order
__global__ void k_reduce(const float2* parts, const int* beg, int M, size_t plane, float2* out) {
  const size_t total = (size_t)M * plane;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int m = (int)(i / plane);
    size_t p = i - (size_t)m * plane;
    float2 a = out[i];
    for (int g = beg[m]; g < beg[m + 1]; ++g) a = c_add(a, parts[(size_t)g * plane + p]);
    out[i] = a;
  }
}

// gradient = unpad(IS + dR^H(IR)) (dReflect.h:58-79, Pad.h:98-107)
__global__ void k_grad(int M, int nz, int nxg, int nx, int pad, const float2* a0, const float2* b0,
                       const float2* a1, const float2* b1, const float2* IR, const float2* IS, float2* g0,
                       float2* g1, int add) {
  const size_t total = (size_t)M * nz * nx;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % nx);
    size_t t = i / nx;
    int z = (int)(t % nz);
    int m = (int)(t / nz);
    size_t p = ((size_t)m * nz + z) * nxg + x + pad;
    float2 v0 = IS[p], v1 = zero2();
    if (z + 1 >= 1 && z + 1 <= nz - 2) {
      v0 = c_add(v0, c_mulc(IR[p + nxg], a0[p + nxg]));
      v1 = c_sub(v1, c_mulc(IR[p + nxg], b1[p + nxg]));
    }
    if (z >= 1 && z <= nz - 2) {
      v0 = c_sub(v0, c_mulc(IR[p], b0[p]));
      v1 = c_add(v1, c_mulc(IR[p], a1[p]));
    }
    g0[i] = add ? c_add(g0[i], v0) : v0;
    g1[i] = add ? c_add(g1[i], v1) : v1;
  }
}

// Window copy between caller bins [nrows][ldu] and the compact bins
// [nrows][nf] of the propagated frequencies (bins off .. off + nf - 1).
// to_user: every caller bin is written (zero outside the window, or left as
// it is with add); otherwise the compact rows take the caller's window
// (zero where it runs past ldu).
__global__ void k_bin_window(const float2* src, float2* dst, int nrows, int ldu, int nf, int off, int to_user,
                             int add) {
  const size_t total = (size_t)nrows * (to_user ? ldu : nf);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    if (to_user) {
      const size_t r = i / ldu;
      const int b = (int)(i - r * ldu), f = b - off;
      const float2 v = (f >= 0 && f < nf) ? src[r * nf + f] : zero2();
      dst[i] = add ? c_add(dst[i], v) : v;
    } else {
      const size_t r = i / nf;
      const int f = (int)(i - r * nf), b = f + off;
      dst[i] = b < ldu ? src[r * ldu + b] : zero2();
    }
  }
}

__global__ void k_copy_rows(const float2* src, int lds, float2* dst, int ldd, int nrows, int ncopy, int add) {
  const size_t total = (size_t)nrows * ldd;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    size_t r = i / ldd;
    int j = (int)(i - r * ldd);
    float2 v = j < ncopy ? src[r * lds + j] : zero2();
    dst[i] = add ? c_add(dst[i], v) : v;
  }
}

__global__ void k_add(float2* y, const float2* x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = c_add(y[i], x[i]);
}

int grid_for(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? (b ? b : 1) : 152 * 32);
}

template <class K>
void set_smem(K kernel, size_t bytes) {
  // the device's bound rather than this launch's size, so concurrent
  // launches of the kernel from several host threads never undercut another
  (void)bytes;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_per_block());
}

size_t al(size_t n) { return (n + 1) & ~size_t(1); }

}  // namespace

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int max_smem_per_block() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

static size_t fft_bufs(const DevCtx& c, int rows, bool third) {
  return (third ? 3 : 2) * al((size_t)rows * c.N);
}

dim3 table_grid(int gx, int nrow, int threads) {
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    return cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0 ? n : 152;
  }();
  const int want = std::max(1, 2 * sms * (2048 / threads) / std::max(gx, 1));
  return dim3(gx, std::min(std::min(nrow, want), 65535));
}

size_t smem_wem(const DevCtx& c, int G) {
  return 8 * (al(c.N) + fft_bufs(c, G, c.nref > 1) + 2 * al((size_t)G * c.nxg));
}
size_t smem_born_fwd(const DevCtx& c, int G) {
  return 8 * (al(c.N) + fft_bufs(c, 2 * G, c.nref > 1 || c.ntaylor > 1) + 2 * al((size_t)2 * G * c.nxg) +
              2 * al((size_t)G * c.nxg));
}
size_t smem_born_adj(const DevCtx& c, int G) {
  return 8 * (al(c.N) + fft_bufs(c, G, c.nref > 1 || c.ntaylor > 1) + 5 * al((size_t)G * c.nxg) + al(c.nxg));
}
size_t smem_rows(const DevCtx& c, int G) { return 8 * (al(c.N) + fft_bufs(c, G, true) + 2 * al((size_t)G * c.nxg)); }

void launch_phase_tables(const DevCtx& c, const float2* sref, float eps, float2* ph, cudaStream_t st) {
  const int nrow = c.nfreq * c.nz * c.nref;
  const dim3 grid = table_grid((c.N + 255) / 256, nrow, 256);
  k_phase<<<grid, 256, 0, st>>>(c, sref, eps, ph);
  note_launch();
}

void launch_fac_tables(const DevCtx& c, const float2* q, float2* fac, cudaStream_t st) {
  const int nrow = c.nfreq * c.nz;
  const dim3 grid = table_grid((c.nxg + 127) / 128, nrow, 128);
  k_fac<<<grid, 128, 0, st>>>(c, q, fac);
  note_launch();
}

void launch_wem(const DevCtx& c, const Group* groups, int ngroups, int G, float2* store, float2* bins,
                cudaStream_t st) {
  size_t sm = smem_wem(c, G);
  set_smem(k_wem, sm);
  k_wem<<<ngroups, kThreads, sm, st>>>(c, groups, G, store, bins);
  note_launch();
}

void launch_born_fwd(const DevCtx& c, const Group* groups, int ngroups, int G, const float2* dm,
                     const float2* drm, float2* storeA, float2* storeB, float2* bins, cudaStream_t st) {
  size_t sm = smem_born_fwd(c, G);
  set_smem(k_born_fwd, sm);
  k_born_fwd<<<ngroups, kThreads, sm, st>>>(c, groups, G, dm, drm, storeA, storeB, bins);
  note_launch();
}

void launch_born_adj(const DevCtx& c, const Group* groups, int ngroups, int G, float2* storeBG, float2* storeT,
                     const float2* bins, float2* imgR, float2* imgS, int compat, cudaStream_t st) {
  size_t sm = smem_born_adj(c, G);
  set_smem(k_born_adj, sm);
  k_born_adj<<<ngroups, kThreads, sm, st>>>(c, groups, G, storeBG, storeT, bins, imgR, imgS, compat);
  note_launch();
}

void launch_onestep(const DevCtx& c, int f, int z, int adj, const float2* in, float2* out, int nrow, int add,
                    int G, cudaStream_t st) {
  size_t sm = smem_rows(c, G);
  set_smem(k_onestep, sm);
  k_onestep<<<(nrow + G - 1) / G, kThreads, sm, st>>>(c, f, z, adj, in, out, nrow, add, G);
  note_launch();
}

void launch_scatter(const DevCtx& c, int f, int z, int adj, int exact, const float2* in, float2* out, int nrow,
                    int add, int G, cudaStream_t st) {
  size_t sm = smem_rows(c, G);
  set_smem(k_scatter, sm);
  int mode = adj ? (exact ? 2 : 1) : 0;
  k_scatter<<<(nrow + G - 1) / G, kThreads, sm, st>>>(c, f, z, mode, in, out, nrow, add, G);
  note_launch();
}

void launch_oneway(const DevCtx& c, int f, int up, int adj, int recursive, const float2* in, float2* out,
                   int nrow, int add, int G, cudaStream_t st) {
  size_t sm = smem_rows(c, G);
  set_smem(k_oneway, sm);
  k_oneway<<<(nrow + G - 1) / G, kThreads, sm, st>>>(c, f, up, adj, recursive, in, out, nrow, add, G);
  note_launch();
}

void launch_pad_model(const float2* in, float2* out, int M, int nz, int nx, int pad, cudaStream_t st) {
  size_t n = (size_t)M * nz * (nx + 2 * pad);
  k_pad_model<<<grid_for(n), 256, 0, st>>>(in, out, M, nz, nx, pad);
  note_launch();
}

void launch_drefl_fwd(const DevCtx& c, int M, const float2* a0, const float2* b0, const float2* a1,
                      const float2* b1, const float2* dm0, const float2* dm1, float2* out, cudaStream_t st) {
  size_t n = (size_t)M * c.nz * c.nxg;
  k_drefl_fwd<<<grid_for(n), 256, 0, st>>>(M, c.nz, c.nxg, a0, b0, a1, b1, dm0, dm1, out);
  note_launch();
}

void launch_reduce_images(const float2* parts, const int* slice_beg, int M, size_t plane, float2* out,
                          cudaStream_t st) {
  size_t n = (size_t)M * plane;
  k_reduce<<<grid_for(n), 256, 0, st>>>(parts, slice_beg, M, plane, out);
  note_launch();
}

void launch_grad_assemble(const DevCtx& c, int M, const float2* a0, const float2* b0, const float2* a1,
                          const float2* b1, const float2* IR, const float2* IS, float2* g0, float2* g1, int nx,
                          int add, cudaStream_t st) {
  size_t n = (size_t)M * c.nz * nx;
  k_grad<<<grid_for(n), 256, 0, st>>>(M, c.nz, c.nxg, nx, c.pad, a0, b0, a1, b1, IR, IS, g0, g1, add);
  note_launch();
}

void launch_bin_window(const float2* src, float2* dst, int nrows, int ldu, int nf, int off, int to_user, int add,
                       cudaStream_t st) {
  const size_t n = (size_t)nrows * (to_user ? ldu : nf);
  k_bin_window<<<grid_for(n), 256, 0, st>>>(src, dst, nrows, ldu, nf, off, to_user, add);
  note_launch();
}

void launch_copy_rows(const float2* src, int lds, float2* dst, int ldd, int nrows, int ncopy, int add,
                      cudaStream_t st) {
  size_t n = (size_t)nrows * ldd;
  k_copy_rows<<<grid_for(n), 256, 0, st>>>(src, lds, dst, ldd, nrows, ncopy, add);
  note_launch();
}

void launch_scale_add(float2* y, const float2* x, size_t n, cudaStream_t st) {
  k_add<<<grid_for(n), 256, 0, st>>>(y, x, n);
  note_launch();
}

}  // namespace wg
