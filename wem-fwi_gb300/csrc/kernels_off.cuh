// Sweep kernels of the subsurface-offset extended reflectivity Born on
// per-shot apertures.  Per (shot, frequency) row, as BornRefl
// (propagator/src/ext_born_refl.cpp:8-105) on the shot's aperture:
//   forward  bg = Down(src); sc(x) = sum_l r_l(x - l) bg(x - 2 l); Up(sc); record
//   adjoint  bg = Down(src); a = Up^H(rec^H d); I_l(x) += conj(bg(x - l)) a(x + l)
// The lag sums live in offset.cu; this file holds the three depth sweeps:
//   mode 0  bg:  W[0] = src(0), W[z+1] = P_z W[z] + src(z+1), every depth stored
//   mode 1  up:  W[nz-1] = sc[nz-1], W[z-1] = P_z W[z] + sc[z-1], recorded at
//                every depth (OneWay.cpp:82, Injection.cpp:69-80)
//   mode 2  Up^H: W[0] = rec(0), W[z+1] = P^H_{z+1} W[z] + rec(z+1), stored
// One warp owns one row in registers (the natural layout of wfft.cuh); the
// rows of a CTA are frequencies of one shot.  Every row has its own phase
// and split-step tables (built once per background by launch_off_tables):
// each warp copies its next depth's rows into its own shared-memory slots
// with cp.async as soon as the current depth has read them, so the copy runs
// under the rest of the step and the next transform.
#pragma once
#include "kernels_w.cuh"
#include "phase.cuh"

namespace wg {
namespace {

// [tw: tw_entries][exchange: kOffRows x wbuf][table slots: kOffRows x (N + nxg_max)]
template <int E>
struct OffCarve {
  float2* tw;
  float2* sb0;
  float2* slots;
  __host__ __device__ static size_t up16(size_t b) { return (b + 15) & ~size_t(15); }
  __host__ __device__ static size_t bytes(int nxg_max) {
    return up16((size_t)tw_entries<E>() * 8) + up16((size_t)kOffRows * wbuf_len<E>() * 8) +
           up16((size_t)kOffRows * (32 * E + nxg_max) * 8);
  }
  __device__ explicit OffCarve(int nxg_max) {
    extern __shared__ float4 smem4[];
    char* p = reinterpret_cast<char*>(smem4);
    auto take = [&](size_t b) {
      char* r = p;
      p += up16(b);
      return r;
    };
    tw = reinterpret_cast<float2*>(take((size_t)tw_entries<E>() * 8));
    sb0 = reinterpret_cast<float2*>(take((size_t)kOffRows * wbuf_len<E>() * 8));
    slots = reinterpret_cast<float2*>(take((size_t)kOffRows * (32 * E + nxg_max) * 8));
  }
};

template <int E, int MODE>
__global__ void __launch_bounds__(kOffRows * 32, 1) kw_off(OffCtx c, const OffGroup* groups, float2* store,
                                                           float2* bins, int nxg_max) {
  constexpr int N = 32 * E;
  const OffCarve<E> sm(nxg_max);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const OffGroup gp = groups[blockIdx.x];
  const int s = gp.s, nz = c.nz;
  const int x0 = c.x0[s], nxg = c.w[s] + 2 * c.pad, tap = c.tap[s];
  // twiddles in wfft.cuh's per-stage layout
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
  __syncthreads();
  const bool act = warp < gp.n;
  if (!act) return;  // no barrier below this point: the warps run on their own
  const int f = gp.f0 + warp;
  const size_t row = (size_t)gp.row0 + warp;
  float2* Fr = store + c.roff[row];          // this row's field [nz][nxg]
  const float2* PH = c.tph + c.poff[row];    // [nz][N]
  const float2* FA = c.tfac + c.roff[row];   // [nz][nxg]
  float2* sb = sm.sb0 + warp * wbuf_len<E>();
  float2* sph = sm.slots + (size_t)warp * (N + nxg_max);
  float2* sfa = sph + N;
  const float2 zero = make_float2(0.f, 0.f);
  const int nsteps = nz - 1;
  auto dep = [&](int i) { return MODE == 0 ? i : (MODE == 1 ? nz - 1 - i : i + 1); };
  // the tables of step i into the slots; every lane commits a group per call
  auto issue_ph = [&](int i) {
    if (i < nsteps) warp_copy(sph, PH + (size_t)dep(i) * N, N * 8, lane);
    cp_commit();
  };
  auto issue_fa = [&](int i) {
    if (i < nsteps) warp_copy(sfa, FA + (size_t)dep(i) * nxg, nxg * 8, lane);
    cp_commit();
  };
  // all but the latest group landed, for every lane of the warp
  auto ready = [&]() {
    cp_wait1();
    __syncwarp();
  };
  // grid index of register j (clamped) and whether it is on the aperture
  auto xat = [&](int j, bool& in) {
    const int x = lane + 32 * j - tap;
    in = (unsigned)x < (unsigned)nxg;
    return in ? x : 0;
  };
  float2 W[E], X[E];

  auto store_row = [&](int z) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xat(j, in);
      if (in) Fr[(size_t)z * nxg + x] = W[j];
    }
  };
  // Injection.cpp:8-19 on the aperture
  auto inject_src = [&](int z) {
    if (c.sz[s] != z) return;
    const float2 wv = c.wave[f];
    const int p0 = c.sptr ? c.sptr[s] : s, p1 = c.sptr ? c.sptr[s + 1] : s + 1;
    for (int pt = p0; pt < p1; ++pt)
      for (int g = -c.ngs; g <= c.ngs; ++g) {
        const int x = c.sx[pt] - x0 + g + c.pad;
        if (x < 0 || x >= nxg) continue;
        const int n = x + tap;
        if ((n & 31) != lane) continue;
        const int jn = n >> 5;
        const float2 a = c_scale(wv, c.gs[g + c.ngs]);
#pragma unroll
        for (int j = 0; j < E; ++j)
          if (j == jn) W[j] = c_add(W[j], a);
      }
  };
  // data[s][i][f] += sum_g gr[g] W[x_i + g] (Injection.cpp:69-80)
  auto record = [&](int z) {
    const int* rp = c.rptr + (size_t)s * (nz + 1);
    const int k0 = rp[z], k1 = rp[z + 1];
    if (k0 == k1) return;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E; ++j) sb[swz<E>(lane + 32 * j)] = W[j];
    __syncwarp();
    for (int k = k0 + lane; k < k1; k += 32) {
      const int xr = c.rxc[k] - x0 + c.pad;
      float2 acc = zero;
      for (int g = -c.ngr; g <= c.ngr; ++g) {
        const int x = xr + g;
        if (x >= 0 && x < nxg) acc = c_add(acc, c_scale(sb[swz<E>(x + tap)], c.gr[g + c.ngr]));
      }
      float2* d = bins + ((size_t)s * c.nr + c.rid[k]) * c.nfreq + f;
      *d = c_add(*d, acc);
    }
    __syncwarp();
  };
  // W += receivers of depth z spreading data[s][.][f] (Injection.cpp:56-67)
  auto inject_rec = [&](int z) {
    const int* rp = c.rptr + (size_t)s * (nz + 1);
    const int k0 = rp[z], k1 = rp[z + 1];
    if (k0 == k1) return;
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xat(j, in);
      if (!in) continue;
      const int lo = x - c.pad + x0 - c.ngr, hi = x - c.pad + x0 + c.ngr;
      int a = k0, b = k1;
      while (a < b) {
        const int mid = (a + b) >> 1;
        if (c.rxc[mid] < lo) a = mid + 1; else b = mid;
      }
      float2 acc = zero;
      for (int k = a; k < k1 && c.rxc[k] <= hi; ++k) {
        const int g = x - c.pad + x0 - c.rxc[k];
        acc = c_add(acc, c_scale(bins[((size_t)s * c.nr + c.rid[k]) * c.nfreq + f], c.gr[g + c.ngr]));
      }
      W[j] = c_add(W[j], acc);
    }
  };
  // W = P_d W (SSF.cpp:8-31 with one reference): FFT, phase, IFFT, split step
  auto step_fwd = [&](int i) {
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = W[j];
    wfft<E, false>(X, sb, sm.tw, lane);
    ready();
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = c_mul(X[j], sph[lane + 32 * j]);
    __syncwarp();
    issue_ph(i + 1);
    wfft<E, true>(X, sb, sm.tw, lane);
    ready();
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xat(j, in);
      const float2 fx = sfa[x];
      W[j] = in ? c_mul(X[j], fx) : zero;
    }
    __syncwarp();
    issue_fa(i + 1);
  };
  // W = P^H_d W (SSF.cpp:33-60): conj(split step), FFT, conj(phase), IFFT
  auto step_adj = [&](int i) {
    ready();
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xat(j, in);
      const float2 fx = sfa[x];
      X[j] = in ? c_mulc(W[j], fx) : zero;
    }
    __syncwarp();
    issue_fa(i + 1);
    wfft<E, false>(X, sb, sm.tw, lane);
    ready();
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = c_mulc(X[j], sph[lane + 32 * j]);
    __syncwarp();
    issue_ph(i + 1);
    wfft<E, true>(X, sb, sm.tw, lane);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      xat(j, in);
      W[j] = in ? X[j] : zero;
    }
  };

  w_zero<E>(W);
  if (MODE == 2) {
    issue_fa(0);
    issue_ph(0);
  } else {
    issue_ph(0);
    issue_fa(0);
  }
  if (MODE == 0) {
    inject_src(0);
    store_row(0);
  } else if (MODE == 1) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xat(j, in);
      const float2 v = Fr[(size_t)(nz - 1) * nxg + x];
      W[j] = in ? v : zero;
    }
    record(nz - 1);
  } else {
    inject_rec(0);
    store_row(0);
  }
  for (int i = 0; i < nsteps; ++i) {
    const int d = dep(i);
    if (MODE == 1) {
      if (lane == 0 && d >= 2) l2_prefetch(Fr + (size_t)(d - 2) * nxg, nxg * 8);
      step_fwd(i);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const int x = xat(j, in);
        const float2 v = Fr[(size_t)(d - 1) * nxg + x];
        if (in) W[j] = c_add(W[j], v);
      }
      record(d - 1);
    } else if (MODE == 0) {
      step_fwd(i);
      inject_src(d + 1);
      store_row(d + 1);
    } else {
      step_adj(i);
      inject_rec(d);
      store_row(d);
    }
  }
  cp_wait0();
}

}  // namespace

template <int E>
void launch_off_w(int mode, const OffCtx& c, const OffGroup* g, int ng, int nxg_max, float2* store, float2* bins,
                  cudaStream_t st) {
  init_w96();
  const size_t sm = OffCarve<E>::bytes(nxg_max);
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<ng, kOffRows * 32, sm, st>>>(c, g, store, bins, nxg_max);
    note_launch();
  };
  if (mode == 0) go(kw_off<E, 0>);
  else if (mode == 1) go(kw_off<E, 1>);
  else go(kw_off<E, 2>);
}

template <int E>
size_t off_smem_w(int nxg_max) {
  return OffCarve<E>::bytes(nxg_max);
}

}  // namespace wg
