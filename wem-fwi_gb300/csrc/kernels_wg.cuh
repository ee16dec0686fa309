// Exact gradient of the nonlinear modelling (wem_prop.cpp:9-78) on the
// warp-per-row kernels: the adjoint-state derivative of
// L = 1/2 |Re IFFT(d(s, rho)) - d_obs|^2 (or of <g_d, d> for a given data
// gradient) with respect to slowness^2 and density.  The reference's own
// FWI gradient is the Born adjoint (a Taylor-scatter linearisation with the
// references held fixed and the dReflect scaling of dReflect.h:18-24); this
// kernel differentiates the modelled data itself, for a finite-difference
// check and for torch autograd.
//
// Per (shot, frequency) row, with D = Down(src), A = R D, U = Up(A) and the
// data d = rec(D) + rec(U), the adjoint fields are those of the Born
// adjoint: wu = Up^H(rec^H g) and wd = Down^H(rec^H g + conj(R) wu).  The
// gradient has three parts:
//  * Reflect (Reflect.h:19-26): IR = sum conj(D) wu, assembled with the exact
//    derivatives of R = (u - v)/(u + v), u = rho_z sqrt(s_{z-1}),
//    v = rho_{z-1} sqrt(s_z);
//  * the split step (SplitStep.cpp:12-14): P_z W = F_z . IFFT(ph_z FFT W) with
//    F_z = taper exp(-i w dz (s - s_ref)/sqrt(s_ref)) / N, so
//    d(P_z W)/ds(x) = c_z (P_z W)(x), c_z = -i w dz / sqrt(s_ref): the image
//    IL[z] = sum conj(c_z P_z D[z]) wd[z+1] + conj(c_z P_z U[z]) wu[z-1];
//  * the reference slowness of each depth (RefSampler.cpp:28-39), sampled
//    from s at one point: through F_z (holomorphic; assembled from IL) and
//    through the phase-shift factor ph_z (phase_shift.ispc:2-32), whose
//    derivative is Gamma = -i dz ph / (2 kz) times a per-depth combination
//    of the real and imaginary parts: per row and depth the kernel leaves
//    w^2 sum_k conj(FFT(conj(F) lambda))[k] Gamma[k] FFT(W)[k].
// The chains run on two warps per row as in kw_born_adj2: the source side
// carries D down and U up, the receiver side wu down and wd up.  The down
// sweep stores D and T = wu - rec and the two spectra the reference term
// needs (FFT D, FFT(conj(F) wu)); with checkpointing (ck > 1) it stores D
// and T every ck depths only, and the up sweep recomputes each segment of
// ck depths from its checkpoint (the same arithmetic, so the result is the
// same bit for bit) into per-row segment buffers.
#pragma once
#include "kernels_w.cuh"

namespace wg {
namespace {

// principal square root (single precision)
__device__ __forceinline__ float2 c_sqrt(float2 a) {
  const float r = hypotf(a.x, a.y);
  const float re = sqrtf(fmaxf(0.5f * (r + a.x), 0.f)), im = sqrtf(fmaxf(0.5f * (r - a.x), 0.f));
  return make_float2(re, a.y < 0.f ? -im : im);
}

// conj(c_z) = i w dz / conj(sqrt(s_ref)) = i w dz sqrt(s_ref) / |s_ref|
__device__ __forceinline__ float2 conj_cz(float2 sref, float wdz) {
  const float2 r = c_sqrt(sref);
  const float m = wdz / (r.x * r.x + r.y * r.y);
  return make_float2(-r.y * m, r.x * m);
}

// sum over the warp of a complex value (every lane gets the sum)
__device__ __forceinline__ float2 warp_csum(float2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// storage of the gradient pass: full depth rows (ck <= 1) or checkpoints
// every ck depths plus a segment of ck + 1 recomputed depths per row
struct GradStore {
  float2 *bg, *t, *sw, *sg;  // full: [rows][nz][nxg] x 2, [rows][nz][N] x 2; checkpoints: bg, t [rows][ncp][nxg]
  float2* seg;               // [rows][(ck + 1)(2 nxg + 2 N) + 2 N] (checkpoints only)
  float2* il;                // [groups][nz][nxg] split-step image
  float2* ir;                // [groups][nz][nxg] Reflect image
  float2* qs;                // [2][rows][nz] reference terms (source side, receiver side)
  int ck, rows_total;
};

template <int E, bool NT, int R>
__global__ void __launch_bounds__(2 * R * 32, 1) kw_wem_grad(DevCtx c, SlotLayout L, const Group* groups,
                                                             GradStore gs, const float2* bins) {
  constexpr int N = 32 * E;
  const Carve<E> sm(c, L, false, 2 * R, true);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, row = warp >> 1;
  const bool recv = warp & 1;
  stage_static<E>(c, sm);
  const int nxg = c.nxg, nz = c.nz, ck = gs.ck;
  const Group gp = groups[blockIdx.x];
  const int nrows = gp.n;
  const bool act = row < nrows;
  float2* xb = sm.sb0 + warp * wbuf_len<E>();
  const WRow w{c, sm.tw, xb, sm.taperN, sm.kx, lane, NT ? 0 : c.tap, NT ? N : c.nxg};
  const int f = gp.f, s = gp.s0 + (act ? row : 0), bin = c.bin[f];
  const size_t rid = (size_t)gp.row0 + (act ? row : 0);
  const size_t plane = (size_t)nz * nxg, splane = (size_t)nz * N;
  const int ncp = ck > 1 ? (nz - 1) / ck + 1 : nz;
  float2* BG = gs.bg + rid * (size_t)ncp * nxg;
  float2* TT = gs.t + rid * (size_t)ncp * nxg;
  float2* SW = ck > 1 ? nullptr : gs.sw + rid * splane;
  float2* SG = ck > 1 ? nullptr : gs.sg + rid * splane;
  float2* SEG = ck > 1 ? gs.seg + rid * ((size_t)(ck + 1) * (2 * nxg + 2 * N) + 2 * N) : nullptr;
  float2* IR = gs.ir + (size_t)blockIdx.x * plane;
  float2* IL = gs.il + (size_t)blockIdx.x * plane;
  float2* QS = gs.qs + rid * nz;                               // source side
  float2* QR = gs.qs + ((size_t)gs.rows_total + rid) * nz;     // receiver side
  const float om = c.omega[f], w2 = om * om, wdz = om * c.dz;
  const bool has_fac = c.fac != nullptr;
  const float2 zero = make_float2(0.f, 0.f);
  const Ring ring{c, L, sm.ring, Src{nullptr, nullptr}, f};
  const float2* xb0 = sm.sb0;
  constexpr int WB = wbuf_len<E>();
  float2 S[E], X[E], Yd[1];
  int zs = -1;  // first depth of the current segment (checkpoints)

  // rows of the stored fields (full storage or the current segment)
  auto bgrow = [&](int z) -> float2* { return ck > 1 ? SEG + (size_t)(z - zs) * nxg : BG + (size_t)z * nxg; };
  auto trow = [&](int z) -> float2* {
    return ck > 1 ? SEG + (size_t)(ck + 1) * nxg + (size_t)(z - zs) * nxg : TT + (size_t)z * nxg;
  };
  auto swrow = [&](int z) -> float2* {
    return ck > 1 ? SEG + (size_t)(ck + 1) * 2 * nxg + (size_t)(z - zs) * N : SW + (size_t)z * N;
  };
  auto sgrow = [&](int z) -> float2* {
    return ck > 1 ? SEG + (size_t)(ck + 1) * (2 * nxg + N) + (size_t)(z - zs) * N : SG + (size_t)z * N;
  };
  auto store_spec = [&](float2* dst, const float2 (&v)[E]) {
#pragma unroll
    for (int j = 0; j < E; ++j) dst[lane + 32 * j] = v[j];
  };
  auto put = [&](const float2 (&v)[E]) {
#pragma unroll
    for (int j = 0; j < E; ++j) {
      bool in;
      const int x = xclamp(w, j, in);
      if (in) xb[x] = v[j];
    }
  };
  // one step of the source side's down recursion: bg = P_z bg + src(z + 1);
  // the spectrum FFT(bg[z]) to spec when given
  auto src_step = [&](const Tabs& T, int z, float2* spec) {
#pragma unroll
    for (int j = 0; j < E; ++j) X[j] = S[j];
    wfft<E, false>(X, w.sb, w.tw, lane);
    if (spec) store_spec(spec, X);
    fwd_mid<E>(w, T, 0, X);
    wfft<E, true>(X, w.sb, w.tw, lane);
    fwd_post<E, false>(w, T, 0, X, S);
    w_inject_src<E>(w, S, s, f, z + 1);
  };
  // one step of the receiver side's down recursion: T[z + 1] = P^H_{z+1} wu
  // (T the tables of depth z + 1); the spectrum FFT(conj(F) wu) to spec
  auto rec_step = [&](const Tabs& T, float2* spec) {
    adj_pre<E, false>(w, T, 0, S, X);
    wfft<E, false>(X, w.sb, w.tw, lane);
    if (spec) store_spec(spec, X);
    adj_mid<E, false>(w, T, 0, X, Yd);
    wfft<E, true>(X, w.sb, w.tw, lane);
    adj_post<E>(w, X, S);
  };

  // ---------------- down sweep: bg (source side), wu (receiver side), IR
  w_zero<E>(S);
  if (act) {
    if (!recv) {
      w_inject_src<E>(w, S, s, f, 0);
      w_store<E>(w, BG, S);
    } else {
      for (int x = lane; x < nxg; x += 32) TT[x] = zero;  // T[0] = 0
      w_inject_rec<E>(w, S, s, bin, 0, bins);
    }
    put(S);
  }
  ring.issue(0);
  ring.issue(1);
  cp_commit();
  cp_wait0();
  __syncthreads();
  auto reduce_down = [&](float2* out) {
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      float2 a = zero;
      for (int r = 0; r < nrows; ++r) a = c_add(a, c_mulc(xb0[(2 * r + 1) * WB + x], xb0[2 * r * WB + x]));
      out[x] = a;
    }
  };
  reduce_down(IR);
  for (int z = 0; z + 1 < nz; ++z) {
    __syncthreads();
    ring.issue(z + 2);
    cp_commit();
    if (act) {
      const bool keep = ck <= 1 || (z + 1) % ck == 0;
      const int zi = ck > 1 ? (z + 1) / ck : z + 1;
      if (!recv) {
        src_step(ring.stabs(z), z, ck > 1 ? nullptr : SW + (size_t)z * N);
        if (keep) w_store<E>(w, BG + (size_t)zi * nxg, S);
      } else {
        rec_step(ring.stabs(z + 1), ck > 1 ? nullptr : SG + (size_t)(z + 1) * N);
        if (keep) w_store<E>(w, TT + (size_t)zi * nxg, S);
        w_inject_rec<E>(w, S, s, bin, z + 1, bins);
      }
      put(S);
    }
    cp_wait0();
    __syncthreads();
    reduce_down(IR + (size_t)(z + 1) * nxg);
  }
  if (nz < 2) return;

  // ---------------- segment recompute (checkpoints): depths z0 .. z1 of
  // bg, T and their spectra from the checkpoint at z0; tables from global.
  // The recompute runs in S: the up sweep's state waits in one of the
  // segment's two last slots meanwhile (one per warp of the row).  Each
  // side reads rows the other side recomputes, so the caller synchronises
  // the block after it.
  auto recompute = [&](int z0, bool keep_state) {
    zs = z0;
    if (!act) return;
    float2* save = SEG + (size_t)(ck + 1) * (2 * nxg + 2 * N) + (recv ? N : 0);
    if (keep_state) store_spec(save, S);
    const int z1 = min(z0 + ck, nz - 1);
    if (!recv) {
      w_load<E>(w, BG + (size_t)(z0 / ck) * nxg, S);
      w_store<E>(w, bgrow(z0), S);
      for (int z = z0; z < z1; ++z) {
        src_step(global_tabs(c, Src{nullptr, nullptr}, f, z), z, swrow(z));
        w_store<E>(w, bgrow(z + 1), S);
      }
    } else {
      w_load<E>(w, TT + (size_t)(z0 / ck) * nxg, S);
      w_store<E>(w, trow(z0), S);
      w_inject_rec<E>(w, S, s, bin, z0, bins);
      for (int z = z0; z < z1; ++z) {
        rec_step(global_tabs(c, Src{nullptr, nullptr}, f, z + 1), sgrow(z + 1));
        w_store<E>(w, trow(z + 1), S);
        w_inject_rec<E>(w, S, s, bin, z + 1, bins);
      }
    }
    __syncwarp();
    if (keep_state) {
#pragma unroll
      for (int j = 0; j < E; ++j) S[j] = save[lane + 32 * j];
    }
  };

  // ---------------- up sweep: iteration z = nz - 1 .. 1.  Source side:
  // bu[z-1] = P_z bu[z] + R[z-1] bg[z-1] with the terms of depth z;
  // receiver side: wd[z-1] = P^H_{z-1} wd[z] + rec + conj(R[z-1]) wu[z-1]
  // with the terms of depth z - 1.
  __syncthreads();  // the down sweep's buffers are summed; the ring is idle
  if (ck > 1) recompute(((nz - 2) / ck) * ck, false);
  ring.issue(nz - 1);
  ring.issue(nz - 2);
  cp_commit();
  cp_wait0();
  __syncthreads();
  if (act) {
    const Tabs Tl = ring.stabs(nz - 1);
    if (!recv) {
      // bu[nz-1] = R bg[nz-1]
      w_load<E>(w, bgrow(nz - 1), S);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const float2 r = Tl.rc[xclamp(w, j, in)];
        S[j] = in ? c_mul(r, S[j]) : zero;
      }
    } else {
      // wd[nz-1] = conj(R) (T[nz-1] + rec) + rec
      w_load<E>(w, trow(nz - 1), X);
      w_inject_rec<E>(w, X, s, bin, nz - 1, bins);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        bool in;
        const float2 r = Tl.rc[xclamp(w, j, in)];
        S[j] = in ? c_mulc(X[j], r) : zero;
      }
      w_inject_rec<E>(w, S, s, bin, nz - 1, bins);
    }
  }
  const float2* sref = c.sref;
  const int gz = c.ext ? f : 0;
  for (int z = nz - 1; z >= 1; --z) {
    __syncthreads();  // the image buffers are summed; slot (z - 2) % 3 is free
    ring.issue(z - 2);
    cp_commit();
    if (ck > 1 && z - 1 < zs) {
      recompute(((z - 1) / ck) * ck, true);
      __syncthreads();  // bg rows for the receiver sides, T rows for the source sides
    }
    if (act) {
      const float2* gam = c.gam + ((size_t)f * nz + (recv ? z - 1 : z)) * N;
      if (!recv) {
        // ---- source side, depth z
        const Tabs Tz = ring.stabs(z);
#pragma unroll
        for (int j = 0; j < E; ++j) X[j] = S[j];
        wfft<E, false>(X, w.sb, w.tw, lane);
        // reference term through the phase factor: conj(FFT(conj(F_z) wu[z-1])) Gamma FFT(bu[z])
        {
          const float2* sg = sgrow(z);
          float2 acc = zero;
#pragma unroll
          for (int j = 0; j < E; ++j) acc = c_fmac(acc, c_mul(gam[lane + 32 * j], X[j]), sg[lane + 32 * j]);
          acc = warp_csum(acc);
          if (lane == 0) QS[z] = c_scale(acc, w2);
        }
        fwd_mid<E>(w, Tz, 0, X);
        wfft<E, true>(X, w.sb, w.tw, lane);
        fwd_post<E, false>(w, ring.stabs(launder(z)), 0, X, S);  // S = P_z bu[z]
        if (has_fac) {
          // split-step term of depth z: conj(c_z P_z bu[z]) wu[z-1]
          const float2 cc = conj_cz(sref[((size_t)gz * nz + z) * c.nref], wdz);
          w_load<E>(w, trow(z - 1), X);
          w_inject_rec<E>(w, X, s, bin, z - 1, bins);
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const int x = xclamp(w, j, in);
            if (in) xb[x] = c_mul(cc, c_mulc(X[j], S[j]));
          }
        }
        // bu[z-1] = P_z bu[z] + R[z-1] bg[z-1]
        const Tabs Tp = ring.stabs(z - 1);
        const float2* bgp = bgrow(z - 1);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          bool in;
          const int x = xclamp(w, j, in);
          const float2 r = Tp.rc[x], b = bgp[x];
          if (in) S[j] = c_add(S[j], c_mul(r, b));
        }
      } else {
        // ---- receiver side, depth z - 1
        const Tabs Tq = ring.stabs(z - 1);
        adj_pre<E, false>(w, Tq, 0, S, X);
        wfft<E, false>(X, w.sb, w.tw, lane);
        {
          const float2* sp = swrow(z - 1);
          float2 acc = zero;
#pragma unroll
          for (int j = 0; j < E; ++j) acc = c_fmac(acc, c_mul(gam[lane + 32 * j], sp[lane + 32 * j]), X[j]);
          acc = warp_csum(acc);
          if (lane == 0) QR[z - 1] = c_scale(acc, w2);
        }
        adj_mid<E, false>(w, Tq, 0, X, Yd);
        wfft<E, true>(X, w.sb, w.tw, lane);
        adj_post<E>(w, X, X);  // q = P^H_{z-1} wd[z]
        const int zl = launder(z);
        if (has_fac) {
          // split-step term of depth z - 1: conj(c_{z-1} (bg[z] - src(z))) wd[z]
          const float2 cc = conj_cz(sref[((size_t)gz * nz + zl - 1) * c.nref], wdz);
          const float2* bgz = bgrow(zl);
          const bool at_src = c.sz[s] == zl;
          const int sx0 = c.sx[s] + c.pad;
          const float2 wv = c.wave[f];
#pragma unroll
          for (int j = 0; j < E; ++j) {
            bool in;
            const int x = xclamp(w, j, in);
            float2 pd = bgz[x];
            const int g = x - sx0;
            if (at_src && g >= -c.ngs && g <= c.ngs) pd = c_sub(pd, c_scale(wv, c.gs[g + c.ngs]));
            if (in) xb[x] = c_mul(cc, c_mulc(S[j], pd));
          }
        }
        // wd[z-1] = q + rec + conj(R[z-1]) (T[z-1] + rec)
        const Tabs Tr = ring.stabs(zl - 1);
#pragma unroll
        for (int j = 0; j < E; ++j) S[j] = X[j];
        w_load<E>(w, trow(zl - 1), X);
        w_inject_rec<E>(w, X, s, bin, zl - 1, bins);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          bool in;
          const float2 r = Tr.rc[xclamp(w, j, in)];
          if (in) S[j] = c_add(S[j], c_mulc(X[j], r));
        }
        w_inject_rec<E>(w, S, s, bin, zl - 1, bins);
      }
    }
    cp_wait0();
    __syncthreads();
    if (has_fac) {
      // IL[z] (+)= source sides' terms (row z got the receiver sides' terms
      // one iteration before, unless z = nz - 1); IL[z-1] = receiver sides'
      for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
        float2 a = z + 1 < nz ? IL[(size_t)z * nxg + x] : zero, b = zero;
        for (int r = 0; r < nrows; ++r) {
          a = c_add(a, xb0[2 * r * WB + x]);
          b = c_add(b, xb0[(2 * r + 1) * WB + x]);
        }
        IL[(size_t)z * nxg + x] = a;
        IL[(size_t)(z - 1) * nxg + x] = b;
      }
    }
  }
}

}  // namespace

template <int E>
void launch_grad_w(const DevCtx& c, const Group* g, int ng, const GradArgs& a, cudaStream_t st) {
  init_w96();
  const SlotLayout L = slot_layout<E>(c, 7, max_smem_per_block());
  const size_t sm = smem_w<E>(c, 7, L);
  GradStore gs{a.bg, a.t, a.sw, a.sg, a.seg, a.il, a.ir, a.qs, a.ck, a.rows_total};
  auto go = [&](auto kern) {
    set_max_smem(kern);
    kern<<<ng, 2 * kRowsAdj2 * 32, sm, st>>>(c, L, g, gs, a.bins);
    note_launch();
  };
  if (c.tap == 0) go(kw_wem_grad<E, true, kRowsAdj2>);
  else go(kw_wem_grad<E, false, kRowsAdj2>);
}

// the gradient pass serves this context: one reference and its shared
// memory (the layout of the two-warp Born adjoint without the Scatter rows)
template <int E>
bool grad_fits_w(const DevCtx& c) {
  if (c.nref != 1) return false;
  const SlotLayout L = slot_layout<E>(c, 7, max_smem_per_block());
  return L.nslots == 3 && (c.fac || L.ref >= 0);
}

}  // namespace wg
