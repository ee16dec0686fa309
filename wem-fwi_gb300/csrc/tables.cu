// Background tables built on the GPU, in double precision: the per-task
// set-up the reference repeats for every shot (propagator/src/wem_prop.cpp:
// 26-41, born_prop.cpp:36-58), computed once per background for all rows.
#include <algorithm>
#include <cmath>

#include "kernels.h"

namespace wg {
namespace {

struct cdd {
  double x, y;
};
__device__ __forceinline__ cdd mk(double x, double y) { return cdd{x, y}; }
__device__ __forceinline__ cdd mk(float2 v) { return cdd{(double)v.x, (double)v.y}; }
__device__ __forceinline__ cdd add(cdd a, cdd b) { return mk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cdd sub(cdd a, cdd b) { return mk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ cdd mul(cdd a, cdd b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cdd dvd(cdd a, cdd b) {
  double d = b.x * b.x + b.y * b.y;
  return mk((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// principal square root
__device__ __forceinline__ cdd csqrt(cdd a) {
  double r = hypot(a.x, a.y);
  double re = sqrt(fmax(0.5 * (r + a.x), 0.0));
  double im = sqrt(fmax(0.5 * (r - a.x), 0.0));
  return mk(re, a.y < 0 ? -im : im);
}
// The complex powers of the tables, exp(p Log a) on the principal branch,
// are written algebraically (no FP64 logarithm, exponential or angle):
// a^-2 = 1 / (a a) and a^(-1/2 - k) = (1 / csqrt(a)) (1 / a)^k.
__device__ __forceinline__ float2 f2(cdd a) { return make_float2((float)a.x, (float)a.y); }

// edge-extended pad along x (operator/src/Pad.h:77-96, extend = true)
__global__ void k_pad_edge(const float2* in, float2* out, int M, int nz, int nx, int pad) {
  const int nxg = nx + 2 * pad;
  const size_t total = (size_t)M * nz * nxg;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % nxg) - pad;
    size_t rz = i / nxg;
    x = x < 0 ? 0 : (x >= nx ? nx - 1 : x);
    out[i] = in[rz * nx + x];
  }
}

// reference slownesses sampled at x = nxg/(2 nref) + j nxg/nref
// (RefSampler.cpp:28-39); the reference refuses a real part <= 0, so the
// smallest flat index of such an entry goes to *bad (atomicMin)
__global__ void k_sref(const float2* sp, float2* sref, int M, int nz, int nxg, int nref, int* bad) {
  const size_t total = (size_t)M * nz * nref;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int j = (int)(i % nref);
    size_t mz = i / nref;
    int off = nxg / (2 * nref) + j * nxg / nref;
    const float2 v = sp[mz * nxg + off];
    sref[i] = v;
    if (bad && !(v.x > 0.f)) atomicMin(bad, (int)i);
  }
}

// RefSampler partition (RefSampler.cpp:41-84) on the device, one CTA per
// model slice.  The reference keeps its reference values in an nx-long
// buffer that survives across depths: every depth overwrites the buffer's
// first nref entries (after the previous depth's sort, its nref smallest)
// with the depth's references and sorts the whole buffer again, so the
// thresholds of depth z are the K = max(nref, 2) smallest values of a
// multiset that starts as nx zeros and, per depth, loses its nref smallest
// values and gains the depth's references.  One thread replays that multiset
// as a zero count plus a binary min-heap in shared memory and writes the K
// thresholds of every depth; when the zeros cannot run out (nx - nz nref >=
// K) every threshold is 0 and the replay is skipped.  Every thread also
// writes, per depth, the references' indices in ascending order of their
// real part (stable, as the float comparisons of the reference).
__global__ void k_refs_hist(const float2* sref, int nz, int nxg, int nref, int K, int replay, float* thr,
                            signed char* rord) {
  extern __shared__ float heap[];
  const int m = blockIdx.x;
  for (int z = threadIdx.x; z < nz; z += blockDim.x) {
    const float2* r = sref + ((size_t)m * nz + z) * nref;
    signed char* o = rord + ((size_t)m * nz + z) * nref;
    for (int j = 0; j < nref; ++j) o[j] = (signed char)j;
    for (int i = 1; i < nref; ++i) {
      const signed char key = o[i];
      const float kv = r[key].x;
      int k = i - 1;
      while (k >= 0 && r[o[k]].x > kv) {
        o[k + 1] = o[k];
        --k;
      }
      o[k + 1] = key;
    }
  }
  float* t = thr + (size_t)m * nz * K;
  if (!replay) {
    for (int i = threadIdx.x; i < nz * K; i += blockDim.x) t[i] = 0.f;
    return;
  }
  if (threadIdx.x != 0) return;
  int zeros = nxg, sz = 0;
  auto push = [&](float v) {
    int i = sz++;
    while (i > 0) {
      const int p = (i - 1) >> 1;
      if (heap[p] <= v) break;
      heap[i] = heap[p];
      i = p;
    }
    heap[i] = v;
  };
  // the smallest value of the multiset (zeros counted apart), removed
  auto pop = [&]() -> float {
    if (zeros > 0 && (sz == 0 || !(heap[0] < 0.f))) {
      --zeros;
      return 0.f;
    }
    const float top = heap[0];
    const float v = heap[--sz];
    int i = 0;
    for (;;) {
      int c = 2 * i + 1;
      if (c >= sz) break;
      if (c + 1 < sz && heap[c + 1] < heap[c]) ++c;
      if (!(heap[c] < v)) break;
      heap[i] = heap[c];
      i = c;
    }
    if (sz > 0) heap[i] = v;
    return top;
  };
  for (int j = 0; j < nref; ++j) pop();  // depth 0 overwrites nref of the initial zeros
  for (int z = 0; z < nz; ++z) {
    const float2* r = sref + ((size_t)m * nz + z) * nref;
    for (int j = 0; j < nref; ++j) push(r[j].x);
    // the K smallest are the thresholds; the nref smallest are also the
    // entries the next depth overwrites, so only the rest go back
    for (int k = 0; k < K; ++k) t[(size_t)z * K + k] = pop();
    for (int k = nref; k < K; ++k) push(t[(size_t)z * K + k]);
  }
}

// reference index of every point: in the as-coded partition the sorted
// slowness is cut where `s - h_j < h_{j+1} - s` (float differences) first
// fails, so a point belongs to the first j < nref - 1 whose test it passes,
// else to the last, and group j is the j-th reference in ascending order
// (nref = 1: points passing the test get none, -1).  The nearest partition
// takes the reference of smallest |s - s_ref| (real parts, double, first of
// equals).
__global__ void k_refs_assign(const float2* sp, const float2* sref, const float* thr, const signed char* rord,
                              int M, int nz, int nxg, int nref, int K, int nearest, signed char* ref) {
  const size_t plane = (size_t)nz * nxg, total = (size_t)M * plane;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t mz = i / nxg;
    const float v = sp[i].x;
    int out;
    if (nearest) {
      const float2* r = sref + mz * nref;
      const double dv = (double)v;
      int best = 0;
      double bd = fabs(dv - (double)r[0].x);
      for (int j = 1; j < nref; ++j) {
        const double d = fabs(dv - (double)r[j].x);
        if (d < bd) {
          bd = d;
          best = j;
        }
      }
      out = best;
    } else {
      const float* h = thr + mz * K;
      if (nref == 1) {
        out = __fsub_rn(v, h[0]) < __fsub_rn(h[1], v) ? -1 : 0;
      } else {
        int g = nref - 1;
        for (int j = 0; j < nref - 1; ++j)
          if (__fsub_rn(v, h[j]) < __fsub_rn(h[j + 1], v)) {
            g = j;
            break;
          }
        out = rord[mz * nref + g];
      }
    }
    ref[i] = (signed char)out;
  }
}

// split step q (SplitStep.cpp:12-13), Reflect (Reflect.h:19-26), Scatter
// coefficients (Scatter.cpp:77-86, Scatter.h:36) and dReflect pairs
// (dReflect.h:18-27, 40-47) of every padded point
__global__ void k_point_tables(int M, int nz, int nxg, int nref, int nt, double eps, const float2* sp,
                               const float2* spr, const float2* dp, const float2* sref, const signed char* ref,
                               float2* q, float2* rc, float2* sc, float2* a0, float2* b0, float2* a1, float2* b1) {
  const size_t plane = (size_t)nz * nxg;
  const size_t total = (size_t)M * plane;
  const double coef[5] = {1., 1. / 2., 3. / 8., 5. / 16., 35. / 128.};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(i / plane);
    const size_t p = i - (size_t)m * plane;
    const int z = (int)(p / nxg);
    const cdd s = mk(sp[i]), d = mk(dp[i]);
    if (q) {
      int j = ref[i];
      cdd v = mk(0, 0);
      if (j >= 0) {
        cdd sr = mk(sref[((size_t)m * nz + z) * nref + j]);
        v = dvd(sub(s, sr), csqrt(sr));
      }
      q[i] = f2(v);
    }
    cdd r = mk(0, 0), va0 = r, vb0 = r, va1 = r, vb1 = r;
    if (z >= 1) {
      const cdd du = mk(dp[i - nxg]);
      {
        // Reflect is built from spr, the slowness before any conformal-map
        // Jacobian (born_prop.cpp:44-47); dReflect, built after the scaling
        // from the same arrays (Born_refl.cpp:10-11), and the split step
        // and Scatter see sp
        const cdd sr = mk(spr[i]), sur = mk(spr[i - nxg]);
        const cdd u = mul(d, csqrt(sur)), w = mul(du, csqrt(sr));
        r = dvd(sub(u, w), add(u, w));
      }
      if (sc) {
        const cdd su = mk(sp[i - nxg]);
        const cdd u = mul(d, csqrt(su)), w = mul(du, csqrt(s));
        // v = (u + w)^-2; dividing by v multiplies by (u + w)^2
        const cdd uw = add(u, w), uw2 = mul(uw, uw);
        cdd s1s2 = mul(mul(du, d), uw2);
        cdd r1r2 = mul(mul(mk(2, 0), mul(su, s)), uw2);
        cdd cc = csqrt(dvd(s, su));
        va0 = mul(cc, s1s2);
        vb0 = mul(dvd(mk(1, 0), cc), s1s2);
        va1 = mul(du, r1r2);
        vb1 = mul(d, r1r2);
      }
    }
    rc[i] = f2(r);
    if (sc) {
      a0[i] = f2(va0);
      b0[i] = f2(vb0);
      a1[i] = f2(va1);
      b1[i] = f2(vb1);
      const cdd base = mk(s.x - eps * s.x, s.y);
      const cdd one = mk(1, 0), inv = dvd(one, base);
      cdd pw = dvd(one, csqrt(base));  // base^(-1/2 - it)
      for (int it = 0; it < nt; ++it) {
        sc[((size_t)m * nt + it) * plane + p] = f2(mul(mk(coef[it], 0), pw));
        pw = mul(pw, inv);
      }
    }
  }
}

int grid_of(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? (b ? b : 1) : 152 * 32);
}

}  // namespace

void launch_pad_edge(const float2* in, float2* out, int M, int nz, int nx, int pad, cudaStream_t st) {
  size_t n = (size_t)M * nz * (nx + 2 * pad);
  k_pad_edge<<<grid_of(n), 256, 0, st>>>(in, out, M, nz, nx, pad);
  note_launch();
}

void launch_sref(const float2* sp, float2* sref, int M, int nz, int nxg, int nref, int* bad, cudaStream_t st) {
  size_t n = (size_t)M * nz * nref;
  k_sref<<<grid_of(n), 256, 0, st>>>(sp, sref, M, nz, nxg, nref, bad);
  note_launch();
}

size_t refs_scratch_floats(int M, int nz, int nref) {
  const int K = nref > 2 ? nref : 2;
  return (size_t)M * nz * K + ((size_t)M * nz * nref + 3) / 4;
}

void launch_refsampler(int nearest, const float2* sp, const float2* sref, int M, int nz, int nxg, int nref,
                       float* scratch, signed char* ref, cudaStream_t st) {
  const int K = nref > 2 ? nref : 2;
  float* thr = scratch;
  signed char* rord = reinterpret_cast<signed char*>(scratch + (size_t)M * nz * K);
  if (!nearest) {
    const int replay = (long long)nxg - (long long)nz * nref >= K ? 0 : 1;
    const size_t smem = replay ? (size_t)nxg * sizeof(float) : 0;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_refs_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_refs_hist<<<M, 128, smem, st>>>(sref, nz, nxg, nref, K, replay, thr, rord);
    note_launch();
  }
  const size_t n = (size_t)M * nz * nxg;
  k_refs_assign<<<grid_of(n), 256, 0, st>>>(sp, sref, thr, rord, M, nz, nxg, nref, K, nearest, ref);
  note_launch();
}

void launch_point_tables(int M, int nz, int nxg, int nref, int ntaylor, float eps, const float2* sp,
                         const float2* sp_refl, const float2* dp, const float2* sref, const signed char* ref,
                         float2* q, float2* rc, float2* sc, float2* a0, float2* b0, float2* a1, float2* b1,
                         cudaStream_t st) {
  size_t n = (size_t)M * nz * nxg;
  k_point_tables<<<grid_of(n), 256, 0, st>>>(M, nz, nxg, nref, ntaylor + 1, (double)eps, sp, sp_refl ? sp_refl : sp,
                                             dp, sref, ref, q, rc, sc, a0, b0, a1, b1);
  note_launch();
}

// ---- subsurface-offset Born: per-shot apertures
namespace {
// grid (nz, ns): aperture row of shot s at depth z, edge-extended by pad
__global__ void k_off_crop(OffCtx c, const float2* s2, float2* sp) {
  const int z = blockIdx.x, s = blockIdx.y;
  const int w = c.w[s], nxg = w + 2 * c.pad, x0 = c.x0[s];
  float2* o = sp + c.toff[s] + (size_t)z * nxg;
  const float2* in = s2 + (size_t)z * c.nx + x0;
  for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
    int k = x - c.pad;
    k = k < 0 ? 0 : (k >= w ? w - 1 : k);
    o[x] = in[k];
  }
}
// q as k_point_tables (double, rounded once), (0, kOffNoRef) without a reference
__global__ void k_off_q(OffCtx c, const float2* sp, const signed char* ref, int ssf, float2* q) {
  const int z = blockIdx.x, s = blockIdx.y;
  const int nxg = c.w[s] + 2 * c.pad;
  const size_t o = c.toff[s] + (size_t)z * nxg;
  const cdd sr = mk(c.sref[(size_t)s * c.nz + z]);
  const cdd rs = csqrt(sr);
  for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
    float2 v = make_float2(0.f, kOffNoRef);
    if (ref[o + x] >= 0) v = ssf ? f2(dvd(sub(mk(sp[o + x]), sr), rs)) : make_float2(0.f, 0.f);
    q[o + x] = v;
  }
}
}  // namespace

void launch_off_crop(const OffCtx& c, const float2* s2, int nxg_max, float2* sp, cudaStream_t st) {
  k_off_crop<<<dim3(c.nz, c.ns), std::min(1024, (nxg_max + 31) / 32 * 32), 0, st>>>(c, s2, sp);
  note_launch();
}

void launch_off_q(const OffCtx& c, const float2* sp, const signed char* ref, int ssf, int nxg_max, float2* q,
                  cudaStream_t st) {
  k_off_q<<<dim3(c.nz, c.ns), std::min(1024, (nxg_max + 31) / 32 * 32), 0, st>>>(c, sp, ref, ssf, q);
  note_launch();
}

// ---- conformal maps
namespace {
__global__ void k_cmap_gather(const float2* in, const int* idx, float2* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = idx[i];
  out[i] = j >= 0 ? in[j] : make_float2(0.f, 0.f);
}
__global__ void k_cmap_gather_add(const float2* in, const int* idx, float2* out, int n, int add) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = idx[i];
  const float2 v = j >= 0 ? in[j] : make_float2(0.f, 0.f);
  out[i] = add ? make_float2(out[i].x + v.x, out[i].y + v.y) : v;
}
// ConformalMap::scaleByJacobian twice on the padded slowness, by flat index
__global__ void k_cmap_jacobian(float2* sp, int n, float js, const float* jl) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float2 v = sp[k];
  for (int rep = 0; rep < 2; ++rep) {
    v.x = __fmul_rn(v.x, js);
    v.y = __fmul_rn(v.y, js);
    if (jl) {
      v.x = __fmul_rn(v.x, jl[k]);
      v.y = __fmul_rn(v.y, jl[k]);
    }
  }
  sp[k] = v;
}
}  // namespace

void launch_cmap_gather(const float2* in, const int* idx, float2* out, int n, int add, cudaStream_t st) {
  if (add < 0) k_cmap_gather<<<(n + 255) / 256, 256, 0, st>>>(in, idx, out, n);
  else k_cmap_gather_add<<<(n + 255) / 256, 256, 0, st>>>(in, idx, out, n, add);
  note_launch();
}

void launch_cmap_jacobian(float2* sp, int n, float js, const float* jl, cudaStream_t st) {
  k_cmap_jacobian<<<(n + 255) / 256, 256, 0, st>>>(sp, n, js, jl);
  note_launch();
}

}  // namespace wg
