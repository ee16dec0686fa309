// Tables and assembly of the exact modelling gradient (kernels_wg.cuh).
//
// The phase-shift factor of a depth (phase_shift.ispc:2-32) is
// ph = exp(-i dz kz) with kz = re + i im the root of a + i b' (b' = -|b| for
// the ISPC law, kz the conjugate root for the exact-kz law), a = w^2 s_re -
// k^2, so d ph = -i dz ph d kz and d kz = (d a + i d b') / (2 kz): every
// derivative of the factor with respect to the reference slowness is
// Gamma = -i dz ph / (2 kz) times w^2 and a per-depth combination of the
// real and imaginary parts of the change.  The kernel sums
// w^2 conj(FFT(conj(F) lambda)) Gamma FFT(W) per row and depth; the
// assembly below turns the sums into the gradient at the reference's sample
// point and adds the split-step and Reflect terms.
#include <cmath>

#include "kernels.h"
#include "wemgpu.h"

namespace wg {
namespace {

// Gamma for every (frequency, depth, reference, k), with the root computed
// exactly as the phase table's (k_phase)
__global__ void k_phase_grad(DevCtx c, const float2* sref, float eps, float2* gam) {
  const int nrow = c.nfreq * c.nz * c.nref;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= c.N) return;
  const float k = c.kx[n];
  for (int r = blockIdx.y; r < nrow; r += gridDim.y) {
    const int j = r % c.nref, z = (r / c.nref) % c.nz, f = r / (c.nref * c.nz);
    const int m = c.ext ? f : 0;
    const float2 s = sref[((size_t)m * c.nz + z) * c.nref + j];
    const float w = c.omega[f], w2 = w * w;
    const float a = fmaf(w2, s.x, -k * k);
    const bool exact = c.phase_law == WEM_PHASE_EXACT_KZ;
    const float b = exact ? fmaf(w2, s.y, 1e-5f) : w2 * fmaf(-eps, s.x, s.y);
    const float cc = sqrtf(fmaf(a, a, b * b));
    float re, im;
    if (a >= 0.f) {
      re = sqrtf(0.5f * (cc + a));
      im = re > 0.f ? -fabsf(b) / (2.f * re) : 0.f;
    } else {
      const float q = sqrtf(0.5f * (cc - a));
      im = -q;
      re = fabsf(b) / (2.f * q);
    }
    if (exact && b < 0.f) im = -im;
    const float e = expf(im * c.dz);
    float sn, cs;
    sincosf(re * c.dz, &sn, &cs);
    const float2 ph = make_float2(e * cs, -e * sn);
    // -i dz ph / (2 kz), kz = re + i im
    const float d = 2.f * (re * re + im * im);
    const float2 q = make_float2((ph.x * re + ph.y * im) / d, (ph.y * re - ph.x * im) / d);  // ph / (2 kz)
    gam[(size_t)r * c.N + n] = make_float2(c.dz * q.y, -c.dz * q.x);
  }
}

// out[z] (+)= sum over rows of both sides' terms, rows in order
__global__ void k_qs_reduce(const float2* qs, int rows, int nz, int add, float2* out) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= nz) return;
  double ax = 0, ay = 0;
  for (int r = 0; r < rows; ++r) {
    const float2 a = qs[(size_t)r * nz + z], b = qs[((size_t)rows + r) * nz + z];
    ax += (double)a.x + (double)b.x;
    ay += (double)a.y + (double)b.y;
  }
  float2 v = make_float2((float)ax, (float)ay);
  if (add) v = make_float2(out[z].x + v.x, out[z].y + v.y);
  out[z] = v;
}

struct cd2 {
  double x, y;
};
__device__ __forceinline__ cd2 mk(double x, double y) { return cd2{x, y}; }
__device__ __forceinline__ cd2 mk(float2 v) { return cd2{(double)v.x, (double)v.y}; }
__device__ __forceinline__ cd2 operator+(cd2 a, cd2 b) { return mk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cd2 operator-(cd2 a, cd2 b) { return mk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ cd2 operator*(cd2 a, cd2 b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cd2 operator/(cd2 a, cd2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return mk((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ cd2 cj(cd2 a) { return mk(a.x, -a.y); }
__device__ __forceinline__ cd2 sq(cd2 a) {
  const double r = hypot(a.x, a.y);
  const double re = sqrt(fmax(0.5 * (r + a.x), 0.0)), im = sqrt(fmax(0.5 * (r - a.x), 0.0));
  return mk(re, a.y < 0 ? -im : im);
}

// the reference terms of every depth: through the split step (holomorphic,
// from IL: sum_x conj(-(s + s_ref) / (2 s_ref)) IL[x] over the points of
// the reference) and through the phase factor (from qsum, with the law's
// combination of real and imaginary parts); one CTA per depth
__global__ void k_exact_ref(DevCtx c, float eps, const float2* sp, const float2* IL, const float2* qsum,
                            float2* gref) {
  const int z = blockIdx.x, nxg = c.nxg;
  __shared__ double rx[256], ry[256];
  const cd2 sr = mk(c.sref[(size_t)z * c.nref]);
  double ax = 0, ay = 0;
  if (c.fac) {
    for (int x = threadIdx.x; x < nxg; x += blockDim.x) {
      if (c.ref[(size_t)z * nxg + x] != 0) continue;
      const cd2 d = mk(0, 0) - (mk(sp[(size_t)z * nxg + x]) + sr) / (mk(2, 0) * sr);
      const cd2 v = cj(d) * mk(IL[(size_t)z * nxg + x]);
      ax += v.x;
      ay += v.y;
    }
  }
  rx[threadIdx.x] = ax;
  ry[threadIdx.x] = ay;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      rx[threadIdx.x] += rx[threadIdx.x + h];
      ry[threadIdx.x] += ry[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double S_re = qsum[z].x, S_im = qsum[z].y;
    double g_re, g_im;
    if (c.phase_law == WEM_PHASE_EXACT_KZ) {
      g_re = S_re;
      g_im = S_im;
    } else {
      // b = w^2 (s_im - eps s_re) and b' = -|b|: d b' = -sign(b) d b
      const double b = (double)sr.y - (double)eps * sr.x;
      const double sb = b > 0 ? 1.0 : -1.0;
      g_re = S_re - sb * eps * S_im;
      g_im = sb * S_im;
    }
    gref[z] = make_float2((float)(rx[0] + g_re), (float)(ry[0] + g_im));
  }
}

// derivatives of R[z] = (u - v)/(u + v), u = rho_z sqrt(s_{z-1}),
// v = rho_{z-1} sqrt(s_z) (Reflect.h:19-26) at padded point (z, x), z >= 1:
// d/ds_z, d/ds_{z-1}, d/drho_z, d/drho_{z-1}
__device__ __forceinline__ void refl_derivs(const float2* sp, const float2* dp, int nxg, int z, int x, cd2& ds_z,
                                            cd2& ds_u, cd2& dr_z, cd2& dr_u) {
  const size_t i = (size_t)z * nxg + x, iu = i - nxg;
  const cd2 s = mk(sp[i]), su = mk(sp[iu]), rh = mk(dp[i]), rhu = mk(dp[iu]);
  const cd2 qs = sq(s), qsu = sq(su);
  const cd2 u = rh * qsu, v = rhu * qs;
  const cd2 D = (u + v) * (u + v);
  ds_z = mk(0, 0) - u * rhu / (qs * D);
  ds_u = v * rh / (qsu * D);
  dr_z = mk(2, 0) * v * qsu / D;
  dr_u = mk(0, 0) - mk(2, 0) * u * qs / D;
}

// gradient on the model grid: per unpadded point, the sum over the padded
// points that the edge extension copies it to (Pad.h:77-96) of
// IL + conj(dR[z]/ds_z) IR[z] + conj(dR[z+1]/ds_z) IR[z+1] (+ the reference
// term at the sample point), and the density's Reflect terms
__global__ void k_exact_grad(DevCtx c, int nx, const float2* sp, const float2* dp, const float2* IR,
                             const float2* IL, const float2* gref, float2* g0, float2* g1, int add) {
  const int nz = c.nz, nxg = c.nxg, pad = c.pad;
  const size_t total = (size_t)nz * nx;
  const int xref = nxg / 2;  // RefSampler.cpp:28-39 with one reference
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(i / nx), xu = (int)(i - (size_t)z * nx);
    const int x0 = xu == 0 ? 0 : xu + pad, x1 = xu == nx - 1 ? nxg - 1 : xu + pad;
    cd2 gs = mk(0, 0), gr = mk(0, 0);
    for (int x = x0; x <= x1; ++x) {
      const size_t k = (size_t)z * nxg + x;
      gs = gs + mk(IL[k]);
      if (z >= 1) {
        cd2 a, b, e, d;
        refl_derivs(sp, dp, nxg, z, x, a, b, e, d);
        const cd2 ir = mk(IR[k]);
        gs = gs + cj(a) * ir;
        gr = gr + cj(e) * ir;
      }
      if (z + 1 < nz) {
        cd2 a, b, e, d;
        refl_derivs(sp, dp, nxg, z + 1, x, a, b, e, d);
        const cd2 ir = mk(IR[k + nxg]);
        gs = gs + cj(b) * ir;
        gr = gr + cj(d) * ir;
      }
      if (x == xref) gs = gs + mk(gref[z]);
    }
    float2 v0 = make_float2((float)gs.x, (float)gs.y), v1 = make_float2((float)gr.x, (float)gr.y);
    if (add) {
      v0 = make_float2(g0[i].x + v0.x, g0[i].y + v0.y);
      v1 = make_float2(g1[i].x + v1.x, g1[i].y + v1.y);
    }
    g0[i] = v0;
    g1[i] = v1;
  }
}

}  // namespace

void launch_phase_grad_tables(const DevCtx& c, const float2* sref, float eps, float2* gam, cudaStream_t st) {
  const int nrow = c.nfreq * c.nz * c.nref;
  const dim3 grid = table_grid((c.N + 255) / 256, nrow, 256);
  k_phase_grad<<<grid, 256, 0, st>>>(c, sref, eps, gam);
  note_launch();
}

void launch_qs_reduce(const float2* qs, int rows, int nz, int add, float2* out, cudaStream_t st) {
  k_qs_reduce<<<(nz + 127) / 128, 128, 0, st>>>(qs, rows, nz, add, out);
  note_launch();
}

void launch_exact_assemble(const DevCtx& c, int nx, float eps, const float2* sp, const float2* dp, const float2* IR,
                           const float2* IL, const float2* qsum, float2* gref, float2* g0, float2* g1, int add,
                           cudaStream_t st) {
  k_exact_ref<<<c.nz, 256, 0, st>>>(c, eps, sp, IL, qsum, gref);
  note_launch();
  const size_t n = (size_t)c.nz * nx;
  const int grid = (int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
  k_exact_grad<<<grid > 0 ? grid : 1, 256, 0, st>>>(c, nx, sp, dp, IR, IL, gref, g0, g1, add);
  note_launch();
}

}  // namespace wg
