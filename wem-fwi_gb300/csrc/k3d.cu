// 3D one-way operators: dispatch of the row and column passes
// (kernels3d.cuh), the column pass of single-line planes (ny = 1), the
// imaging condition, the quadrant phase tables and the 3D edge padding.
#include <algorithm>

#include "fft.cuh"
#include "kernels.h"
#include "phase.cuh"

namespace wg {

template <int E>
void launch_k3_rows_e(const Ctx3&, const Pass3&, int, cudaStream_t);
template <int E>
void launch_k3_cols_e(const Ctx3&, int, int, const float2*, float2*, cudaStream_t);

namespace {

__device__ __forceinline__ int quad1(int i, int n) { return i < n / 2 ? i : (i == n / 2 ? 0 : n - i); }

// column pass of planes of one line (Ny = 1): the transform along y is the
// identity, the phase shift of each reference is applied per point
__global__ void k3_cols1(Ctx3 c, int z, int adj, const float2* in, float2* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)c.rows * c.Nx) return;
  const int r = (int)(i / c.Nx), x = (int)(i % c.Nx), f = r / c.ns;
  const size_t plane = (size_t)c.rows * c.Nx;
  const size_t tab = ((size_t)f * c.nz + z) * c.nref;
  const size_t qsz = (size_t)c.Qy * c.Qx;
  const int ix = quad1(x, c.Nx);
  if (!adj) {
    const float2 v = in[i];
    for (int j = 0; j < c.nref; ++j) out[(size_t)j * plane + i] = c_mul(v, c.ph[(tab + j) * qsz + ix]);
  } else {
    float2 acc = make_float2(0.f, 0.f);
    for (int j = 0; j < c.nref; ++j) acc = c_add(acc, c_mulc(in[(size_t)j * plane + i], c.ph[(tab + j) * qsz + ix]));
    out[i] = acc;
  }
}

// one thread per model point (y, x) of depth z; rows in order
__global__ void k3_image(Ctx3 c, int z, const float2* bg, const float2* a, float2* img, int add) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.ny * c.nx) return;
  const int ym = i / c.nx, xm = i % c.nx;
  const size_t fp = (size_t)c.nyg * c.nxg, o = (size_t)(ym + c.pady) * c.nxg + xm + c.pad;
  float2 acc = make_float2(0.f, 0.f);
  for (int r = 0; r < c.rows; ++r) acc = c_fmac(acc, a[(size_t)r * fp + o], bg[(size_t)r * fp + o]);
  float2* p = img + (size_t)z * c.ny * c.nx + i;
  *p = add ? c_add(*p, acc) : acc;
}

// ph[f][z][j][iy][ix] = phase_factor_k2(w^2, sref[z][j], kx[ix]^2 + ky[iy]^2)
__global__ void k3_phase(Ctx3 c, const float2* sref, const float* kx, const float* ky, float eps, int law,
                         float2* ph) {
  const size_t qsz = (size_t)c.Qy * c.Qx;
  const size_t nt = (size_t)c.nfreq * c.nz * c.nref;
  for (size_t t = blockIdx.y; t < nt; t += gridDim.y) {  // (f, z, j)
    const int j = (int)(t % c.nref), z = (int)((t / c.nref) % c.nz), f = (int)(t / ((size_t)c.nref * c.nz));
    const float w = c.omega[f];
    const float2 s = sref[(size_t)z * c.nref + j];
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < qsz; k += (size_t)gridDim.x * blockDim.x) {
      const int iy = (int)(k / c.Qx), ix = (int)(k % c.Qx);
      const float k2 = __fadd_rn(__fmul_rn(kx[ix], kx[ix]), __fmul_rn(ky[iy], ky[iy]));
      ph[t * qsz + k] = phase_factor_k2(w * w, s, k2, eps, c.dz, law);
    }
  }
}

__global__ void k_pad3(const float2* in, float2* out, int nz, int ny, int nx, int pady, int pad) {
  const int nyg = ny + 2 * pady, nxg = nx + 2 * pad;
  const size_t total = (size_t)nz * nyg * nxg;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % nxg) - pad, y = (int)((i / nxg) % nyg) - pady;
    const size_t z = i / ((size_t)nxg * nyg);
    x = x < 0 ? 0 : (x >= nx ? nx - 1 : x);
    y = y < 0 ? 0 : (y >= ny ? ny - 1 : y);
    out[i] = in[(z * ny + y) * nx + x];
  }
}

int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 65535); }

}  // namespace

bool k3_supported(int Nx, int Ny) {
  auto ok = [](int n) { return n == 256 || n == 384 || n == 512 || n == 768 || n == 1024; };
  return ok(Nx) && (Ny == 1 || ok(Ny));
}

void launch_k3_rows(const Ctx3& c, const Pass3& a, int adj, cudaStream_t st) {
  switch (c.Nx / 32) {
    case 8: launch_k3_rows_e<8>(c, a, adj, st); break;
    case 12: launch_k3_rows_e<12>(c, a, adj, st); break;
    case 16: launch_k3_rows_e<16>(c, a, adj, st); break;
    case 24: launch_k3_rows_e<24>(c, a, adj, st); break;
    case 32: launch_k3_rows_e<32>(c, a, adj, st); break;
  }
}

void launch_k3_cols(const Ctx3& c, int z, int adj, const float2* in, float2* out, cudaStream_t st) {
  if (c.Ny == 1) {
    const long long n = (long long)c.rows * c.Nx;
    k3_cols1<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(c, z, adj, in, out);
    note_launch();
    return;
  }
  switch (c.Ny / 32) {
    case 8: launch_k3_cols_e<8>(c, z, adj, in, out, st); break;
    case 12: launch_k3_cols_e<12>(c, z, adj, in, out, st); break;
    case 16: launch_k3_cols_e<16>(c, z, adj, in, out, st); break;
    case 24: launch_k3_cols_e<24>(c, z, adj, in, out, st); break;
    case 32: launch_k3_cols_e<32>(c, z, adj, in, out, st); break;
  }
}

void launch_k3_image(const Ctx3& c, int z, const float2* bg, const float2* a, float2* img, int add, cudaStream_t st) {
  const int n = c.ny * c.nx;
  k3_image<<<(n + 255) / 256, 256, 0, st>>>(c, z, bg, a, img, add);
  note_launch();
}

void launch_k3_phase(const Ctx3& c, const float2* sref, const float* kx, const float* ky, float eps, int law,
                     float2* ph, cudaStream_t st) {
  const size_t nt = (size_t)c.nfreq * c.nz * c.nref;
  const size_t qsz = (size_t)c.Qy * c.Qx;
  const dim3 grid((unsigned)std::min<size_t>((qsz + 255) / 256, 64), (unsigned)std::min<size_t>(nt, 65535));
  k3_phase<<<grid, 256, 0, st>>>(c, sref, kx, ky, eps, law, ph);
  note_launch();
}

void launch_pad3(const float2* in, float2* out, int nz, int ny, int nx, int pady, int pad, cudaStream_t st) {
  const size_t n = (size_t)nz * (ny + 2 * pady) * (nx + 2 * pad);
  k_pad3<<<grid_for(n), 256, 0, st>>>(in, out, nz, ny, nx, pady, pad);
  note_launch();
}

}  // namespace wg
