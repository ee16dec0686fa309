// Model-space interpolation operators of the FWI preconditioner
// (scripts/fwi.py:45-68): a coarse 2D complex model is interpolated to the
// fine modelling grid with separable filters,
//   data[i2][i1] = sum_j2 F2[i2][j2] sum_j1 F1[i1][j1] model[j2][j1],
// F1 [nd1][nm1] along the fast axis and F2 [nd2][nm2] along the slow one.
//
//   LanczosInterpolation2D (operator/src/LanczosInterpolation2D.h:14-125):
//     windowed sinc of half width a[k] coarse samples, mirrored at the first
//     samples of each axis;
//   Spline2D (operator/src/Spline2D.h:14-130): the two-parameter cubic
//     (a, b) on the coarse spacing, with the reference's edge terms; its
//     adjoint then copies the edge columns and rows of the model from their
//     neighbours (Spline2D.h:84-92), so it is not the exact transpose there.
//
// Both filters depend only on the samplings (the axes' origins are not
// used, as in the reference) and are built once on the host in float, the
// reference's arithmetic.  They are banded: each fine sample sees a few
// coarse ones.  The GPU applies them as two banded contractions with the
// intermediate [nm2][nd1] held in HBM; every output element is one thread's
// fixed-order sum, so results do not depend on the launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "kernels.h"
#include "planner.h"
#include "wemgpu.h"

namespace wg {
void set_last_error(const char* msg);

namespace {

constexpr int kInterpThreads = 128;

struct Axis1 {
  int n;
  float d;
};

// windowed-sinc weight at offset x != 0 (LanczosInterpolation2D.h:99-100),
// evaluated in the reference's mixed float/double arithmetic
float lanczos_weight(float x, float dm, float a) {
  const double pi = 4.0 * std::atan(1.0);
  return (float)((double)(dm * a) * std::sin(pi * x / dm) * std::sin(pi * x / a) / (pi * pi * x * x));
}

// filter [nd][nm] of one axis; a = half width in units of the axis
// (LanczosInterpolation2D.h:91-121)
std::vector<float> lanczos_filter(Axis1 dax, Axis1 max, float a) {
  const int nf = (int)(2 * a / dax.d + 1);
  const int na = (nf - 1) / 2;
  const float half = na * dax.d;
  std::vector<float> f((size_t)dax.n * max.n, 0.f);
  for (int i = 0; i < dax.n; ++i)
    for (int j = 0; j < max.n; ++j) {
      const float x = i * dax.d - j * max.d;
      if (std::fabs(x) <= half) f[(size_t)i * max.n + j] = (x == 0) ? 1.f : lanczos_weight(x, max.d, a);
    }
  // the samples before the first coarse node see its mirror image
  for (int i = 0; i < na && i < dax.n; ++i)
    for (int j = 0; j < max.n; ++j) {
      const float x = i * dax.d - j * max.d;
      const float xx = i * dax.d + j * max.d;
      if (std::fabs(xx) < half && x != xx) {
        const float w = lanczos_weight(xx, max.d, a);
        f[(size_t)i * max.n + j] += w;
        f[(size_t)(dax.n - i - 1) * max.n + (max.n - j - 1)] += w;
      }
    }
  return f;
}

// two-parameter cubic at distance y (coarse samples) (Spline2D.h:101-107)
float spline_weight(float y, float a, float b) {
  if (y < 1) return ((-6 * a - 9 * b + 12) * y * y * y + (6 * a + 12 * b - 18) * y * y - 2 * b + 6) / 6;
  if (y < 2) return ((-6 * a - b) * y * y * y + (30 * a + 6 * b) * y * y + (-48 * a - 12 * b) * y + 24 * a + 8 * b) / 6;
  return 0.f;
}

// filter [nd][nm] of one axis (Spline2D.h:96-125)
std::vector<float> spline_filter(Axis1 dax, Axis1 max, float a, float b) {
  std::vector<float> f((size_t)dax.n * max.n, 0.f);
  for (int i = 0; i < dax.n; ++i)
    for (int j = 0; j < max.n; ++j) {
      const float x = std::fabs(i * dax.d - j * max.d);
      f[(size_t)i * max.n + j] = spline_weight(x / max.d, a, b);
    }
  for (int i = 0; i < dax.n; ++i)
    for (int j = 1; j < max.n - 1; ++j) {
      const float xx = i * dax.d + j * max.d;
      const float w = spline_weight(std::fabs(xx) / max.d, a, b);
      f[(size_t)i * max.n + j] += w;
      f[(size_t)(dax.n - i - 1) * max.n + (max.n - j - 1)] += w;
    }
  return f;
}

// nonzero range [lo, hi) of every row (by_row) or column of f [nr][nc]
void bands(const std::vector<float>& f, int nr, int nc, bool by_row, std::vector<int>& lo, std::vector<int>& hi) {
  const int n = by_row ? nr : nc, m = by_row ? nc : nr;
  lo.assign(n, 0);
  hi.assign(n, 0);
  for (int u = 0; u < n; ++u) {
    int a = m, b = 0;
    for (int v = 0; v < m; ++v) {
      const float w = by_row ? f[(size_t)u * nc + v] : f[(size_t)v * nc + u];
      if (w != 0.f) {
        a = std::min(a, v);
        b = v + 1;
      }
    }
    lo[u] = a < b ? a : 0;
    hi[u] = a < b ? b : 0;
  }
}

__device__ __forceinline__ float2 fma2(float w, float2 x, float2 acc) {
  return make_float2(fmaf(w, x.x, acc.x), fmaf(w, x.y, acc.y));
}

// T[j2][i1] = sum_j1 F1[i1][j1] M[j2][j1]; F1 stored transposed [nm1][nd1]
__global__ void k_interp_a(const float* __restrict__ f1t, const int* __restrict__ lo, const int* __restrict__ hi,
                           const float2* __restrict__ m, float2* __restrict__ t, int nd1, int nm1) {
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
  const int j2 = blockIdx.y;
  if (i1 >= nd1) return;
  const float2* mr = m + (size_t)j2 * nm1;
  float2 acc = make_float2(0.f, 0.f);
  for (int j1 = lo[i1]; j1 < hi[i1]; ++j1) acc = fma2(f1t[(size_t)j1 * nd1 + i1], mr[j1], acc);
  t[(size_t)j2 * nd1 + i1] = acc;
}

// D[i2][i1] (+)= sum_j2 F2[i2][j2] T[j2][i1]
__global__ void k_interp_b(const float* __restrict__ f2, const int* __restrict__ lo, const int* __restrict__ hi,
                           const float2* __restrict__ t, float2* __restrict__ d, int nd1, int nm2, int add) {
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
  const int i2 = blockIdx.y;
  if (i1 >= nd1) return;
  float2 acc = make_float2(0.f, 0.f);
  for (int j2 = lo[i2]; j2 < hi[i2]; ++j2) acc = fma2(f2[(size_t)i2 * nm2 + j2], t[(size_t)j2 * nd1 + i1], acc);
  float2* o = d + (size_t)i2 * nd1 + i1;
  *o = add ? make_float2(o->x + acc.x, o->y + acc.y) : acc;
}

// U[j2][i1] = sum_i2 F2[i2][j2] D[i2][i1]
__global__ void k_interp_at(const float* __restrict__ f2, const int* __restrict__ lo, const int* __restrict__ hi,
                            const float2* __restrict__ d, float2* __restrict__ u, int nd1, int nm2) {
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
  const int j2 = blockIdx.y;
  if (i1 >= nd1) return;
  float2 acc = make_float2(0.f, 0.f);
  for (int i2 = lo[j2]; i2 < hi[j2]; ++i2) acc = fma2(f2[(size_t)i2 * nm2 + j2], d[(size_t)i2 * nd1 + i1], acc);
  u[(size_t)j2 * nd1 + i1] = acc;
}

// M[j2][j1] (+)= sum_i1 F1[i1][j1] U[j2][i1]
__global__ void k_interp_bt(const float* __restrict__ f1t, const int* __restrict__ lo, const int* __restrict__ hi,
                            const float2* __restrict__ u, float2* __restrict__ m, int nd1, int nm1, int add) {
  const int j1 = blockIdx.x * blockDim.x + threadIdx.x;
  const int j2 = blockIdx.y;
  if (j1 >= nm1) return;
  const float2* ur = u + (size_t)j2 * nd1;
  const float* fr = f1t + (size_t)j1 * nd1;
  float2 acc = make_float2(0.f, 0.f);
  for (int i1 = lo[j1]; i1 < hi[j1]; ++i1) acc = fma2(fr[i1], ur[i1], acc);
  float2* o = m + (size_t)j2 * nm1 + j1;
  *o = add ? make_float2(o->x + acc.x, o->y + acc.y) : acc;
}

// Spline2D adjoint edges: first and last column from their neighbours, then
// first and last row (Spline2D.h:84-92, in that order)
__global__ void k_edge_cols(float2* m, int nm1, int nm2) {
  const int j2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (j2 >= nm2) return;
  float2* r = m + (size_t)j2 * nm1;
  r[0] = r[1];
  r[nm1 - 1] = r[nm1 - 2];
}
__global__ void k_edge_rows(float2* m, int nm1, int nm2) {
  const int j1 = blockIdx.x * blockDim.x + threadIdx.x;
  if (j1 >= nm1) return;
  m[j1] = m[(size_t)nm1 + j1];
  m[(size_t)(nm2 - 1) * nm1 + j1] = m[(size_t)(nm2 - 2) * nm1 + j1];
}

void check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  throw Fail(e == cudaErrorMemoryAllocation ? WEM_ENOMEM : WEM_EDEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

bool on_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

struct DevMem {
  void* p = nullptr;
  DevMem() = default;
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() {
    if (p) cudaFree(p);
  }
  void alloc(size_t bytes) {
    if (p) cudaFree(p);
    p = nullptr;
    check(cudaMalloc(&p, bytes ? bytes : 16), "cudaMalloc");
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

template <class T>
void put(DevMem& d, const std::vector<T>& v) {
  d.alloc(v.size() * sizeof(T));
  if (!v.empty()) check(cudaMemcpy(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
}

}  // namespace

class Interp2D {
 public:
  Interp2D(bool spline, Axis1 m1, Axis1 m2, Axis1 d1, Axis1 d2, const std::vector<float>& f1,
           const std::vector<float>& f2)
      : spline_(spline), nm1_(m1.n), nm2_(m2.n), nd1_(d1.n), nd2_(d2.n) {
    std::vector<float> f1t((size_t)nm1_ * nd1_);
    for (int i = 0; i < nd1_; ++i)
      for (int j = 0; j < nm1_; ++j) f1t[(size_t)j * nd1_ + i] = f1[(size_t)i * nm1_ + j];
    std::vector<int> lo, hi;
    put(f1t_, f1t);
    put(f2_, f2);
    bands(f1, nd1_, nm1_, true, lo, hi);
    put(r1lo_, lo);
    put(r1hi_, hi);
    bands(f1, nd1_, nm1_, false, lo, hi);
    put(c1lo_, lo);
    put(c1hi_, hi);
    bands(f2, nd2_, nm2_, true, lo, hi);
    put(r2lo_, lo);
    put(r2hi_, hi);
    bands(f2, nd2_, nm2_, false, lo, hi);
    put(c2lo_, lo);
    put(c2hi_, hi);
    tmp_.alloc((size_t)nm2_ * nd1_ * sizeof(float2));
  }

  void forward(const void* model, void* data, int add) {
    const size_t mb = (size_t)nm1_ * nm2_ * 8, db = (size_t)nd1_ * nd2_ * 8;
    const float2* m = stage_in(model, mb, hm_);
    float2* d = stage_out(data, db, hd_, add != 0);
    const dim3 ga((nd1_ + kInterpThreads - 1) / kInterpThreads, nm2_);
    k_interp_a<<<ga, kInterpThreads>>>(f1t_.as<float>(), r1lo_.as<int>(), r1hi_.as<int>(), m, tmp_.as<float2>(),
                                       nd1_, nm1_);
    note_launch();
    const dim3 gb((nd1_ + kInterpThreads - 1) / kInterpThreads, nd2_);
    k_interp_b<<<gb, kInterpThreads>>>(f2_.as<float>(), r2lo_.as<int>(), r2hi_.as<int>(), tmp_.as<float2>(), d,
                                       nd1_, nm2_, add);
    note_launch();
    check(cudaGetLastError(), "interpolation forward");
    finish(data, db, hd_);
  }

  void adjoint(void* model, const void* data, int add) {
    const size_t mb = (size_t)nm1_ * nm2_ * 8, db = (size_t)nd1_ * nd2_ * 8;
    const float2* d = stage_in(data, db, hd_);
    float2* m = stage_out(model, mb, hm_, add != 0);
    const dim3 ga((nd1_ + kInterpThreads - 1) / kInterpThreads, nm2_);
    k_interp_at<<<ga, kInterpThreads>>>(f2_.as<float>(), c2lo_.as<int>(), c2hi_.as<int>(), d, tmp_.as<float2>(),
                                        nd1_, nm2_);
    note_launch();
    const dim3 gb((nm1_ + kInterpThreads - 1) / kInterpThreads, nm2_);
    k_interp_bt<<<gb, kInterpThreads>>>(f1t_.as<float>(), c1lo_.as<int>(), c1hi_.as<int>(), tmp_.as<float2>(), m,
                                        nd1_, nm1_, add);
    note_launch();
    if (spline_) {
      k_edge_cols<<<(nm2_ + kInterpThreads - 1) / kInterpThreads, kInterpThreads>>>(m, nm1_, nm2_);
      k_edge_rows<<<(nm1_ + kInterpThreads - 1) / kInterpThreads, kInterpThreads>>>(m, nm1_, nm2_);
      note_launch();
      note_launch();
    }
    check(cudaGetLastError(), "interpolation adjoint");
    finish(model, mb, hm_);
  }

 private:
  struct Host {
    DevMem mem;
    size_t bytes = 0;
    bool host = false;
  };
  const float2* stage_in(const void* p, size_t bytes, Host& h) {
    h.host = !on_device(p);
    if (!h.host) return reinterpret_cast<const float2*>(p);
    if (h.bytes != bytes) {
      h.mem.alloc(bytes);
      h.bytes = bytes;
    }
    check(cudaMemcpy(h.mem.p, p, bytes, cudaMemcpyHostToDevice), "H2D");
    return h.mem.as<float2>();
  }
  float2* stage_out(void* p, size_t bytes, Host& h, bool need) {
    h.host = !on_device(p);
    if (!h.host) return reinterpret_cast<float2*>(p);
    if (h.bytes != bytes) {
      h.mem.alloc(bytes);
      h.bytes = bytes;
    }
    if (need) check(cudaMemcpy(h.mem.p, p, bytes, cudaMemcpyHostToDevice), "H2D");
    return h.mem.as<float2>();
  }
  void finish(void* p, size_t bytes, Host& h) {
    if (h.host) check(cudaMemcpy(p, h.mem.p, bytes, cudaMemcpyDeviceToHost), "D2H");
    else check(cudaStreamSynchronize(0), "interpolation");
  }

  bool spline_;
  int nm1_, nm2_, nd1_, nd2_;
  DevMem f1t_, f2_, r1lo_, r1hi_, c1lo_, c1hi_, r2lo_, r2hi_, c2lo_, c2hi_, tmp_;
  Host hm_, hd_;
};

}  // namespace wg

struct interp2d_handle {
  std::unique_ptr<wg::Interp2D> op;
};

namespace {

template <class Fn>
int interp_guard(Fn fn) {
  try {
    fn();
    return WEM_OK;
  } catch (const wg::Fail& e) {
    wg::set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    wg::set_last_error("host allocation failed");
    return WEM_ENOMEM;
  } catch (const std::exception& e) {
    wg::set_last_error(e.what());
    return WEM_EINVAL;
  }
}

void check_axes(int nm1, float dm1, int nm2, float dm2, int nd1, float dd1, int nd2, float dd2) {
  wg::require(nm1 >= 2 && nm2 >= 2 && nd1 >= 1 && nd2 >= 1, "interpolation: need at least 2 coarse samples per axis");
  wg::require(dm1 > 0 && dm2 > 0 && dd1 > 0 && dd2 > 0, "interpolation: sampling intervals must be positive");
}

}  // namespace

extern "C" {

int lanczos2d_create(int nm1, float dm1, int nm2, float dm2, int nd1, float dd1, int nd2, float dd2, const float* a,
                     interp2d_handle** out) {
  return interp_guard([&] {
    wg::require(out && a, "NULL argument");
    *out = nullptr;
    check_axes(nm1, dm1, nm2, dm2, nd1, dd1, nd2, dd2);
    wg::require(a[0] > 0 && a[1] > 0, "lanczos2d: half widths must be positive");
    // half widths in the units of each axis (LanczosInterpolation2D.h:16-17)
    const float a1 = a[0] * dm1, a2 = a[1] * dm2;
    auto h = std::make_unique<interp2d_handle>();
    h->op = std::make_unique<wg::Interp2D>(false, wg::Axis1{nm1, dm1}, wg::Axis1{nm2, dm2}, wg::Axis1{nd1, dd1},
                                           wg::Axis1{nd2, dd2},
                                           wg::lanczos_filter({nd1, dd1}, {nm1, dm1}, a1),
                                           wg::lanczos_filter({nd2, dd2}, {nm2, dm2}, a2));
    *out = h.release();
  });
}

int spline2d_create(int nm1, float dm1, int nm2, float dm2, int nd1, float dd1, int nd2, float dd2, float a, float b,
                    interp2d_handle** out) {
  return interp_guard([&] {
    wg::require(out != nullptr, "NULL argument");
    *out = nullptr;
    check_axes(nm1, dm1, nm2, dm2, nd1, dd1, nd2, dd2);
    auto h = std::make_unique<interp2d_handle>();
    h->op = std::make_unique<wg::Interp2D>(true, wg::Axis1{nm1, dm1}, wg::Axis1{nm2, dm2}, wg::Axis1{nd1, dd1},
                                           wg::Axis1{nd2, dd2}, wg::spline_filter({nd1, dd1}, {nm1, dm1}, a, b),
                                           wg::spline_filter({nd2, dd2}, {nm2, dm2}, a, b));
    *out = h.release();
  });
}

void interp2d_destroy(interp2d_handle* h) { delete h; }

int interp2d_forward(interp2d_handle* h, const void* model, void* data, int add) {
  return interp_guard([&] {
    wg::require(h && model && data, "NULL argument");
    h->op->forward(model, data, add);
  });
}

int interp2d_adjoint(interp2d_handle* h, void* model, const void* data, int add) {
  return interp_guard([&] {
    wg::require(h && model && data, "NULL argument");
    h->op->adjoint(model, data, add);
  });
}

}  // extern "C"
