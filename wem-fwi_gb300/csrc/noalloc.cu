// One SSF/PSPI depth step that allocates no memory.
//
// Who needs it: code that cannot call cudaMalloc while it runs — a caller
// that owns all device memory up front (a fixed arena or memory pool, an
// embedded or real-time loop that must not touch the allocator), or one
// whose allocator is unavailable at that point.  wemop_onestep needs a
// handle whose tables were allocated with cudaMalloc; this entry point takes
// the depth's inputs directly and keeps its per-call tables (twiddles, k
// grid, taper, phase-shift and split-step factors) in the file-scope device
// array below, sized for rows up to N = 4096 points and 16 references.
//
// The array exists once per GPU that loads the library and stays allocated
// until the process exits.  Every call reuses it and overwrites what the
// previous call left there, so two calls that overlap on the GPU (on
// different streams, or from different host threads) race on it: serialise
// them.  The first call on a device looks the array up with
// cudaGetSymbolAddress; make that first call before any stream capture.  The
// address is kept per device together with the id of the context it was
// looked up in, and looked up again only when the device's context has
// changed (after cudaDeviceReset, say), which a later call then also must
// not do under capture.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.h"
#include "wemgpu.h"

namespace wg {
void set_last_error(const char* msg);
}

namespace {

constexpr int kMaxN = 4096;
constexpr int kMaxRef = 16;
constexpr size_t kScratchBytes = (size_t)1 << 20;  // 1 MiB per device

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
// per device: the array's address and the id of the context it belongs to
struct ScratchSlot {
  void* addr = nullptr;
  unsigned long long ctx = 0;
};
ScratchSlot g_slot[kMaxDevices];
std::mutex g_scratch_mutex;

// id of the calling thread's current context (0: none, or the driver does
// not say), through the driver entry points the runtime hands out, so the
// library does not link the driver library itself
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// byte layout of the scratch for one call
struct Layout {
  size_t tw, kx, taper, omega, q, fac, ph, ref, end;
};

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

Layout layout_of(int N, int nxg, int nref) {
  Layout L{};
  size_t o = 0;
  L.tw = o;    o += al256((size_t)N * 8);
  L.kx = o;    o += al256((size_t)N * 4);
  L.taper = o; o += al256((size_t)nxg * 4);
  L.omega = o; o += al256(4);
  L.q = o;     o += al256((size_t)nxg * 8);
  L.fac = o;   o += al256((size_t)nxg * 8);
  L.ph = o;    o += al256((size_t)nref * N * 8);
  L.ref = o;   o += al256((size_t)nxg);
  L.end = o;
  return L;
}

// twiddles, k grid (Phshift_cmplx.cpp:13,21-24), taper / N (Taper.h:11-23),
// omega, and the split-step argument q = (s - s_ref)/sqrt(s_ref) of each
// point's reference (SplitStep.cpp:12-13), all in double; the caller's
// reference indices are copied with every entry outside [-1, nref) made -1
__global__ void k_noalloc_setup(int N, int nxg, int pad, double dx, float freq, int nref,
                                const float2* slow, const float2* sref, const signed char* ref, float2* tw, float* kx,
                                float* taper, float* omega, float2* q, signed char* ref_ok) {
  const double pi = 3.14159265358979323846;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int t = tid; t < N; t += nth) {
    double s, c;
    sincospi(-2.0 * t / N, &s, &c);
    tw[t] = make_float2((float)c, (float)s);
    const double dk = 2 * pi / (dx * (N - 1));
    double k = 0;
    if (t < N / 2) k = t * dk;
    else if (t > N - N / 2) k = -(N - t) * dk;
    kx[t] = (float)k;
  }
  for (int x = tid; x < nxg; x += nth) {
    double tp = 1.0;
    const int i = x < nxg - 1 - x ? x : nxg - 1 - x;
    if (i < pad) tp = .5 * (1 - cos(pi * i / (pad - 1)));
    taper[x] = (float)(tp / N);
    const int j = ref[x] >= -1 && ref[x] < nref ? ref[x] : -1;
    ref_ok[x] = (signed char)j;
    float2 v = make_float2(0.f, 0.f);
    if (j >= 0 && j < nref) {
      const double sr = sref[j].x, si = sref[j].y;
      // principal square root of s_ref
      const double r = hypot(sr, si);
      const double a = sqrt(fmax(0.5 * (r + sr), 0.0)), b0 = sqrt(fmax(0.5 * (r - sr), 0.0));
      const double b = si < 0 ? -b0 : b0;
      const double nr = (double)slow[x].x - sr, ni = (double)slow[x].y - si;
      const double d = a * a + b * b;
      v = make_float2((float)((nr * a + ni * b) / d), (float)((ni * a - nr * b) / d));
    }
    q[x] = v;
  }
  if (tid == 0) omega[0] = (float)(2 * pi * (double)freq);
}

// device memory of GPU `dev` (the current one), or managed memory
bool device_ptr(const void* p, int dev) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

int fail(int code, const char* msg) {
  wg::set_last_error(msg);
  return code;
}

// radix plan without heap use: 4s, 2, then odd factors
bool plan_of(int n, wg::FftPlan& P) {
  P.n = n;
  P.nstage = 0;
  int m = n;
  auto push = [&](int r) {
    if (P.nstage >= wg::kMaxStages) return false;
    P.radix[P.nstage++] = r;
    return true;
  };
  while (m % 4 == 0) { if (!push(4)) return false; m /= 4; }
  while (m % 2 == 0) { if (!push(2)) return false; m /= 2; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) { if (!push(f)) return false; m /= f; }
  return true;
}

}  // namespace

extern "C" int wemop_onestep_noalloc(const wem_params* p, const void* slow_row, const void* sref,
                                     const signed char* refidx, int nxg, float freq, int adj, const void* in,
                                     void* out, int nrow, int add, void* stream) {
  if (!p || !slow_row || !sref || !refidx || !in || !out) return fail(WEM_EINVAL, "NULL argument");
  if (nxg < 2 || nrow < 0 || p->tap < 0 || p->pad < 0 || p->pad == 1 || 2 * p->pad > nxg || p->nref < 1 ||
      !(p->dx > 0) || !(p->dz > 0) || (p->prop != WEM_PROP_SSF && p->prop != WEM_PROP_PSPI) ||
      (p->phase_law != WEM_PHASE_ISPC && p->phase_law != WEM_PHASE_EXACT_KZ))
    return fail(WEM_EINVAL, "invalid parameters for the depth step");
  const int N = nxg + 2 * p->tap;
  if (N > kMaxN || p->nref > kMaxRef)
    return fail(WEM_EINVAL, "wemop_onestep_noalloc: rows are limited to N = nxg + 2 tap <= 4096 and nref <= 16");
  const Layout L = layout_of(N, nxg, p->nref);
  if (L.end > kScratchBytes) return fail(WEM_EINVAL, "wemop_onestep_noalloc: tables exceed the 1 MiB scratch");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(WEM_EDEVICE, "wemop_onestep_noalloc: no usable current device");
  }
  if (!device_ptr(slow_row, dev) || !device_ptr(sref, dev) || !device_ptr(refidx, dev) || !device_ptr(in, dev) ||
      !device_ptr(out, dev))
    return fail(WEM_EINVAL, "wemop_onestep_noalloc: every array must be device memory of the current device");
  if (nrow == 0) return WEM_OK;
  wg::FftPlan plan;
  if (!plan_of(N, plan)) return fail(WEM_EINVAL, "FFT length has too many factors");

  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    ScratchSlot& slot = g_slot[dev];
    const unsigned long long ctx = slot.addr ? current_context_id() : 0;
    if (!slot.addr || ctx == 0 || ctx != slot.ctx) {
      void* a = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&a, g_scratch);
      if (e != cudaSuccess || !a) {
        cudaGetLastError();
        return fail(WEM_EDEVICE, "wemop_onestep_noalloc: cannot get the scratch address");
      }
      slot.addr = a;
      slot.ctx = current_context_id();
    }
    base = static_cast<unsigned char*>(slot.addr);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2* tw = reinterpret_cast<float2*>(base + L.tw);
  float* kx = reinterpret_cast<float*>(base + L.kx);
  float* taper = reinterpret_cast<float*>(base + L.taper);
  float* omega = reinterpret_cast<float*>(base + L.omega);
  float2* q = reinterpret_cast<float2*>(base + L.q);
  float2* fac = reinterpret_cast<float2*>(base + L.fac);
  float2* ph = reinterpret_cast<float2*>(base + L.ph);
  signed char* ref_ok = reinterpret_cast<signed char*>(base + L.ref);

  k_noalloc_setup<<<8, 256, 0, st>>>(N, nxg, p->pad, (double)p->dx, freq, p->nref,
                                     static_cast<const float2*>(slow_row), static_cast<const float2*>(sref), refidx,
                                     tw, kx, taper, omega, q, ref_ok);
  wg::note_launch();
  // one depth, one frequency: the depth-step kernels index the tables at (f, z) = (0, 0)
  wg::DevCtx c{};
  c.plan = plan;
  c.N = N;
  c.nxg = nxg;
  c.tap = p->tap;
  c.pad = p->pad;
  c.nz = 1;
  c.nref = p->nref;
  c.prop = p->prop;
  c.ntaylor = p->ntaylor;
  c.phase_law = p->phase_law;
  c.nfreq = 1;
  c.ext = 0;
  c.dz = p->dz;
  c.invN = 1.0f / N;
  c.tw = tw;
  c.kx = kx;
  c.taperN = taper;
  c.omega = omega;
  c.ref = ref_ok;
  wg::launch_phase_tables(c, static_cast<const float2*>(sref), p->eps, ph, st);
  c.ph = ph;
  if (p->prop == WEM_PROP_SSF) {
    wg::launch_fac_tables(c, q, fac, st);
    c.fac = fac;
  }
  int G = 8;
  const int lim = wg::max_smem_per_block();
  while (G > 1 && (int)wg::smem_rows(c, G) > lim) --G;
  if ((int)wg::smem_rows(c, G) > lim) return fail(WEM_EINVAL, "row too long for one CTA's shared memory");
  wg::launch_onestep(c, 0, 0, adj, static_cast<const float2*>(in), static_cast<float2*>(out), nrow, add, G, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char msg[256];
    std::snprintf(msg, sizeof msg, "wemop_onestep_noalloc: %s", cudaGetErrorString(e));
    return fail(WEM_EDEVICE, msg);
  }
  return WEM_OK;
}
