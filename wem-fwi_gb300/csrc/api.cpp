// C ABI of the GB300 one-way wave-equation library (include/wemgpu.h).
//
// An Engine owns the device tables of one parameter set and one background
// (or one background per frequency for the extended operators), the group
// schedule and the workspaces.  Every public call validates its arguments
// on the host, turns every failure into a status code and never throws
// across the boundary.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "cmap.h"
#include "kernels.h"
#include "planner.h"
#include "wemgpu.h"

namespace wg {
namespace {

thread_local std::string g_error;

// per-kernel CUDA-event timing (wem_stats_*)
struct KStat {
  double ms = 0;
  long long n = 0;
};
bool g_stats_on = false;
bool g_plain = false;
int g_path = 0;  // 0 automatic, 1 shared-memory kernels, 2 warp-per-row kernels
int g_rows = 0;  // 0 automatic, 1 grouped rows per CTA, 2 one-row CTAs
bool g_split_off = false;  // fwi_gradient: the Born adjoint recomputes the source field
std::vector<std::pair<std::string, KStat>> g_stats;

std::mutex g_stats_mu;  // engines may run on several host threads

KStat& stat_of(const std::string& name) {
  for (auto& kv : g_stats)
    if (kv.first == name) return kv.second;
  g_stats.emplace_back(name, KStat{});
  return g_stats.back().second;
}

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  int code = (e == cudaErrorMemoryAllocation) ? WEM_ENOMEM : WEM_EDEVICE;
  throw Fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// growable device buffer
struct Buf {
  void* p = nullptr;
  size_t cap = 0;
  ~Buf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  void* get(size_t bytes) {
    if (bytes > cap) {
      release();
      cuda_check(cudaMalloc(&p, bytes ? bytes : 16), "cudaMalloc");
      cap = bytes;
    }
    return p;
  }
  template <class T> T* as(size_t n) { return reinterpret_cast<T*>(get(n * sizeof(T))); }
};

// page-locked host memory for the values a call reads back when it ends:
// the loss (double at byte 0) and the background status (int at byte 8,
// kNoBad when every reference slowness was positive)
constexpr int kNoBad = 0x7f7f7f7f;
struct Pinned {
  void* p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
  char* get() {
    if (!p) {
      cuda_check(cudaMallocHost(&p, 64), "cudaMallocHost");
      std::memset(p, 0, 64);
      *reinterpret_cast<int*>(static_cast<char*>(p) + 8) = kNoBad;
    }
    return static_cast<char*>(p);
  }
};

template <class T>
T* upload(Buf& b, const std::vector<T>& v) {
  T* d = b.as<T>(v.size());
  if (!v.empty()) cuda_check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
  return d;
}

std::vector<float2> to_f2(const std::vector<cd>& v) {
  std::vector<float2> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = make_float2((float)v[i].real(), (float)v[i].imag());
  return o;
}

FftPlan make_plan(int n) {
  FftPlan P{};
  P.n = n;
  std::vector<int> r = fft_radices(n);
  require((int)r.size() <= kMaxStages, "FFT length has too many factors");
  P.nstage = (int)r.size();
  for (size_t i = 0; i < r.size(); ++i) P.radix[i] = r[i];
  return P;
}

// host view of a caller buffer: device pointers are used in place, host
// buffers are staged through a device buffer
struct Staged {
  Buf own;
  void* dev = nullptr;
  bool host = false;
  size_t bytes = 0;
  void in(const void* p, size_t nbytes) {
    bytes = nbytes;
    host = !is_device_ptr(p);
    if (!host) {
      dev = const_cast<void*>(p);
      return;
    }
    dev = own.get(nbytes);
    cuda_check(cudaMemcpy(dev, p, nbytes, cudaMemcpyHostToDevice), "H2D");
  }
  // output buffer: when add is set the current contents are needed
  void out(void* p, size_t nbytes, bool need_contents) {
    bytes = nbytes;
    host = !is_device_ptr(p);
    if (!host) {
      dev = p;
      return;
    }
    dev = own.get(nbytes);
    if (need_contents) cuda_check(cudaMemcpy(dev, p, nbytes, cudaMemcpyHostToDevice), "H2D");
  }
  void finish(void* p) {
    if (host) cuda_check(cudaMemcpy(p, dev, bytes, cudaMemcpyDeviceToHost), "D2H");
  }
};

// launches `fn` on stream 0, bracketed by events when timing is enabled
template <class Fn>
void timed(const char* name, Fn fn) {
  if (!g_stats_on) {
    fn();
    return;
  }
  cudaEvent_t a, b;
  cuda_check(cudaEventCreate(&a), "event");
  cuda_check(cudaEventCreate(&b), "event");
  cuda_check(cudaEventRecord(a, 0), "event");
  fn();
  cuda_check(cudaEventRecord(b, 0), "event");
  cuda_check(cudaEventSynchronize(b), "event");
  float ms = 0;
  cuda_check(cudaEventElapsedTime(&ms, a, b), "event");
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  std::lock_guard<std::mutex> lock(g_stats_mu);
  KStat& k = stat_of(name);
  k.ms += ms;
  k.n += 1;
}

std::vector<float> host_floats(const void* p, size_t nfloat) {
  std::vector<float> h(nfloat);
  if (is_device_ptr(p)) cuda_check(cudaMemcpy(h.data(), p, nfloat * 4, cudaMemcpyDeviceToHost), "D2H");
  else std::memcpy(h.data(), p, nfloat * 4);
  return h;
}

// The traces' time <-> frequency transform over n samples for nf
// propagated bins from b0: the FFT plan with its per-stage twiddle tables
// ([r - 1][l] per stage, in double rounded once) and the natural table of the
// restricted DFT; the launch shape for ntr traces
TimeFreq make_timefreq(int n, int nt, int nf, int b0, int ntr, Buf& tftw, Buf& tfwn, TfShape& shape) {
  TimeFreq t{};
  t.n = n;
  t.nt = nt;
  t.nf = nf;
  t.b0 = b0;
  t.sc = (float)(1.0 / std::sqrt((double)n));
  t.wn = upload(tfwn, to_f2(twiddles(n)));
  // radices, largest first: 16, 12, 8, 6 (in-register DFTs), then 4, 3, 2, 5, 7
  std::vector<int> rad;
  int m = n;
  for (int r : {16, 12, 8, 6, 4, 3, 2, 5, 7})
    while (m % r == 0) {
      rad.push_back(r);
      m /= r;
    }
  t.fft = m == 1 && (int)rad.size() <= kMaxStages && n <= 16384;
  if (t.fft) {
    const long double pi = 3.14159265358979323846264338327950288L;
    std::vector<float2> tws;
    t.plan.n = n;
    t.plan.nstage = (int)rad.size();
    int L = 1;
    for (size_t s = 0; s < rad.size(); ++s) {
      TfStage& S = t.st[s];
      S.R = rad[s];
      t.plan.radix[s] = S.R;
      S.L = L;
      S.nb = n / S.R;
      S.ld = n + (n >> 4) + 1;
      S.twoff = (int)tws.size();
      S.mag_nb = (unsigned)((((unsigned long long)1 << 32) + S.nb - 1) / S.nb);
      S.mag_L = (unsigned)((((unsigned long long)1 << 32) + L - 1) / L);
      for (int k = 0; k < 7; ++k)
        S.w7[k] = make_float2((float)std::cos(-2 * pi * k / 7), (float)std::sin(-2 * pi * k / 7));
      for (int r = 1; r < S.R; ++r)
        for (int l = 0; l < L; ++l) {
          const long double a = -2 * pi * (long double)(r * l) / ((long double)L * S.R);
          tws.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
        }
      L *= S.R;
    }
    t.tw_len = (int)tws.size();
    t.tws = upload(tftw, tws);
  }
  shape = timefreq_shape(t, ntr);
  require(shape.ok, "time axis too long for the time-frequency kernels' shared memory");
  return t;
}

class Engine {
 public:
  // kind: 0 BornFull / WEM, 1 BornRefl, 2 BornTomo (propagator/src/ext_born_refl.cpp,
  // ext_born_tomo.cpp); the variants run on the Born passes with the
  // switches of DevCtx
  Engine(const wem_params& p_in, const float* wavelet, bool ext, bool born, int kind = 0)
      : p_(refl_conventions(p_in, kind)), ext_(ext), born_(born), kind_(kind),
        taper_w_(p_in.pad) {
    const wem_params& p = p_;
    require(wavelet != nullptr, "wavelet is NULL");
    require(taper_w_ != 1, "pad == 1 makes the taper divide by zero (Taper.h:19)");
    geo_ = make_geometry(p, wavelet);
    F_ = geo_.nfreq();
    M_ = ext ? F_ : 1;
    M_img_ = (ext || kind == 1) ? F_ : 1;
    // conformal maps (wem_prop.cpp:19-45, born_prop.cpp:28-70): every shot
    // propagates on its own mapped grid, so each gets an engine of one shot
    // with that grid, its mapped devices and its gather tables
    std::vector<ShotMap> maps;
    if (p.cmap != WEM_CMAP_NONE) {
      require(!ext && kind == 0, "cmap applies to WEM and BornFull only");
      maps = make_shot_maps(p, geo_);
    }
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (!maps.empty()) {
      // the shots run on `workers_` host threads (shot s on thread s mod
      // workers_, in order), each thread with its own large buffers
      workers_ = std::max(1, std::min(geo_.ns, kShotWorkers));
      for (int w = 0; w < workers_; ++w) worker_ws_.push_back(std::make_shared<Scratch>());
      acc_.resize(workers_);
      for (int s = 0; s < geo_.ns; ++s) {
        const ShotMap& m = maps[s];
        wem_params ps = p;
        ps.cmap = WEM_CMAP_NONE;
        ps.ns = 1;
        ps.ox = m.o1;
        ps.dx = m.d1;
        ps.oz = m.o2;
        ps.dz = m.d2;
        Geometry gs = geo_;
        gs.ns = 1;
        gs.sx = m.src_x;
        gs.sz = {m.src_z};
        gs.sptr = {0, (int)m.src_x.size()};
        gs.rx = m.rec_x;
        gs.rz = m.rec_z;
        shots_.push_back(std::unique_ptr<Engine>(new Engine(ps, gs, m, born, worker_ws_[s % workers_])));
      }
      return;
    }
    build_static();
    ctx_.ext_model = kind == 1 ? 1 : 0;
    ctx_.no_fwd_record = kind == 2 ? 1 : 0;
    ctx_.last_rule = kind == 2 ? 1 : 0;
  }

  ~Engine() {
    for (cudaStream_t st : ostreams_) cudaStreamDestroy(st);
    for (cudaEvent_t ev : oevents_) cudaEventDestroy(ev);
  }

  int nfreq() const { return F_; }
  const wem_params& params() const { return p_; }

  // BornRefl and BornTomo (ext_born_refl.cpp:18-25, ext_born_tomo.cpp:20-25)
  // propagate on the model grid itself: Down/Up are built on the unpadded
  // slowness, so `pad` is only the width of OneStep's taper (OneStep.h:27-35),
  // the source spreads over the reference's "ng" cells (here `ngs`) and the
  // receivers are points (Injection's default ng = 0), none offset by a pad.
  // The offset Born (kind 3) is BornRefl on each shot's cropped model and
  // keeps these conventions.
  static wem_params refl_conventions(wem_params p, int kind) {
    if (kind == 1 || kind == 2 || kind == 3) {
      p.pad = 0;
      p.ngr = 0;
    }
    return p;
  }

  void set_background(const void* s2, const void* rho) {
    require(s2 && rho, "background model is NULL");
    if (!shots_.empty()) {
      // kept here; every shot maps it onto its grid when it runs
      const size_t nm = (size_t)p_.nz * p_.nx * 8;
      Staged a, b;
      a.in(s2, nm);
      b.in(rho, nm);
      cuda_check(cudaMemcpy(cm_bg0_.get(nm), a.dev, nm, cudaMemcpyDeviceToDevice), "copy background");
      cuda_check(cudaMemcpy(cm_bg1_.get(nm), b.dev, nm, cudaMemcpyDeviceToDevice), "copy background");
    } else if (kind_ == 3) {
      off_background(s2);
    } else {
      build_background(s2, rho);
    }
    have_bg_ = true;
  }

  bool warp_path() const {
    if (g_path == 1) return false;
    bool ok = warp_path_supported(ctx_);
    require(ok || g_path != 2, "warp-per-row kernels need N = 32 E with E in {8,12,16,24,32} and ntaylor <= 1");
    return ok;
  }

  int warp_G(int which) const { return g_plain ? 1 : std::min(geo_.ns, warp_rows_per_group(ctx_, which)); }

  // Rows per CTA of the single-reference warp kernels.  A launch with no
  // more (shot, frequency) rows than the GPU has SMs runs one row per CTA,
  // so the rows spread over as many SMs as there are rows instead of
  // sharing a few grouped CTAs; larger launches group rows of a frequency.
  // The shots of a conformal-map operator always run one-row CTAs.
  void pick_row_ctas() {
    if (map_) return;
    int dev = 0, sms = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    const long long rows = (long long)F_ * geo_.ns;
    ctx_.one_row = g_rows == 2 ? 1 : (g_rows == 1 ? 0 : (rows <= sms ? 1 : 0));
  }

  void wem_forward(const void* s2, const void* rho, void* data, int kind, int add) {
    if (!shots_.empty()) {
      require(s2 && rho && data, "NULL argument");
      const size_t nm = (size_t)p_.nz * p_.nx * 8;
      Staged a, b;
      a.in(s2, nm);
      b.in(rho, nm);
      for_shots([&](int s, int) { shots_[s]->wem_forward(a.dev, b.dev, shot_data(data, kind, s), kind, add); });
      return;
    }
    set_background(s2, rho);
    zero_bins();
    wem_pass();
    emit(data, kind, add);
  }

  // modelling of the current background into the internal bins
  // bg_for_adjoint: the modelling also stores its down field in the
  // adjoint's first stored field (ws_->store1), keeping its own rows of R bg
  // in ws_->store4
  void wem_pass(bool bg_for_adjoint = false) {
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    const bool wp = warp_path();
    if (wp) pick_row_ctas();
    int G = wp ? warp_G(0) : pick_G([&](int g) { return smem_wem(ctx_, g); });
    int chunks = 0;
    wem_rows_all_ = false;
    for_chunks(G, plane * 8, [&](const Group* gd, int ng, int rows) {
      wem_rows_all_ = ++chunks == 1 && (size_t)rows == (size_t)F_ * geo_.ns;
      const bool keep_bg = bg_for_adjoint && wp;
      float2* A = (keep_bg ? ws_->store4 : ws_->store1).as<float2>((size_t)rows * plane);
      ctx_.bg_store = keep_bg ? ws_->store1.as<float2>((size_t)rows * plane) : nullptr;
      if (wp) timed("k_wem", [&] { launch_pass_warp(0, ctx_, gd, ng, nullptr, nullptr, A, nullptr, nullptr, bins_, nullptr, nullptr, 0, 0); });
      else timed("k_wem", [&] { launch_wem(ctx_, gd, ng, G, A, bins_, 0); });
      ctx_.bg_store = nullptr;
      cuda_check(cudaGetLastError(), "k_wem launch");
    }, wp);
  }

  // FWI objective and gradient in one call: modelling, residual and loss on
  // the device, Born adjoint of the residual at the same background (its
  // tables built once for both passes)
  double fwi_gradient(const void* s2, const void* rho, const void* dobs, void* g_s2, void* g_rho) {
    require(s2 && rho && dobs && g_s2 && g_rho, "NULL argument");
    if (!shots_.empty()) {
      const size_t nm = (size_t)p_.nz * p_.nx;
      Staged a, b, ob, o0, o1;
      a.in(s2, nm * 8);
      b.in(rho, nm * 8);
      ob.in(dobs, (size_t)geo_.ns * geo_.nr * p_.nt * 4);
      o0.out(g_s2, nm * 8, false);
      o1.out(g_rho, nm * 8, false);
      std::vector<double> losses(geo_.ns, 0.0);
      for_shots([&](int s, int w) {
        Engine& e = *shots_[s];
        ShotAcc& A = acc_[w];
        float2* g0 = A.g0.as<float2>(nm);
        float2* g1 = A.g1.as<float2>(nm);
        losses[s] = e.fwi_gradient(a.dev, b.dev, shot_data(ob.dev, WEM_DATA_TIME, s), g0, g1);
        e.image_back(g0, A.s0.as<float2>(nm), s >= workers_);
        e.image_back(g1, A.s1.as<float2>(nm), s >= workers_);
        cuda_check(cudaStreamSynchronize(0), "fwi_gradient");
      });
      sum_workers((float2*)o0.dev, (float2*)o1.dev, nm, false);
      o0.finish(g_s2);
      o1.finish(g_rho);
      double loss = 0;
      for (double v : losses) loss += v;
      return loss;
    }
    set_background(s2, rho);
    zero_bins();
    // The modelling's down sweep computes the Born adjoint's source field bg
    // (the same background, tables and kernels): with both passes in one
    // launch of the warp kernels, rows numbered alike, the modelling stores
    // bg itself and the adjoint runs only the receiver side's down sweep
    const bool split = split_gradient();
    wem_pass(split);
    // residual r = WEM(m) - d_obs in time, loss = 1/2 |r|^2, r back to bins
    const size_t nd = (size_t)geo_.ns * geo_.nr * p_.nt;
    Staged obs;
    obs.in(dobs, nd * 4);
    double* loss_h = residual_bins((const float*)obs.dev);
    // the adjoint takes the stored bg only when the modelling ran every row
    // in one launch and its own launch holds every row too (adj_pass)
    adj_split_req_ = split && wem_rows_all_;
    adj_pass();
    adj_split_req_ = false;
    grad_out(g_s2, g_rho, 0);  // ends with the stream synchronised
    return *loss_h;
  }

  // fwi_gradient may hand the source field from the modelling to the Born
  // adjoint: warp kernels with grouped CTAs and one reference, the as-coded
  // adjoint; the passes check that each ran every row in one launch (rows
  // numbered frequency-major in both; the modelling's stored rows are the
  // adjoint's first stored field, ws_->store1)
  bool split_gradient() {
    if (g_plain || g_split_off || !warp_path() || p_.nref != 1 || ext_ || kind_ != 0) return false;
    if (p_.adjoint_mode != WEM_ADJ_COMPAT) return false;
    pick_row_ctas();
    if (!warp_adj_split(ctx_)) return false;
    return true;
  }

  void born_forward(const void* ds2, const void* drho, void* data, int kind, int add) {
    require(have_bg_, "background not set");
    if (!shots_.empty()) {
      require(ds2 && drho && data, "NULL argument");
      const size_t nm = (size_t)p_.nz * p_.nx * 8;
      Staged a, b;
      a.in(ds2, nm);
      b.in(drho, nm);
      for_shots([&](int s, int) {
        shots_[s]->set_background(cm_bg0_.p, cm_bg1_.p);
        shots_[s]->born_forward(a.dev, b.dev, shot_data(data, kind, s), kind, add);
      });
      return;
    }
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    float2* dm0 = dm0_.as<float2>((size_t)M_ * plane);
    float2* dm1 = dm1_.as<float2>((size_t)M_ * plane);
    pad_perturbation(ds2, dm0, M_);
    pad_perturbation(drho, dm1, M_);
    float2* drm = drm_.as<float2>((size_t)M_ * plane);
    launch_drefl_fwd(ctx_, M_, a0_, b0_, a1_, b1_, dm0, dm1, drm, 0);
    zero_bins();
    born_fwd_pass(dm0, drm);
    emit(data, kind, add);
  }

  // Born forward of the slowness perturbation rows dm0 and the reflectivity
  // perturbation rows drm into the internal bins
  void born_fwd_pass(const float2* dm0, const float2* drm) {
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    const bool wp = warp_path();
    int G = wp ? warp_G(1) : pick_G([&](int g) { return smem_born_fwd(ctx_, g); });
    for_chunks(G, 2 * plane * 8, [&](const Group* gd, int ng, int rows) {
      float2* A = ws_->store1.as<float2>((size_t)rows * plane);
      float2* B = ws_->store2.as<float2>((size_t)rows * plane);
      if (wp) timed("k_born_fwd", [&] { launch_pass_warp(1, ctx_, gd, ng, dm0, drm, A, B, nullptr, bins_, nullptr, nullptr, 0, 0); });
      else timed("k_born_fwd", [&] { launch_born_fwd(ctx_, gd, ng, G, dm0, drm, A, B, bins_, 0); });
      cuda_check(cudaGetLastError(), "k_born_fwd launch");
    }, wp);
  }

  // ------------------------------------------------ BornRefl, BornTomo
  // BornRefl (ext_born_refl.cpp:8-105): the model is a reflectivity per
  // frequency [F][nz][nx]; forward records Up(bg m_f), adjoint gives
  // sum_s conj(bg) Up^H(rec) per frequency.  On the Born passes: no slowness
  // perturbation, the model in place of dR(dm), the reflectivity image out.
  void refl_forward(const void* model, void* data, int kind, int add) {
    require(have_bg_, "background not set");
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    float2* drm = drm_.as<float2>((size_t)F_ * plane);
    pad_perturbation(model, drm, F_);
    float2* dm0 = dm0_.as<float2>((size_t)F_ * plane);
    cuda_check(cudaMemsetAsync(dm0, 0, (size_t)F_ * plane * 8, 0), "memset");
    zero_bins();
    born_fwd_pass(dm0, drm);
    emit(data, kind, add);
  }
  void refl_adjoint(void* model, const void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(model && data, "NULL argument");
    absorb(data, kind);
    adj_pass();
    image_out(ir_, model, add);
  }

  // ---- subsurface-offset extended reflectivity Born (kind 3; no reference
  // counterpart).  BornRefl with the imaging condition extended over nh
  // horizontal lags, every shot on its own aperture of model columns [x0, x0
  // + w) (the cropped-model mechanism of WEM.from_subspace,
  // propagator/src/python/WEM.py:24-30), padded by pad (edge-extended) and
  // zero-padded to the row length N = 32 E >= w + 2 pad + 2 tap of the warp
  // kernels, equally on both sides.  Receivers outside a shot's aperture
  // record zero and are ignored by the adjoint.  One reference slowness.
  void off_init(int nh, const int* ax0, const int* aw) {
    require(kind_ == 3, "not an offset-Born engine");
    require(nh >= 1 && nh % 2 == 1 && nh <= 41, "nh must be odd and at most 41");
    require(p_.nref == 1, "the offset Born operator takes one reference slowness (nref = 1)");
    require(p_.cmap == WEM_CMAP_NONE, "the offset Born operator has no conformal maps");
    const Geometry& g = geo_;
    const int ns = g.ns, nz = p_.nz, pad = p_.pad;
    onh_ = nh;
    osh_.assign(ns, OffShot{});
    for (int s = 0; s < ns; ++s) {
      OffShot& o = osh_[s];
      o.x0 = ax0 ? ax0[s] : 0;
      o.w = aw ? aw[s] : p_.nx;
      require(o.x0 >= 0 && o.w >= 2 && o.x0 + o.w <= p_.nx, "aperture of shot " + std::to_string(s) +
                                                                 " outside the model");
      require(o.w % 2 == 0, "aperture widths must be even (shot " + std::to_string(s) + ")");
      const int p0 = g.sptr.empty() ? s : g.sptr[s], p1 = g.sptr.empty() ? s + 1 : g.sptr[s + 1];
      for (int pt = p0; pt < p1; ++pt)
        require(g.sx[pt] >= o.x0 && g.sx[pt] < o.x0 + o.w,
                "source of shot " + std::to_string(s) + " outside its aperture");
      const int nxg = o.w + 2 * pad;
      o.N = off_row_length(nxg + 2 * p_.tap);
      require(o.N > 0, "aperture of shot " + std::to_string(s) + " too wide: w + 2 tap must be <= 1024");
      o.tap = (o.N - nxg) / 2;
    }
    // rows: shots by row length, then shot, then frequency
    std::vector<int> order(ns);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return osh_[a].N < osh_[b].N; });
    std::vector<int> rowbase(ns), tpo(ns), x0(ns), w(ns), tap(ns);
    std::vector<long long> toff(ns), roff, poff;
    std::vector<int> rowshot;
    std::vector<float> tpr;
    long long t = 0, r = 0;
    onxg_max_ = 0;
    for (int s = 0; s < ns; ++s) {
      const OffShot& o = osh_[s];
      const int nxg = o.w + 2 * pad;
      x0[s] = o.x0;
      w[s] = o.w;
      tap[s] = o.tap;
      toff[s] = t;
      t += (long long)nz * nxg;
      tpo[s] = (int)tpr.size();
      const std::vector<double> tp = taper(nxg, taper_w_);
      for (int i = 0; i < nxg; ++i) tpr.push_back((float)(tp[i] / o.N));
      onxg_max_ = std::max(onxg_max_, nxg);
    }
    otab_elems_ = (size_t)t;
    t = 0;
    long long tp = 0;
    obuckets_.clear();
    for (int s : order) {
      const OffShot& o = osh_[s];
      rowbase[s] = (int)r;
      if (obuckets_.empty() || obuckets_.back().E != o.N / 32) {
        obuckets_.emplace_back();
        obuckets_.back().E = o.N / 32;
        obuckets_.back().row0 = (int)r;
      }
      for (int f = 0; f < F_; ++f) {
        roff.push_back(t);  // t: running offset of the rows' fields
        t += (long long)nz * (o.w + 2 * pad);
        poff.push_back(tp);  // tp: running offset of the rows' phase tables
        tp += (long long)nz * o.N;
        rowshot.push_back(s);
        ++r;
      }
      obuckets_.back().nrows = (int)r - obuckets_.back().row0;
      obuckets_.back().nxg_max = std::max(obuckets_.back().nxg_max, o.w + 2 * pad);
      for (int f0 = 0; f0 < F_; f0 += kOffRows)
        obuckets_.back().groups.push_back(OffGroup{s, f0, std::min(kOffRows, F_ - f0), rowbase[s] + f0});
    }
    ostore_elems_ = (size_t)t;
    oph_elems_ = (size_t)tp;
    // receivers of each shot inside its aperture, by (depth, column, id)
    std::vector<int> rptr((size_t)ns * (nz + 1), 0), rid, rxc;
    for (int s = 0; s < ns; ++s) {
      const OffShot& o = osh_[s];
      std::vector<int> in;
      for (int i = 0; i < g.nr; ++i)
        if (g.rx[i] >= o.x0 && g.rx[i] < o.x0 + o.w) in.push_back(i);
      std::stable_sort(in.begin(), in.end(), [&](int a, int b) {
        return g.rz[a] != g.rz[b] ? g.rz[a] < g.rz[b] : g.rx[a] < g.rx[b];
      });
      int* rp = rptr.data() + (size_t)s * (nz + 1);
      const int base = (int)rid.size();
      for (int i : in) {
        rp[g.rz[i] + 1]++;
        rid.push_back(i);
        rxc.push_back(g.rx[i]);
      }
      rp[0] = base;
      for (int z = 0; z < nz; ++z) rp[z + 1] += rp[z];
    }
    OffCtx& c = octx_;
    c = OffCtx{};
    c.nz = nz;
    c.nx = p_.nx;
    c.pad = pad;
    c.prop = p_.prop;
    c.phase_law = p_.phase_law;
    c.nh = nh;
    c.nfreq = F_;
    c.ns = ns;
    c.nr = g.nr;
    c.ngs = p_.ngs;
    c.ngr = p_.ngr;
    c.dz = p_.dz;
    c.eps = p_.eps;
    c.omega = ctx_.omega;
    c.wave = ctx_.wave;
    c.x0 = upload(ox0_, x0);
    c.w = upload(ow_, w);
    c.tap = upload(otap_, tap);
    c.toff = upload(otoff_, toff);
    c.taperN = upload(otaper_, tpr);
    c.tpo = upload(otpo_, tpo);
    c.sx = ctx_.sx;
    c.sptr = ctx_.sptr;
    c.sz = ctx_.sz;
    c.gs = ctx_.gs;
    c.gr = ctx_.gr;
    c.rptr = upload(orptr_, rptr);
    c.rid = upload(orid_, rid.empty() ? std::vector<int>{0} : rid);
    c.rxc = upload(orxc_, rxc.empty() ? std::vector<int>{0} : rxc);
    c.rowbase = upload(orowbase_, rowbase);
    c.roff = upload(oroff_, roff);
    c.poff = upload(opoff_, poff);
    c.rowshot = upload(orowshot_, rowshot);
    // per row length: k grid, twiddles and the groups on the device
    for (OffBucket& b : obuckets_) {
      const int N = 32 * b.E;
      std::vector<double> k = k_grid(N, p_.dx);
      b.kx = upload(*b.kxb, std::vector<float>(k.begin(), k.end()));
      b.tw = upload(*b.twb, to_f2(twiddles(N)));
      b.dg = upload(*b.gb, b.groups);
      require(off_smem_bytes(b.E, b.nxg_max) <= (size_t)max_smem_per_block(),
              "aperture rows do not fit one CTA's shared memory");
    }
  }

  // row length and leading zero pad of every shot's aperture row
  void off_rows(int* row_len, int* tap) const {
    require(kind_ == 3 && !osh_.empty(), "not an offset-Born engine");
    for (size_t s = 0; s < osh_.size(); ++s) {
      if (row_len) row_len[s] = osh_[s].N;
      if (tap) tap[s] = osh_[s].tap;
    }
  }

  void off_forward(const void* model, void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(model && data, "NULL argument");
    Staged m;
    m.in(model, (size_t)onh_ * p_.nz * p_.nx * 8);
    float2* A = ostoreA_.as<float2>(ostore_elems_);
    float2* B = ostoreB_.as<float2>(ostore_elems_);
    zero_bins();
    off_sweeps(0, A);
    timed("k_off_source", [&] { launch_off_source(octx_, (const float2*)m.dev, A, B, onxg_max_, 0); });
    off_sweeps(1, B);
    cuda_check(cudaGetLastError(), "offset Born launches");
    emit(data, kind, add);
  }

  void off_adjoint(void* model, const void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(model && data, "NULL argument");
    absorb(data, kind);
    float2* A = ostoreA_.as<float2>(ostore_elems_);
    float2* B = ostoreB_.as<float2>(ostore_elems_);
    off_sweeps(0, A);
    off_sweeps(2, B);
    Staged o;
    const size_t nm = (size_t)onh_ * p_.nz * p_.nx;
    o.out(model, nm * 8, add != 0);
    timed("k_off_image", [&] { launch_off_image(octx_, A, B, (float2*)o.dev, add, 0); });
    cuda_check(cudaGetLastError(), "offset Born launches");
    cuda_check(cudaStreamSynchronize(0), "offset Born adjoint");
    o.finish(model);
    check_background();
  }

  // BornTomo (ext_born_tomo.cpp:9-119): the model is a slowness perturbation
  // [nz][nx]; the down- and up-scattering terms of BornFull with the given
  // reflectivity per frequency in place of R, without the forward-scattering
  // record and the reflectivity perturbation.
  void tomo_set_refl(const void* refl) {
    require(refl != nullptr, "reflectivity is NULL");
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    Staged s;
    s.in(refl, (size_t)F_ * p_.nz * p_.nx * 8);
    float2* rcf = rcf_.as<float2>((size_t)F_ * plane);
    launch_pad_edge((const float2*)s.dev, rcf, F_, p_.nz, p_.nx, p_.pad, 0);
    cuda_check(cudaGetLastError(), "pad launch");
    cuda_check(cudaStreamSynchronize(0), "set_refl");
    ctx_.rcf = rcf;
  }
  void tomo_forward(const void* dm, void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(ctx_.rcf != nullptr, "reflectivity not set");
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    float2* dm0 = dm0_.as<float2>(plane);
    pad_perturbation(dm, dm0, 1);
    float2* drm = drm_.as<float2>(plane);
    cuda_check(cudaMemsetAsync(drm, 0, plane * 8, 0), "memset");
    zero_bins();
    born_fwd_pass(dm0, drm);
    emit(data, kind, add);
  }
  void tomo_adjoint(void* dm, const void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(ctx_.rcf != nullptr, "reflectivity not set");
    require(dm && data, "NULL argument");
    absorb(data, kind);
    adj_pass();
    image_out(is_, dm, add);
  }

  // an image [M_img][nz][nxg] unpadded into the caller's [M_img][nz][nx]
  void image_out(Buf& img, void* out, int add) {
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    const size_t nm = (size_t)M_img_ * p_.nz * p_.nx;
    float2* I = img.as<float2>((size_t)M_img_ * plane);
    Staged o;
    o.out(out, nm * 8, add != 0);
    launch_copy_rows(I + p_.pad, geo_.nxg, (float2*)o.dev, p_.nx, M_img_ * p_.nz, p_.nx, add, 0);
    cuda_check(cudaGetLastError(), "image launch");
    cuda_check(cudaStreamSynchronize(0), "image");
    o.finish(out);
    check_background();
  }

  void born_adjoint(void* ds2, void* drho, const void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(ds2 && drho && data, "NULL argument");
    if (!shots_.empty()) {
      // every shot's gradient is brought back to the model grid by the
      // inverse map (born_prop.cpp:217-232); each worker thread sums its
      // shots in order, then the workers' sums are added in worker order
      const size_t nm = (size_t)p_.nz * p_.nx;
      Staged o0, o1;
      o0.out(ds2, nm * 8, add != 0);
      o1.out(drho, nm * 8, add != 0);
      for_shots([&](int s, int w) {
        Engine& e = *shots_[s];
        ShotAcc& A = acc_[w];
        float2* g0 = A.g0.as<float2>(nm);
        float2* g1 = A.g1.as<float2>(nm);
        e.set_background(cm_bg0_.p, cm_bg1_.p);
        e.born_adjoint(g0, g1, shot_data(data, kind, s), kind, 0);
        e.image_back(g0, A.s0.as<float2>(nm), s >= workers_);
        e.image_back(g1, A.s1.as<float2>(nm), s >= workers_);
        cuda_check(cudaStreamSynchronize(0), "born_adjoint");
      });
      sum_workers((float2*)o0.dev, (float2*)o1.dev, nm, add != 0);
      o0.finish(ds2);
      o1.finish(drho);
      return;
    }
    absorb(data, kind);
    adj_pass();
    grad_out(ds2, drho, add);
  }

  // Born adjoint of the internal bins into the images IR, IS
  void adj_pass() {
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    float2* IR = ir_.as<float2>((size_t)M_img_ * plane);
    float2* IS = is_.as<float2>((size_t)M_img_ * plane);
    cuda_check(cudaMemsetAsync(IR, 0, (size_t)M_img_ * plane * 8, 0), "memset");
    cuda_check(cudaMemsetAsync(IS, 0, (size_t)M_img_ * plane * 8, 0), "memset");
    const bool wp = warp_path();
    if (wp) pick_row_ctas();
    int G = wp ? warp_G(2) : pick_G([&](int g) { return smem_born_adj(ctx_, g); });
    const int compat = p_.adjoint_mode == WEM_ADJ_COMPAT ? 1 : 0;
    const bool reuse = wp && !g_plain && warp_adj_reuse(ctx_, compat);
    const int nfield = reuse ? 3 : 2;
    // per row: two stored fields (three with spectral reuse); per group: two partial images
    for_chunks(G, nfield * plane * 8 + (2 * plane * 8 + G - 1) / G, [&](const Group* gd, int ng, int rows) {
      float2* BG = ws_->store1.as<float2>((size_t)rows * plane);
      float2* T = ws_->store2.as<float2>((size_t)rows * plane);
      float2* SG = reuse ? ws_->store3.as<float2>((size_t)rows * plane) : nullptr;
      float2* pr = ws_->part1.as<float2>((size_t)ng * plane);
      float2* ps = ws_->part2.as<float2>((size_t)ng * plane);
      // rows numbered as the modelling's: the stored bg lines up
      ctx_.adj_split = adj_split_req_ && wp && (size_t)rows == (size_t)F_ * geo_.ns ? 1 : 0;
      if (wp) timed("k_born_adj", [&] { launch_pass_warp(2, ctx_, gd, ng, nullptr, nullptr, BG, T, SG, bins_, pr, ps, compat, 0); });
      else timed("k_born_adj", [&] { launch_born_adj(ctx_, gd, ng, G, BG, T, bins_, pr, ps, compat, 0); });
      ctx_.adj_split = 0;
      cuda_check(cudaGetLastError(), "k_born_adj launch");
      // chunk-local group ranges of each image slice
      std::vector<int> beg(M_img_ + 1, 0);
      if (M_img_ == 1) {
        beg[1] = ng;
      } else {
        int g = 0;
        for (int m = 0; m <= M_img_; ++m) {
          while (g < ng && chunk_[g].f < m) ++g;
          beg[m] = g;
        }
      }
      int* dbeg = upload(begbuf_, beg);
      launch_reduce_images(pr, dbeg, M_img_, plane, IR, 0);
      launch_reduce_images(ps, dbeg, M_img_, plane, IS, 0);
      cuda_check(cudaGetLastError(), "reduce launch");
    }, wp);
  }

  // images -> gradient [M][nz][nx] x 2 (dR^H of IR plus IS, unpadded)
  void grad_out(void* ds2, void* drho, int add) {
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    const size_t nm = (size_t)M_ * p_.nz * p_.nx;
    float2* IR = ir_.as<float2>((size_t)M_ * plane);
    float2* IS = is_.as<float2>((size_t)M_ * plane);
    Staged o0, o1;
    o0.out(ds2, nm * 8, add != 0);
    o1.out(drho, nm * 8, add != 0);
    launch_grad_assemble(ctx_, M_, a0_, b0_, a1_, b1_, IR, IS, (float2*)o0.dev, (float2*)o1.dev, p_.nx, add, 0);
    cuda_check(cudaGetLastError(), "grad launch");
    cuda_check(cudaStreamSynchronize(0), "born_adjoint");
    o0.finish(ds2);
    o1.finish(drho);
    check_background();
  }

  // ---------------------------------- exact gradient of the modelling
  // (kernels_wg.cuh, grad.cu): the adjoint-state derivative of the modelled
  // data (wem_prop.cpp:9-78) through Reflect, the split step, the phase
  // shift and the reference slowness; ck > 1 stores every ck-th depth and
  // recomputes the segments between
  void require_exact(bool tables) const {
    if (!shots_.empty() || ext_ || kind_ != 0)
      throw Fail(WEM_ENOTIMPL, "the exact gradient covers WEM without conformal maps or per-frequency models");
    if (p_.nref != 1) throw Fail(WEM_ENOTIMPL, "the exact gradient needs one reference slowness (nref = 1)");
    if (tables && !grad_warp_supported(ctx_))
      throw Fail(WEM_ENOTIMPL, "the exact gradient runs on the warp kernels: N = 32 E, E in {8, 12, 16, 24, 32}, "
                               "ntaylor <= 1, and its tables in shared memory");
  }

  // the images IR, IL and the per-depth reference sums of the data
  // gradient held in the internal bins
  void exact_pass(int ck) {
    require(ck >= 0 && ck < p_.nz, "checkpoint interval must be in [0, nz)");
    const int nz = p_.nz, nxg = geo_.nxg, N = geo_.N;
    const size_t plane = (size_t)nz * nxg, splane = (size_t)nz * N;
    if (!gam_ok_) {
      float2* gam = gam_.as<float2>((size_t)F_ * nz * N);
      launch_phase_grad_tables(ctx_, ctx_.sref, p_.eps, gam, 0);
      ctx_.gam = gam;
      gam_ok_ = true;
    }
    const int cke = ck > 1 ? ck : 0;
    const int ncp = cke ? (nz - 1) / cke + 1 : nz;
    const size_t segl = (size_t)(cke + 1) * (2 * nxg + 2 * N) + 2 * N;
    const int G = std::min(geo_.ns, grad_rows_per_group());
    const size_t row_store = cke ? (2 * (size_t)ncp * nxg + segl) * 8 : (2 * plane + 2 * splane) * 8;
    float2* IR = ir_.as<float2>(plane);
    float2* IL = is_.as<float2>(plane);
    float2* qsum = qsum_.as<float2>(nz);
    cuda_check(cudaMemsetAsync(IR, 0, plane * 8, 0), "memset");
    cuda_check(cudaMemsetAsync(IL, 0, plane * 8, 0), "memset");
    cuda_check(cudaMemsetAsync(qsum, 0, (size_t)nz * 8, 0), "memset");
    ctx_.one_row = 0;
    for_chunks(G, row_store + (2 * plane * 8 + G - 1) / G + 2 * (size_t)nz * 8, [&](const Group* gd, int ng, int rows) {
      GradArgs a{};
      a.bg = ws_->store1.as<float2>((size_t)rows * ncp * nxg);
      a.t = ws_->store2.as<float2>((size_t)rows * ncp * nxg);
      if (cke) {
        a.seg = ws_->store3.as<float2>((size_t)rows * segl);
      } else {
        a.sw = ws_->store3.as<float2>((size_t)rows * splane);
        a.sg = ws_->store4.as<float2>((size_t)rows * splane);
      }
      a.ir = ws_->part1.as<float2>((size_t)ng * plane);
      a.il = ws_->part2.as<float2>((size_t)ng * plane);
      if (!ctx_.fac) cuda_check(cudaMemsetAsync(a.il, 0, (size_t)ng * plane * 8, 0), "memset");
      a.qs = qsbuf_.as<float2>((size_t)2 * rows * nz);
      cuda_check(cudaMemsetAsync(a.qs, 0, (size_t)2 * rows * nz * 8, 0), "memset");
      a.bins = bins_;
      a.ck = cke;
      a.rows_total = rows;
      timed("k_wem_grad", [&] { launch_grad_warp(ctx_, gd, ng, a, 0); });
      cuda_check(cudaGetLastError(), "k_wem_grad launch");
      int* dbeg = upload(begbuf_, std::vector<int>{0, ng});
      launch_reduce_images(a.ir, dbeg, 1, plane, IR, 0);
      launch_reduce_images(a.il, dbeg, 1, plane, IL, 0);
      launch_qs_reduce(a.qs, rows, nz, 1, qsum, 0);
      cuda_check(cudaGetLastError(), "reduce launch");
    }, true);
  }

  void exact_grad_out(void* g_s2, void* g_rho, int add) {
    const size_t plane = (size_t)p_.nz * geo_.nxg;
    const size_t nm = (size_t)p_.nz * p_.nx;
    Staged o0, o1;
    o0.out(g_s2, nm * 8, add != 0);
    o1.out(g_rho, nm * 8, add != 0);
    launch_exact_assemble(ctx_, p_.nx, p_.eps, static_cast<const float2*>(sp_.p), static_cast<const float2*>(dp_.p),
                          ir_.as<float2>(plane), is_.as<float2>(plane), qsum_.as<float2>(p_.nz),
                          gref_.as<float2>(p_.nz), (float2*)o0.dev, (float2*)o1.dev, add, 0);
    cuda_check(cudaGetLastError(), "gradient launch");
    cuda_check(cudaStreamSynchronize(0), "gradient");
    o0.finish(g_s2);
    o1.finish(g_rho);
    check_background();
  }

  // the FWI objective and its exact gradient in one call
  double fwi_gradient_exact(const void* s2, const void* rho, const void* dobs, void* g_s2, void* g_rho, int ck) {
    require(s2 && rho && dobs && g_s2 && g_rho, "NULL argument");
    require_exact(false);
    set_background(s2, rho);
    require_exact(true);
    zero_bins();
    wem_pass();
    const size_t nd = (size_t)geo_.ns * geo_.nr * p_.nt;
    Staged obs;
    obs.in(dobs, nd * 4);
    double* loss_h = residual_bins((const float*)obs.dev);
    exact_pass(ck);
    exact_grad_out(g_s2, g_rho, 0);
    return *loss_h;
  }

  // (g_s2, g_rho) (+)= J^H g: the adjoint of the modelling's derivative at
  // (s2, rho) applied to the data gradient g (time traces or bins)
  void wem_gradient(const void* s2, const void* rho, const void* data, int kind, void* g_s2, void* g_rho, int add,
                    int ck) {
    require(s2 && rho && data && g_s2 && g_rho, "NULL argument");
    require_exact(false);
    set_background(s2, rho);
    require_exact(true);
    absorb(data, kind);
    exact_pass(ck);
    exact_grad_out(g_s2, g_rho, add);
  }

  // a model-grid field of this shot's mapped grid back onto the model grid
  // (the conformal map's inverse), into or onto out
  void image_back(const float2* mapped, float2* out, bool add) {
    require(map_ != nullptr, "not a conformal-map shot");
    launch_cmap_gather(mapped, map_->inv.as<int>(map_->n), out, map_->n, add ? 1 : 0, 0);
    cuda_check(cudaGetLastError(), "cmap gather launch");
  }

 private:
  // the large buffers: stored fields, per-group partial images and the
  // per-frequency phase / split-step tables.  The shots of a conformal-map
  // operator run one after another and rebuild their tables before every
  // pass, so they share one set.
  struct Scratch {
    Buf store1, store2, store3, store4, part1, part2, ph, fac;
  };
  std::shared_ptr<Scratch> ws_ = std::make_shared<Scratch>();

  // one shot of a conformal-map operator: its mapped grid (p.dx, p.dz) and
  // devices (g) and the gather tables of its map
  Engine(const wem_params& p, const Geometry& g, const ShotMap& m, bool born, std::shared_ptr<Scratch> ws)
      : p_(p), ext_(false), born_(born), kind_(0), taper_w_(p.pad) {
    ws_ = std::move(ws);
    geo_ = g;
    F_ = geo_.nfreq();
    M_ = 1;
    M_img_ = 1;
    build_static();
    ctx_.one_row = 1;  // one shot: every group is one (shot, frequency) row
    map_.reset(new MapDev);
    map_->n = p.nx * p.nz;
    upload(map_->fwd, m.fwd);
    upload(map_->inv, m.inv);
    map_->js = m.js;
    map_->scale = m.js != 1.f || !m.jl.empty();
    if (!m.jl.empty()) map_->jl_d = upload(map_->jl, m.jl);
  }

  // fn(shot, worker) for every shot, on workers_ host threads: worker w
  // runs shots w, w + workers_, ... in order on its own default stream;
  // the first failure is rethrown here once every thread has stopped
  template <class Fn>
  void for_shots(Fn fn) {
    const int ns = (int)shots_.size();
    if (workers_ <= 1) {
      for (int s = 0; s < ns; ++s) fn(s, 0);
      return;
    }
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    // work the caller queued before (its inputs) precedes the workers' streams
    cuda_check(cudaDeviceSynchronize(), "cmap inputs");
    std::mutex mu;
    std::exception_ptr err;
    std::vector<std::thread> th;
    for (int w = 0; w < workers_; ++w)
      th.emplace_back([&, w] {
        try {
          cuda_check(cudaSetDevice(dev), "cudaSetDevice");
          for (int s = w; s < ns; s += workers_) {
            {
              std::lock_guard<std::mutex> lock(mu);
              if (err) return;
            }
            fn(s, w);
          }
        } catch (...) {
          std::lock_guard<std::mutex> lock(mu);
          if (!err) err = std::current_exception();
        }
      });
    for (auto& t : th) t.join();
    if (err) std::rethrow_exception(err);
  }

  // out0/out1 (+)= the workers' sums, in worker order
  void sum_workers(float2* out0, float2* out1, size_t nm, bool add) {
    for (int w = 0; w < workers_ && w < (int)shots_.size(); ++w) {
      const float2* s0 = acc_[w].s0.as<float2>(nm);
      const float2* s1 = acc_[w].s1.as<float2>(nm);
      if (w == 0 && !add) {
        cuda_check(cudaMemcpyAsync(out0, s0, nm * 8, cudaMemcpyDeviceToDevice, 0), "copy");
        cuda_check(cudaMemcpyAsync(out1, s1, nm * 8, cudaMemcpyDeviceToDevice, 0), "copy");
      } else {
        launch_scale_add(out0, s0, nm, 0);
        launch_scale_add(out1, s1, nm, 0);
      }
    }
    cuda_check(cudaGetLastError(), "sum kernels");
    cuda_check(cudaStreamSynchronize(0), "sum");
  }

  // a shot's slice of caller data
  void* shot_data(const void* data, int kind, int s) const {
    const size_t per = (size_t)geo_.nr * (kind == WEM_DATA_TIME ? (size_t)p_.nt * 4 : (size_t)geo_.nbin * 8);
    return (char*)const_cast<void*>(data) + per * s;
  }

  struct MapDev {
    int n = 0;
    Buf fwd, inv, jl;
    float js = 1;
    const float* jl_d = nullptr;
    bool scale = false;
  };
  std::unique_ptr<MapDev> map_;                // this engine is one shot of a conformal-map operator
  std::vector<std::unique_ptr<Engine>> shots_;  // this operator runs one engine per mapped shot
  static constexpr int kShotWorkers = 8;        // host threads that run the shots side by side
  int workers_ = 1;
  std::vector<std::shared_ptr<Scratch>> worker_ws_;
  struct ShotAcc {
    Buf g0, g1, s0, s1;  // a shot's mapped gradient; the worker's running sum on the model grid
  };
  std::vector<ShotAcc> acc_;
  Buf cm_bg0_, cm_bg1_, cm_map0_, cm_map1_, cm_map2_, spr_, sptr_;

  wem_params p_;
  bool ext_, born_;
  int kind_ = 0;
  int taper_w_ = 0;  // OneStep's taper width: the reference's `pad`
  bool wem_rows_all_ = false;   // the last modelling pass ran every row in one launch
  bool adj_split_req_ = false;  // fwi_gradient: the stored rows hold bg for the adjoint
  int M_img_ = 1;  // image slices: per frequency for the extended operators and BornRefl
  bool have_bg_ = false;
  Geometry geo_;
  int F_ = 0, M_ = 1;
  DevCtx ctx_{};
  // static tables
  Buf tw_, kx_, taper_, omega_, bin_, wave_, sx_, sz_, gs_, gr_, rptr_, rid_, rxs_, tftw_, tfwn_;
  TimeFreq tf_{};  // the traces' time <-> frequency transform (timefreq.cu)
  TfShape tfs_{};
  // background tables
  Buf sref_, ref_, q_, sc_, rc_, a0b_, b0b_, a1b_, b1b_, sp_, dp_, badbuf_, refscr_;
  float2 *a0_ = nullptr, *b0_ = nullptr, *a1_ = nullptr, *b1_ = nullptr;
  // workspaces
  std::vector<Group> chunk_;  // host copy of the groups of the current launch
  Buf rcf_, binsbuf_, groups_, lossbuf_, dm0_, dm1_, drm_, ir_, is_, begbuf_, stage_;
  Buf gam_, qsum_, qsbuf_, gref_;  // exact gradient: phase-factor derivatives and reference sums
  bool gam_ok_ = false;
  Pinned pinned_;
  float2* bins_ = nullptr;

  // offset Born (kind 3)
  struct OffShot {
    int x0 = 0, w = 0, N = 0, tap = 0;
  };
  struct OffBucket {
    int E = 0, row0 = 0, nrows = 0, nxg_max = 0;
    std::vector<OffGroup> groups;
    std::shared_ptr<Buf> kxb = std::make_shared<Buf>(), twb = std::make_shared<Buf>(), gb = std::make_shared<Buf>();
    const float* kx = nullptr;
    const float2* tw = nullptr;
    const OffGroup* dg = nullptr;
  };
  std::vector<OffShot> osh_;
  std::vector<OffBucket> obuckets_;
  OffCtx octx_{};
  int onh_ = 1, onxg_max_ = 0;
  size_t otab_elems_ = 0, ostore_elems_ = 0, oph_elems_ = 0;
  Buf ox0_, ow_, otap_, otoff_, otaper_, otpo_, orptr_, orid_, orxc_, orowbase_, oroff_, opoff_, orowshot_;
  Buf osp_, osref_, oref_, oq_, obad_, oscr_, ostoreA_, ostoreB_, otph_, otfac_;
  // one stream per row length: the launches of a sweep run side by side
  std::vector<cudaStream_t> ostreams_;
  std::vector<cudaEvent_t> oevents_;

  void off_streams() {
    while (ostreams_.size() < obuckets_.size()) {
      cudaStream_t st;
      cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
      ostreams_.push_back(st);
    }
    while (oevents_.size() < obuckets_.size() + 1) {
      cudaEvent_t ev;
      cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
      oevents_.push_back(ev);
    }
  }

  // one sweep over every row: a launch per row length, each on its own
  // stream after the work before it on stream 0, which waits for them all
  void off_sweeps(int mode, float2* store) {
    static const char* names[3] = {"k_off_down", "k_off_up", "k_off_upadj"};
    off_streams();
    timed(names[mode], [&] {
      cuda_check(cudaEventRecord(oevents_.back(), 0), "event");
      for (size_t i = 0; i < obuckets_.size(); ++i) {
        const OffBucket& b = obuckets_[i];
        OffCtx c = octx_;
        c.kx = b.kx;
        c.tw = b.tw;
        cuda_check(cudaStreamWaitEvent(ostreams_[i], oevents_.back(), 0), "stream wait");
        launch_off_sweep(mode, b.E, c, b.dg, (int)b.groups.size(), b.nxg_max, store, bins_, ostreams_[i]);
        cuda_check(cudaEventRecord(oevents_[i], ostreams_[i]), "event");
      }
      for (size_t i = 0; i < obuckets_.size(); ++i)
        cuda_check(cudaStreamWaitEvent(0, oevents_[i], 0), "stream wait");
    });
  }

  // aperture tables: edge-padded slowness of every aperture, its RefSampler
  // (RefSampler.cpp:10-91 on the aperture, one reference) and the split-step
  // exponents; a reference slowness <= 0 is reported when the call ends
  void off_background(const void* s2) {
    require(!osh_.empty(), "offset apertures not set");
    const int nz = p_.nz, ns = geo_.ns, pad = p_.pad;
    Staged ss;
    ss.in(s2, (size_t)nz * p_.nx * 8);
    float2* sp = osp_.as<float2>(otab_elems_);
    launch_off_crop(octx_, (const float2*)ss.dev, onxg_max_, sp, 0);
    float2* sref = osref_.as<float2>((size_t)ns * nz);
    signed char* ref = oref_.as<signed char>(otab_elems_);
    int* bad = obad_.as<int>(ns);
    cuda_check(cudaMemsetAsync(bad, 0x7f, (size_t)ns * sizeof(int), 0), "memset");
    float* scr = oscr_.as<float>(refs_scratch_floats(1, nz, 1));
    long long t = 0;
    for (int s = 0; s < ns; ++s) {
      const int nxg = osh_[s].w + 2 * pad;
      launch_sref(sp + t, sref + (size_t)s * nz, 1, nz, nxg, 1, bad + s, 0);
      launch_refsampler(p_.refs_mode == WEM_REFS_NEAREST ? 1 : 0, sp + t, sref + (size_t)s * nz, 1, nz, nxg, 1, scr,
                        ref + t, 0);
      t += (long long)nz * nxg;
    }
    octx_.sref = sref;
    float2* q = oq_.as<float2>(otab_elems_);
    launch_off_q(octx_, sp, ref, p_.prop == WEM_PROP_SSF ? 1 : 0, onxg_max_, q, 0);
    octx_.q = q;
    // every row's phase and split-step tables
    octx_.tph = otph_.as<float2>(oph_elems_);
    octx_.tfac = otfac_.as<float2>(ostore_elems_);
    for (const OffBucket& b : obuckets_) {
      OffCtx c = octx_;
      c.kx = b.kx;
      launch_off_tables(c, b.row0, b.nrows, 32 * b.E, 0);
    }
    cuda_check(cudaGetLastError(), "aperture table kernels");
    ss.own.release();
    cuda_check(cudaStreamSynchronize(0), "aperture tables");
  }

  void off_check() {
    if (!have_bg_) return;
    const int ns = geo_.ns;
    std::vector<int> bad(ns);
    cuda_check(cudaMemcpy(bad.data(), obad_.p, (size_t)ns * sizeof(int), cudaMemcpyDeviceToHost), "D2H status");
    for (int s = 0; s < ns; ++s) {
      if (bad[s] == kNoBad) continue;
      float2 v{};
      cuda_check(cudaMemcpy(&v, static_cast<const float2*>(osref_.p) + (size_t)s * p_.nz + bad[s], sizeof v,
                            cudaMemcpyDeviceToHost),
                 "D2H sref");
      throw Fail(WEM_EINVAL, "Ref velocity " + std::to_string(v.x) + " at the layer " + std::to_string(bad[s]) +
                                 " (aperture of shot " + std::to_string(s) + ")");
    }
  }

  void build_static() {
    const Geometry& g = geo_;
    std::vector<cd> tw = twiddles(g.N);
    std::vector<double> k = k_grid(g.N, p_.dx), tp = taper(g.nxg, taper_w_);
    std::vector<float> kf(k.begin(), k.end()), tpf(g.nxg), om(F_);
    for (int i = 0; i < g.nxg; ++i) tpf[i] = (float)(tp[i] / g.N);
    for (int f = 0; f < F_; ++f) om[f] = (float)(2 * 3.14159265358979323846 * (double)g.freq[f]);
    std::vector<float> gsf(g.gs.begin(), g.gs.end()), grf(g.gr.begin(), g.gr.end());
    // receivers sorted by (depth, x, id)
    std::vector<int> ord(g.nr);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
      return g.rz[a] != g.rz[b] ? g.rz[a] < g.rz[b] : g.rx[a] < g.rx[b];
    });
    std::vector<int> rptr(p_.nz + 1, 0), rxs(g.nr);
    for (int i = 0; i < g.nr; ++i) rptr[g.rz[ord[i]] + 1]++;
    for (int z = 0; z < p_.nz; ++z) rptr[z + 1] += rptr[z];
    for (int i = 0; i < g.nr; ++i) rxs[i] = g.rx[ord[i]];
    ctx_.plan = make_plan(g.N);
    ctx_.N = g.N;
    ctx_.nxg = g.nxg;
    ctx_.tap = p_.tap;
    ctx_.pad = p_.pad;
    ctx_.nz = p_.nz;
    ctx_.nref = p_.nref;
    ctx_.prop = p_.prop;
    ctx_.ntaylor = p_.ntaylor;
    ctx_.phase_law = p_.phase_law;
    ctx_.nfreq = F_;
    ctx_.ext = ext_ ? 1 : 0;
    ctx_.ns = g.ns;
    ctx_.nr = g.nr;
    ctx_.ngs = p_.ngs;
    ctx_.ngr = p_.ngr;
    ctx_.nbin = F_;  // internal bins are compact: the propagated frequencies only
    ctx_.dz = p_.dz;
    ctx_.invN = 1.0f / g.N;
    ctx_.tw = upload(tw_, to_f2(tw));
    ctx_.kx = upload(kx_, kf);
    ctx_.taperN = upload(taper_, tpf);
    ctx_.omega = upload(omega_, om);
    std::vector<int> fidx(F_);
    std::iota(fidx.begin(), fidx.end(), 0);
    ctx_.bin = upload(bin_, fidx);
    ctx_.wave = upload(wave_, to_f2(g.wave_at));
    ctx_.sx = upload(sx_, g.sx);
    ctx_.sptr = g.sptr.empty() ? nullptr : upload(sptr_, g.sptr);
    ctx_.sz = upload(sz_, g.sz);
    ctx_.gs = upload(gs_, gsf);
    ctx_.gr = upload(gr_, grf);
    ctx_.rptr = upload(rptr_, rptr);
    ctx_.rid = upload(rid_, ord);
    ctx_.rxs = upload(rxs_, rxs);
    // time <-> frequency over n = nt + tpad samples; the propagated bins are
    // the window [bin[0], bin[0] + F)
    build_timefreq(g.nt_pad);
    bins_ = binsbuf_.as<float2>((size_t)g.ns * g.nr * F_);
  }

  // Background tables on the device: edge-padded model, RefSampler (on the
  // host only when its sort can change the partition: nref > 1, or the
  // as-coded history running out for nref == 1), point tables, and the
  // per-(frequency, depth) phase-shift and split-step tables.
  void build_background(const void* s2, const void* rho) {
    const int nz = p_.nz, nx = p_.nx, nxg = geo_.nxg, nref = p_.nref;
    const size_t plane = (size_t)nz * nxg, n = (size_t)M_ * nz * nx;
    Staged ss, sr;
    ss.in(s2, n * 8);
    sr.in(rho, n * 8);
    const float2 *s_in = (const float2*)ss.dev, *r_in = (const float2*)sr.dev;
    if (map_) {
      // the model on this shot's mapped grid (wem_prop.cpp:24-25)
      float2* ms = cm_map0_.as<float2>(n);
      float2* mr = cm_map1_.as<float2>(n);
      launch_cmap_gather(s_in, map_->fwd.as<int>(n), ms, (int)n, -1, 0);
      launch_cmap_gather(r_in, map_->fwd.as<int>(n), mr, (int)n, -1, 0);
      s_in = ms;
      r_in = mr;
    }
    float2* sp = sp_.as<float2>((size_t)M_ * plane);
    float2* dp = dp_.as<float2>((size_t)M_ * plane);
    launch_pad_edge(s_in, sp, M_, nz, nx, p_.pad, 0);
    launch_pad_edge(r_in, dp, M_, nz, nx, p_.pad, 0);
    // Reflect keeps the padded slowness as mapped; the Jacobian then scales
    // it, by flat index of the padded grid, for everything else
    // (wem_prop.cpp:35-40, born_prop.cpp:44-48)
    const float2* spr = nullptr;
    if (map_ && map_->scale) {
      float2* u = spr_.as<float2>(plane);
      cuda_check(cudaMemcpyAsync(u, sp, plane * 8, cudaMemcpyDeviceToDevice, 0), "copy slowness");
      launch_cmap_jacobian(sp, nz * nx, map_->js, map_->jl_d, 0);
      spr = u;
    }
    float2* dsref = sref_.as<float2>((size_t)M_ * nz * nref);
    signed char* dref = ref_.as<signed char>((size_t)M_ * plane);
    // RefSampler on the device; a reference slowness <= 0 is reported when
    // the call ends (check_background), not by a copy in mid-call
    int* bad = badbuf_.as<int>(1);
    cuda_check(cudaMemsetAsync(bad, 0x7f, sizeof(int), 0), "memset");
    launch_sref(sp, dsref, M_, nz, nxg, nref, bad, 0);
    cuda_check(cudaMemcpyAsync(pinned_bad(), bad, sizeof(int), cudaMemcpyDeviceToHost, 0), "D2H status");
    launch_refsampler(p_.refs_mode == WEM_REFS_NEAREST ? 1 : 0, sp, dsref, M_, nz, nxg, nref,
                      refscr_.as<float>(refs_scratch_floats(M_, nz, nref)), dref, 0);
    ctx_.ref = dref;
    ctx_.sref = dsref;
    gam_ok_ = false;
    const bool ssf = p_.prop == WEM_PROP_SSF;
    float2* q = ssf ? q_.as<float2>((size_t)M_ * plane) : nullptr;
    float2* rc = rc_.as<float2>((size_t)M_ * plane);
    float2* sc = nullptr;
    if (born_) {
      sc = sc_.as<float2>((size_t)M_ * (p_.ntaylor + 1) * plane);
      a0_ = a0b_.as<float2>((size_t)M_ * plane);
      b0_ = b0b_.as<float2>((size_t)M_ * plane);
      a1_ = a1b_.as<float2>((size_t)M_ * plane);
      b1_ = b1b_.as<float2>((size_t)M_ * plane);
    }
    launch_point_tables(M_, nz, nxg, nref, p_.ntaylor, p_.eps, sp, spr, dp, dsref, dref, q, rc, sc, a0_, b0_, a1_, b1_,
                        0);
    ctx_.rc = rc;
    ctx_.sc = sc;
    float2* ph = ws_->ph.as<float2>((size_t)F_ * nz * nref * geo_.N);
    launch_phase_tables(ctx_, dsref, p_.eps, ph, 0);
    ctx_.ph = ph;
    if (ssf) {
      float2* fac = ws_->fac.as<float2>((size_t)F_ * plane);
      launch_fac_tables(ctx_, q, fac, 0);
      ctx_.fac = fac;
    } else {
      ctx_.fac = nullptr;
    }
    cuda_check(cudaGetLastError(), "table kernels");
  }

  template <class F>
  int pick_G(F smem_of) {
    int lim = max_smem_per_block();
    int G = g_plain ? 1 : std::min(geo_.ns, 8);
    while (G > 1 && (int)smem_of(G) > lim) --G;
    require((int)smem_of(G) <= lim, "row too long for one CTA's shared memory");
    return G;
  }

  // split the ns shots of frequency f into q groups of near-equal size
  void split_shots(std::vector<Group>& out, int f, int q) const {
    const int ns = geo_.ns, base = ns / q, extra = ns % q;
    for (int i = 0, s0 = 0; i < q; ++i) {
      const int n = base + (i < extra ? 1 : 0);
      out.push_back(Group{f, s0, n, 0});
      s0 += n;
    }
  }

  // Groups of one launch whose CTAs run one per SM.  With full groups of G
  // the last wave would hold only NG mod SMs CTAs of full length; instead the
  // frequencies that fill whole waves keep full groups and the remaining
  // frequencies are split into smaller groups that together fill one wave,
  // placed last in the grid, so the tail is a wave of shorter CTAs.
  std::vector<Group> shaped_groups(int G) const {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int ns = geo_.ns, gpf = (ns + G - 1) / G;
    const long long ng = (long long)F_ * gpf;
    std::vector<Group> all;
    const long long waves = sms > 0 ? ng / sms : 0;
    const int ff = waves > 0 ? (int)std::min<long long>(F_, waves * sms / gpf) : F_;
    const int fr = F_ - ff;
    const int q = fr > 0 ? std::min(ns, sms / fr) : 0;
    if (fr == 0 || ng % sms == 0 || q <= gpf) {
      for (int f = 0; f < F_; ++f)
        for (int s0 = 0; s0 < ns; s0 += G) all.push_back(Group{f, s0, std::min(G, ns - s0), 0});
      return all;
    }
    for (int f = 0; f < ff; ++f) split_shots(all, f, gpf);
    for (int f = ff; f < F_; ++f) split_shots(all, f, q);
    return all;
  }

  // groups of up to G shots of one frequency, sorted by frequency, run in
  // chunks whose storage fits the memory budget; a pass that fits one launch
  // of the warp kernels gets the shaped tail of shaped_groups
  // rows whose storage fits the memory budget (60 % of free HBM, at most 96 GB)
  size_t max_rows_of(size_t bytes_per_row, int G) const {
    size_t freeb = 0, totalb = 0;
    cuda_check(cudaMemGetInfo(&freeb, &totalb), "cudaMemGetInfo");
    size_t budget = std::min<size_t>((size_t)(0.6 * (double)freeb), (size_t)96 << 30);
    return std::max<size_t>(G, budget / std::max<size_t>(bytes_per_row, 1));
  }

  template <class F>
  void for_chunks(int G, size_t bytes_per_row, F run, bool shape = false) {
    size_t max_rows = max_rows_of(bytes_per_row, G);
    if (g_plain) max_rows = 1;  // one row per launch
    std::vector<Group> all;
    if (shape && !g_plain && (size_t)F_ * geo_.ns <= max_rows) {
      all = shaped_groups(G);
    } else {
      for (int f = 0; f < F_; ++f)
        for (int s0 = 0; s0 < geo_.ns; s0 += G) all.push_back(Group{f, s0, std::min(G, geo_.ns - s0), 0});
    }
    size_t i = 0;
    while (i < all.size()) {
      std::vector<Group> chunk;
      int rows = 0;
      while (i < all.size() && (size_t)(rows + all[i].n) <= max_rows) {
        Group g = all[i++];
        g.row0 = rows;
        rows += g.n;
        chunk.push_back(g);
      }
      if (chunk.empty()) {
        Group g = all[i++];
        g.row0 = 0;
        rows = g.n;
        chunk.push_back(g);
      }
      Group* gd = upload(groups_, chunk);
      chunk_ = chunk;
      run(gd, (int)chunk.size(), rows);
    }
  }

  float2* zero_bins() {
    cuda_check(cudaMemsetAsync(bins_, 0, (size_t)geo_.ns * geo_.nr * F_ * 8, 0), "memset");
    return bins_;
  }

  void pad_perturbation(const void* m, float2* out, int slices) {
    require(m != nullptr, "perturbation is NULL");
    Staged s;
    const size_t n = (size_t)slices * p_.nz * p_.nx;
    s.in(m, n * 8);
    const float2* src = (const float2*)s.dev;
    if (map_) {
      // the perturbation on this shot's mapped grid, unscaled (born_prop.cpp:50-51)
      float2* t = cm_map2_.as<float2>(n);
      launch_cmap_gather(src, map_->fwd.as<int>(n), t, (int)n, -1, 0);
      src = t;
    }
    launch_pad_model(src, out, slices, p_.nz, p_.nx, p_.pad, 0);
    cuda_check(cudaGetLastError(), "pad launch");
    cuda_check(cudaStreamSynchronize(0), "pad");
  }

  // internal bins [ns][nr][F] -> time traces [ns][nr][nt] on the device
  void bins_to_time(float* t, int add) {
    launch_timefreq(0, tf_, tfs_, bins_, t, nullptr, geo_.ns * geo_.nr, add, nullptr, 0);
  }

  // time traces on the device -> internal bins
  void time_to_bins(const float* t) {
    launch_timefreq(1, tf_, tfs_, bins_, const_cast<float*>(t), nullptr, geo_.ns * geo_.nr, 0, nullptr, 0);
  }

  int* pinned_bad() { return reinterpret_cast<int*>(pinned_.get() + 8); }

 public:
  // once the stream has passed the last background build: a reference
  // slowness whose real part is not > 0 fails the call as the reference's
  // RefSampler does (RefSampler.cpp:35-36)
  void check_background() {
    if (kind_ == 3) {
      off_check();
      return;
    }
    if (have_bg_ && shots_.empty()) cuda_check(cudaStreamSynchronize(0), "background");
    if (!shots_.empty() || !pinned_.p) return;
    const int i = *pinned_bad();
    if (i == kNoBad) return;
    float2 v{};
    cuda_check(cudaMemcpy(&v, static_cast<const float2*>(sref_.p) + i, sizeof v, cudaMemcpyDeviceToHost), "D2H sref");
    throw Fail(WEM_EINVAL, "Ref velocity " + std::to_string(v.x) + " at the layer " +
                               std::to_string((i / p_.nref) % p_.nz));
  }

 private:
  void build_timefreq(int n) { tf_ = make_timefreq(n, p_.nt, F_, geo_.bin[0], geo_.ns * geo_.nr, tftw_, tfwn_, tfs_); }

  // bins <- bins of (the bins' time traces - obs); the loss 1/2 |residual|^2
  // lands in page-locked host memory once the stream has reached it (the
  // per-CTA sums added in a fixed order)
  double* residual_bins(const float* obs) {
    double* part = lossbuf_.as<double>((size_t)tfs_.grid + 1);
    launch_timefreq(2, tf_, tfs_, bins_, nullptr, obs, geo_.ns * geo_.nr, 0, part, 0);
    launch_half_sum(part, tfs_.grid, part + tfs_.grid, 0);
    cuda_check(cudaGetLastError(), "residual launch");
    double* h = reinterpret_cast<double*>(pinned_.get());
    cuda_check(cudaMemcpyAsync(h, part + tfs_.grid, sizeof(double), cudaMemcpyDeviceToHost, 0), "D2H loss");
    return h;
  }

  // internal bins -> caller data: time traces by the inverse transform,
  // frequency data by a window copy
  void emit(void* data, int kind, int add) {
    require(data != nullptr, "data is NULL");
    const int ntr = geo_.ns * geo_.nr;
    Staged o;
    if (kind == WEM_DATA_TIME) {
      o.out(data, (size_t)ntr * p_.nt * 4, add != 0);
      bins_to_time((float*)o.dev, add);
    } else {
      require(kind == WEM_DATA_FREQ, "unknown data kind");
      o.out(data, (size_t)ntr * geo_.nbin * 8, add != 0);
      launch_bin_window(bins_, (float2*)o.dev, ntr, geo_.nbin, F_, geo_.bin[0], 1, add, 0);
    }
    cuda_check(cudaGetLastError(), "emit launch");
    cuda_check(cudaStreamSynchronize(0), "operator");
    o.finish(data);
    check_background();
  }

  // caller data -> internal bins
  void absorb(const void* data, int kind) {
    const int ntr = geo_.ns * geo_.nr;
    Staged s;
    if (kind == WEM_DATA_TIME) {
      s.in(data, (size_t)ntr * p_.nt * 4);
      time_to_bins((const float*)s.dev);
    } else {
      require(kind == WEM_DATA_FREQ, "unknown data kind");
      s.in(data, (size_t)ntr * geo_.nbin * 8);
      launch_bin_window((const float2*)s.dev, bins_, ntr, geo_.nbin, F_, geo_.bin[0], 0, 0, 0);
    }
    cuda_check(cudaGetLastError(), "absorb launch");
    cuda_check(cudaStreamSynchronize(0), "absorb");
  }
};

// ------------------------------------------------------------ 3D
// 3D one-way modelling and reflectivity Born on planes of ny x nx points per
// depth (no reference counterpart; at ny = 1 the 2D WEM and BornRefl).  The
// depth recursions run as per-depth batched passes over every (shot,
// frequency) row (kernels3d.cuh); forward-type fields keep their spectrum
// along x (S) and the per-reference planes after the column pass (T).
class Engine3D {
 public:
  // refl: the reflectivity Born / migration pair, which keeps the 2D
  // BornRefl conventions (ext_born_refl.cpp:18-25): propagation on the model
  // plane itself, pad and pad_y the taper widths only, point receivers
  Engine3D(const wem3d_params& q, const float* wavelet, bool refl = false) : p_(q.p) {
    require(wavelet != nullptr, "wavelet is NULL");
    const int twx = p_.pad, twy = q.pad_y;
    if (refl) {
      p_.pad = 0;
      p_.ngr = 0;
    }
    require(q.ny >= 1 && q.dy > 0, "ny must be >= 1 and dy > 0");
    require(q.pad_y >= 0 && q.tap_y >= 0 && q.pad_y != 1, "pad_y/tap_y must be >= 0 (pad_y != 1)");
    require(q.ny > 1 || (q.pad_y == 0 && q.tap_y == 0), "a single line (ny = 1) takes no y padding");
    require(p_.src_x && p_.src_z && p_.rec_x && p_.rec_z && q.src_y && q.rec_y,
            "3D devices need x, y and z coordinate arrays");
    require(p_.cmap == WEM_CMAP_NONE, "3D operators have no conformal maps");
    geo_ = make_geometry(p_, wavelet);
    ny_ = q.ny;
    pady_ = refl ? 0 : q.pad_y;
    const int nx = p_.nx, nz = p_.nz;
    nxg_ = nx + 2 * p_.pad;
    nyg_ = ny_ + 2 * pady_;
    Nx_ = nxg_ + 2 * p_.tap;
    Ny_ = nyg_ + 2 * q.tap_y;
    require(k3_supported(Nx_, Ny_), refl ? "3D reflectivity planes need Nx = nx + 2 tap and Ny = ny + 2 tap_y "
                                           "in {256, 384, 512, 768, 1024} (or Ny = 1 for ny = 1)"
                                         : "3D planes need Nx = nx + 2 pad + 2 tap and Ny = ny + 2 pad_y + 2 tap_y "
                                           "in {256, 384, 512, 768, 1024} (or Ny = 1 for ny = 1)");
    require(p_.nref <= nxg_ * nyg_, "nref larger than the padded slice");
    F_ = geo_.nfreq();
    const int ns = geo_.ns, nr = geo_.nr;
    rows_ = F_ * ns;
    auto yidx = [&](float y) {
      const int j = (int)((y - q.oy) / q.dy + .5f);
      require(j >= 0 && j < ny_, "Device is out of bounds!");
      return j;
    };
    std::vector<int> sy(ns), ry(nr);
    for (int s = 0; s < ns; ++s) sy[s] = yidx(q.src_y[s]);
    for (int i = 0; i < nr; ++i) ry[i] = yidx(q.rec_y[i]);
    // receivers by (depth, padded line, column)
    std::vector<int> ord(nr);
    std::iota(ord.begin(), ord.end(), 0);
    auto key = [&](int i) { return ((long long)geo_.rz[i] * nyg_ + ry[i] + pady_) * (nxg_ + 1) + geo_.rx[i]; };
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return key(a) < key(b); });
    std::vector<int> rptr((size_t)nz * nyg_ + 1, 0), rxs(nr);
    for (int i = 0; i < nr; ++i) rptr[(size_t)geo_.rz[ord[i]] * nyg_ + ry[ord[i]] + pady_ + 1]++;
    for (size_t k = 0; k + 1 < rptr.size(); ++k) rptr[k + 1] += rptr[k];
    for (int i = 0; i < nr; ++i) rxs[i] = geo_.rx[ord[i]];
    for (int s = 0; s < ns; ++s) require(geo_.rx.size() > 0 && geo_.sx[s] < nx, "source outside the model");
    // static tables
    std::vector<double> kx = k_grid(Nx_, p_.dx), ky = k_grid(Ny_, q.dy);
    c_.Qx = Nx_ / 2;
    c_.Qy = std::max(Ny_ / 2, 1);
    std::vector<float> kxq(kx.begin(), kx.begin() + c_.Qx), kyq(ky.begin(), ky.begin() + c_.Qy);
    std::vector<double> tx = taper(nxg_, twx), ty = taper(nyg_, twy);
    std::vector<float> tp((size_t)nyg_ * nxg_);
    for (int y = 0; y < nyg_; ++y)
      for (int x = 0; x < nxg_; ++x) tp[(size_t)y * nxg_ + x] = (float)(tx[x] * ty[y] / ((double)Nx_ * Ny_));
    std::vector<float> om(F_);
    for (int f = 0; f < F_; ++f) om[f] = (float)(2 * 3.14159265358979323846 * (double)geo_.freq[f]);
    Ctx3& c = c_;
    c.Nx = Nx_;
    c.Ny = Ny_;
    c.nxg = nxg_;
    c.nyg = nyg_;
    c.tapx = p_.tap;
    c.tapy = q.tap_y;
    c.pad = p_.pad;
    c.pady = pady_;
    c.nx = nx;
    c.ny = ny_;
    c.nz = nz;
    c.nref = p_.nref;
    c.prop = p_.prop;
    c.ns = ns;
    c.nr = nr;
    c.nfreq = F_;
    c.ngs = p_.ngs;
    c.ngr = p_.ngr;
    c.rows = rows_;
    c.dz = p_.dz;
    c.twx = upload(twx_, to_f2(twiddles(Nx_)));
    c.twy = upload(twy_, to_f2(twiddles(Ny_)));
    c.taper = upload(taper_, tp);
    c.omega = upload(om_, om);
    c.wave = upload(wave_, to_f2(geo_.wave_at));
    c.sx = upload(sx_, geo_.sx);
    c.sy = upload(sy_, sy);
    c.sz = upload(sz_, geo_.sz);
    std::vector<float> gsf(geo_.gs.begin(), geo_.gs.end()), grf(geo_.gr.begin(), geo_.gr.end());
    c.gs = upload(gs_, gsf);
    c.gr = upload(gr_, grf);
    c.rptr = upload(rptr_, rptr);
    c.rid = upload(rid_, ord);
    c.rxs = upload(rxs_, rxs);
    kxq_ = upload(kxb_, kxq);
    kyq_ = upload(kyb_, kyq);
    tf_ = make_timefreq(geo_.nt_pad, p_.nt, F_, geo_.bin[0], ns * nr, tftw_, tfwn_, tfs_);
    bins_ = binsbuf_.as<float2>((size_t)ns * nr * F_);
  }

  int nfreq() const { return F_; }

  // background [nz][ny][nx] slowness^2 and density: padded slices, the
  // RefSampler of each flattened slice, split-step exponents, Reflect and the
  // quadrant phase tables
  void set_background(const void* s2, const void* rho) {
    require(s2 && rho, "background model is NULL");
    const int nz = p_.nz, nref = p_.nref;
    const size_t n = (size_t)nz * ny_ * p_.nx, plane = (size_t)nyg_ * nxg_;
    Staged ss, sr;
    ss.in(s2, n * 8);
    sr.in(rho, n * 8);
    float2* sp = sp_.as<float2>((size_t)nz * plane);
    float2* dp = dp_.as<float2>((size_t)nz * plane);
    launch_pad3((const float2*)ss.dev, sp, nz, ny_, p_.nx, pady_, p_.pad, 0);
    launch_pad3((const float2*)sr.dev, dp, nz, ny_, p_.nx, pady_, p_.pad, 0);
    const int K = std::max(nref, 2);
    require((long long)plane - (long long)nz * nref >= K || plane * 4 <= (size_t)max_smem_per_block(),
            "slice too large for the RefSampler history of this depth count");
    float2* sref = sref_.as<float2>((size_t)nz * nref);
    signed char* ref = ref_.as<signed char>((size_t)nz * plane);
    int* bad = bad_.as<int>(1);
    cuda_check(cudaMemsetAsync(bad, 0x7f, sizeof(int), 0), "memset");
    launch_sref(sp, sref, 1, nz, (int)plane, nref, bad, 0);
    launch_refsampler(p_.refs_mode == WEM_REFS_NEAREST ? 1 : 0, sp, sref, 1, nz, (int)plane, nref,
                      scr_.as<float>(refs_scratch_floats(1, nz, nref)), ref, 0);
    const bool ssf = p_.prop == WEM_PROP_SSF;
    float2* q = ssf ? q_.as<float2>((size_t)nz * plane) : nullptr;
    float2* rc = rc_.as<float2>((size_t)nz * plane);
    launch_point_tables(1, nz, (int)plane, nref, 0, p_.eps, sp, nullptr, dp, sref, ref, q, rc, nullptr, nullptr, nullptr,
                        nullptr, nullptr, 0);
    c_.ref = ref;
    c_.q = q;
    c_.rc = rc;
    float2* ph = ph_.as<float2>((size_t)F_ * nz * nref * c_.Qy * c_.Qx);
    launch_k3_phase(c_, sref, kxq_, kyq_, p_.eps, p_.phase_law, ph, 0);
    c_.ph = ph;
    cuda_check(cudaGetLastError(), "3D table kernels");
    int hbad = 0;
    cuda_check(cudaMemcpy(&hbad, bad, sizeof hbad, cudaMemcpyDeviceToHost), "D2H status");
    if (hbad != kNoBad) {
      float2 v{};
      cuda_check(cudaMemcpy(&v, sref + hbad, sizeof v, cudaMemcpyDeviceToHost), "D2H sref");
      throw Fail(WEM_EINVAL, "Ref velocity " + std::to_string(v.x) + " at the layer " + std::to_string(hbad / nref));
    }
    have_bg_ = true;
  }

  // background slowness^2 with unit density (the reflectivity Born takes no
  // density, as BornRefl)
  void set_background_unit(const void* s2) {
    std::vector<float> ones((size_t)2 * p_.nz * ny_ * p_.nx, 0.f);
    for (size_t i = 0; i < ones.size(); i += 2) ones[i] = 1.f;
    set_background(s2, ones.data());
  }

  // nonlinear modelling (wem_prop.cpp:52-74 on planes): down sweep recording
  // the direct field and keeping R D; up sweep of the reflections recorded.
  // checkpoint k > 1: D kept every k depths, R D recomputed per segment
  void wem_forward(const void* s2, const void* rho, void* data, int kind, int add, int ck) {
    set_background(s2, rho);
    zero_bins();
    forward_two_sweeps(ck, true, nullptr);
    emit(data, kind, add);
  }

  // reflectivity Born (ext_born_refl.cpp:8-57 with one reflectivity for all
  // frequencies): bg = Down(src); record Up(r bg)
  void refl_forward(const void* model, void* data, int kind, int add, int ck) {
    require(have_bg_, "background not set");
    require(model && data, "NULL argument");
    Staged m;
    m.in(model, (size_t)p_.nz * ny_ * p_.nx * 8);
    zero_bins();
    forward_two_sweeps(ck, false, (const float2*)m.dev);
    emit(data, kind, add);
  }

  // its adjoint (ext_born_refl.cpp:60-105): image = sum conj(bg) Up^H(rec^H d),
  // both fields marching down together
  void refl_adjoint(void* model, const void* data, int kind, int add) {
    require(have_bg_, "background not set");
    require(model && data, "NULL argument");
    absorb(data, kind);
    const int nz = p_.nz;
    const size_t fp = (size_t)rows_ * nyg_ * nxg_;
    Planes A = planes(0), B = planes(1);
    float2* wb = wsp_[0].as<float2>(fp);
    float2* wa = wsp_[1].as<float2>(fp);
    Staged o;
    o.out(model, (size_t)nz * ny_ * p_.nx * 8, add != 0);
    for (int z = 0; z < nz; ++z) {
      Pass3 a{};
      a.z = z;
      a.zt = z - 1;
      a.init = z == 0 ? 1 : 0;
      a.src = 1;
      a.spatial = wb;
      a.tin = A.T;
      a.tout = A.S;
      a.last = z == nz - 1;
      launch_k3_rows(c_, a, 0, 0);
      Pass3 b{};
      b.z = z;
      b.zt = z + 1 < nz ? z + 1 : -1;
      b.init = z == 0 ? 1 : 0;
      b.rec_in = 1;
      b.spatial = wa;
      b.tin = B.S;
      b.tout = B.T;
      b.bins = bins_;
      b.last = z == nz - 1;
      launch_k3_rows(c_, b, 1, 0);
      launch_k3_image(c_, z, wb, wa, (float2*)o.dev, add, 0);
      if (z + 1 < nz) {
        launch_k3_cols(c_, z, 0, A.S, A.T, 0);
        launch_k3_cols(c_, z + 1, 1, B.T, B.S, 0);
      }
    }
    cuda_check(cudaGetLastError(), "3D launches");
    cuda_check(cudaStreamSynchronize(0), "3D adjoint");
    o.finish(model);
  }

 private:
  struct Planes {
    float2 *S, *T;
  };
  wem_params p_;
  Geometry geo_;
  int ny_ = 1, pady_ = 0, nxg_ = 0, nyg_ = 0, Nx_ = 0, Ny_ = 0, F_ = 0, rows_ = 0;
  bool have_bg_ = false;
  Ctx3 c_{};
  const float* kxq_ = nullptr;
  const float* kyq_ = nullptr;
  Buf twx_, twy_, taper_, om_, wave_, sx_, sy_, sz_, gs_, gr_, rptr_, rid_, rxs_, kxb_, kyb_, tftw_, tfwn_, binsbuf_;
  Buf sp_, dp_, sref_, ref_, bad_, scr_, q_, rc_, ph_;
  Buf pl_[2][2], wsp_[2], store_, seg_, lossbuf_;
  TimeFreq tf_{};
  TfShape tfs_{};
  float2* bins_ = nullptr;

  // plane set k: S [rows][Ny][Nx] and nref T planes
  Planes planes(int k) {
    const size_t plane = (size_t)rows_ * Ny_ * Nx_;
    return Planes{pl_[k][0].as<float2>(plane), pl_[k][1].as<float2>(plane * p_.nref)};
  }

  // down sweep of the source field over depths z0..z1 on plane set P (from
  // zero, or from the stored field `load` at z0); `at` sets each depth's
  // stores and records
  template <class F>
  void down(int z0, int z1, const float2* load, Planes P, F at) {
    for (int z = z0; z <= z1; ++z) {
      Pass3 a{};
      a.z = z;
      a.zt = z == z0 ? -1 : z - 1;
      a.init = z == z0 ? (load ? 2 : 1) : 0;
      a.load = load;
      a.src = (z == z0 && load) ? 0 : 1;
      a.tin = P.T;
      a.tout = P.S;
      a.last = z == z1;
      a.bins = bins_;
      at(z, a);
      launch_k3_rows(c_, a, 0, 0);
      if (z < z1) launch_k3_cols(c_, z, 0, P.S, P.T, 0);
    }
  }

  // WEM (wem = true: record the down field, up sweep of R D) or the
  // reflectivity Born (refl: up sweep of refl bg), with stored or
  // checkpointed down fields
  void forward_two_sweeps(int ck, bool wem, const float2* refl) {
    const int nz = p_.nz;
    const size_t fp = (size_t)rows_ * nyg_ * nxg_;
    const bool cp = ck > 1;
    const int ncp = cp ? (nz - 1) / ck + 1 : nz;
    float2* st = store_.as<float2>((size_t)ncp * fp);
    Planes A = planes(0);
    down(0, nz - 1, nullptr, A, [&](int z, Pass3& a) {
      a.record = wem ? 1 : 0;
      if (!cp || z % ck == 0) {
        a.store = st + (size_t)(cp ? z / ck : z) * fp;
        a.store_rw = (wem && !cp) ? 1 : 0;
      }
    });
    // up sweep: U[nz-1] = src(nz-1), U[z-1] = P_z U[z] + src(z-1), recorded,
    // src(z) = R[z] D[z] (WEM) or refl[z] bg[z]
    float2* seg = cp ? seg_.as<float2>((size_t)(ck + 1) * fp) : nullptr;
    int zs = nz;  // first depth of the recomputed segment
    Planes B = cp ? planes(1) : Planes{};
    for (int z = nz - 1; z >= 0; --z) {
      if (cp && z < zs) {
        const int z0 = (z / ck) * ck;
        down(z0, z, st + (size_t)(z0 / ck) * fp, B, [&](int d, Pass3& a) { a.store = seg + (size_t)(d - z0) * fp; });
        zs = z0;
      }
      Pass3 a{};
      a.z = z;
      a.zt = z == nz - 1 ? -1 : z + 1;
      a.init = z == nz - 1 ? 1 : 0;
      a.add = cp ? seg + (size_t)(z - zs) * fp : st + (size_t)z * fp;
      a.add_rw = (wem && cp) ? 1 : 0;
      a.refl = wem ? nullptr : refl;
      a.record = 1;
      a.tin = A.T;
      a.tout = A.S;
      a.bins = bins_;
      a.last = z == 0;
      launch_k3_rows(c_, a, 0, 0);
      if (z > 0) launch_k3_cols(c_, z, 0, A.S, A.T, 0);
    }
    cuda_check(cudaGetLastError(), "3D launches");
  }

  void zero_bins() {
    cuda_check(cudaMemsetAsync(bins_, 0, (size_t)geo_.ns * geo_.nr * F_ * 8, 0), "memset");
  }

  void emit(void* data, int kind, int add) {
    require(data != nullptr, "data is NULL");
    const int ntr = geo_.ns * geo_.nr;
    Staged o;
    if (kind == WEM_DATA_TIME) {
      o.out(data, (size_t)ntr * p_.nt * 4, add != 0);
      launch_timefreq(0, tf_, tfs_, bins_, (float*)o.dev, nullptr, ntr, add, nullptr, 0);
    } else {
      require(kind == WEM_DATA_FREQ, "unknown data kind");
      o.out(data, (size_t)ntr * geo_.nbin * 8, add != 0);
      launch_bin_window(bins_, (float2*)o.dev, ntr, geo_.nbin, F_, geo_.bin[0], 1, add, 0);
    }
    cuda_check(cudaGetLastError(), "emit launch");
    cuda_check(cudaStreamSynchronize(0), "operator");
    o.finish(data);
  }

  void absorb(const void* data, int kind) {
    const int ntr = geo_.ns * geo_.nr;
    Staged s;
    if (kind == WEM_DATA_TIME) {
      s.in(data, (size_t)ntr * p_.nt * 4);
      launch_timefreq(1, tf_, tfs_, bins_, const_cast<float*>((const float*)s.dev), nullptr, ntr, 0, nullptr, 0);
    } else {
      require(kind == WEM_DATA_FREQ, "unknown data kind");
      s.in(data, (size_t)ntr * geo_.nbin * 8);
      launch_bin_window((const float2*)s.dev, bins_, ntr, geo_.nbin, F_, geo_.bin[0], 0, 0, 0);
    }
    cuda_check(cudaGetLastError(), "absorb launch");
    cuda_check(cudaStreamSynchronize(0), "absorb");
  }
};

// ------------------------------------------------------------ wemop
// RefSampler tables of one padded slowness grid [nz][nxg] on the device,
// brought back to the host (the row-level operators build their other
// tables there)
void device_refsampler(const wem_params& p, const float2* slow_d, int nxg, std::vector<cd>& sref,
                       std::vector<signed char>& ref) {
  require(p.nref >= 1 && p.nref <= 127 && p.nref <= nxg, "nref must be in [1, min(127, nxg)]");
  const int nz = p.nz, nref = p.nref;
  Buf sb, rb, bb, scr;
  float2* dsref = sb.as<float2>((size_t)nz * nref);
  signed char* dref = rb.as<signed char>((size_t)nz * nxg);
  int* bad = bb.as<int>(1);
  cuda_check(cudaMemsetAsync(bad, 0x7f, sizeof(int), 0), "memset");
  launch_sref(slow_d, dsref, 1, nz, nxg, nref, bad, 0);
  launch_refsampler(p.refs_mode == WEM_REFS_NEAREST ? 1 : 0, slow_d, dsref, 1, nz, nxg, nref,
                    scr.as<float>(refs_scratch_floats(1, nz, nref)), dref, 0);
  cuda_check(cudaGetLastError(), "refsampler kernels");
  std::vector<float2> hs((size_t)nz * nref);
  int hbad = 0;
  cuda_check(cudaMemcpy(hs.data(), dsref, hs.size() * 8, cudaMemcpyDeviceToHost), "D2H sref");
  cuda_check(cudaMemcpy(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost), "D2H status");
  if (hbad != kNoBad)
    throw Fail(WEM_EINVAL, "Ref velocity " + std::to_string(hs[hbad].x) + " at the layer " +
                               std::to_string(hbad / nref));
  ref.resize((size_t)nz * nxg);
  cuda_check(cudaMemcpy(ref.data(), dref, ref.size(), cudaMemcpyDeviceToHost), "D2H ref");
  sref.resize(hs.size());
  for (size_t i = 0; i < hs.size(); ++i) sref[i] = cd(hs[i].x, hs[i].y);
}

class RowOps {
 public:
  RowOps(const wem_params& p, const void* slow, int nxg) : p_(p), nxg_(nxg) {
    require(slow != nullptr, "slowness is NULL");
    require(nxg >= 2 && p.nz > 1, "bad grid");
    require(p.pad >= 0 && p.tap >= 0 && p.pad != 1 && 2 * p.pad <= nxg, "bad pad/tap");
    require(p.ntaylor >= 0 && p.ntaylor <= 4, "ntaylor must be in [0,4]");
    require(p.phase_law == WEM_PHASE_ISPC || p.phase_law == WEM_PHASE_EXACT_KZ, "phase_law must be 0 or 1");
    std::vector<float> hs = host_floats(slow, 2 * (size_t)p.nz * nxg);
    std::vector<cd> sp((size_t)p.nz * nxg), dp(sp.size(), cd(1.0, 0.0));
    for (size_t i = 0; i < sp.size(); ++i) sp[i] = cd(hs[2 * i], hs[2 * i + 1]);
    std::vector<float2> sf(sp.size());
    for (size_t i = 0; i < sp.size(); ++i) sf[i] = make_float2(hs[2 * i], hs[2 * i + 1]);
    slow_d_ = upload(slow_, sf);
    // the partition from the operators' own device RefSampler
    std::vector<cd> sref;
    std::vector<signed char> ref;
    device_refsampler(p, slow_d_, nxg, sref, ref);
    t_ = make_slice_tables(p, sp, dp, nxg, true, sref, ref);
    N_ = nxg + 2 * p.tap;
    std::vector<double> k = k_grid(N_, p.dx), tp = taper(nxg, p.pad);
    std::vector<float> kf(k.begin(), k.end()), tpf(nxg);
    for (int i = 0; i < nxg; ++i) tpf[i] = (float)(tp[i] / N_);
    c_.plan = make_plan(N_);
    c_.N = N_;
    c_.nxg = nxg;
    c_.tap = p.tap;
    c_.pad = p.pad;
    c_.nz = p.nz;
    c_.nref = p.nref;
    c_.prop = p.prop;
    c_.ntaylor = p.ntaylor;
    c_.phase_law = p.phase_law;
    c_.nfreq = 1;
    c_.ext = 0;
    c_.dz = p.dz;
    c_.invN = 1.0f / N_;
    c_.tw = upload(tw_, to_f2(twiddles(N_)));
    c_.kx = upload(kx_, kf);
    c_.taperN = upload(taper_, tpf);
    c_.ref = upload(ref_, t_.ref);
    c_.sc = upload(sc_, to_f2(t_.sc));
    c_.rc = upload(rc_, to_f2(t_.rc));
    sref_d_ = upload(sref_, to_f2(t_.sref));
    q_d_ = upload(q_, to_f2(t_.q));
  }

  void set_freq(float freq) {
    if (have_freq_ && freq == freq_) return;
    float om = (float)(2 * 3.14159265358979323846 * (double)freq);
    c_.omega = upload(omega_, std::vector<float>{om});
    c_.ph = nullptr;
    float2* ph = ph_.as<float2>((size_t)p_.nz * p_.nref * N_);
    launch_phase_tables(c_, sref_d_, p_.eps, ph, 0);
    c_.ph = ph;
    if (p_.prop == WEM_PROP_SSF) {
      float2* fac = fac_.as<float2>((size_t)p_.nz * nxg_);
      launch_fac_tables(c_, q_d_, fac, 0);
      c_.fac = fac;
    } else {
      c_.fac = nullptr;
    }
    cuda_check(cudaGetLastError(), "table kernels");
    freq_ = freq;
    have_freq_ = true;
  }

  int G() const {
    int lim = max_smem_per_block(), G = 8;
    while (G > 1 && (int)smem_rows(c_, G) > lim) --G;
    require((int)smem_rows(c_, G) <= lim, "row too long for one CTA's shared memory");
    return G;
  }

  template <class L>
  void run_rows(const void* in, void* out, size_t per_row, int nrow, int add, L launch) {
    require(in && out && nrow >= 0, "bad arguments");
    const bool alias = in == out;
    Staged si, so;
    so.out(out, per_row * nrow * 8, add != 0 || alias);
    if (alias) si.dev = so.dev; else si.in(in, per_row * nrow * 8);
    launch((const float2*)si.dev, (float2*)so.dev, alias);
    cuda_check(cudaGetLastError(), "row kernel");
    cuda_check(cudaStreamSynchronize(0), "row kernel");
    so.finish(out);
  }

  // LinDown (LinOneWay.cpp:33-85) of one field [nz][nxg]: per depth the
  // imaging condition with the background row, the Taylor scatter and the
  // depth step, added into the next row; the adjoint runs the transposed
  // chain upwards.  As in the reference, the forward clears the first output
  // row whatever add says, and the compat adjoint the last one (the exact
  // adjoint, the transpose, leaves it).
  void lindown(const void* bg, float freq, int adj, const void* in, void* out, int add) {
    require(bg && in && out, "NULL argument");
    require(in != out, "lindown needs distinct model and data");
    set_freq(freq);
    const int nz = p_.nz, nx = nxg_;
    const size_t plane = (size_t)nz * nx;
    Staged sb, si, so;
    sb.in(bg, plane * 8);
    si.in(in, plane * 8);
    so.out(out, plane * 8, add != 0);
    const float2* b = (const float2*)sb.dev;
    const float2* x = (const float2*)si.dev;
    float2* o = (float2*)so.dev;
    float2* t = row_.as<float2>(2 * (size_t)nx);
    float2* u = t + nx;
    const int G = this->G();
    const int exact = p_.adjoint_mode == WEM_ADJ_EXACT ? 1 : 0;
    if (!add) cuda_check(cudaMemsetAsync(o, 0, plane * 8, 0), "memset");
    if (!adj) {
      cuda_check(cudaMemsetAsync(o, 0, (size_t)nx * 8, 0), "memset");
      for (int iz = 0; iz < nz - 1; ++iz) {
        launch_diag_rows(x + (size_t)iz * nx, b + (size_t)iz * nx, t, nx, 1, 0, 0, 0);
        launch_scatter(c_, 0, iz, 0, exact, t, u, 1, 0, G, 0);
        launch_onestep(c_, 0, iz, 0, u, t, 1, 0, G, 0);
        launch_scale_add(o + (size_t)(iz + 1) * nx, t, nx, 0);
      }
    } else {
      if (!exact) cuda_check(cudaMemsetAsync(o + (size_t)(nz - 1) * nx, 0, (size_t)nx * 8, 0), "memset");
      for (int iz = nz - 1; iz > 0; --iz) {
        launch_onestep(c_, 0, iz - 1, 1, x + (size_t)iz * nx, t, 1, 0, G, 0);
        launch_scatter(c_, 0, iz - 1, 1, exact, t, u, 1, 0, G, 0);
        launch_diag_rows(u, b + (size_t)(iz - 1) * nx, t, nx, 1, 1, 0, 0);
        launch_scale_add(o + (size_t)(iz - 1) * nx, t, nx, 0);
      }
    }
    cuda_check(cudaGetLastError(), "lindown kernels");
    cuda_check(cudaStreamSynchronize(0), "lindown");
    so.finish(out);
  }

  wem_params p_;
  int nxg_, N_ = 0;
  SliceTables t_;
  DevCtx c_{};
  Buf tw_, kx_, taper_, ref_, sc_, rc_, sref_, q_, omega_, ph_, fac_, slow_, row_;
  float2 *sref_d_ = nullptr, *q_d_ = nullptr, *slow_d_ = nullptr;
  float freq_ = 0;
  bool have_freq_ = false;
};

template <class Fn>
int guard(Fn fn) {
  try {
    fn();
    return WEM_OK;
  } catch (const Fail& e) {
    g_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_error = "host allocation failed";
    return WEM_ENOMEM;
  } catch (const std::exception& e) {
    g_error = e.what();
    return WEM_EINVAL;
  }
}

}  // namespace

// error text of a failed call on this thread (also used by noalloc.cu)
void set_last_error(const char* msg) { g_error = msg; }

}  // namespace wg

using namespace wg;

struct wem_handle { std::unique_ptr<Engine> e; };
struct born_handle { std::unique_ptr<Engine> e; };
struct extwem_handle { std::unique_ptr<Engine> e; };
struct extborn_handle { std::unique_ptr<Engine> e; };
struct fwi_handle { std::unique_ptr<Engine> e; };
struct bornrefl_handle { std::unique_ptr<Engine> e; };
struct borntomo_handle { std::unique_ptr<Engine> e; };
struct bornoff_handle { std::unique_ptr<Engine> e; };
struct wem3d_handle { std::unique_ptr<Engine3D> e; };
struct refl3d_handle { std::unique_ptr<Engine3D> e; };
struct wemop_handle { std::unique_ptr<RowOps> r; };

extern "C" {

void wem_params_default(wem_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->prop = WEM_PROP_SSF;
  p->nref = 1;
  p->ntaylor = 1;
  p->eps = 0.04f;
  p->fmin = 1.0f;
  p->adjoint_mode = WEM_ADJ_COMPAT;
  p->refs_mode = WEM_REFS_ASCODED;
  p->phase_law = WEM_PHASE_ISPC;
  p->cmap = WEM_CMAP_NONE;
  p->eps_log = 0.01f;
}

const char* wem_last_error(void) { return g_error.c_str(); }

int wem_stats_enable(int on) {
  g_stats_on = on != 0;
  return WEM_OK;
}
int wem_stats_get(const char* kernel, double* total_ms, long long* launches) {
  return guard([&] {
    require(kernel && total_ms && launches, "NULL argument");
    std::lock_guard<std::mutex> lock(g_stats_mu);
    KStat& k = stat_of(kernel);
    *total_ms = k.ms;
    *launches = k.n;
  });
}
int wem_set_kernel_path(int path) {
  return guard([&] {
    require(path >= 0 && path <= 2, "path must be 0, 1 or 2");
    g_path = path;
  });
}
int wem_set_row_ctas(int mode) {
  return guard([&] {
    require(mode >= 0 && mode <= 2, "mode must be 0, 1 or 2");
    g_rows = mode;
  });
}
int wem_set_gradient_split(int on) {
  return guard([&] {
    require(on == 0 || on == 1, "on must be 0 or 1");
    g_split_off = on == 0;
  });
}
int wem_set_plain(int plain) {
  g_plain = plain != 0;
  return WEM_OK;
}
int wem_stats_reset(void) {
  std::lock_guard<std::mutex> lock(g_stats_mu);
  g_stats.clear();
  return WEM_OK;
}
long long wem_launch_count(void) { return launch_count(); }
const char* wem_version(void) { return "wemgpu 0.1 (sm_103a)"; }

int wem_count_freqs(const wem_params* p, const float* wavelet, int* nfreq) {
  (void)wavelet;
  return guard([&] {
    require(p && nfreq, "NULL argument");
    *nfreq = count_frequencies(*p);
  });
}

// ---- WEM
int wem_create(const wem_params* p, const float* wavelet, wem_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<wem_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, false, false);
    *out = h.release();
  });
}
void wem_destroy(wem_handle* h) { delete h; }
int wem_get_nfreq(wem_handle* h, int* n) {
  return guard([&] { require(h && n, "NULL argument"); *n = h->e->nfreq(); });
}
int wem_forward(wem_handle* h, const void* s2, const void* rho, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->wem_forward(s2, rho, data, kind, add); });
}

// ---- Born
int born_create(const wem_params* p, const float* wavelet, const void* s2, const void* rho, born_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<born_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, false, true);
    h->e->set_background(s2, rho);
    h->e->check_background();
    *out = h.release();
  });
}
void born_destroy(born_handle* h) { delete h; }
int born_set_background(born_handle* h, const void* s2, const void* rho) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    h->e->set_background(s2, rho);
    h->e->check_background();
  });
}
int born_forward(born_handle* h, const void* ds2, const void* drho, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->born_forward(ds2, drho, data, kind, add); });
}
int born_adjoint(born_handle* h, void* ds2, void* drho, const void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->born_adjoint(ds2, drho, data, kind, add); });
}

// ---- extended
int extwem_create(const wem_params* p, const float* wavelet, extwem_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<extwem_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, true, false);
    *out = h.release();
  });
}
void extwem_destroy(extwem_handle* h) { delete h; }
int extwem_forward(extwem_handle* h, const void* s2, const void* rho, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->wem_forward(s2, rho, data, kind, add); });
}
// background of the variants: slowness^2 with unit density (the reference's
// BornRefl / BornTomo take no density; it only enters the tables they replace)
static void set_bg_unit_rho(Engine& e, const wem_params& p, const void* s2) {
  std::vector<float> ones((size_t)2 * p.nz * p.nx, 0.f);
  for (size_t i = 0; i < ones.size(); i += 2) ones[i] = 1.f;
  e.set_background(s2, ones.data());
  e.check_background();
}

int bornrefl_create(const wem_params* p, const float* wavelet, const void* s2, bornrefl_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<bornrefl_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, false, true, 1);
    set_bg_unit_rho(*h->e, *p, s2);
    *out = h.release();
  });
}
void bornrefl_destroy(bornrefl_handle* h) { delete h; }
int bornrefl_set_background(bornrefl_handle* h, const void* s2) {
  return guard([&] { require(h != nullptr, "NULL handle"); set_bg_unit_rho(*h->e, h->e->params(), s2); });
}
int bornrefl_forward(bornrefl_handle* h, const void* model, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->refl_forward(model, data, kind, add); });
}
int bornrefl_adjoint(bornrefl_handle* h, void* model, const void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->refl_adjoint(model, data, kind, add); });
}

int bornoff_create(const wem_params* p, const float* wavelet, const void* s2, int nh, const int* ap_x0,
                   const int* ap_w, bornoff_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<bornoff_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, false, false, 3);
    h->e->off_init(nh, ap_x0, ap_w);
    set_bg_unit_rho(*h->e, *p, s2);
    *out = h.release();
  });
}
void bornoff_destroy(bornoff_handle* h) { delete h; }
int bornoff_set_background(bornoff_handle* h, const void* s2) {
  return guard([&] { require(h != nullptr, "NULL handle"); set_bg_unit_rho(*h->e, h->e->params(), s2); });
}
int bornoff_forward(bornoff_handle* h, const void* model, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->off_forward(model, data, kind, add); });
}
int bornoff_adjoint(bornoff_handle* h, void* model, const void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->off_adjoint(model, data, kind, add); });
}
int bornoff_rows(bornoff_handle* h, int* row_len, int* tap) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->off_rows(row_len, tap); });
}

int wem3d_create(const wem3d_params* p, const float* wavelet, wem3d_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<wem3d_handle>();
    h->e = std::make_unique<Engine3D>(*p, wavelet);
    *out = h.release();
  });
}
void wem3d_destroy(wem3d_handle* h) { delete h; }
int wem3d_forward(wem3d_handle* h, const void* s2, const void* rho, void* data, int kind, int add, int checkpoint) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->wem_forward(s2, rho, data, kind, add, checkpoint); });
}
int refl3d_create(const wem3d_params* p, const float* wavelet, const void* s2, refl3d_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<refl3d_handle>();
    h->e = std::make_unique<Engine3D>(*p, wavelet, true);
    h->e->set_background_unit(s2);
    *out = h.release();
  });
}
void refl3d_destroy(refl3d_handle* h) { delete h; }
int refl3d_set_background(refl3d_handle* h, const void* s2) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    h->e->set_background_unit(s2);
  });
}
int refl3d_forward(refl3d_handle* h, const void* model, void* data, int kind, int add, int checkpoint) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->refl_forward(model, data, kind, add, checkpoint); });
}
int refl3d_adjoint(refl3d_handle* h, void* model, const void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->refl_adjoint(model, data, kind, add); });
}
int wem3d_get_nfreq(wem3d_handle* h, int* n) {
  return guard([&] {
    require(h && n, "NULL argument");
    *n = h->e->nfreq();
  });
}

int borntomo_create(const wem_params* p, const float* wavelet, const void* s2, borntomo_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<borntomo_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, false, true, 2);
    set_bg_unit_rho(*h->e, *p, s2);
    *out = h.release();
  });
}
void borntomo_destroy(borntomo_handle* h) { delete h; }
int borntomo_set_background(borntomo_handle* h, const void* s2) {
  return guard([&] { require(h != nullptr, "NULL handle"); set_bg_unit_rho(*h->e, h->e->params(), s2); });
}
int borntomo_set_refl(borntomo_handle* h, const void* refl) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->tomo_set_refl(refl); });
}
int borntomo_forward(borntomo_handle* h, const void* dm, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->tomo_forward(dm, data, kind, add); });
}
int borntomo_adjoint(borntomo_handle* h, void* dm, const void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->tomo_adjoint(dm, data, kind, add); });
}

int fwi_create(const wem_params* p, const float* wavelet, fwi_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<fwi_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, false, true);
    *out = h.release();
  });
}
void fwi_destroy(fwi_handle* h) { delete h; }
int fwi_gradient(fwi_handle* h, const void* s2, const void* rho, const void* d_obs, void* g_s2, void* g_rho,
                 double* loss) {
  return guard([&] {
    require(h != nullptr && loss != nullptr, "NULL argument");
    *loss = h->e->fwi_gradient(s2, rho, d_obs, g_s2, g_rho);
  });
}

int fwi_gradient_exact(fwi_handle* h, const void* s2, const void* rho, const void* d_obs, void* g_s2, void* g_rho,
                       double* loss, int checkpoint) {
  return guard([&] {
    require(h != nullptr && loss != nullptr, "NULL argument");
    *loss = h->e->fwi_gradient_exact(s2, rho, d_obs, g_s2, g_rho, checkpoint);
  });
}

int wem_gradient(wem_handle* h, const void* s2, const void* rho, const void* data_grad, int kind, void* g_s2,
                 void* g_rho, int add, int checkpoint) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    h->e->wem_gradient(s2, rho, data_grad, kind, g_s2, g_rho, add, checkpoint);
  });
}

int extborn_create(const wem_params* p, const float* wavelet, const void* s2, const void* rho,
                   extborn_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<extborn_handle>();
    h->e = std::make_unique<Engine>(*p, wavelet, true, true);
    h->e->set_background(s2, rho);
    h->e->check_background();
    *out = h.release();
  });
}
void extborn_destroy(extborn_handle* h) { delete h; }
int extborn_set_background(extborn_handle* h, const void* s2, const void* rho) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    h->e->set_background(s2, rho);
    h->e->check_background();
  });
}
int extborn_forward(extborn_handle* h, const void* ds2, const void* drho, void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->born_forward(ds2, drho, data, kind, add); });
}
int extborn_adjoint(extborn_handle* h, void* ds2, void* drho, const void* data, int kind, int add) {
  return guard([&] { require(h != nullptr, "NULL handle"); h->e->born_adjoint(ds2, drho, data, kind, add); });
}

// ---- row-level operators
int wemop_create(const wem_params* p, const void* slow, int nxg, wemop_handle** out) {
  return guard([&] {
    require(p && out, "NULL argument");
    auto h = std::make_unique<wemop_handle>();
    h->r = std::make_unique<RowOps>(*p, slow, nxg);
    *out = h.release();
  });
}
void wemop_destroy(wemop_handle* h) { delete h; }

int wemop_onestep(wemop_handle* h, int iz, float freq, int adj, const void* in, void* out, int nrow, int add) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    RowOps& R = *h->r;
    require(iz >= 0 && iz < R.p_.nz, "depth index out of range");
    R.set_freq(freq);
    int G = R.G();
    R.run_rows(in, out, R.nxg_, nrow, add, [&](const float2* a, float2* b, bool alias) {
      require(!alias, "onestep needs distinct input and output");
      launch_onestep(R.c_, 0, iz, adj, a, b, nrow, add, G, 0);
    });
  });
}

int wemop_oneway(wemop_handle* h, int up, float freq, int adj, const void* in, void* out, int nrow, int add) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    RowOps& R = *h->r;
    R.set_freq(freq);
    int G = R.G();
    R.run_rows(in, out, (size_t)R.nxg_ * R.p_.nz, nrow, add, [&](const float2* a, float2* b, bool alias) {
      launch_oneway(R.c_, 0, up, adj, alias ? 1 : 0, a, b, nrow, add, G, 0);
    });
  });
}

int wemop_scatter(wemop_handle* h, int iz, float freq, int adj, const void* in, void* out, int nrow, int add) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    RowOps& R = *h->r;
    require(iz >= 0 && iz < R.p_.nz, "depth index out of range");
    R.set_freq(freq);
    int G = R.G();
    int exact = R.p_.adjoint_mode == WEM_ADJ_EXACT ? 1 : 0;
    R.run_rows(in, out, R.nxg_, nrow, add, [&](const float2* a, float2* b, bool alias) {
      require(!alias, "scatter needs distinct input and output");
      launch_scatter(R.c_, 0, iz, adj, exact, a, b, nrow, add, G, 0);
    });
  });
}

int wemop_refsampler(wemop_handle* h, void* sref, int* refidx) {
  return guard([&] {
    require(h && sref && refidx, "NULL argument");
    RowOps& R = *h->r;
    float* s = (float*)sref;
    for (size_t i = 0; i < R.t_.sref.size(); ++i) {
      s[2 * i] = (float)R.t_.sref[i].real();
      s[2 * i + 1] = (float)R.t_.sref[i].imag();
    }
    for (size_t i = 0; i < R.t_.ref.size(); ++i) refidx[i] = R.t_.ref[i];
  });
}

int wemop_splitstep(wemop_handle* h, int iz, float freq, float sref_re, float sref_im, const int* loc, int nloc,
                    int adj, const void* in, void* out, int nrow, int add) {
  return guard([&] {
    require(h && in && out && (loc || nloc == 0), "NULL argument");
    RowOps& R = *h->r;
    require(iz >= 0 && iz < R.p_.nz, "depth index out of range");
    require(nloc >= 0 && nrow >= 0, "negative count");
    require(!(sref_re == 0.f && sref_im == 0.f), "reference slowness is zero");
    std::vector<int> hl(loc, loc + nloc);
    for (int x : hl) require(x >= 0 && x < R.nxg_, "split-step location out of the row");
    Buf lb;
    const int* dl = upload(lb, hl);
    const size_t per = R.nxg_;
    const bool alias = in == out;
    Staged si, so;
    // points off the list keep the output's contents (zero without add)
    so.out(out, per * nrow * 8, add != 0 || alias);
    if (alias) si.dev = so.dev; else si.in(in, per * nrow * 8);
    if (!add) cuda_check(cudaMemsetAsync(so.dev, 0, per * nrow * 8, 0), "memset");
    const float w = (float)(2 * 3.14159265358979323846 * (double)freq);
    launch_splitstep(R.slow_d_ + (size_t)iz * R.nxg_, dl, nloc, R.nxg_, nrow, (double)(w * R.p_.dz), sref_re,
                     sref_im, adj, (const float2*)si.dev, (float2*)so.dev, 0);
    cuda_check(cudaGetLastError(), "splitstep kernel");
    cuda_check(cudaStreamSynchronize(0), "splitstep");
    so.finish(out);
  });
}

int wemop_lindown(wemop_handle* h, const void* bg, float freq, int adj, const void* in, void* out, int add) {
  return guard([&] {
    require(h != nullptr, "NULL handle");
    h->r->lindown(bg, freq, adj, in, out, add);
  });
}

int wem_ic(const void* bg, int n, int adj, const void* in, void* out, int add) {
  return guard([&] {
    require(bg && in && out && n >= 0, "bad arguments");
    Staged sb, si, so;
    sb.in(bg, (size_t)n * 8);
    so.out(out, (size_t)n * 8, add != 0 || in == out);
    if (in == out) si.dev = so.dev; else si.in(in, (size_t)n * 8);
    launch_diag_rows((const float2*)si.dev, (const float2*)sb.dev, (float2*)so.dev, n, 1, adj ? 1 : 0, add, 0);
    cuda_check(cudaGetLastError(), "ic kernel");
    cuda_check(cudaStreamSynchronize(0), "ic");
    so.finish(out);
  });
}

int wem_phshift(const wem_params* p, int n, float dx, float dz, float freq, float s_re, float s_im, int adj,
                const void* in, void* out, int nrow, int add) {
  return guard([&] {
    require(p && in && out, "NULL argument");
    require(n >= 2 && nrow >= 0 && dx > 0, "bad row length or spacing");
    require(p->phase_law == WEM_PHASE_ISPC || p->phase_law == WEM_PHASE_EXACT_KZ, "phase_law must be 0 or 1");
    // the factor of every k sample from the depth step's phase-table kernel
    // on a one-row table, then applied to the rows
    Buf kb, ob, sb, fb;
    std::vector<double> k = k_grid(n, dx);
    DevCtx c{};
    c.N = n;
    c.nz = 1;
    c.nref = 1;
    c.nfreq = 1;
    c.dz = dz;
    c.phase_law = p->phase_law;
    c.kx = upload(kb, std::vector<float>(k.begin(), k.end()));
    c.omega = upload(ob, std::vector<float>{(float)(2 * 3.14159265358979323846 * (double)freq)});
    const float2* sref = upload(sb, std::vector<float2>{make_float2(s_re, s_im)});
    float2* f = fb.as<float2>(n);
    launch_phase_tables(c, sref, p->eps, f, 0);
    const bool alias = in == out;
    Staged si, so;
    so.out(out, (size_t)n * nrow * 8, add != 0 || alias);
    if (alias) si.dev = so.dev; else si.in(in, (size_t)n * nrow * 8);
    launch_diag_rows((const float2*)si.dev, f, (float2*)so.dev, n, nrow, adj ? 1 : 0, add, 0);
    cuda_check(cudaGetLastError(), "phshift kernels");
    cuda_check(cudaStreamSynchronize(0), "phshift");
    so.finish(out);
  });
}

// Reflect / dReflect coefficients of one grid from the point-table kernel
struct ReflTables {
  Buf s, d, rc, sc, a0, b0, a1, b1;
  DevCtx c{};
  ReflTables(const void* slow2, const void* rho, int nx, int nz, bool born) {
    require(slow2 && rho && nx >= 1 && nz >= 2, "bad reflectivity arguments");
    const size_t n = (size_t)nx * nz;
    Staged ss, sr;
    ss.in(slow2, n * 8);
    sr.in(rho, n * 8);
    float2* sp = s.as<float2>(n);
    float2* dp = d.as<float2>(n);
    cuda_check(cudaMemcpy(sp, ss.dev, n * 8, cudaMemcpyDeviceToDevice), "copy");
    cuda_check(cudaMemcpy(dp, sr.dev, n * 8, cudaMemcpyDeviceToDevice), "copy");
    launch_point_tables(1, nz, nx, 1, 0, 0.f, sp, nullptr, dp, nullptr, nullptr, nullptr, rc.as<float2>(n),
                        born ? sc.as<float2>(n) : nullptr, born ? a0.as<float2>(n) : nullptr,
                        born ? b0.as<float2>(n) : nullptr, born ? a1.as<float2>(n) : nullptr,
                        born ? b1.as<float2>(n) : nullptr, 0);
    cuda_check(cudaGetLastError(), "point tables");
    c.nz = nz;
    c.nxg = nx;
    c.pad = 0;
  }
};

// Injection.h:53-65: the cos^2 window in the reference's float arithmetic
static std::vector<float> inject_window(int ng) {
  std::vector<float> g(2 * ng + 1, 1.f);
  if (ng == 0) return g;
  const float pi = (float)(4 * std::atan(1.));
  const int sz = 2 * ng + 1;
  for (int i = 0; i < sz / 2; ++i) g[i] = (-std::cos(pi / ng * i) + 1) / 2;
  for (int i = sz / 2; i < sz; ++i) g[i] = (std::cos(pi / ng * (i - sz + ng + 1)) + 1) / 2;
  return g;
}

int wem_inject(const int* iz, const int* ix, int npt, int ng, int tap, int nx, int nz, int nt, int nshot, int step,
               int shot, int adj, void* model, void* data, int add) {
  return guard([&] {
    require(model && data && model != data && npt >= 0 && (npt == 0 || (iz && ix)), "bad arguments");
    require(nx > 0 && nz > 0 && nt > 0 && ng >= 0 && nshot >= 0, "bad sizes");
    require(step >= 0 && step < nt, "step outside the model's time axis");
    require(nshot == 0 || (shot >= 0 && shot < nshot), "shot outside the model's shot axis");
    for (int i = 0; i < npt; ++i) require(iz[i] >= 0 && iz[i] < nz, "a point's depth index is outside the rows");
    Buf gb, zb, xb;
    const float* g = upload(gb, inject_window(ng));
    const int* zd = upload(zb, std::vector<int>(iz, iz + npt));
    const int* xd = upload(xb, std::vector<int>(ix, ix + npt));
    // the 1D model [nt] gives every point model[step]; the 3D one
    // [nshot][npt][nt] gives point i model[shot][i][step]
    const size_t msize = (size_t)(nshot ? (size_t)nshot * npt : 1) * nt * 8, dsize = (size_t)nz * nx * 8;
    const size_t off0 = nshot ? ((size_t)shot * npt) * nt + step : (size_t)step;
    const size_t stride = nshot ? (size_t)nt : 0;
    Staged sm, sd;
    if (!adj) {
      sm.in(model, msize);
      sd.out(data, dsize, add != 0);
      launch_inject(zd, xd, npt, g, ng, tap, nx, nz, 0, (float2*)sm.dev, off0, stride, (float2*)sd.dev, add, 0);
      cuda_check(cudaGetLastError(), "inject kernel");
      cuda_check(cudaStreamSynchronize(0), "inject");
      sd.finish(data);
    } else {
      sd.in(data, dsize);
      sm.out(model, msize, add != 0);
      // the reference clears the whole model unless adding (Injection.cpp:22,65)
      if (!add) cuda_check(cudaMemsetAsync(sm.dev, 0, msize, 0), "memset");
      launch_inject(zd, xd, npt, g, ng, tap, nx, nz, 1, (float2*)sm.dev, off0, stride, (float2*)sd.dev, add, 0);
      cuda_check(cudaGetLastError(), "inject kernel");
      cuda_check(cudaStreamSynchronize(0), "inject");
      sm.finish(model);
    }
  });
}

int wem_reflect(const void* slow2, const void* rho, int nx, int nz, int adj, const void* in, void* out) {
  return guard([&] {
    require(in && out, "NULL argument");
    ReflTables T(slow2, rho, nx, nz, false);
    const size_t n = (size_t)nx * nz;
    const bool alias = in == out;
    Staged si, so;
    so.out(out, n * 8, alias);
    if (alias) si.dev = so.dev; else si.in(in, n * 8);
    // Reflect.h:34-47 assigns r m (conj(r) d): the output never accumulates
    launch_diag_rows((const float2*)si.dev, (const float2*)T.rc.p, (float2*)so.dev, (int)n, 1, adj ? 1 : 0, 0, 0);
    cuda_check(cudaGetLastError(), "reflect kernel");
    cuda_check(cudaStreamSynchronize(0), "reflect");
    so.finish(out);
  });
}

int wem_dreflect(const void* slow2, const void* rho, int nx, int nz, int adj, void* dslow2, void* drho, void* data,
                 int add) {
  return guard([&] {
    require(dslow2 && drho && data, "NULL argument");
    ReflTables T(slow2, rho, nx, nz, true);
    const size_t n = (size_t)nx * nz;
    const float2 *a0 = (const float2*)T.a0.p, *b0 = (const float2*)T.b0.p;
    const float2 *a1 = (const float2*)T.a1.p, *b1 = (const float2*)T.b1.p;
    if (!adj) {
      Staged m0, m1, d;
      m0.in(dslow2, n * 8);
      m1.in(drho, n * 8);
      d.out(data, n * 8, add != 0);
      Buf tb;
      float2* t = add ? tb.as<float2>(n) : (float2*)d.dev;
      launch_drefl_fwd(T.c, 1, a0, b0, a1, b1, (const float2*)m0.dev, (const float2*)m1.dev, t, 0);
      if (add) launch_scale_add((float2*)d.dev, t, n, 0);
      cuda_check(cudaGetLastError(), "dreflect kernels");
      cuda_check(cudaStreamSynchronize(0), "dreflect");
      d.finish(data);
    } else {
      Staged d, g0, g1;
      d.in(data, n * 8);
      g0.out(dslow2, n * 8, add != 0);
      g1.out(drho, n * 8, add != 0);
      Buf zb;
      float2* zero = zb.as<float2>(n);
      cuda_check(cudaMemsetAsync(zero, 0, n * 8, 0), "memset");
      launch_grad_assemble(T.c, 1, a0, b0, a1, b1, (const float2*)d.dev, zero, (float2*)g0.dev, (float2*)g1.dev, nx,
                           add, 0);
      cuda_check(cudaGetLastError(), "dreflect kernels");
      cuda_check(cudaStreamSynchronize(0), "dreflect");
      g0.finish(dslow2);
      g1.finish(drho);
    }
  });
}

}  // extern "C"
