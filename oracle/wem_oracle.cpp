// ORACLE — test infrastructure only (see wem_oracle.hpp).  Drivers of the
// CPU restatement and the extern "C" surface that tests/ and bench.py reach
// through ctypes.  PARITY PINNED to the reference run (tests/test_ref_pin.py).
//
// Drivers follow the reference's per-(shot, frequency) call sequence
// literally, without the algebraic fusions the GPU library makes, so that
// those fusions are checked rather than restated.

#include <atomic>
#include <functional>
#include <thread>

#include "cmap_oracle.hpp"
#include "wem_oracle.hpp"

namespace wo {
namespace {

thread_local std::string g_err;

template <class Fn>
void parallel_for(int ntask, int nthreads, Fn fn) {
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  nthreads = std::max(1, std::min(nthreads, ntask));
  if (nthreads == 1) {
    for (int t = 0; t < ntask; ++t) fn(t, 0);
    return;
  }
  // static block partition, as tbb::static_partitioner over a blocked range
  // (propagator/src/wem_prop.cpp:11,76)
  std::vector<std::thread> th;
  std::exception_ptr err;
  std::atomic<bool> failed{false};
  for (int i = 0; i < nthreads; ++i) {
    int b = (int)((long long)ntask * i / nthreads), e = (int)((long long)ntask * (i + 1) / nthreads);
    th.emplace_back([&, b, e, i] {
      try {
        for (int t = b; t < e; ++t) fn(t, i);
      } catch (...) {
        if (!failed.exchange(true)) err = std::current_exception();
      }
    });
  }
  for (auto& t : th) t.join();
  if (err) std::rethrow_exception(err);
}

template <class R>
std::vector<C<R>> load(const float* p, size_t n) {
  std::vector<C<R>> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = C<R>((R)p[2 * i], (R)p[2 * i + 1]);
  return v;
}

template <class R>
void store(float* p, const C<R>* v, size_t n, bool add) {
  for (size_t i = 0; i < n; ++i) {
    float re = (float)v[i].real(), im = (float)v[i].imag();
    if (add) { p[2 * i] += re; p[2 * i + 1] += im; } else { p[2 * i] = re; p[2 * i + 1] = im; }
  }
}

// Quantities every driver derives from the parameters (PropParam.h:24-85,
// Device.h), for one real type.
template <class R>
struct Problem {
  wem_params p;
  Freqs F;
  Devices src, rec;
  int nxg, nbin;
  std::vector<C<R>> wave_f;  // unitary FFT of the time-padded wavelet

  Problem(const wem_params& p_, const float* wavelet) : p(p_) {
    check(p.nx > 0 && p.nz > 1, "model must have nx > 0 and nz > 1");
    check(p.dx > 0 && p.dz > 0, "grid spacing must be positive");
    check(p.nref >= 1, "nref must be >= 1");
    check(p.pad >= 0 && p.tap >= 0 && p.tpad >= 0, "pad/tap/tpad must be >= 0");
    check(p.pad != 1, "pad == 1 makes the taper divide by zero (Taper.h:19)");
    F = make_freqs(p);
    src = make_devices(p, true);
    rec = make_devices(p, false);
    nxg = p.nx + 2 * p.pad;
    nbin = p.nbin ? p.nbin : F.nt_pad;
    for (int b : F.bin) check(b >= 0 && b < F.nt_pad && b < nbin, "frequency bin beyond the data axis");
    // FFT1_r forward of the wavelet (FFT1_r.cpp:74-83 via PropParam.h:49-54)
    Fft<R> fft(F.nt_pad);
    wave_f.assign(F.nt_pad, C<R>(0));
    for (int i = 0; i < p.nt; ++i) wave_f[i] = C<R>((R)wavelet[i], 0);
    std::vector<C<R>> scr(F.nt_pad);
    fft.run(wave_f.data(), -1, scr.data());
    R s = (R)(1.0 / std::sqrt((double)F.nt_pad));
    for (auto& v : wave_f) v *= s;
  }
  int nfreq() const { return (int)F.freq.size(); }
  Inject<R> src_inj(int is) const { return Inject<R>({src.ix[is]}, {src.iz[is]}, p.ngs, p.pad); }
  Inject<R> rec_inj() const { return Inject<R>(rec.ix, rec.iz, p.ngr, p.pad); }
};

// Complex bins <-> real time traces (FFT1_r.cpp, WEMnl.cpp:39-65,
// BornFull.cpp:80-102).  data_f [ns][nr][nt_pad].
template <class R>
void bins_to_time(const Problem<R>& P, const std::vector<C<R>>& df, float* dt, bool add, int nthreads) {
  int ntr = P.p.ns * P.p.nr, n = P.F.nt_pad, nt = P.p.nt;
  Fft<R> fft(n);
  R s = (R)(1.0 / std::sqrt((double)n));
  parallel_for(ntr, nthreads, [&](int tr, int) {
    std::vector<C<R>> x(df.begin() + (size_t)tr * n, df.begin() + (size_t)(tr + 1) * n), scr(n);
    fft.run(x.data(), +1, scr.data());
    float* o = dt + (size_t)tr * nt;
    for (int t = 0; t < nt; ++t) {
      float v = (float)(x[t].real() * s);
      o[t] = add ? o[t] + v : v;
    }
  });
}

template <class R>
std::vector<C<R>> time_to_bins(const Problem<R>& P, const float* dt, int nthreads) {
  int ntr = P.p.ns * P.p.nr, n = P.F.nt_pad, nt = P.p.nt;
  std::vector<C<R>> df((size_t)ntr * n);
  Fft<R> fft(n);
  R s = (R)(1.0 / std::sqrt((double)n));
  parallel_for(ntr, nthreads, [&](int tr, int) {
    C<R>* x = df.data() + (size_t)tr * n;
    for (int t = 0; t < n; ++t) x[t] = C<R>(t < nt ? (R)dt[(size_t)tr * nt + t] : R(0), 0);
    std::vector<C<R>> scr(n);
    fft.run(x, -1, scr.data());
    for (int t = 0; t < n; ++t) x[t] *= s;
  });
  return df;
}

// complex data view [ns][nr][nb]
template <class R>
struct DataF {
  std::vector<C<R>> v;
  int ns, nr, nb;
  C<R>* at(int is, int ir, int b) { return &v[((size_t)is * nr + ir) * nb + b]; }
};

// the source of shot is: the acquisition's point, or the points of a
// conformal map (several points of one shot all carry the wavelet)
template <class R>
void spread_source(const Problem<R>& P, int is, const Inject<R>* src_ov, C<R>* W, int nx, C<R> wv) {
  if (!src_ov) {
    P.src_inj(is).spread(W, nx, &wv);
    return;
  }
  std::vector<C<R>> vals(src_ov->ix.size(), wv);
  src_ov->spread(W, nx, vals.data());
}

// ------------------------------------------------------------ WEM forward
// WEM::full_fwd (propagator/src/wem_prop.cpp:9-78) for one padded model.
template <class R>
void wem_row(const Problem<R>& P, const Core<R>& core, const std::vector<C<R>>& r, int is, int f,
             DataF<R>& D, int bin_col, std::vector<C<R>>& W, Work<R>& wk, const Inject<R>* src_ov = nullptr,
             const Inject<R>* rec_ov = nullptr) {
  const int nx = core.nxg, nz = core.nz;
  R w = Core<R>::omega(P.F.freq[f]);
  std::fill(W.begin(), W.end(), C<R>(0));
  C<R> wv = P.wave_f[P.F.bin[f]];
  spread_source(P, is, src_ov, W.data(), nx, wv);
  down_fwd(core, w, W.data(), W.data(), true, wk);
  Inject<R> rec = rec_ov ? *rec_ov : P.rec_inj();
  std::vector<C<R>> vals(rec.ix.size());
  auto record = [&]() {
    for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin_col);
    rec.gather(W.data(), nx, vals.data());
    for (size_t i = 0; i < vals.size(); ++i) *D.at(is, (int)i, bin_col) = vals[i];
  };
  record();
  for (size_t i = 0; i < W.size(); ++i) W[i] = r[i] * W[i];
  up_fwd(core, w, W.data(), W.data(), true, wk);
  record();
  (void)nz;
}

// data in/out helpers shared by all drivers
template <class R>
DataF<R> new_dataf(const Problem<R>& P) {
  DataF<R> D;
  D.ns = P.p.ns; D.nr = P.p.nr; D.nb = P.F.nt_pad;
  D.v.assign((size_t)D.ns * D.nr * D.nb, C<R>(0));
  return D;
}

template <class R>
void emit_data(const Problem<R>& P, DataF<R>& D, void* data, int kind, bool add, int nthreads) {
  if (kind == WEM_DATA_TIME) {
    bins_to_time(P, D.v, (float*)data, add, nthreads);
  } else {
    float* o = (float*)data;
    for (int is = 0; is < D.ns; ++is)
      for (int ir = 0; ir < D.nr; ++ir)
        for (int b = 0; b < P.nbin; ++b) {
          size_t k = (((size_t)is * D.nr + ir) * P.nbin + b) * 2;
          C<R> v = b < D.nb ? *D.at(is, ir, b) : C<R>(0);
          if (add) { o[k] += (float)v.real(); o[k + 1] += (float)v.imag(); }
          else { o[k] = (float)v.real(); o[k + 1] = (float)v.imag(); }
        }
  }
}

template <class R>
DataF<R> absorb_data(const Problem<R>& P, const void* data, int kind, int nthreads) {
  DataF<R> D = new_dataf(P);
  if (kind == WEM_DATA_TIME) {
    D.v = time_to_bins(P, (const float*)data, nthreads);
  } else {
    const float* s = (const float*)data;
    for (int is = 0; is < D.ns; ++is)
      for (int ir = 0; ir < D.nr; ++ir)
        for (int b = 0; b < std::min(P.nbin, D.nb); ++b) {
          size_t k = (((size_t)is * D.nr + ir) * P.nbin + b) * 2;
          *D.at(is, ir, b) = C<R>((R)s[k], (R)s[k + 1]);
        }
  }
  return D;
}

template <class R>
void wem_forward(const wem_params& p, const float* wavelet, const float* s2, const float* rho,
                 void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz;
  std::vector<C<R>> s = load<R>(s2, (size_t)p.nx * nz), d = load<R>(rho, (size_t)p.nx * nz);
  std::vector<C<R>> sp((size_t)nx * nz), dp((size_t)nx * nz);
  pad_x(s.data(), sp.data(), nz, p.nx, p.pad, true);
  pad_x(d.data(), dp.data(), nz, p.nx, p.pad, true);
  std::vector<C<R>> r = reflect_coefs(sp.data(), dp.data(), nx, nz);
  Core<R> core(p, sp.data(), nx, nz);
  DataF<R> D = new_dataf(P);
  int nf = P.nfreq(), ns = p.ns;
  parallel_for(ns * nf, nthreads, [&](int t, int) {
    int is = t / nf, f = t % nf;
    Work<R> wk(core.N, nx);
    std::vector<C<R>> W((size_t)nx * nz);
    wem_row(P, core, r, is, f, D, P.F.bin[f], W, wk);
  });
  emit_data(P, D, data, kind, add, nthreads);
}

// -------------------------------------------------------------- Born
// One shot/frequency-range task state (born_prop.cpp:11-235).
template <class R>
struct BornBg {
  std::vector<C<R>> sp, dp, r;  // padded background and reflection coefficients
  Core<R>* core = nullptr;
  DRefl<R>* drefl = nullptr;
};

template <class R>
void born_row_fwd(const Problem<R>& P, const Core<R>& core, const std::vector<C<R>>& r, const DRefl<R>& dR,
                  const std::vector<C<R>>& gm0, const std::vector<C<R>>& gm1, int is, int f, DataF<R>& D,
                  std::vector<C<R>>& bg, std::vector<C<R>>& sc, std::vector<C<R>>& dr, Work<R>& wk,
                  const Inject<R>* src_ov = nullptr, const Inject<R>* rec_ov = nullptr) {
  const int nx = core.nxg;
  const int bin = P.F.bin[f];
  R w = Core<R>::omega(P.F.freq[f]);
  Inject<R> rec = rec_ov ? *rec_ov : P.rec_inj();
  std::vector<C<R>> vals(rec.ix.size());
  auto record = [&](const std::vector<C<R>>& W) {
    for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin);
    rec.gather(W.data(), nx, vals.data());
    for (size_t i = 0; i < vals.size(); ++i) *D.at(is, (int)i, bin) = vals[i];
  };
  // down background wavefield
  std::fill(bg.begin(), bg.end(), C<R>(0));
  C<R> wv = P.wave_f[bin];
  spread_source(P, is, src_ov, bg.data(), nx, wv);
  down_fwd(core, w, bg.data(), bg.data(), true, wk);
  // forward scattering
  lindown_fwd(core, w, bg.data(), gm0.data(), sc.data(), false, wk);
  down_fwd(core, w, sc.data(), sc.data(), true, wk);
  record(sc);
  // linearisation of the reflectivity: Born_refl::forward (Born_refl.cpp:19-27)
  std::fill(dr.begin(), dr.end(), C<R>(0));
  dR.fwd(gm0.data(), gm1.data(), dr.data());
  for (size_t i = 0; i < sc.size(); ++i) sc[i] = bg[i] * dr[i];
  up_fwd(core, w, sc.data(), sc.data(), true, wk);
  record(sc);
  // down-scattering
  lindown_fwd(core, w, bg.data(), gm0.data(), sc.data(), false, wk);
  down_fwd(core, w, sc.data(), sc.data(), true, wk);
  for (size_t i = 0; i < sc.size(); ++i) sc[i] = r[i] * sc[i];
  up_fwd(core, w, sc.data(), sc.data(), true, wk);
  record(sc);
  // up background wavefield
  for (size_t i = 0; i < bg.size(); ++i) bg[i] = r[i] * bg[i];
  up_fwd(core, w, bg.data(), bg.data(), true, wk);
  // up-scattering
  linup_fwd(core, w, bg.data(), gm0.data(), sc.data(), false, wk);
  up_fwd(core, w, sc.data(), sc.data(), true, wk);
  record(sc);
}

template <class R>
void born_row_adj(const Problem<R>& P, const Core<R>& core, const std::vector<C<R>>& r, const DRefl<R>& dR,
                  std::vector<C<R>>& gm0, std::vector<C<R>>& gm1, int is, int f, DataF<R>& D, bool exact,
                  bool ext_order, std::vector<C<R>>& bg, std::vector<C<R>>& sc, std::vector<C<R>>& dr,
                  Work<R>& wk, const Inject<R>* src_ov = nullptr, const Inject<R>* rec_ov = nullptr) {
  const int nx = core.nxg;
  const int bin = P.F.bin[f];
  R w = Core<R>::omega(P.F.freq[f]);
  Inject<R> rec = rec_ov ? *rec_ov : P.rec_inj();
  std::vector<C<R>> vals(rec.ix.size());
  auto inject_data = [&]() {  // Injection::forward 3D, add = 0
    std::fill(sc.begin(), sc.end(), C<R>(0));
    for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin);
    rec.spread(sc.data(), nx, vals.data());
  };
  auto born_refl_adj = [&]() {  // Born_refl::adjoint (Born_refl.cpp:29-40)
    inject_data();
    up_adj(core, w, sc.data(), sc.data(), true, wk);
    for (size_t i = 0; i < sc.size(); ++i) dr[i] = std::conj(bg[i]) * sc[i];
    dR.adj(gm0.data(), gm1.data(), dr.data());
  };
  auto fwd_scatter_adj = [&]() {
    inject_data();
    down_adj(core, w, sc.data(), sc.data(), true, wk);
    lindown_adj(core, w, bg.data(), gm0.data(), sc.data(), true, exact, wk);
  };
  std::fill(bg.begin(), bg.end(), C<R>(0));
  C<R> wv = P.wave_f[bin];
  spread_source(P, is, src_ov, bg.data(), nx, wv);
  down_fwd(core, w, bg.data(), bg.data(), true, wk);
  // born_prop.cpp:193-199 reflectivity first; ext_born_prop.cpp:159-165 the
  // forward-scattering term first
  if (ext_order) { fwd_scatter_adj(); born_refl_adj(); }
  else { born_refl_adj(); fwd_scatter_adj(); }
  // down-scattering
  inject_data();
  up_adj(core, w, sc.data(), sc.data(), true, wk);
  for (size_t i = 0; i < sc.size(); ++i) sc[i] = std::conj(r[i]) * sc[i];
  down_adj(core, w, sc.data(), sc.data(), true, wk);
  lindown_adj(core, w, bg.data(), gm0.data(), sc.data(), true, exact, wk);
  // up background wavefield
  for (size_t i = 0; i < bg.size(); ++i) bg[i] = r[i] * bg[i];
  up_fwd(core, w, bg.data(), bg.data(), true, wk);
  // up-scattering
  inject_data();
  up_adj(core, w, sc.data(), sc.data(), true, wk);
  linup_adj(core, w, bg.data(), gm0.data(), sc.data(), true, exact, wk);
}

template <class R>
struct PaddedModel {
  std::vector<C<R>> s, d;
  PaddedModel(const wem_params& p, const float* s2, const float* rho, bool extend, size_t nslices = 1) {
    int nxg = p.nx + 2 * p.pad;
    size_t n = (size_t)p.nx * p.nz, ng = (size_t)nxg * p.nz;
    s.resize(ng * nslices); d.resize(ng * nslices);
    for (size_t k = 0; k < nslices; ++k) {
      std::vector<C<R>> a = load<R>(s2 + 2 * n * k, n), b = load<R>(rho + 2 * n * k, n);
      pad_x(a.data(), s.data() + ng * k, p.nz, p.nx, p.pad, extend);
      pad_x(b.data(), d.data() + ng * k, p.nz, p.nx, p.pad, extend);
    }
  }
};

template <class R>
void born_forward(const wem_params& p, const float* wavelet, const float* bs2, const float* brho,
                  const float* ds2, const float* drho, void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz;
  PaddedModel<R> bgm(p, bs2, brho, true), dm(p, ds2, drho, false);
  std::vector<C<R>> r = reflect_coefs(bgm.s.data(), bgm.d.data(), nx, nz);
  DRefl<R> dR(bgm.s.data(), bgm.d.data(), nx, nz);
  Core<R> core(p, bgm.s.data(), nx, nz);
  DataF<R> D = new_dataf(P);
  int nf = P.nfreq(), ns = p.ns;
  parallel_for(ns * nf, nthreads, [&](int t, int) {
    int is = t / nf, f = t % nf;
    Work<R> wk(core.N, nx);
    std::vector<C<R>> bg((size_t)nx * nz), sc((size_t)nx * nz), dr((size_t)nx * nz);
    born_row_fwd(P, core, r, dR, dm.s, dm.d, is, f, D, bg, sc, dr, wk);
  });
  emit_data(P, D, data, kind, add, nthreads);
}

// fchunks: tasks per shot over the frequency axis.  1 reproduces the
// compat semantics exactly (the shot's frequencies in order in one task);
// more chunks only change the last depth row of the compat gradient.
template <class R>
void born_adjoint(const wem_params& p, const float* wavelet, const float* bs2, const float* brho,
                  float* ds2, float* drho, const void* data, int kind, bool add, int nthreads, int fchunks) {
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz;
  const bool exact = p.adjoint_mode == WEM_ADJ_EXACT;
  PaddedModel<R> bgm(p, bs2, brho, true);
  std::vector<C<R>> r = reflect_coefs(bgm.s.data(), bgm.d.data(), nx, nz);
  DRefl<R> dR(bgm.s.data(), bgm.d.data(), nx, nz);
  Core<R> core(p, bgm.s.data(), nx, nz);
  DataF<R> D = absorb_data(P, data, kind, nthreads);
  int nf = P.nfreq(), ns = p.ns;
  fchunks = std::max(1, std::min(fchunks, nf));
  int ntask = ns * fchunks;
  size_t ng = (size_t)nx * nz;
  std::vector<std::vector<C<R>>> g0(ntask), g1(ntask);
  parallel_for(ntask, nthreads, [&](int t, int) {
    int is = t / fchunks, ch = t % fchunks;
    int fb = (int)((long long)nf * ch / fchunks), fe = (int)((long long)nf * (ch + 1) / fchunks);
    Work<R> wk(core.N, nx);
    std::vector<C<R>> bg(ng), sc(ng), dr(ng);
    g0[t].assign(ng, C<R>(0));
    g1[t].assign(ng, C<R>(0));
    for (int f = fb; f < fe; ++f)
      born_row_adj(P, core, r, dR, g0[t], g1[t], is, f, D, exact, false, bg, sc, dr, wk);
  });
  // unpad (Pad::adjoint, Pad.h:98-107) and sum the tasks in order: the
  // reference adds them without a lock (born_prop.cpp:220-232)
  size_t nm = (size_t)p.nx * nz;
  std::vector<C<R>> m0(nm, 0), m1(nm, 0);
  for (int t = 0; t < ntask; ++t)
    for (int iz = 0; iz < nz; ++iz)
      for (int ix = 0; ix < p.nx; ++ix) {
        m0[(size_t)iz * p.nx + ix] += g0[t][(size_t)iz * nx + ix + p.pad];
        m1[(size_t)iz * p.nx + ix] += g1[t][(size_t)iz * nx + ix + p.pad];
      }
  store(ds2, m0.data(), nm, add);
  store(drho, m1.data(), nm, add);
}

// ------------------------------------------------------- conformal maps
// One shot of a cmap operator: its chain of maps, the shot's parameters on
// the mapped grid, its devices there, and the mapped background
// (wem_prop.cpp:19-45, born_prop.cpp:28-70).
template <class R>
struct CmapShot {
  cm::ShotChain chain;
  wem_params ps{};
  Inject<R> src, rec;
  std::vector<C<R>> sp, dp, r;
  std::unique_ptr<Core<R>> core;
  std::unique_ptr<DRefl<R>> drefl;
};

template <class R>
void cmap_shot_setup(const Problem<R>& P, int is, const float* s2, const float* rho, bool born, CmapShot<R>& S) {
  const wem_params& p = P.p;
  check(p.cmap == 1 || p.cmap == 2, "cmap must be 0, 1 or 2");
  check(p.cmap != 2 || p.cmap_angles != nullptr, "cmap 2 needs cmap_angles");
  check(p.cmap != 1 || p.nr >= 2, "cmap 1 needs at least 2 receivers");
  const cm::Hyper model{p.nx, p.nz, p.ox, p.dx, p.oz, p.dz};
  S.chain = cm::shot_chain(p.cmap, model, P.src.iz[is], P.src.ix[is], p.eps_log,
                           p.cmap == 2 ? p.cmap_angles[is] : 0.f);
  const cm::Hyper& h = S.chain.out();
  S.ps = p;
  S.ps.ns = 1;
  S.ps.cmap = 0;
  S.ps.ox = h.o1;
  S.ps.dx = h.d1;
  S.ps.oz = h.o2;
  S.ps.dz = h.d2;
  // devices on the mapped grid
  std::vector<int> sz, sx, rz, rx;
  S.chain.points({P.src.iz[is]}, {P.src.ix[is]}, sz, sx);
  S.chain.points(P.rec.iz, P.rec.ix, rz, rx);
  for (size_t i = 0; i < rz.size(); ++i)
    check(rz[i] >= 0 && rz[i] < h.n2 && rx[i] >= 0 && rx[i] < h.n1, "cmap: a receiver maps outside the grid");
  for (size_t i = 1; i < sz.size(); ++i) check(sz[i] == sz[0], "cmap: source points of a shot at several depths");
  S.src = Inject<R>(sx, sz, p.ngs, p.pad);
  S.rec = Inject<R>(rx, rz, p.ngr, p.pad);
  // background: mapped, edge padded; Reflect from it; then the Jacobian,
  // twice, by flat index of the padded grid; the rest sees the scaled grid
  const size_t n = (size_t)p.nx * p.nz;
  std::vector<C<R>> ms = S.chain.forward(load<R>(s2, n)), mr = S.chain.forward(load<R>(rho, n));
  const int nxg = P.nxg;
  S.sp.assign((size_t)nxg * p.nz, C<R>(0));
  S.dp.assign((size_t)nxg * p.nz, C<R>(0));
  pad_x(ms.data(), S.sp.data(), p.nz, p.nx, p.pad, true);
  pad_x(mr.data(), S.dp.data(), p.nz, p.nx, p.pad, true);
  S.r = reflect_coefs(S.sp.data(), S.dp.data(), nxg, p.nz);
  S.chain.scale_by_jacobian(S.sp.data());
  S.chain.scale_by_jacobian(S.sp.data());
  S.core = std::make_unique<Core<R>>(S.ps, S.sp.data(), nxg, p.nz);
  if (born) S.drefl = std::make_unique<DRefl<R>>(S.sp.data(), S.dp.data(), nxg, p.nz);
}

// a perturbation on the shot's mapped grid, zero padded (born_prop.cpp:50-57)
template <class R>
std::vector<C<R>> cmap_perturbation(const Problem<R>& P, const CmapShot<R>& S, const float* m) {
  const wem_params& p = P.p;
  std::vector<C<R>> mm = S.chain.forward(load<R>(m, (size_t)p.nx * p.nz));
  std::vector<C<R>> out((size_t)P.nxg * p.nz, C<R>(0));
  pad_x(mm.data(), out.data(), p.nz, p.nx, p.pad, false);
  return out;
}

template <class R>
void cmap_wem_forward(const wem_params& p, const float* wavelet, const float* s2, const float* rho, void* data,
                      int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  DataF<R> D = new_dataf(P);
  const int nf = P.nfreq();
  parallel_for(p.ns, nthreads, [&](int is, int) {
    CmapShot<R> S;
    cmap_shot_setup(P, is, s2, rho, false, S);
    Work<R> wk(S.core->N, P.nxg);
    std::vector<C<R>> W((size_t)P.nxg * p.nz);
    for (int f = 0; f < nf; ++f) wem_row(P, *S.core, S.r, is, f, D, P.F.bin[f], W, wk, &S.src, &S.rec);
  });
  emit_data(P, D, data, kind, add, nthreads);
}

template <class R>
void cmap_born_forward(const wem_params& p, const float* wavelet, const float* bs2, const float* brho,
                       const float* ds2, const float* drho, void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  DataF<R> D = new_dataf(P);
  const int nf = P.nfreq();
  const size_t ng = (size_t)P.nxg * p.nz;
  parallel_for(p.ns, nthreads, [&](int is, int) {
    CmapShot<R> S;
    cmap_shot_setup(P, is, bs2, brho, true, S);
    std::vector<C<R>> gm0 = cmap_perturbation(P, S, ds2), gm1 = cmap_perturbation(P, S, drho);
    Work<R> wk(S.core->N, P.nxg);
    std::vector<C<R>> bg(ng), sc(ng), dr(ng);
    for (int f = 0; f < nf; ++f)
      born_row_fwd(P, *S.core, S.r, *S.drefl, gm0, gm1, is, f, D, bg, sc, dr, wk, &S.src, &S.rec);
  });
  emit_data(P, D, data, kind, add, nthreads);
}

// every shot's gradient, unpadded on its mapped grid, comes back through the
// inverse map and the shots are summed in order (born_prop.cpp:217-232)
template <class R>
void cmap_born_adjoint(const wem_params& p, const float* wavelet, const float* bs2, const float* brho, float* ds2,
                       float* drho, const void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  DataF<R> D = absorb_data(P, data, kind, nthreads);
  const bool exact = p.adjoint_mode == WEM_ADJ_EXACT;
  const int nf = P.nfreq(), nx = P.nxg, nz = p.nz;
  const size_t ng = (size_t)nx * nz, nm = (size_t)p.nx * nz;
  std::vector<std::vector<C<R>>> back0(p.ns), back1(p.ns);
  parallel_for(p.ns, nthreads, [&](int is, int) {
    CmapShot<R> S;
    cmap_shot_setup(P, is, bs2, brho, true, S);
    Work<R> wk(S.core->N, nx);
    std::vector<C<R>> bg(ng), sc(ng), dr(ng), g0(ng, C<R>(0)), g1(ng, C<R>(0));
    for (int f = 0; f < nf; ++f)
      born_row_adj(P, *S.core, S.r, *S.drefl, g0, g1, is, f, D, exact, false, bg, sc, dr, wk, &S.src, &S.rec);
    std::vector<C<R>> m0(nm), m1(nm);
    for (int iz = 0; iz < nz; ++iz)
      for (int ix = 0; ix < p.nx; ++ix) {
        m0[(size_t)iz * p.nx + ix] = g0[(size_t)iz * nx + ix + p.pad];
        m1[(size_t)iz * p.nx + ix] = g1[(size_t)iz * nx + ix + p.pad];
      }
    back0[is] = S.chain.inverse(m0);
    back1[is] = S.chain.inverse(m1);
  });
  std::vector<C<R>> t0(nm, C<R>(0)), t1(nm, C<R>(0));
  for (int is = 0; is < p.ns; ++is)
    for (size_t i = 0; i < nm; ++i) {
      t0[i] += back0[is][i];
      t1[i] += back1[is][i];
    }
  store(ds2, t0.data(), nm, add);
  store(drho, t1.data(), nm, add);
}

// --------------------------------------------------- frequency-extended
// extWEM::full_fwd (ext_wem_prop.cpp:8-59): one model slice per frequency.
template <class R>
void extwem_forward(const wem_params& p, const float* wavelet, const float* s2, const float* rho,
                    void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  PaddedModel<R> m(p, s2, rho, true, nf);
  size_t ng = (size_t)nx * nz;
  DataF<R> D = new_dataf(P);
  parallel_for(nf, nthreads, [&](int f, int) {
    const C<R>* sp = m.s.data() + ng * f;
    const C<R>* dp = m.d.data() + ng * f;
    Core<R> core(p, sp, nx, nz);
    std::vector<C<R>> r = reflect_coefs(sp, dp, nx, nz);
    Work<R> wk(core.N, nx);
    std::vector<C<R>> W(ng);
    for (int is = 0; is < p.ns; ++is) wem_row(P, core, r, is, f, D, P.F.bin[f], W, wk);
  });
  emit_data(P, D, data, kind, add, nthreads);
}

template <class R>
void extborn_forward(const wem_params& p, const float* wavelet, const float* bs2, const float* brho,
                     const float* ds2, const float* drho, void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  PaddedModel<R> bgm(p, bs2, brho, true, nf), dm(p, ds2, drho, false, nf);
  size_t ng = (size_t)nx * nz;
  DataF<R> D = new_dataf(P);
  parallel_for(nf, nthreads, [&](int f, int) {
    const C<R>* sp = bgm.s.data() + ng * f;
    const C<R>* dp = bgm.d.data() + ng * f;
    Core<R> core(p, sp, nx, nz);
    std::vector<C<R>> r = reflect_coefs(sp, dp, nx, nz);
    DRefl<R> dR(sp, dp, nx, nz);
    std::vector<C<R>> g0(dm.s.begin() + ng * f, dm.s.begin() + ng * (f + 1));
    std::vector<C<R>> g1(dm.d.begin() + ng * f, dm.d.begin() + ng * (f + 1));
    Work<R> wk(core.N, nx);
    std::vector<C<R>> bg(ng), sc(ng), dr(ng);
    for (int is = 0; is < p.ns; ++is) born_row_fwd(P, core, r, dR, g0, g1, is, f, D, bg, sc, dr, wk);
  });
  emit_data(P, D, data, kind, add, nthreads);
}

template <class R>
void extborn_adjoint(const wem_params& p, const float* wavelet, const float* bs2, const float* brho,
                     float* ds2, float* drho, const void* data, int kind, bool add, int nthreads) {
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  const bool exact = p.adjoint_mode == WEM_ADJ_EXACT;
  PaddedModel<R> bgm(p, bs2, brho, true, nf);
  size_t ng = (size_t)nx * nz, nm = (size_t)p.nx * nz;
  DataF<R> D = absorb_data(P, data, kind, nthreads);
  std::vector<C<R>> m0(nm * nf), m1(nm * nf);
  parallel_for(nf, nthreads, [&](int f, int) {
    const C<R>* sp = bgm.s.data() + ng * f;
    const C<R>* dp = bgm.d.data() + ng * f;
    Core<R> core(p, sp, nx, nz);
    std::vector<C<R>> r = reflect_coefs(sp, dp, nx, nz);
    DRefl<R> dR(sp, dp, nx, nz);
    std::vector<C<R>> g0(ng, 0), g1(ng, 0);
    Work<R> wk(core.N, nx);
    std::vector<C<R>> bg(ng), sc(ng), dr(ng);
    for (int is = 0; is < p.ns; ++is) born_row_adj(P, core, r, dR, g0, g1, is, f, D, exact, true, bg, sc, dr, wk);
    for (int iz = 0; iz < nz; ++iz)
      for (int ix = 0; ix < p.nx; ++ix) {
        m0[nm * f + (size_t)iz * p.nx + ix] = g0[(size_t)iz * nx + ix + p.pad];
        m1[nm * f + (size_t)iz * p.nx + ix] = g1[(size_t)iz * nx + ix + p.pad];
      }
  });
  store(ds2, m0.data(), nm * nf, add);
  store(drho, m1.data(), nm * nf, add);
}

// ------------------------------------------- BornRefl / BornTomo (f3)
// One complex field [slices][nz][nx] padded to [slices][nz][nxg].
template <class R>
std::vector<C<R>> pad_field(const wem_params& p, const float* a, int slices, bool extend) {
  const int nxg = p.nx + 2 * p.pad;
  const size_t n = (size_t)p.nx * p.nz, ng = (size_t)nxg * p.nz;
  std::vector<C<R>> out(ng * slices);
  for (int k = 0; k < slices; ++k) {
    std::vector<C<R>> v = load<R>(a + 2 * n * k, n);
    pad_x(v.data(), out.data() + ng * k, p.nz, p.nx, p.pad, extend);
  }
  return out;
}

// BornRefl and BornTomo propagate on the model grid itself
// (ext_born_refl.cpp:18-25, ext_born_tomo.cpp:20-25: Down/Up on the unpadded
// slowness): `pad` is only OneStep's taper width (OneStep.h:27-35), the
// source spreads over "ng" cells (here ngs) and the receivers are points
// (Injection's default ng = 0), with no pad offset.  The returned block drives
// the geometry; the caller's block, with its pad, drives Core's taper.
inline wem_params refl_grid(const wem_params& p) {
  check(p.pad != 1, "pad == 1 makes the taper divide by zero (Taper.h:19)");
  wem_params q = p;
  q.pad = 0;
  q.ngr = 0;
  return q;
}

// a block whose `pad` is the taper width `w` (Core reads the taper from it)
inline wem_params with_taper(wem_params p, int w) {
  p.pad = w;
  return p;
}

// BornRefl::fwd_propagate (ext_born_refl.cpp:8-57): per (frequency, shot)
// bg = Down(src); sc = bg m_f (IC::forward); Up in place; record.
template <class R>
void bornrefl_forward(const wem_params& p_in, const float* wavelet, const float* bs2, const float* model, void* data,
                      int kind, bool add, int nthreads) {
  const wem_params p = refl_grid(p_in);
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  std::vector<C<R>> sp = pad_field<R>(p, bs2, 1, true);
  std::vector<C<R>> m = pad_field<R>(p, model, nf, false);
  Core<R> core(p_in, sp.data(), nx, nz);
  DataF<R> D = new_dataf(P);
  const size_t ng = (size_t)nx * nz;
  parallel_for(nf, nthreads, [&](int f, int) {
    const int bin = P.F.bin[f];
    R w = Core<R>::omega(P.F.freq[f]);
    Inject<R> rec = P.rec_inj();
    std::vector<C<R>> vals(rec.ix.size()), bg(ng), sc(ng);
    Work<R> wk(core.N, nx);
    for (int is = 0; is < p.ns; ++is) {
      std::fill(bg.begin(), bg.end(), C<R>(0));
      C<R> wv = P.wave_f[bin];
      P.src_inj(is).spread(bg.data(), nx, &wv);
      down_fwd(core, w, bg.data(), bg.data(), true, wk);
      for (size_t i = 0; i < ng; ++i) sc[i] = bg[i] * m[ng * f + i];
      up_fwd(core, w, sc.data(), sc.data(), true, wk);
      for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin);
      rec.gather(sc.data(), nx, vals.data());
      for (size_t i = 0; i < vals.size(); ++i) *D.at(is, (int)i, bin) = vals[i];
    }
  });
  emit_data(P, D, data, kind, add, nthreads);
}

// BornRefl::adj_propagate (ext_born_refl.cpp:60-105): image_f += conj(bg) Up^H(rec)
template <class R>
void bornrefl_adjoint(const wem_params& p_in, const float* wavelet, const float* bs2, float* model, const void* data,
                      int kind, bool add, int nthreads) {
  const wem_params p = refl_grid(p_in);
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  std::vector<C<R>> sp = pad_field<R>(p, bs2, 1, true);
  Core<R> core(p_in, sp.data(), nx, nz);
  DataF<R> D = absorb_data(P, data, kind, nthreads);
  const size_t ng = (size_t)nx * nz, nm = (size_t)p.nx * nz;
  std::vector<C<R>> out(nm * nf);
  parallel_for(nf, nthreads, [&](int f, int) {
    const int bin = P.F.bin[f];
    R w = Core<R>::omega(P.F.freq[f]);
    Inject<R> rec = P.rec_inj();
    std::vector<C<R>> vals(rec.ix.size()), bg(ng), sc(ng), img(ng, C<R>(0));
    Work<R> wk(core.N, nx);
    for (int is = 0; is < p.ns; ++is) {
      std::fill(bg.begin(), bg.end(), C<R>(0));
      C<R> wv = P.wave_f[bin];
      P.src_inj(is).spread(bg.data(), nx, &wv);
      down_fwd(core, w, bg.data(), bg.data(), true, wk);
      std::fill(sc.begin(), sc.end(), C<R>(0));
      for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin);
      rec.spread(sc.data(), nx, vals.data());
      up_adj(core, w, sc.data(), sc.data(), true, wk);
      for (size_t i = 0; i < ng; ++i) img[i] += std::conj(bg[i]) * sc[i];
    }
    for (int iz = 0; iz < nz; ++iz)
      for (int ix = 0; ix < p.nx; ++ix) out[nm * f + (size_t)iz * p.nx + ix] = img[(size_t)iz * nx + ix + p.pad];
  });
  store(model, out.data(), nm * nf, add);
}

// ------------------------------- subsurface-offset extended Born (C4)
// No reference counterpart.  Per shot, BornRefl (ext_born_refl.cpp:8-105) on
// the cropped model of the shot's aperture, as WEM.from_subspace builds a
// sub-propagator (propagator/src/python/WEM.py:24-30): the aperture's model
// columns [x0, x0 + w) with BornRefl's conventions (refl_grid: no model pad,
// `pad` the taper width, point receivers), a row of w + 2 tap_s points, its
// own RefSampler; the shot's devices inside the aperture.  The imaging
// condition IC (ic.cpp:5-29) is extended over horizontal lags l = -hm .. hm:
// forward sc(x) = sum_l r_l(x - l) bg(x - 2l), adjoint
// image_l(y) += conj(bg(y - l)) a(y + l), r, bg and a zero off the aperture.
template <class R>
struct Aperture {
  wem_params ps;             // the cropped problem: nx = w, tap = tap_s
  int x0 = 0, w = 0, nxg = 0;
  std::vector<C<R>> sp;      // padded aperture slowness [nz][nxg]
  std::vector<int> rec;      // receivers inside the aperture
  Inject<R> src, recinj;
};

template <class R>
Aperture<R> make_aperture(const Problem<R>& P, const float* bs2, int is, int x0, int w, int tap) {
  const wem_params& p = P.p;
  check(x0 >= 0 && w >= 2 && x0 + w <= p.nx, "aperture outside the model");
  Aperture<R> a;
  a.ps = p;
  a.ps.nx = w;
  a.ps.tap = tap;
  a.x0 = x0;
  a.w = w;
  a.nxg = w + 2 * p.pad;
  std::vector<float> crop((size_t)2 * p.nz * w);
  for (int z = 0; z < p.nz; ++z)
    for (int x = 0; x < w; ++x) {
      crop[2 * ((size_t)z * w + x)] = bs2[2 * ((size_t)z * p.nx + x0 + x)];
      crop[2 * ((size_t)z * w + x) + 1] = bs2[2 * ((size_t)z * p.nx + x0 + x) + 1];
    }
  a.sp = pad_field<R>(a.ps, crop.data(), 1, true);
  const int sx = P.src.ix[is];
  check(sx >= x0 && sx < x0 + w, "source outside its aperture");
  a.src = Inject<R>({sx - x0}, {P.src.iz[is]}, p.ngs, p.pad);
  std::vector<int> ix, iz;
  for (size_t i = 0; i < P.rec.ix.size(); ++i)
    if (P.rec.ix[i] >= x0 && P.rec.ix[i] < x0 + w) {
      a.rec.push_back((int)i);
      ix.push_back(P.rec.ix[i] - x0);
      iz.push_back(P.rec.iz[i]);
    }
  a.recinj = Inject<R>(ix, iz, p.ngr, p.pad);
  return a;
}

template <class R>
void offborn_forward(const wem_params& p_in, const float* wavelet, const float* bs2, int nh, const int* ax0,
                     const int* aw, const int* atap, const float* model, void* data, int kind, bool add,
                     int nthreads) {
  const wem_params p = refl_grid(p_in);
  check(nh >= 1 && nh % 2 == 1, "nh must be odd");
  check(p.nref == 1, "one reference slowness");
  Problem<R> P(p, wavelet);
  const int nz = p.nz, nf = P.nfreq(), hm = (nh - 1) / 2;
  const size_t nm = (size_t)p.nx * nz;
  std::vector<C<R>> r = load<R>(model, nm * nh);
  DataF<R> D = new_dataf(P);
  for (int is = 0; is < p.ns; ++is) {
    Aperture<R> A = make_aperture(P, bs2, is, ax0[is], aw[is], atap[is]);
    const int nxg = A.nxg;
    Core<R> core(with_taper(A.ps, p_in.pad), A.sp.data(), nxg, nz);
    const size_t ng = (size_t)nxg * nz;
    parallel_for(nf, nthreads, [&](int f, int) {
      const int bin = P.F.bin[f];
      const R w = Core<R>::omega(P.F.freq[f]);
      std::vector<C<R>> bg(ng, C<R>(0)), sc(ng, C<R>(0)), vals(A.rec.size(), C<R>(0));
      Work<R> wk(core.N, nxg);
      C<R> wv = P.wave_f[bin];
      A.src.spread(bg.data(), nxg, &wv);
      down_fwd(core, w, bg.data(), bg.data(), true, wk);
      for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nxg; ++x) {
          C<R> acc(0);
          for (int l = -hm; l <= hm; ++l) {
            const int y = x - l, xb = x - 2 * l;
            if (y < p.pad || y >= p.pad + A.w || xb < 0 || xb >= nxg) continue;
            acc += r[(size_t)(l + hm) * nm + (size_t)z * p.nx + A.x0 + y - p.pad] * bg[(size_t)z * nxg + xb];
          }
          sc[(size_t)z * nxg + x] = acc;
        }
      up_fwd(core, w, sc.data(), sc.data(), true, wk);
      A.recinj.gather(sc.data(), nxg, vals.data());
      for (size_t i = 0; i < vals.size(); ++i) *D.at(is, A.rec[i], bin) += vals[i];
    });
  }
  emit_data(P, D, data, kind, add, nthreads);
}

template <class R>
void offborn_adjoint(const wem_params& p_in, const float* wavelet, const float* bs2, int nh, const int* ax0,
                     const int* aw, const int* atap, float* model, const void* data, int kind, bool add,
                     int nthreads) {
  const wem_params p = refl_grid(p_in);
  check(nh >= 1 && nh % 2 == 1, "nh must be odd");
  check(p.nref == 1, "one reference slowness");
  Problem<R> P(p, wavelet);
  const int nz = p.nz, nf = P.nfreq(), hm = (nh - 1) / 2;
  const size_t nm = (size_t)p.nx * nz;
  DataF<R> D = absorb_data(P, data, kind, nthreads);
  // per-frequency images, summed in frequency order at the end
  std::vector<std::vector<C<R>>> img(nf, std::vector<C<R>>(nm * nh, C<R>(0)));
  for (int is = 0; is < p.ns; ++is) {
    Aperture<R> A = make_aperture(P, bs2, is, ax0[is], aw[is], atap[is]);
    const int nxg = A.nxg;
    Core<R> core(with_taper(A.ps, p_in.pad), A.sp.data(), nxg, nz);
    const size_t ng = (size_t)nxg * nz;
    parallel_for(nf, nthreads, [&](int f, int) {
      const int bin = P.F.bin[f];
      const R w = Core<R>::omega(P.F.freq[f]);
      std::vector<C<R>> bg(ng, C<R>(0)), a(ng, C<R>(0)), vals(A.rec.size());
      Work<R> wk(core.N, nxg);
      C<R> wv = P.wave_f[bin];
      A.src.spread(bg.data(), nxg, &wv);
      down_fwd(core, w, bg.data(), bg.data(), true, wk);
      for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, A.rec[i], bin);
      A.recinj.spread(a.data(), nxg, vals.data());
      up_adj(core, w, a.data(), a.data(), true, wk);
      std::vector<C<R>>& I = img[f];
      for (int z = 0; z < nz; ++z)
        for (int y = p.pad; y < p.pad + A.w; ++y)
          for (int l = -hm; l <= hm; ++l) {
            const int yb = y - l, ya = y + l;
            if (yb < 0 || yb >= nxg || ya < 0 || ya >= nxg) continue;
            I[(size_t)(l + hm) * nm + (size_t)z * p.nx + A.x0 + y - p.pad] +=
                std::conj(bg[(size_t)z * nxg + yb]) * a[(size_t)z * nxg + ya];
          }
    });
  }
  std::vector<C<R>> out(nm * nh, C<R>(0));
  for (int f = 0; f < nf; ++f)
    for (size_t i = 0; i < out.size(); ++i) out[i] += img[f][i];
  store(model, out.data(), out.size(), add);
}

// BornTomo::fwd_propagate (ext_born_tomo.cpp:9-57): Born_down (LinDown,
// Down, reflectivity, Up, record; Born_down.cpp:14-27) and Born_up on the
// up background Up(refl_f bg) (Born_up.cpp:14-22)
template <class R>
void borntomo_forward(const wem_params& p_in, const float* wavelet, const float* bs2, const float* refl,
                      const float* dm, void* data, int kind, bool add, int nthreads) {
  const wem_params p = refl_grid(p_in);
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  std::vector<C<R>> sp = pad_field<R>(p, bs2, 1, true);
  std::vector<C<R>> rf = pad_field<R>(p, refl, nf, true);
  std::vector<C<R>> g = pad_field<R>(p, dm, 1, false);
  Core<R> core(p_in, sp.data(), nx, nz);
  DataF<R> D = new_dataf(P);
  const size_t ng = (size_t)nx * nz;
  parallel_for(nf, nthreads, [&](int f, int) {
    const int bin = P.F.bin[f];
    R w = Core<R>::omega(P.F.freq[f]);
    Inject<R> rec = P.rec_inj();
    std::vector<C<R>> vals(rec.ix.size()), bg(ng), sc(ng);
    const C<R>* r = rf.data() + ng * f;
    Work<R> wk(core.N, nx);
    auto record = [&](int is) {
      for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin);
      rec.gather(sc.data(), nx, vals.data());
      for (size_t i = 0; i < vals.size(); ++i) *D.at(is, (int)i, bin) = vals[i];
    };
    for (int is = 0; is < p.ns; ++is) {
      std::fill(bg.begin(), bg.end(), C<R>(0));
      C<R> wv = P.wave_f[bin];
      P.src_inj(is).spread(bg.data(), nx, &wv);
      down_fwd(core, w, bg.data(), bg.data(), true, wk);
      lindown_fwd(core, w, bg.data(), g.data(), sc.data(), false, wk);
      down_fwd(core, w, sc.data(), sc.data(), true, wk);
      for (size_t i = 0; i < ng; ++i) sc[i] = r[i] * sc[i];
      up_fwd(core, w, sc.data(), sc.data(), true, wk);
      record(is);
      for (size_t i = 0; i < ng; ++i) bg[i] = r[i] * bg[i];
      up_fwd(core, w, bg.data(), bg.data(), true, wk);
      linup_fwd(core, w, bg.data(), g.data(), sc.data(), false, wk);
      up_fwd(core, w, sc.data(), sc.data(), true, wk);
      record(is);
    }
  });
  emit_data(P, D, data, kind, add, nthreads);
}

// BornTomo::adj_propagate (ext_born_tomo.cpp:62-119).  All (frequency, shot)
// terms add into one model.  As coded, every LinDown^H zeroes that model's
// last depth row (LinOneWay.cpp:64-65): in the reference's order (frequencies,
// then shots) the row ends with the LinUp^H term of the last (f, s) alone, so
// the as-coded mode runs the terms in that order in one task.
template <class R>
void borntomo_adjoint(const wem_params& p_in, const float* wavelet, const float* bs2, const float* refl, float* dm,
                      const void* data, int kind, bool add, int nthreads) {
  const wem_params p = refl_grid(p_in);
  Problem<R> P(p, wavelet);
  const int nx = P.nxg, nz = p.nz, nf = P.nfreq();
  const bool exact = p.adjoint_mode == WEM_ADJ_EXACT;
  std::vector<C<R>> sp = pad_field<R>(p, bs2, 1, true);
  std::vector<C<R>> rf = pad_field<R>(p, refl, nf, true);
  Core<R> core(p_in, sp.data(), nx, nz);
  DataF<R> D = absorb_data(P, data, kind, nthreads);
  const size_t ng = (size_t)nx * nz, nm = (size_t)p.nx * nz;
  const int ntask = exact ? nf : 1;
  std::vector<std::vector<C<R>>> part(ntask, std::vector<C<R>>(ng, C<R>(0)));
  parallel_for(ntask, nthreads, [&](int t, int) {
    const int fb = exact ? t : 0, fe = exact ? t + 1 : nf;
    Inject<R> rec = P.rec_inj();
    std::vector<C<R>> vals(rec.ix.size()), bg(ng), sc(ng);
    std::vector<C<R>>& M = part[t];
    Work<R> wk(core.N, nx);
    for (int f = fb; f < fe; ++f) {
      const int bin = P.F.bin[f];
      R w = Core<R>::omega(P.F.freq[f]);
      const C<R>* r = rf.data() + ng * f;
      auto inject_data = [&](int is) {
        std::fill(sc.begin(), sc.end(), C<R>(0));
        for (size_t i = 0; i < vals.size(); ++i) vals[i] = *D.at(is, (int)i, bin);
        rec.spread(sc.data(), nx, vals.data());
      };
      for (int is = 0; is < p.ns; ++is) {
        std::fill(bg.begin(), bg.end(), C<R>(0));
        C<R> wv = P.wave_f[bin];
        P.src_inj(is).spread(bg.data(), nx, &wv);
        down_fwd(core, w, bg.data(), bg.data(), true, wk);
        // Born_down::adjoint (Born_down.cpp:29-41)
        inject_data(is);
        up_adj(core, w, sc.data(), sc.data(), true, wk);
        for (size_t i = 0; i < ng; ++i) sc[i] = std::conj(r[i]) * sc[i];
        down_adj(core, w, sc.data(), sc.data(), true, wk);
        lindown_adj(core, w, bg.data(), M.data(), sc.data(), true, exact, wk);
        // up background, then Born_up::adjoint (Born_up.cpp:24-31)
        for (size_t i = 0; i < ng; ++i) bg[i] = r[i] * bg[i];
        up_fwd(core, w, bg.data(), bg.data(), true, wk);
        inject_data(is);
        up_adj(core, w, sc.data(), sc.data(), true, wk);
        linup_adj(core, w, bg.data(), M.data(), sc.data(), true, exact, wk);
      }
    }
  });
  std::vector<C<R>> out(nm, C<R>(0));
  for (int t = 0; t < ntask; ++t)
    for (int iz = 0; iz < nz; ++iz)
      for (int ix = 0; ix < p.nx; ++ix) out[(size_t)iz * p.nx + ix] += part[t][(size_t)iz * nx + ix + p.pad];
  store(dm, out.data(), nm, add);
}

// ---------------------------------------------------- row-level operators
template <class R>
struct RowOp {
  std::vector<C<R>> s;
  Core<R> core;
  RowOp(const wem_params& p, const float* slow, int nxg)
      : s(load<R>(slow, (size_t)nxg * p.nz)), core(p, s.data(), nxg, p.nz) {}
};

int run_guarded(const std::function<void()>& fn) {
  try {
    fn();
    return WEM_OK;
  } catch (const Error& e) {
    g_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_err = e.what();
    return WEM_EINVAL;
  }
}

}  // namespace
}  // namespace wo

using namespace wo;

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_count_freqs(const wem_params* p, int* nfreq, int* bins, float* freqs) {
  return run_guarded([&] {
    Freqs F = make_freqs(*p);
    *nfreq = (int)F.freq.size();
    if (bins) std::copy(F.bin.begin(), F.bin.end(), bins);
    if (freqs) std::copy(F.freq.begin(), F.freq.end(), freqs);
  });
}

int oracle_devices(const wem_params* p, int* sx, int* sz, int* rx, int* rz) {
  return run_guarded([&] {
    Devices s = make_devices(*p, true), r = make_devices(*p, false);
    std::copy(s.ix.begin(), s.ix.end(), sx);
    std::copy(s.iz.begin(), s.iz.end(), sz);
    std::copy(r.ix.begin(), r.ix.end(), rx);
    std::copy(r.iz.begin(), r.iz.end(), rz);
  });
}

// double-precision transform for checking the FFT against numpy
int oracle_fft(int n, double* x, int sign) {
  return run_guarded([&] {
    Fft<double> f(n);
    std::vector<C<double>> v(n), scr(n);
    for (int i = 0; i < n; ++i) v[i] = C<double>(x[2 * i], x[2 * i + 1]);
    f.run(v.data(), sign, scr.data());
    for (int i = 0; i < n; ++i) { x[2 * i] = v[i].real(); x[2 * i + 1] = v[i].imag(); }
  });
}

int oracle_wem_forward(const wem_params* p, const float* wavelet, const float* s2, const float* rho,
                       void* data, int kind, int add, int prec, int nthreads) {
  return run_guarded([&] {
    if (p->cmap) {
      if (prec == 64) cmap_wem_forward<double>(*p, wavelet, s2, rho, data, kind, add, nthreads);
      else cmap_wem_forward<float>(*p, wavelet, s2, rho, data, kind, add, nthreads);
    } else if (prec == 64) {
      wem_forward<double>(*p, wavelet, s2, rho, data, kind, add, nthreads);
    } else {
      wem_forward<float>(*p, wavelet, s2, rho, data, kind, add, nthreads);
    }
  });
}

int oracle_born_forward(const wem_params* p, const float* wavelet, const float* bs2, const float* brho,
                        const float* ds2, const float* drho, void* data, int kind, int add, int prec,
                        int nthreads) {
  return run_guarded([&] {
    if (p->cmap) {
      if (prec == 64) cmap_born_forward<double>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
      else cmap_born_forward<float>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
    } else if (prec == 64) {
      born_forward<double>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
    } else {
      born_forward<float>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
    }
  });
}

int oracle_born_adjoint(const wem_params* p, const float* wavelet, const float* bs2, const float* brho,
                        float* ds2, float* drho, const void* data, int kind, int add, int prec, int nthreads,
                        int fchunks) {
  return run_guarded([&] {
    if (p->cmap) {
      if (prec == 64) cmap_born_adjoint<double>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
      else cmap_born_adjoint<float>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
    } else if (prec == 64) {
      born_adjoint<double>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads, fchunks);
    } else {
      born_adjoint<float>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads, fchunks);
    }
  });
}

int oracle_extwem_forward(const wem_params* p, const float* wavelet, const float* s2, const float* rho,
                          void* data, int kind, int add, int prec, int nthreads) {
  return run_guarded([&] {
    if (prec == 64) extwem_forward<double>(*p, wavelet, s2, rho, data, kind, add, nthreads);
    else extwem_forward<float>(*p, wavelet, s2, rho, data, kind, add, nthreads);
  });
}

int oracle_extborn_forward(const wem_params* p, const float* wavelet, const float* bs2, const float* brho,
                           const float* ds2, const float* drho, void* data, int kind, int add, int prec,
                           int nthreads) {
  return run_guarded([&] {
    if (prec == 64) extborn_forward<double>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
    else extborn_forward<float>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
  });
}

int oracle_bornrefl_forward(const wem_params* p, const float* wavelet, const float* bs2, const float* model,
                            void* data, int kind, int add, int prec, int nthreads) {
  return run_guarded([&] {
    if (prec == 64) bornrefl_forward<double>(*p, wavelet, bs2, model, data, kind, add, nthreads);
    else bornrefl_forward<float>(*p, wavelet, bs2, model, data, kind, add, nthreads);
  });
}
int oracle_bornrefl_adjoint(const wem_params* p, const float* wavelet, const float* bs2, float* model,
                            const void* data, int kind, int add, int prec, int nthreads) {
  return run_guarded([&] {
    if (prec == 64) bornrefl_adjoint<double>(*p, wavelet, bs2, model, data, kind, add, nthreads);
    else bornrefl_adjoint<float>(*p, wavelet, bs2, model, data, kind, add, nthreads);
  });
}
int oracle_offborn_forward(const wem_params* p, const float* wavelet, const float* bs2, int nh, const int* ax0,
                           const int* aw, const int* atap, const float* model, void* data, int kind, int add, int prec,
                           int nthreads) {
  return run_guarded([&] {
    if (prec == 64) offborn_forward<double>(*p, wavelet, bs2, nh, ax0, aw, atap, model, data, kind, add, nthreads);
    else offborn_forward<float>(*p, wavelet, bs2, nh, ax0, aw, atap, model, data, kind, add, nthreads);
  });
}
int oracle_offborn_adjoint(const wem_params* p, const float* wavelet, const float* bs2, int nh, const int* ax0,
                           const int* aw, const int* atap, float* model, const void* data, int kind, int add, int prec,
                           int nthreads) {
  return run_guarded([&] {
    if (prec == 64) offborn_adjoint<double>(*p, wavelet, bs2, nh, ax0, aw, atap, model, data, kind, add, nthreads);
    else offborn_adjoint<float>(*p, wavelet, bs2, nh, ax0, aw, atap, model, data, kind, add, nthreads);
  });
}
int oracle_borntomo_forward(const wem_params* p, const float* wavelet, const float* bs2, const float* refl,
                            const float* dm, void* data, int kind, int add, int prec, int nthreads) {
  return run_guarded([&] {
    if (prec == 64) borntomo_forward<double>(*p, wavelet, bs2, refl, dm, data, kind, add, nthreads);
    else borntomo_forward<float>(*p, wavelet, bs2, refl, dm, data, kind, add, nthreads);
  });
}
int oracle_borntomo_adjoint(const wem_params* p, const float* wavelet, const float* bs2, const float* refl,
                            float* dm, const void* data, int kind, int add, int prec, int nthreads) {
  return run_guarded([&] {
    if (prec == 64) borntomo_adjoint<double>(*p, wavelet, bs2, refl, dm, data, kind, add, nthreads);
    else borntomo_adjoint<float>(*p, wavelet, bs2, refl, dm, data, kind, add, nthreads);
  });
}

int oracle_extborn_adjoint(const wem_params* p, const float* wavelet, const float* bs2, const float* brho,
                           float* ds2, float* drho, const void* data, int kind, int add, int prec,
                           int nthreads) {
  return run_guarded([&] {
    if (prec == 64) extborn_adjoint<double>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
    else extborn_adjoint<float>(*p, wavelet, bs2, brho, ds2, drho, data, kind, add, nthreads);
  });
}

// ---- row-level operators over a padded slowness [nz][nxg]
extern "C++" {
template <class R>
static void onestep_rows(const wem_params& p, const float* slow, int nxg, int iz, float freq, int adj,
                         const float* in, float* out, int nrow, int add) {
  RowOp<R> op(p, slow, nxg);
  Work<R> wk(op.core.N, nxg);
  R w = Core<R>::omega(freq);
  for (int r = 0; r < nrow; ++r) {
    std::vector<C<R>> a = load<R>(in + 2 * (size_t)r * nxg, nxg), b(nxg, C<R>(0));
    if (add) b = load<R>(out + 2 * (size_t)r * nxg, nxg);
    if (!adj) onestep_fwd(op.core, iz, w, a.data(), b.data(), add != 0, wk);
    else onestep_adj(op.core, iz, w, b.data(), a.data(), add != 0, wk);
    store(out + 2 * (size_t)r * nxg, b.data(), nxg, false);
  }
}
}  // extern "C++"

int oracle_onestep(const wem_params* p, const float* slow, int nxg, int iz, float freq, int adj,
                   const float* in, float* out, int nrow, int add, int prec) {
  return run_guarded([&] {
    check(iz >= 0 && iz < p->nz, "depth index out of range");
    if (prec == 64) onestep_rows<double>(*p, slow, nxg, iz, freq, adj, in, out, nrow, add);
    else onestep_rows<float>(*p, slow, nxg, iz, freq, adj, in, out, nrow, add);
  });
}

extern "C++" {
template <class R>
static void oneway_rows(const wem_params& p, const float* slow, int nxg, int up, float freq, int adj,
                        const float* in, float* out, int nrow, int add) {
  RowOp<R> op(p, slow, nxg);
  Work<R> wk(op.core.N, nxg);
  R w = Core<R>::omega(freq);
  size_t n = (size_t)nxg * p.nz;
  const bool inplace = (in == out);
  for (int r = 0; r < nrow; ++r) {
    std::vector<C<R>> a = load<R>(in + 2 * n * r, n);
    std::vector<C<R>> b = inplace ? a : load<R>(out + 2 * n * r, n);
    C<R>* A = a.data();
    C<R>* B = inplace ? a.data() : b.data();
    if (!adj) {
      if (up) up_fwd(op.core, w, A, B, add != 0, wk); else down_fwd(op.core, w, A, B, add != 0, wk);
    } else {
      if (up) up_adj(op.core, w, B, A, add != 0, wk); else down_adj(op.core, w, B, A, add != 0, wk);
    }
    store(out + 2 * n * r, B, n, false);
  }
}
}  // extern "C++"

int oracle_oneway(const wem_params* p, const float* slow, int nxg, int up, float freq, int adj,
                  const float* in, float* out, int nrow, int add, int prec) {
  return run_guarded([&] {
    if (prec == 64) oneway_rows<double>(*p, slow, nxg, up, freq, adj, in, out, nrow, add);
    else oneway_rows<float>(*p, slow, nxg, up, freq, adj, in, out, nrow, add);
  });
}

extern "C++" {
template <class R>
static void scatter_rows(const wem_params& p, const float* slow, int nxg, int iz, float freq, int adj,
                         const float* in, float* out, int nrow, int add) {
  RowOp<R> op(p, slow, nxg);
  Work<R> wk(op.core.N, nxg);
  R w = Core<R>::omega(freq);
  bool exact = p.adjoint_mode == WEM_ADJ_EXACT;
  for (int r = 0; r < nrow; ++r) {
    std::vector<C<R>> a = load<R>(in + 2 * (size_t)r * nxg, nxg), b(nxg, C<R>(0));
    if (add) b = load<R>(out + 2 * (size_t)r * nxg, nxg);
    if (!adj) scatter_fwd(op.core, iz, w, a.data(), b.data(), add != 0, wk);
    else scatter_adj(op.core, iz, w, b.data(), a.data(), add != 0, exact, wk);
    store(out + 2 * (size_t)r * nxg, b.data(), nxg, false);
  }
}
}  // extern "C++"

int oracle_scatter(const wem_params* p, const float* slow, int nxg, int iz, float freq, int adj,
                   const float* in, float* out, int nrow, int add, int prec) {
  return run_guarded([&] {
    check(iz >= 0 && iz < p->nz, "depth index out of range");
    if (prec == 64) scatter_rows<double>(*p, slow, nxg, iz, freq, adj, in, out, nrow, add);
    else scatter_rows<float>(*p, slow, nxg, iz, freq, adj, in, out, nrow, add);
  });
}

extern "C++" {
// Phshift::forward/adjoint (Phshift_cmplx.cpp:47-113): rows of n k samples,
// k grid of a row of n points at spacing dx (Phshift_cmplx.cpp:8-24)
template <class R>
static void phshift_rows(const wem_params& p, int n, float dx, float dz, float freq, float sre, float sim, int adj,
                         const float* in, float* out, int nrow, int add) {
  std::vector<R> k(n, R(0));
  const R dk = (R)(2 * kPi / ((double)dx * (n - 1)));
  for (int ik = 0; ik < n / 2; ++ik) k[ik] = ik * dk;
  for (int ik = 1; ik < n / 2; ++ik) k[n - ik] = -k[ik];
  const R w = Core<R>::omega(freq);
  const C<R> s((R)sre, (R)sim);
  for (int r = 0; r < nrow; ++r)
    for (int ik = 0; ik < n; ++ik) {
      C<R> f = ps_factor(w, k[ik], (R)dz, s, (R)p.eps, p.phase_law);
      if (adj) f = std::conj(f);
      const size_t i = (size_t)r * n + ik;
      C<R> v = f * C<R>((R)in[2 * i], (R)in[2 * i + 1]);
      if (add) v += C<R>((R)out[2 * i], (R)out[2 * i + 1]);
      out[2 * i] = (float)v.real();
      out[2 * i + 1] = (float)v.imag();
    }
}

// SplitStep::forward/adjoint (SplitStep.cpp:5-29) at depth iz of the grid
template <class R>
static void splitstep_rows(const wem_params& p, const float* slow, int nxg, int iz, float freq, float sre,
                           float sim, const int* loc, int nloc, int adj, const float* in, float* out, int nrow,
                           int add) {
  const R w = Core<R>::omega(freq);
  const C<R> sref((R)sre, (R)sim), I(0, 1);
  for (int r = 0; r < nrow; ++r) {
    float* o = out + 2 * (size_t)r * nxg;
    const float* a = in + 2 * (size_t)r * nxg;
    std::vector<float> src(a, a + 2 * (size_t)nxg);  // in may alias out
    if (!add) std::fill(o, o + 2 * (size_t)nxg, 0.f);
    for (int i = 0; i < nloc; ++i) {
      const int x = loc[i];
      const C<R> st((R)slow[2 * ((size_t)iz * nxg + x)], (R)slow[2 * ((size_t)iz * nxg + x) + 1]);
      const C<R> u = (st - sref) / std::sqrt(sref);
      const C<R> corr = adj ? I * w * (R)p.dz * std::conj(u) : -I * w * (R)p.dz * u;
      const C<R> v = C<R>((R)src[2 * x], (R)src[2 * x + 1]) * std::exp(corr);
      o[2 * x] = (float)v.real();
      o[2 * x + 1] = (float)v.imag();
    }
  }
}

template <class R>
static void lindown_field(const wem_params& p, const float* slow, int nxg, const float* bg, float freq, int adj,
                          const float* in, float* out, int add) {
  RowOp<R> op(p, slow, nxg);
  Work<R> wk(op.core.N, nxg);
  const size_t n = (size_t)nxg * p.nz;
  std::vector<C<R>> b = load<R>(bg, n), x = load<R>(in, n), y = load<R>(out, n);
  const R w = Core<R>::omega(freq);
  if (!adj) lindown_fwd(op.core, w, b.data(), x.data(), y.data(), add != 0, wk);
  else lindown_adj(op.core, w, b.data(), y.data(), x.data(), add != 0, p.adjoint_mode == WEM_ADJ_EXACT, wk);
  store(out, y.data(), n, false);
}
}

int oracle_phshift(const wem_params* p, int n, float dx, float dz, float freq, float sre, float sim, int adj,
                   const float* in, float* out, int nrow, int add, int prec) {
  return run_guarded([&] {
    check(n >= 2 && dx > 0, "bad row");
    if (prec == 64) phshift_rows<double>(*p, n, dx, dz, freq, sre, sim, adj, in, out, nrow, add);
    else phshift_rows<float>(*p, n, dx, dz, freq, sre, sim, adj, in, out, nrow, add);
  });
}

int oracle_splitstep(const wem_params* p, const float* slow, int nxg, int iz, float freq, float sre, float sim,
                     const int* loc, int nloc, int adj, const float* in, float* out, int nrow, int add, int prec) {
  return run_guarded([&] {
    check(iz >= 0 && iz < p->nz, "depth index out of range");
    for (int i = 0; i < nloc; ++i) check(loc[i] >= 0 && loc[i] < nxg, "location out of the row");
    if (prec == 64) splitstep_rows<double>(*p, slow, nxg, iz, freq, sre, sim, loc, nloc, adj, in, out, nrow, add);
    else splitstep_rows<float>(*p, slow, nxg, iz, freq, sre, sim, loc, nloc, adj, in, out, nrow, add);
  });
}

int oracle_lindown(const wem_params* p, const float* slow, int nxg, const float* bg, float freq, int adj,
                   const float* in, float* out, int add, int prec) {
  return run_guarded([&] {
    if (prec == 64) lindown_field<double>(*p, slow, nxg, bg, freq, adj, in, out, add);
    else lindown_field<float>(*p, slow, nxg, bg, freq, adj, in, out, add);
  });
}

// Reflect (Reflect.h:12-48): out = r in / conj(r) in
int oracle_reflect(const float* slow2, const float* rho, int nx, int nz, int adj, const float* in, float* out) {
  return run_guarded([&] {
    const size_t n = (size_t)nx * nz;
    std::vector<C<double>> s = load<double>(slow2, n), d = load<double>(rho, n), x = load<double>(in, n);
    std::vector<C<double>> r = reflect_coefs(s.data(), d.data(), nx, nz);
    for (size_t i = 0; i < n; ++i) x[i] = (adj ? std::conj(r[i]) : r[i]) * x[i];
    store(out, x.data(), n, false);
  });
}

// dReflect (dReflect.h:11-84): data (+)= dR(m0, m1) or (m0, m1) (+)= dR^H data
int oracle_dreflect(const float* slow2, const float* rho, int nx, int nz, int adj, float* m0, float* m1, float* data,
                    int add) {
  return run_guarded([&] {
    const size_t n = (size_t)nx * nz;
    std::vector<C<double>> s = load<double>(slow2, n), d = load<double>(rho, n);
    DRefl<double> dr(s.data(), d.data(), nx, nz);
    if (!adj) {
      std::vector<C<double>> a = load<double>(m0, n), b = load<double>(m1, n), y(n, C<double>(0));
      if (add) y = load<double>(data, n);
      dr.fwd(a.data(), b.data(), y.data());
      store(data, y.data(), n, false);
    } else {
      std::vector<C<double>> y = load<double>(data, n), a(n, C<double>(0)), b(n, C<double>(0));
      if (add) {
        a = load<double>(m0, n);
        b = load<double>(m1, n);
      }
      dr.adj(a.data(), b.data(), y.data());
      store(m0, a.data(), n, false);
      store(m1, b.data(), n, false);
    }
  });
}

int oracle_refsampler(const wem_params* p, const float* slow, int nxg, float* sref, int* refidx) {
  return run_guarded([&] {
    std::vector<C<float>> s = load<float>(slow, (size_t)nxg * p->nz);
    RefSampler<float> rs(s.data(), nxg, p->nz, p->nref, p->refs_mode);
    for (size_t i = 0; i < rs.sref.size(); ++i) { sref[2 * i] = rs.sref[i].real(); sref[2 * i + 1] = rs.sref[i].imag(); }
    std::fill(refidx, refidx + (size_t)nxg * p->nz, -1);
    for (int iz = 0; iz < p->nz; ++iz)
      for (int j = 0; j < p->nref; ++j)
        for (int x : rs.loc[(size_t)iz * p->nref + j]) refidx[(size_t)iz * nxg + x] = j;
  });
}

}  // extern "C"
