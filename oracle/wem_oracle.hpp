// ORACLE — test infrastructure only.  Nothing in the product links, imports
// or executes this code: only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg use it, and only as the checker.
//
// CPU restatement of arustam92/wem-fwi's one-way depth-continuation path, in
// the reference's own call order, templated on the real type so the same code
// gives the fp32 restatement (the parity target) and its fp64 twin (the
// accuracy oracle).  Each function cites the reference file:line it follows.
//
// PARITY PINNED to the reference run: the reference's own propagator
// sources, compiled unchanged by oracle/ref/Makefile against stand-ins for
// FFTW, TBB, Boost and the SEP libraries, give the golden outputs of
// tests/golden/ref_*.npz (tests/test_ref_pin.py: this restatement within 5e-5
// of them for WEM, BornFull, BornRefl, BornTomo, extWEM and extBornFull).
// Also: the reference's known-answer test (extWEM on a frequency-constant
// model equals WEM bit for bit, propagator/test/test_wem_ops.py:268-282),
// dot-product tests on the reference's set-ups, the fp64 twin, numpy.fft.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "wemgpu.h"

namespace wo {

template <class R> using C = std::complex<R>;
constexpr double kPi = 3.14159265358979323846264338327950288;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ------------------------------------------------------------------ FFT
// Unnormalised c2c DFT, sign -1 = FFTW_FORWARD, +1 = FFTW_BACKWARD (the
// transforms FFTW3f performs at operator/src/FFT1_c.cpp:80,99).  Stockham
// autosort, any length (radix 4, 2, 3, 5, then any prime by direct DFT).
template <class R>
struct Fft {
  int n = 0;
  std::vector<int> radix;
  std::vector<C<R>> w;  // w[t] = exp(-2 pi i t / n)

  explicit Fft(int n_ = 1) : n(n_) {
    if (n < 1) throw Error(WEM_EINVAL, "FFT length < 1");
    int m = n;
    while (m % 4 == 0) { radix.push_back(4); m /= 4; }
    while (m % 2 == 0) { radix.push_back(2); m /= 2; }
    for (int f = 3; m > 1; f += 2)
      while (m % f == 0) { radix.push_back(f); m /= f; }
    w.resize(n);
    for (int t = 0; t < n; ++t) {
      long double a = -2.0L * (long double)kPi * (long double)t / (long double)n;
      w[t] = C<R>((R)std::cos(a), (R)std::sin(a));
    }
  }

  // in place; scratch must hold n values
  void run(C<R>* x, int sign, C<R>* scratch) const {
    C<R>* in = x;
    C<R>* out = scratch;
    int L = 1;
    C<R> t[64], y[64];
    std::vector<C<R>> tv, yv;
    for (int R_ : radix) {
      C<R>* tp = t;
      C<R>* yp = y;
      if (R_ > 64) { tv.resize(R_); yv.resize(R_); tp = tv.data(); yp = yv.data(); }
      const int nb = n / R_;
      const int Lp = L * R_;
      const int tws = n / Lp;
      for (int b = 0; b < nb; ++b) {
        const int l = b % L;
        for (int r = 0; r < R_; ++r) {
          C<R> v = in[b + r * nb];
          if (r && l) {
            C<R> tw = w[(size_t)r * l * tws];
            if (sign > 0) tw = std::conj(tw);
            v *= tw;
          }
          tp[r] = v;
        }
        dft_small(tp, yp, R_, sign);
        const int ob = (b / L) * Lp + l;
        for (int q = 0; q < R_; ++q) out[ob + q * L] = yp[q];
      }
      std::swap(in, out);
      L = Lp;
    }
    if (in != x) std::copy(in, in + n, x);
  }

  void dft_small(const C<R>* a, C<R>* y, int p, int sign) const {
    if (p == 2) { y[0] = a[0] + a[1]; y[1] = a[0] - a[1]; return; }
    if (p == 4) {
      C<R> s0 = a[0] + a[2], d0 = a[0] - a[2];
      C<R> s1 = a[1] + a[3], d1 = a[1] - a[3];
      // multiply d1 by -i*sign... forward (sign -1): W4 = -i
      C<R> jd1 = (sign < 0) ? C<R>(d1.imag(), -d1.real()) : C<R>(-d1.imag(), d1.real());
      y[0] = s0 + s1; y[2] = s0 - s1; y[1] = d0 + jd1; y[3] = d0 - jd1;
      return;
    }
    const int step = n / p;
    for (int q = 0; q < p; ++q) {
      C<R> acc = a[0];
      for (int r = 1; r < p; ++r) {
        C<R> tw = w[(size_t)((r * q) % p) * step];
        if (sign > 0) tw = std::conj(tw);
        acc += a[r] * tw;
      }
      y[q] = acc;
    }
  }
};

// ------------------------------------------------------ parameter set-up
inline void check(bool ok, const std::string& msg) {
  if (!ok) throw Error(WEM_EINVAL, msg);
}

// Device index lists (propagator/src/Device.h:39-85).  Float arithmetic and
// the +.5f truncating round of the reference.
struct Devices {
  std::vector<int> ix, iz;
};

inline Devices make_devices(const wem_params& p, bool src) {
  Devices d;
  const float* ax = src ? p.src_x : p.rec_x;
  const float* az = src ? p.src_z : p.rec_z;
  int n = src ? p.ns : p.nr;
  check(n > 0, std::string("Number of devices ") + (src ? "s" : "r") + " is zero!");
  for (int i = 0; i < n; ++i) {
    float x, z;
    if (ax) {
      x = ax[i]; z = az[i];
    } else {
      float bx = src ? p.osx : p.orx, bz = src ? p.osz : p.orz;
      float sx = src ? p.dsx : p.drx, sz = src ? p.dsz : p.drz;
      check(bx >= p.ox && bz >= p.oz, "Devices start outside of the model!");
      check(sx != 0.f || sz != 0.f || n == 1, "Devices have spacing equal to zero!");
      x = bx + i * sx;
      z = bz + i * sz;
    }
    int indx = (int)((x - p.ox) / p.dx + .5f);
    int indz = (int)((z - p.oz) / p.dz + .5f);
    check(indx >= 0 && indz >= 0, "Device is out of bounds!");
    check(indz < p.nz, "Device depth index beyond the model");
    d.ix.push_back(indx);
    d.iz.push_back(indz);
  }
  return d;
}

// Frequencies and wavelet bins (propagator/src/PropParam.h:45-85).
struct Freqs {
  std::vector<float> freq;
  std::vector<int> bin;
  int nt_pad = 0;
  float tmax = 0;
};

inline Freqs make_freqs(const wem_params& p) {
  Freqs F;
  F.nt_pad = p.nt + p.tpad;
  F.tmax = p.ot + (p.dt * (F.nt_pad - 1));
  int fmin, fmax;
  if (p.fmax == 0) {
    fmin = 1;
    fmax = p.nfreq;
    if (fmax == 0) fmax = F.nt_pad / 2 + 1;
  } else {
    fmin = (int)(p.fmin * F.tmax);
    fmax = (int)(p.fmax * F.tmax + .5f);
  }
  int nf = fmax - fmin + 1;
  check(nf > 0, "no frequency to propagate");
  for (int i = 0; i < nf; ++i) {
    F.freq.push_back(p.fmin + float(i) / F.tmax);
    F.bin.push_back(i + fmin);
  }
  return F;
}

// Cosine-squared spreading window (propagator/src/Injection.h:53-65).
template <class R>
std::vector<R> gauss_window(int ng) {
  std::vector<R> g(2 * ng + 1);
  R pi = (R)(4 * std::atan(1.));
  if (ng == 0) { g[0] = 1; return g; }
  int sz = (int)g.size();
  for (int i = 0; i < sz / 2; ++i) g[i] = (-std::cos(pi / ng * i) + 1) / 2;
  for (int i = sz / 2; i < sz; ++i) g[i] = (std::cos(pi / ng * (i - sz + ng + 1)) + 1) / 2;
  return g;
}

// Edge-extended (extend=true) or zero (extend=false) pad along x of a 2D
// field [nz][nx] -> [nz][nx+2pad] (operator/src/Pad.h:77-96).
template <class R>
void pad_x(const C<R>* in, C<R>* out, int nz, int nx, int pad, bool extend) {
  int nxg = nx + 2 * pad;
  for (int iz = 0; iz < nz; ++iz) {
    const C<R>* a = in + (size_t)iz * nx;
    C<R>* b = out + (size_t)iz * nxg;
    for (int i = 0; i < nx; ++i) b[i + pad] = a[i];
    C<R> bv = extend ? b[pad] : C<R>(0), ev = extend ? b[nx - 1 + pad] : C<R>(0);
    for (int i = 0; i < pad; ++i) { b[i] = bv; b[nx + i + pad] = ev; }
  }
}

// ------------------------------------------------------------ RefSampler
// propagator/src/RefSampler.cpp:10-84.  sref[z][j] = s[z][o + j nx / nref]
// with o = nx/(2 nref); the partition sorts the x values of each depth and
// splits them with the midpoints of the (history-polluted) sorted reference
// buffer exactly as coded; see the deviation note at the while loops.
template <class R>
struct RefSampler {
  int nx = 0, nz = 0, nref = 0;
  std::vector<C<R>> sref;              // [nz][nref]
  std::vector<std::vector<int>> loc;   // [nz*nref]

  RefSampler() = default;
  RefSampler(const C<R>* s, int nx_, int nz_, int nref_, int mode) : nx(nx_), nz(nz_), nref(nref_) {
    check(nref >= 1 && nref <= nx && nx >= 2, "nref out of range");
    sref.resize((size_t)nz * nref);
    loc.resize((size_t)nz * nref);
    int o = nx / (2 * nref);
    for (int iz = 0; iz < nz; ++iz)
      for (int j = 0; j < nref; ++j) {
        int off = o + j * nx / nref;
        sref[(size_t)iz * nref + j] = s[(size_t)iz * nx + off];
        if (!((float)sref[(size_t)iz * nref + j].real() > 0))
          throw Error(WEM_EINVAL, "Ref velocity " + std::to_string((double)sref[(size_t)iz * nref + j].real()) +
                                      " at the layer " + std::to_string(iz));
      }
    if (mode == WEM_REFS_NEAREST) nearest(s); else ascoded(s);
  }

  void ascoded(const C<R>* s) {
    // float buffers like the reference's float1D members, for both real types:
    // the partition is a discrete choice of the operator, not arithmetic
    std::vector<float> slice(nx), rslice(nx, 0.f);  // boost::multi_array zero-initialises
    std::vector<int> is(nx), isr(nref);
    for (int iz = 0; iz < nz; ++iz) {
      for (int ix = 0; ix < nx; ++ix) slice[ix] = (float)s[(size_t)iz * nx + ix].real();
      for (int j = 0; j < nref; ++j) rslice[j] = (float)sref[(size_t)iz * nref + j].real();
      std::iota(is.begin(), is.end(), 0);
      std::iota(isr.begin(), isr.end(), 0);
      std::stable_sort(is.begin(), is.end(), [&](int a, int b) { return slice[a] < slice[b]; });
      std::stable_sort(isr.begin(), isr.end(), [&](int a, int b) { return rslice[a] < rslice[b]; });
      std::sort(slice.begin(), slice.end());
      std::sort(rslice.begin(), rslice.end());
      // The reference's while loops have no bound; they can only run past
      // the end when nref == 1 and the zero history is used up (nz >= nx-1).
      // Stopping at nx is the one deviation from the code as written.
      int off = 0;
      while (off < nx && slice[off] - rslice[0] < rslice[1] - slice[off]) off++;
      std::vector<std::vector<int>> grp(nref);
      grp[isr[0]].assign(is.begin(), is.begin() + off);
      int beg = off;
      for (int j = 1; j < nref - 1; ++j) {
        while (off < nx && slice[off] - rslice[j] < rslice[j + 1] - slice[off]) off++;
        grp[isr[j]].assign(is.begin() + beg, is.begin() + off);
        beg = off;
      }
      grp[isr[nref - 1]].assign(is.begin() + off, is.end());
      for (int j = 0; j < nref; ++j) {
        std::sort(grp[j].begin(), grp[j].end());
        loc[(size_t)iz * nref + j] = grp[j];
      }
    }
  }

  void nearest(const C<R>* s) {
    for (int iz = 0; iz < nz; ++iz) {
      std::vector<std::vector<int>> grp(nref);
      for (int ix = 0; ix < nx; ++ix) {
        R v = s[(size_t)iz * nx + ix].real();
        int best = 0;
        R bd = std::abs(v - sref[(size_t)iz * nref].real());
        for (int j = 1; j < nref; ++j) {
          R d = std::abs(v - sref[(size_t)iz * nref + j].real());
          if (d < bd) { bd = d; best = j; }
        }
        grp[best].push_back(ix);
      }
      for (int j = 0; j < nref; ++j) loc[(size_t)iz * nref + j] = grp[j];
    }
  }
};

// --------------------------------------------------------- depth step core
// One padded slowness grid with its RefSampler, k grid and taper: the state
// shared by SSF/PSPI (OneStep.h:19-38), SplitStep and Scatter.
template <class R>
struct Core {
  int nxg = 0, nz = 0, N = 0, tap = 0, pad = 0, nref = 1, prop = WEM_PROP_SSF, ntaylor = 1;
  R dx = 1, dz = 1, eps = 0.04f;
  int law = WEM_PHASE_ISPC;
  const C<R>* slow = nullptr;  // [nz][nxg], owned by the caller
  RefSampler<R> refs;
  std::vector<R> k;      // Phshift k grid, propagator/src/Phshift_cmplx.cpp:13,21-24
  std::vector<R> taper;  // operator/src/Taper.h:11-23
  Fft<R> fft;

  Core(const wem_params& p, const C<R>* s, int nxg_, int nz_)
      : nxg(nxg_), nz(nz_), N(nxg_ + 2 * p.tap), tap(p.tap), pad(p.pad), nref(p.nref),
        prop(p.prop), ntaylor(p.ntaylor), dx(p.dx), dz(p.dz), eps(p.eps), law(p.phase_law), slow(s),
        refs(s, nxg_, nz_, p.nref, p.refs_mode), fft(nxg_ + 2 * p.tap) {
    check(p.ntaylor >= 0 && p.ntaylor <= 4, "ntaylor must be in [0,4]");
    k.assign(N, R(0));
    R dk = (R)(2 * kPi / ((double)dx * (N - 1)));
    for (int ik = 0; ik < N / 2; ++ik) k[ik] = ik * dk;
    for (int ik = 1; ik < N / 2; ++ik) k[N - ik] = -k[ik];
    taper.assign(nxg, R(1));
    for (int i = 0; i < pad; ++i) {
      taper[i] = (R)(.5f * (1 - std::cos(kPi * i / (pad - 1))));
      taper[nxg - 1 - i] = taper[i];
    }
  }
  static R omega(float f) { return (R)(2 * kPi * (double)f); }
};

// Per-thread scratch for one row.
template <class R>
struct Work {
  std::vector<C<R>> a, b, c, d, e, f, scr;
  explicit Work(int N, int nxg) : a(N), b(N), c(N), d(nxg), e(nxg), f(nxg), scr(N) {}
};

// phase_shift.ispc:2-16 (ps_fwd) / :18-32 (ps_adj): one k bin.
// law WEM_PHASE_EXACT_KZ: extPropagator/src/Phshift.cpp:59,81, forward factor
// exp(-i dz kz) with kz = conj(sqrt(w^2 s - k^2 + i 1e-5)) (complex s; the
// reference's s there is real).
template <class R>
inline C<R> ps_factor(R w, R k, R dz, C<R> s, R eps, int law = WEM_PHASE_ISPC) {
  if (law == WEM_PHASE_EXACT_KZ) {
    const C<R> I(0, 1);
    C<R> kz = std::conj(std::sqrt(w * w * s - k * k + I * R(1e-5)));
    return std::exp(-I * dz * kz);
  }
  R a = w * w * s.real() - k * k;
  R b = w * w * (s.imag() - eps * s.real());
  R c = std::sqrt(a * a + b * b);
  R re = std::sqrt((c + a) / 2);
  R im = -std::sqrt((c - a) / 2);
  R e = std::exp(im * dz);
  return C<R>(e * std::cos(re * dz), -e * std::sin(re * dz));
}

// Unitary FFT wrapper without the origin phase: FFT1_c.cpp:73-103 multiplies
// by exp(i o1 k) after the forward transform and divides it out before the
// inverse one; every use on this path brackets only diagonal operators, so
// the factors cancel and are left out here.
template <class R>
inline void fft_unitary(const Core<R>& c, C<R>* x, int sign, Work<R>& wk) {
  c.fft.run(x, sign, wk.scr.data());
  R s = (R)(1.0 / std::sqrt((double)c.N));
  for (int i = 0; i < c.N; ++i) x[i] *= s;
}

// SSF::forward / PSPI::forward (SSF.cpp:8-32, PSPI.cpp:8-29) with
// SplitStep::forward (SplitStep.cpp:5-16) and Selector::forward (Selector.cpp:5-10).
template <class R>
void onestep_fwd(const Core<R>& c, int iz, R w, const C<R>* model, C<R>* data, bool add, Work<R>& wk) {
  const int N = c.N, nxg = c.nxg, tap = c.tap;
  C<R>* mp = wk.a.data();
  C<R>* wp = wk.b.data();
  C<R>* wr = wk.d.data();
  C<R>* out = wk.e.data();  // data may alias model
  if (add) std::copy(data, data + nxg, out); else std::fill(out, out + nxg, C<R>(0));
  std::fill(mp, mp + N, C<R>(0));
  for (int i = 0; i < nxg; ++i) mp[i + tap] = model[i];
  fft_unitary(c, mp, -1, wk);
  for (int j = 0; j < c.nref; ++j) {
    C<R> sr = c.refs.sref[(size_t)iz * c.nref + j];
    for (int ik = 0; ik < N; ++ik) wp[ik] = mp[ik] * ps_factor(w, c.k[ik], c.dz, sr, c.eps, c.law);
    fft_unitary(c, wp, +1, wk);
    for (int i = 0; i < nxg; ++i) wr[i] = wp[i + tap] * c.taper[i];
    const std::vector<int>& loc = c.refs.loc[(size_t)iz * c.nref + j];
    if (c.prop == WEM_PROP_SSF) {
      const C<R> I(0, 1);
      for (int x : loc) {
        C<R> st = c.slow[(size_t)iz * nxg + x];
        C<R> corr = -I * w * c.dz * (st - sr) / std::sqrt(sr);
        wr[x] = wr[x] * std::exp(corr);
      }
    }
    for (int x : loc) out[x] = wr[x];
  }
  std::copy(out, out + nxg, data);
}

// SSF::adjoint / PSPI::adjoint (SSF.cpp:34-60, PSPI.cpp:31-53).
template <class R>
void onestep_adj(const Core<R>& c, int iz, R w, C<R>* model, const C<R>* data, bool add, Work<R>& wk) {
  const int N = c.N, nxg = c.nxg, tap = c.tap;
  C<R>* mp = wk.a.data();
  C<R>* wp = wk.b.data();
  C<R>* wr = wk.d.data();
  C<R>* out = wk.e.data();
  if (add) std::copy(model, model + nxg, out); else std::fill(out, out + nxg, C<R>(0));
  std::fill(mp, mp + N, C<R>(0));
  const C<R> I(0, 1);
  for (int j = 0; j < c.nref; ++j) {
    C<R> sr = c.refs.sref[(size_t)iz * c.nref + j];
    const std::vector<int>& loc = c.refs.loc[(size_t)iz * c.nref + j];
    std::fill(wr, wr + nxg, C<R>(0));
    for (int x : loc) wr[x] = data[x];
    if (c.prop == WEM_PROP_SSF) {
      for (int x : loc) {
        C<R> st = c.slow[(size_t)iz * nxg + x];
        C<R> corr = I * w * c.dz * std::conj((st - sr) / std::sqrt(sr));
        wr[x] = wr[x] * std::exp(corr);
      }
    }
    for (int i = 0; i < nxg; ++i) wr[i] *= c.taper[i];
    std::fill(wp, wp + N, C<R>(0));
    for (int i = 0; i < nxg; ++i) wp[i + tap] = wr[i];
    fft_unitary(c, wp, -1, wk);
    for (int ik = 0; ik < N; ++ik) mp[ik] += wp[ik] * std::conj(ps_factor(w, c.k[ik], c.dz, sr, c.eps, c.law));
  }
  fft_unitary(c, mp, +1, wk);
  for (int i = 0; i < nxg; ++i) out[i] += mp[i + tap];
  std::copy(out, out + nxg, model);
}

// Down / Up (OneWay.cpp:32-109).  Fields [nz][nxg]; model and data may be the
// same array, which turns the loops into the in-place recursions the drivers use.
template <class R>
void down_fwd(const Core<R>& c, R w, const C<R>* M, C<R>* D, bool add, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(D, D + (size_t)nx * nz, C<R>(0));
  std::copy(M, M + nx, D);
  for (int iz = 0; iz < nz - 1; ++iz) {
    std::copy(M + (size_t)iz * nx, M + (size_t)(iz + 1) * nx, wk.f.begin());
    onestep_fwd(c, iz, w, wk.f.data(), wk.f.data(), false, wk);
    for (int i = 0; i < nx; ++i) D[(size_t)(iz + 1) * nx + i] = wk.f[i] + M[(size_t)(iz + 1) * nx + i];
  }
}

template <class R>
void down_adj(const Core<R>& c, R w, C<R>* M, const C<R>* D, bool add, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(M, M + (size_t)nx * nz, C<R>(0));
  std::copy(D + (size_t)(nz - 1) * nx, D + (size_t)nz * nx, M + (size_t)(nz - 1) * nx);
  for (int iz = nz - 1; iz > 0; --iz) {
    std::copy(D + (size_t)iz * nx, D + (size_t)(iz + 1) * nx, wk.f.begin());
    onestep_adj(c, iz - 1, w, wk.f.data(), wk.f.data(), false, wk);
    for (int i = 0; i < nx; ++i) M[(size_t)(iz - 1) * nx + i] = wk.f[i] + D[(size_t)(iz - 1) * nx + i];
  }
}

template <class R>
void up_fwd(const Core<R>& c, R w, const C<R>* M, C<R>* D, bool add, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(D, D + (size_t)nx * nz, C<R>(0));
  std::copy(M + (size_t)(nz - 1) * nx, M + (size_t)nz * nx, D + (size_t)(nz - 1) * nx);
  for (int iz = nz - 1; iz > 0; --iz) {
    std::copy(M + (size_t)iz * nx, M + (size_t)(iz + 1) * nx, wk.f.begin());
    onestep_fwd(c, iz, w, wk.f.data(), wk.f.data(), false, wk);
    for (int i = 0; i < nx; ++i) D[(size_t)(iz - 1) * nx + i] = wk.f[i] + M[(size_t)(iz - 1) * nx + i];
  }
}

template <class R>
void up_adj(const Core<R>& c, R w, C<R>* M, const C<R>* D, bool add, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(M, M + (size_t)nx * nz, C<R>(0));
  std::copy(D, D + nx, M);
  for (int iz = 0; iz < nz - 1; ++iz) {
    std::copy(D + (size_t)iz * nx, D + (size_t)(iz + 1) * nx, wk.f.begin());
    onestep_adj(c, iz + 1, w, wk.f.data(), wk.f.data(), false, wk);
    for (int i = 0; i < nx; ++i) M[(size_t)(iz + 1) * nx + i] = wk.f[i] + D[(size_t)(iz + 1) * nx + i];
  }
}

// ------------------------------------------------------------- Scatter
// propagator/src/Scatter.cpp:6-111 (coefficients Scatter.h:36).
template <class R>
inline C<R> scatter_coef(const Core<R>& c, int iz, int ix, int it) {
  static const R coef[5] = {(R)1., (R)(1. / 2.), (R)(3. / 8.), (R)(5. / 16.), (R)(35. / 128.)};
  C<R> s = c.slow[(size_t)iz * c.nxg + ix];
  return coef[it] * std::pow(s - c.eps * s.real(), (R)(-.5f - it));
}

// (k/w)^(2 it) filter (Scatter.cpp:68-75)
template <class R>
inline R scatter_kfilter(const Core<R>& c, int ik, R w, int it) {
  return (R)std::pow((double)(c.k[ik] / w), 2 * it);
}

// forward: data += sum_it -i w dz c_it(x) unpad(IFFT(K_it FFT(pad(model))))
template <class R>
void scatter_fwd(const Core<R>& c, int iz, R w, const C<R>* model, C<R>* data, bool add, Work<R>& wk) {
  const int N = c.N, nx = c.nxg, tap = c.tap;
  C<R>* kx = wk.a.data();
  C<R>* wp = wk.b.data();
  C<R>* wr = wk.d.data();
  C<R>* out = wk.e.data();
  if (add) std::copy(data, data + nx, out); else std::fill(out, out + nx, C<R>(0));
  std::fill(kx, kx + N, C<R>(0));
  for (int i = 0; i < nx; ++i) kx[i + tap] = model[i];
  fft_unitary(c, kx, -1, wk);
  for (int it = 0; it <= c.ntaylor; ++it) {
    for (int ik = 0; ik < N; ++ik) wp[ik] = kx[ik] * scatter_kfilter(c, ik, w, it);
    fft_unitary(c, wp, +1, wk);
    for (int i = 0; i < nx; ++i) wr[i] = scatter_coef(c, iz, i, it) * wp[i + tap];
    for (int i = 0; i < nx; ++i) {  // set_next_wfld, sign -1
      R re = w * c.dz * wr[i].imag();
      R im = -w * c.dz * wr[i].real();
      out[i] = C<R>(out[i].real() + re, out[i].imag() + im);
    }
  }
  std::copy(out, out + nx, data);
}

// adjoint.  exact=false: the reference's order, k-filter before the
// conjugate slowness scaling (Scatter.cpp:52-66); exact=true: the transpose.
template <class R>
void scatter_adj(const Core<R>& c, int iz, R w, C<R>* model, const C<R>* data, bool add, bool exact, Work<R>& wk) {
  const int N = c.N, nx = c.nxg, tap = c.tap;
  C<R>* kx = wk.a.data();
  C<R>* wp = wk.b.data();
  C<R>* wr = wk.d.data();
  C<R>* out = wk.e.data();
  if (add) std::copy(model, model + nx, out); else std::fill(out, out + nx, C<R>(0));
  if (!exact) {
    std::fill(kx, kx + N, C<R>(0));
    for (int i = 0; i < nx; ++i) kx[i + tap] = data[i];
    fft_unitary(c, kx, -1, wk);
  }
  for (int it = 0; it <= c.ntaylor; ++it) {
    if (!exact) {
      for (int ik = 0; ik < N; ++ik) wp[ik] = kx[ik] * scatter_kfilter(c, ik, w, it);
      fft_unitary(c, wp, +1, wk);
      for (int i = 0; i < nx; ++i) wr[i] = std::conj(scatter_coef(c, iz, i, it)) * wp[i + tap];
    } else {
      std::fill(wp, wp + N, C<R>(0));
      for (int i = 0; i < nx; ++i) wp[i + tap] = std::conj(scatter_coef(c, iz, i, it)) * data[i];
      fft_unitary(c, wp, -1, wk);
      for (int ik = 0; ik < N; ++ik) wp[ik] *= scatter_kfilter(c, ik, w, it);
      fft_unitary(c, wp, +1, wk);
      for (int i = 0; i < nx; ++i) wr[i] = wp[i + tap];
    }
    for (int i = 0; i < nx; ++i) {  // set_next_wfld, sign +1
      R re = -w * c.dz * wr[i].imag();
      R im = w * c.dz * wr[i].real();
      out[i] = C<R>(out[i].real() + re, out[i].imag() + im);
    }
  }
  std::copy(out, out + nx, model);
}

// ------------------------------------------- Reflect / dReflect / IC
// Reflect (Reflect.h:12-48): r[z] from the padded [s, rho]; r[0] = 0.
template <class R>
std::vector<C<R>> reflect_coefs(const C<R>* s, const C<R>* rho, int nx, int nz) {
  std::vector<C<R>> r((size_t)nx * nz, C<R>(0));
  for (int iz = 1; iz < nz; ++iz)
    for (int ix = 0; ix < nx; ++ix) {
      size_t a = (size_t)iz * nx + ix, b = (size_t)(iz - 1) * nx + ix;
      C<R> num = rho[a] * std::sqrt(s[b]) - rho[b] * std::sqrt(s[a]);
      C<R> den = rho[a] * std::sqrt(s[b]) + rho[b] * std::sqrt(s[a]);
      r[a] = num / den;
    }
  return r;
}

// dReflect (dReflect.h:11-84): the per-point coefficient pairs used by
// forward and adjoint, rows 1..nz-2.
template <class R>
struct DRefl {
  int nx = 0, nz = 0;
  std::vector<C<R>> a0, b0, a1, b1;  // [nz][nx]
  DRefl(const C<R>* s, const C<R>* rho, int nx_, int nz_) : nx(nx_), nz(nz_) {
    size_t n = (size_t)nx * nz;
    a0.assign(n, 0); b0.assign(n, 0); a1.assign(n, 0); b1.assign(n, 0);
    for (int iz = 1; iz < nz; ++iz)
      for (int ix = 0; ix < nx; ++ix) {
        size_t a = (size_t)iz * nx + ix, b = (size_t)(iz - 1) * nx + ix;
        C<R> v = std::pow(rho[a] * std::sqrt(s[b]) + rho[b] * std::sqrt(s[a]), -2);
        C<R> s1s2 = (rho[b] * rho[a]) / v;
        C<R> r1r2 = (R)2 * (s[b] * s[a]) / v;
        C<R> cc = std::sqrt(s[a] / s[b]);
        a0[a] = cc * s1s2;
        b0[a] = (R)1 / cc * s1s2;
        a1[a] = rho[b] * r1r2;
        b1[a] = rho[a] * r1r2;
      }
  }
  // data += dR(m0, m1)
  void fwd(const C<R>* m0, const C<R>* m1, C<R>* d) const {
    for (int iz = 1; iz < nz - 1; ++iz)
      for (int ix = 0; ix < nx; ++ix) {
        size_t a = (size_t)iz * nx + ix, b = (size_t)(iz - 1) * nx + ix;
        d[a] += a0[a] * m0[b] - b0[a] * m0[a];
        d[a] += a1[a] * m1[a] - b1[a] * m1[b];
      }
  }
  void adj(C<R>* m0, C<R>* m1, const C<R>* d) const {
    for (int iz = 1; iz < nz - 1; ++iz)
      for (int ix = 0; ix < nx; ++ix) {
        size_t a = (size_t)iz * nx + ix, b = (size_t)(iz - 1) * nx + ix;
        m0[b] += std::conj(a0[a]) * d[a];
        m0[a] += -std::conj(b0[a]) * d[a];
        m1[a] += std::conj(a1[a]) * d[a];
        m1[b] += -std::conj(b1[a]) * d[a];
      }
  }
};

// ------------------------------------------------------- LinDown / LinUp
// propagator/src/LinOneWay.cpp:33-142; IC row ops ic.cpp:30-45.
template <class R>
void lindown_fwd(const Core<R>& c, R w, const C<R>* bg, const C<R>* M, C<R>* D, bool add, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(D, D + (size_t)nx * nz, C<R>(0));
  std::fill(D, D + nx, C<R>(0));
  std::vector<C<R>> prev(nx), next(nx);
  for (int iz = 0; iz < nz - 1; ++iz) {
    for (int i = 0; i < nx; ++i) prev[i] = bg[(size_t)iz * nx + i] * M[(size_t)iz * nx + i];
    scatter_fwd(c, iz, w, prev.data(), next.data(), false, wk);
    onestep_fwd(c, iz, w, next.data(), prev.data(), false, wk);
    for (int i = 0; i < nx; ++i) D[(size_t)(iz + 1) * nx + i] = prev[i] + D[(size_t)(iz + 1) * nx + i];
  }
}

template <class R>
void lindown_adj(const Core<R>& c, R w, const C<R>* bg, C<R>* M, const C<R>* D, bool add, bool exact, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(M, M + (size_t)nx * nz, C<R>(0));
  if (!exact) std::fill(M + (size_t)(nz - 1) * nx, M + (size_t)nz * nx, C<R>(0));
  std::vector<C<R>> prev(nx), next(nx);
  for (int iz = nz - 1; iz > 0; --iz) {
    std::copy(D + (size_t)iz * nx, D + (size_t)(iz + 1) * nx, prev.begin());
    onestep_adj(c, iz - 1, w, next.data(), prev.data(), false, wk);
    scatter_adj(c, iz - 1, w, prev.data(), next.data(), false, exact, wk);
    for (int i = 0; i < nx; ++i)
      M[(size_t)(iz - 1) * nx + i] += std::conj(bg[(size_t)(iz - 1) * nx + i]) * prev[i];
  }
}

template <class R>
void linup_fwd(const Core<R>& c, R w, const C<R>* bg, const C<R>* M, C<R>* D, bool add, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(D, D + (size_t)nx * nz, C<R>(0));
  std::fill(D + (size_t)(nz - 1) * nx, D + (size_t)nz * nx, C<R>(0));
  std::vector<C<R>> prev(nx), next(nx);
  for (int iz = nz - 1; iz > 0; --iz) {
    for (int i = 0; i < nx; ++i) prev[i] = bg[(size_t)iz * nx + i] * M[(size_t)iz * nx + i];
    scatter_fwd(c, iz, w, prev.data(), next.data(), false, wk);
    onestep_fwd(c, iz, w, next.data(), prev.data(), false, wk);
    for (int i = 0; i < nx; ++i) D[(size_t)(iz - 1) * nx + i] = prev[i] + D[(size_t)(iz - 1) * nx + i];
  }
}

template <class R>
void linup_adj(const Core<R>& c, R w, const C<R>* bg, C<R>* M, const C<R>* D, bool add, bool exact, Work<R>& wk) {
  const int nx = c.nxg, nz = c.nz;
  if (!add) std::fill(M, M + (size_t)nx * nz, C<R>(0));
  std::vector<C<R>> prev(nx), next(nx);
  for (int iz = 0; iz < nz - 1; ++iz) {
    std::copy(D + (size_t)iz * nx, D + (size_t)(iz + 1) * nx, prev.begin());
    onestep_adj(c, iz + 1, w, next.data(), prev.data(), false, wk);
    scatter_adj(c, iz + 1, w, prev.data(), next.data(), false, exact, wk);
    for (int i = 0; i < nx; ++i)
      M[(size_t)(iz + 1) * nx + i] += std::conj(bg[(size_t)(iz + 1) * nx + i]) * prev[i];
  }
}

// ------------------------------------------------------------ Injection
// propagator/src/Injection.cpp:8-80.  Source (1D wavelet model) and
// receiver (3D data model) forms for one (shot, bin).
template <class R>
struct Inject {
  std::vector<int> ix, iz;
  int ng = 0, tap = 0;
  std::vector<R> g;
  Inject() = default;
  Inject(std::vector<int> ix_, std::vector<int> iz_, int ng_, int tap_)
      : ix(std::move(ix_)), iz(std::move(iz_)), ng(ng_), tap(tap_), g(gauss_window<R>(ng_)) {}
  // wavefield += spread(value) at every device (Injection.cpp:8-19 / 56-67)
  void spread(C<R>* W, int nx, const C<R>* vals) const {
    for (int ig = -ng; ig <= ng; ++ig)
      for (size_t i = 0; i < ix.size(); ++i) {
        int off = ix[i] + ig + tap;
        if (off >= 0 && off < nx) W[(size_t)iz[i] * nx + off] += g[ig + ng] * vals[i];
      }
  }
  // vals[i] += gather of the wavefield (Injection.cpp:21-32 / 69-80)
  void gather(const C<R>* W, int nx, C<R>* vals) const {
    for (int ig = -ng; ig <= ng; ++ig)
      for (size_t i = 0; i < ix.size(); ++i) {
        int off = ix[i] + ig + tap;
        if (off >= 0 && off < nx) vals[i] += g[ig + ng] * W[(size_t)iz[i] * nx + off];
      }
  }
};

}  // namespace wo
