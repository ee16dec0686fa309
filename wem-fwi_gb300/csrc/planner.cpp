// Host planner (see planner.h).  All background tables are computed in
// double and rounded once when uploaded.
#include "planner.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace wg {

static const double kPi = 3.14159265358979323846;

std::vector<int> fft_radices(int n) {
  require(n >= 1, "FFT length must be >= 1");
  std::vector<int> r;
  int m = n;
  while (m % 4 == 0) { r.push_back(4); m /= 4; }
  while (m % 2 == 0) { r.push_back(2); m /= 2; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) { r.push_back(f); m /= f; }
  return r;
}

std::vector<cd> twiddles(int n) {
  std::vector<cd> w(n);
  for (int t = 0; t < n; ++t) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * t / n;
    w[t] = cd((double)std::cos(a), (double)std::sin(a));
  }
  return w;
}

// Device.h:39-85 — float arithmetic and the truncating +.5f round
static void device_indices(const wem_params& p, bool src, std::vector<int>& ix, std::vector<int>& iz) {
  const float* ax = src ? p.src_x : p.rec_x;
  const float* az = src ? p.src_z : p.rec_z;
  int n = src ? p.ns : p.nr;
  require(n > 0, std::string("Number of devices ") + (src ? "s" : "r") + " is zero!");
  for (int i = 0; i < n; ++i) {
    float x, z;
    if (ax) {
      require(az != nullptr, "irregular geometry needs both x and z coordinates");
      x = ax[i];
      z = az[i];
    } else {
      float bx = src ? p.osx : p.orx, bz = src ? p.osz : p.orz;
      float dx = src ? p.dsx : p.drx, dz = src ? p.dsz : p.drz;
      require(bx >= p.ox && bz >= p.oz, "Devices start outside of the model!");
      require(dx != 0.f || dz != 0.f || n == 1, "Devices have spacing equal to zero!");
      x = bx + i * dx;
      z = bz + i * dz;
    }
    int jx = (int)((x - p.ox) / p.dx + .5f);
    int jz = (int)((z - p.oz) / p.dz + .5f);
    require(jx >= 0 && jz >= 0, "Device is out of bounds!");
    require(jz < p.nz, "Device depth index beyond the model");
    ix.push_back(jx);
    iz.push_back(jz);
  }
}

// PropParam.h:45-85
static void frequencies(const wem_params& p, std::vector<float>& freq, std::vector<int>& bin, int& nt_pad) {
  nt_pad = p.nt + p.tpad;
  require(p.nt > 0 && p.dt > 0, "wavelet needs nt > 0 and dt > 0");
  float tmax = p.ot + (p.dt * (nt_pad - 1));
  int fmin, fmax;
  if (p.fmax == 0) {
    fmin = 1;
    fmax = p.nfreq ? p.nfreq : nt_pad / 2 + 1;
  } else {
    fmin = (int)(p.fmin * tmax);
    fmax = (int)(p.fmax * tmax + .5f);
  }
  require(fmax >= fmin, "no frequency to propagate");
  for (int i = 0; i <= fmax - fmin; ++i) {
    freq.push_back(p.fmin + float(i) / tmax);
    bin.push_back(i + fmin);
  }
}

int count_frequencies(const wem_params& p) {
  std::vector<float> f;
  std::vector<int> b;
  int n;
  frequencies(p, f, b, n);
  return (int)f.size();
}

// Injection.h:53-65 cos^2 window
static std::vector<double> window(int ng) {
  std::vector<double> g(2 * ng + 1, 1.0);
  if (ng == 0) return g;
  int sz = 2 * ng + 1;
  for (int i = 0; i < sz / 2; ++i) g[i] = (1 - std::cos(kPi / ng * i)) / 2;
  for (int i = sz / 2; i < sz; ++i) g[i] = (std::cos(kPi / ng * (i - sz + ng + 1)) + 1) / 2;
  return g;
}

Geometry make_geometry(const wem_params& p, const float* wavelet) {
  require(p.nx > 0 && p.nz > 1, "model must have nx > 0 and nz > 1");
  require(p.dx > 0 && p.dz > 0, "grid spacing must be positive");
  require(p.nref >= 1, "nref must be >= 1");
  require(p.pad >= 0 && p.tap >= 0 && p.tpad >= 0, "pad/tap/tpad must be >= 0");
  require(p.pad != 1, "pad == 1 makes the taper divide by zero (Taper.h:19)");
  require(p.ntaylor >= 0 && p.ntaylor <= 4, "ntaylor must be in [0,4]");
  require(p.phase_law == WEM_PHASE_ISPC || p.phase_law == WEM_PHASE_EXACT_KZ, "phase_law must be 0 or 1");
  require(p.ngs >= 0 && p.ngr >= 0, "ngs/ngr must be >= 0");
  require(p.prop == WEM_PROP_SSF || p.prop == WEM_PROP_PSPI, "prop must be ssf or pspi");
  Geometry g;
  g.nx = p.nx;
  g.nz = p.nz;
  g.pad = p.pad;
  g.tap = p.tap;
  g.nxg = p.nx + 2 * p.pad;
  g.N = g.nxg + 2 * p.tap;
  require(p.nref <= g.nxg && g.nxg >= 2, "nref larger than the padded grid");
  frequencies(p, g.freq, g.bin, g.nt_pad);
  g.nbin = p.nbin ? p.nbin : g.nt_pad;
  for (int b : g.bin)
    require(b >= 0 && b < g.nt_pad && b < g.nbin, "frequency bin beyond the wavelet/data axis");
  device_indices(p, true, g.sx, g.sz);
  device_indices(p, false, g.rx, g.rz);
  g.ns = (int)g.sx.size();
  g.nr = (int)g.rx.size();
  g.gs = window(p.ngs);
  g.gr = window(p.ngr);
  // unitary DFT of the time-padded wavelet at the propagated bins
  // (FFT1_r.cpp:74-83 via PropParam.h:49-54)
  if (wavelet) {
    for (int b : g.bin) {
      cd acc = 0;
      for (int t = 0; t < p.nt; ++t) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * ((long long)b * t % g.nt_pad) / g.nt_pad;
        acc += (double)wavelet[t] * cd((double)std::cos(a), (double)std::sin(a));
      }
      g.wave_at.push_back(acc / std::sqrt((double)g.nt_pad));
    }
  }
  return g;
}

std::vector<cd> pad_model(const float* m, int nz, int nx, int pad, bool extend) {
  int nxg = nx + 2 * pad;
  std::vector<cd> out((size_t)nz * nxg);
  for (int iz = 0; iz < nz; ++iz) {
    const float* a = m + 2 * (size_t)iz * nx;
    cd* b = out.data() + (size_t)iz * nxg;
    for (int i = 0; i < nx; ++i) b[i + pad] = cd(a[2 * i], a[2 * i + 1]);
    cd bv = extend ? b[pad] : cd(0), ev = extend ? b[nx - 1 + pad] : cd(0);
    for (int i = 0; i < pad; ++i) {
      b[i] = bv;
      b[nx + i + pad] = ev;
    }
  }
  return out;
}

std::vector<double> k_grid(int N, double dx) {
  std::vector<double> k(N, 0.0);
  double dk = 2 * kPi / (dx * (N - 1));
  for (int i = 0; i < N / 2; ++i) k[i] = i * dk;
  for (int i = 1; i < N / 2; ++i) k[N - i] = -k[i];
  return k;
}

std::vector<double> taper(int nxg, int pad) {
  std::vector<double> t(nxg, 1.0);
  for (int i = 0; i < pad; ++i) {
    t[i] = .5 * (1 - std::cos(kPi * i / (pad - 1)));
    t[nxg - 1 - i] = t[i];
  }
  return t;
}

SliceTables make_slice_tables(const wem_params& p, const std::vector<cd>& sp, const std::vector<cd>& dp,
                              int nxg, bool need_born, const std::vector<cd>& sref,
                              const std::vector<signed char>& ref) {
  const int nz = p.nz;
  const size_t ng = (size_t)nz * nxg;
  require(p.nref <= 127, "nref must be <= 127");
  require(sref.size() == (size_t)nz * p.nref && ref.size() == ng, "RefSampler tables of the wrong size");
  SliceTables t;
  t.sref = sref;
  t.ref = ref;
  // SplitStep (SplitStep.cpp:11-15): q = (s - sref)/sqrt(sref) of the point's reference
  t.q.assign(ng, 0);
  for (int iz = 0; iz < nz; ++iz)
    for (int ix = 0; ix < nxg; ++ix) {
      int j = t.ref[(size_t)iz * nxg + ix];
      if (j < 0) continue;
      cd sr = t.sref[(size_t)iz * p.nref + j];
      t.q[(size_t)iz * nxg + ix] = (sp[(size_t)iz * nxg + ix] - sr) / std::sqrt(sr);
    }
  // Reflect (Reflect.h:19-26)
  t.rc.assign(ng, 0);
  for (int iz = 1; iz < nz; ++iz)
    for (int ix = 0; ix < nxg; ++ix) {
      size_t a = (size_t)iz * nxg + ix, b = a - nxg;
      cd u = dp[a] * std::sqrt(sp[b]), v = dp[b] * std::sqrt(sp[a]);
      t.rc[a] = (u - v) / (u + v);
    }
  if (!need_born) return t;
  // Scatter coefficients c_it = coef[it] (s - eps Re s)^(-1/2 - it)
  // (Scatter.cpp:77-86, coefficients Scatter.h:36)
  static const double coef[5] = {1., 1. / 2., 3. / 8., 5. / 16., 35. / 128.};
  const int nt = p.ntaylor + 1;
  t.sc.assign((size_t)nt * ng, 0);
  const double eps = (double)p.eps;
  for (int it = 0; it < nt; ++it)
    for (size_t i = 0; i < ng; ++i) {
      cd s = sp[i];
      t.sc[(size_t)it * ng + i] = coef[it] * std::pow(s - eps * s.real(), -.5 - it);
    }
  // dReflect coefficient pairs (dReflect.h:18-27, 40-47)
  t.a0.assign(ng, 0); t.b0.assign(ng, 0); t.a1.assign(ng, 0); t.b1.assign(ng, 0);
  for (int iz = 1; iz < nz; ++iz)
    for (int ix = 0; ix < nxg; ++ix) {
      size_t a = (size_t)iz * nxg + ix, b = a - nxg;
      cd v = std::pow(dp[a] * std::sqrt(sp[b]) + dp[b] * std::sqrt(sp[a]), -2.0);
      cd s1s2 = (dp[b] * dp[a]) / v;
      cd r1r2 = 2.0 * (sp[b] * sp[a]) / v;
      cd c = std::sqrt(sp[a] / sp[b]);
      t.a0[a] = c * s1s2;
      t.b0[a] = 1.0 / c * s1s2;
      t.a1[a] = dp[b] * r1r2;
      t.b1[a] = dp[a] * r1r2;
    }
  return t;
}

}  // namespace wg
