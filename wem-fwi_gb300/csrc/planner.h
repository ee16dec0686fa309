// Host planner: everything the GPU passes need that depends only on the
// parameters and the background model, computed once per background in
// double precision.  Mirrors the per-task set-up of the reference drivers
// (propagator/src/wem_prop.cpp:19-50, born_prop.cpp:28-70): padded model,
// RefSampler, Reflect/dReflect coefficients, injection geometry, wavelet
// spectrum.
#pragma once
#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include "wemgpu.h"

namespace wg {

using cd = std::complex<double>;

struct Fail : std::runtime_error {
  int code;
  Fail(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
inline void require(bool ok, const std::string& m) {
  if (!ok) throw Fail(WEM_EINVAL, m);
}

// radix sequence of an FFT length: 4s, 2, then odd primes ascending
std::vector<int> fft_radices(int n);
// exp(-2 pi i t / n), t < n
std::vector<cd> twiddles(int n);

struct Geometry {
  int nx, nz, pad, tap, nxg, N, ns, nr;
  std::vector<float> freq;   // Hz, PropParam.h:75-78
  std::vector<int> bin;      // wavelet/data bin of each frequency
  int nt_pad = 0, nbin = 0;
  std::vector<int> sx, sz, rx, rz;  // device grid indices (unpadded x)
  // several source points per shot: shot s injects at sx[sptr[s] .. sptr[s+1])
  // and depth sz[s]; empty: one point per shot, sx[s]
  std::vector<int> sptr;
  std::vector<double> gs, gr;       // cos^2 spreading windows
  std::vector<cd> wave_at;          // wavelet spectrum at bin[f]
  int nfreq() const { return (int)freq.size(); }
};

Geometry make_geometry(const wem_params& p, const float* wavelet);
int count_frequencies(const wem_params& p);

// Background-dependent tables for one padded slowness/density slice.
struct SliceTables {
  std::vector<cd> sref;          // [nz][nref]
  std::vector<signed char> ref;  // [nz][nxg], -1 = no reference
  std::vector<cd> q;             // [nz][nxg] split-step (s - sref)/sqrt(sref)
  std::vector<cd> sc;            // [ntaylor+1][nz][nxg] Scatter coefficients
  std::vector<cd> rc;            // [nz][nxg] Reflect coefficients
  std::vector<cd> a0, b0, a1, b1;  // [nz][nxg] dReflect coefficient pairs
};

// sp, dp: padded [nz][nxg] slowness^2 and density; sref [nz][nref] and ref
// [nz][nxg]: the RefSampler tables of sp (from the device RefSampler)
SliceTables make_slice_tables(const wem_params& p, const std::vector<cd>& sp, const std::vector<cd>& dp,
                              int nxg, bool need_born, const std::vector<cd>& sref,
                              const std::vector<signed char>& ref);

// edge- or zero-pad [nz][nx] complex floats to [nz][nx+2pad] doubles
std::vector<cd> pad_model(const float* m, int nz, int nx, int pad, bool extend);

// k grid of the phase shift and the Scatter filter (Phshift_cmplx.cpp:13,21-24)
std::vector<double> k_grid(int N, double dx);
// cosine taper of width pad on a row of nxg (Taper.h:11-23)
std::vector<double> taper(int nxg, int pad);

}  // namespace wg
