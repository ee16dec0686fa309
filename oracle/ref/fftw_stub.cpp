// Test infrastructure only: the FFTW 3 single-precision calls of the
// reference (fftwf_plan_dft_1d, fftwf_plan_many_dft of rank 1, execute,
// execute_dft) over a DFT evaluated in double precision: a recursive
// mixed-radix decimation in time (radices 2, 3, 5, 7; a direct sum over any
// larger prime factor) with twiddles from an exact table of the n-th roots
// of unity, so the transform adds no error beyond one float rounding per
// output (and double-precision rounding inside).  Unnormalised, FFTW's sign
// convention: out[k] = sum_j in[j] exp(sign 2 pi i j k / n).
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "fftw3.h"

namespace {

using cd = std::complex<double>;

struct Dft {
  int n, sign;
  std::vector<cd> w;  // exp(sign 2 pi i m / n), m < n
  std::vector<int> radix;
  Dft(int n_, int sign_) : n(n_), sign(sign_), w(n_) {
    const double pi = 3.14159265358979323846264338327950288;
    for (int m = 0; m < n; ++m) w[m] = cd(std::cos(2.0 * pi * m / n), sign * std::sin(2.0 * pi * m / n));
    int r = n;
    for (int p : {2, 3, 5, 7})
      while (r % p == 0) {
        radix.push_back(p);
        r /= p;
      }
    if (r > 1) radix.push_back(r);  // remaining factor: a direct sum
  }
  // out[k] = sum_j in[j * stride] w_n^(j k) for the length len = n / step
  // sub-transform (its roots are every step-th of this table)
  void run(const cd* in, int stride, cd* out, int len, int step, size_t level) const {
    if (len == 1) {
      out[0] = in[0];
      return;
    }
    const int p = radix[level], m = len / p;
    // p interleaved sub-transforms of length m
    for (int q = 0; q < p; ++q) run(in + (size_t)q * stride, stride * p, out + (size_t)q * m, m, step * p, level + 1);
    std::vector<cd> t(p);
    for (int k = 0; k < m; ++k) {
      for (int q = 0; q < p; ++q) t[q] = out[(size_t)q * m + k] * w[(size_t)q * k * step % n];
      for (int r = 0; r < p; ++r) {
        cd acc = 0.0;
        for (int q = 0; q < p; ++q) acc += t[q] * w[(size_t)q * (r * m) * step % n];
        out[(size_t)r * m + k] = acc;
      }
    }
  }
};

}  // namespace

struct fftwf_plan_s {
  int n, howmany, istride, idist, ostride, odist, sign;
  fftwf_complex *in, *out;
  Dft dft;
};

extern "C" {
void* fftwf_malloc(std::size_t n) { return std::malloc(n); }
void fftwf_free(void* p) { std::free(p); }

fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                               int istride, int idist, fftwf_complex* out, const int* onembed, int ostride,
                               int odist, int sign, unsigned) {
  if (rank != 1 || inembed || onembed) throw std::runtime_error("fftw stub: rank-1 plans without embeds only");
  return new fftwf_plan_s{n[0], howmany, istride, idist, ostride, odist, sign, in, out, Dft(n[0], sign)};
}

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags) {
  return fftwf_plan_many_dft(1, &n, 1, in, nullptr, 1, n, out, nullptr, 1, n, sign, flags);
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out) {
  const int n = p->n;
  std::vector<cd> x(n), y(n);
  for (int h = 0; h < p->howmany; ++h) {
    const fftwf_complex* a = in + (std::ptrdiff_t)h * p->idist;
    fftwf_complex* b = out + (std::ptrdiff_t)h * p->odist;
    for (int j = 0; j < n; ++j) x[j] = cd(a[(std::ptrdiff_t)j * p->istride][0], a[(std::ptrdiff_t)j * p->istride][1]);
    p->dft.run(x.data(), 1, y.data(), n, 1, 0);
    for (int k = 0; k < n; ++k) {
      b[(std::ptrdiff_t)k * p->ostride][0] = (float)y[k].real();
      b[(std::ptrdiff_t)k * p->ostride][1] = (float)y[k].imag();
    }
  }
}

void fftwf_execute(const fftwf_plan p) { fftwf_execute_dft(p, p->in, p->out); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
void fftwf_cleanup(void) {}
}
