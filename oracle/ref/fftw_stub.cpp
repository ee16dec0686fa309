// Test infrastructure only: the FFTW 3 single-precision calls of the
// reference (fftwf_plan_dft_1d, fftwf_plan_many_dft of rank 1, execute,
// execute_dft) over a plain DFT evaluated in double precision with an exact
// twiddle table, so the transform adds no error beyond one float rounding
// per output.  Unnormalised, FFTW's sign convention: out[k] = sum_j in[j]
// exp(sign 2 pi i j k / n).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "fftw3.h"

struct fftwf_plan_s {
  int n, howmany, istride, idist, ostride, odist, sign;
  fftwf_complex *in, *out;
  std::vector<double> c, s;  // cos, sin of 2 pi m / n
};

extern "C" {
void* fftwf_malloc(std::size_t n) { return std::malloc(n); }
void fftwf_free(void* p) { std::free(p); }

fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                               int istride, int idist, fftwf_complex* out, const int* onembed, int ostride,
                               int odist, int sign, unsigned) {
  if (rank != 1 || inembed || onembed) throw std::runtime_error("fftw stub: rank-1 plans without embeds only");
  auto* p = new fftwf_plan_s{n[0], howmany, istride, idist, ostride, odist, sign, in, out, {}, {}};
  const double pi = 3.14159265358979323846264338327950288;
  p->c.resize(p->n);
  p->s.resize(p->n);
  for (int m = 0; m < p->n; ++m) {
    p->c[m] = std::cos(2.0 * pi * m / p->n);
    p->s[m] = std::sin(2.0 * pi * m / p->n);
  }
  return p;
}

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags) {
  return fftwf_plan_many_dft(1, &n, 1, in, nullptr, 1, n, out, nullptr, 1, n, sign, flags);
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out) {
  const int n = p->n;
  std::vector<double> xr(n), xi(n);
  for (int h = 0; h < p->howmany; ++h) {
    const fftwf_complex* a = in + (std::ptrdiff_t)h * p->idist;
    fftwf_complex* b = out + (std::ptrdiff_t)h * p->odist;
    for (int j = 0; j < n; ++j) {
      xr[j] = a[(std::ptrdiff_t)j * p->istride][0];
      xi[j] = a[(std::ptrdiff_t)j * p->istride][1];
    }
    for (int k = 0; k < n; ++k) {
      double re = 0.0, im = 0.0;
      long long m = 0;
      for (int j = 0; j < n; ++j) {
        const double c = p->c[m], s = p->sign * p->s[m];
        re += xr[j] * c - xi[j] * s;
        im += xr[j] * s + xi[j] * c;
        m += k;
        if (m >= n) m -= n;
      }
      b[(std::ptrdiff_t)k * p->ostride][0] = (float)re;
      b[(std::ptrdiff_t)k * p->ostride][1] = (float)im;
    }
  }
}

void fftwf_execute(const fftwf_plan p) { fftwf_execute_dft(p, p->in, p->out); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
void fftwf_cleanup(void) {}
}
