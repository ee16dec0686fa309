// Stand-in for the single-precision FFTW 3 API the reference calls (test
// infrastructure only).  Plans hold their layout; execution is a DFT in
// double precision, rounded to float once per output (fftw_stub.cpp).
#pragma once
#include <cstddef>
typedef float fftwf_complex[2];
struct fftwf_plan_s;
typedef fftwf_plan_s* fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE (0U)
extern "C" {
void* fftwf_malloc(std::size_t n);
void fftwf_free(void* p);
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                               int istride, int idist, fftwf_complex* out, const int* onembed, int ostride,
                               int odist, int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
void fftwf_cleanup(void);
}
