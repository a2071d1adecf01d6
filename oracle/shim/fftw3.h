/* Test infrastructure (oracle): the subset of the FFTW3 API that the
 * reference's FFT.cpp uses (complex 1-D plans, execute, malloc/free), backed by
 * the project's CPU FFT (oracle/cpu_fft.hpp). */
#pragma once
#include <cstddef>
typedef double fftw_complex[2];
typedef struct owt_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
