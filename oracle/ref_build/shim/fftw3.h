// Stand-in for FFTW 3's complex 1-D interface as the reference uses it: plans of
// fftw_plan_dft_1d (FFTW_ESTIMATE), fftw_execute_dft on other arrays, fftw_malloc and
// fftw_free. The transform is the definition FFTW computes (unnormalised, sign -1
// forward and +1 backward), evaluated as a direct sum in extended precision by
// fftw_shim.cpp, so results carry FFTW's definition but not its rounding.
#pragma once
#include <cstddef>

typedef double fftw_complex[2];
typedef struct shim_fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);
