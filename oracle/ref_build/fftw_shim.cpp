// FFTW 3 stand-in for the reference build (test infrastructure, not product code).
//
// X[k] = sum_j x[j] exp(sign * 2 pi i j k / n), unnormalised, as FFTW defines
// fftw_plan_dft_1d. Evaluated as a direct sum in long double with twiddles
// exp(sign 2 pi i m / n) taken at m = (j k) mod n, so the result carries the
// definition with about 1e-18 relative rounding instead of FFTW's own
// (about 1e-16). In-place use (in == out) is supported, as the reference uses it.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "fftw3.h"

struct shim_fftw_plan_s {
    int n;
    int sign;
    std::vector<long double> c, s;  // cos / sin of sign * 2 pi m / n
};

fftw_plan fftw_plan_dft_1d(int n, fftw_complex*, fftw_complex*, int sign, unsigned) {
    fftw_plan p = new shim_fftw_plan_s;
    p->n = n;
    p->sign = sign;
    p->c.resize(n);
    p->s.resize(n);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int m = 0; m < n; ++m) {
        const long double a = two_pi * (long double)m / (long double)n;
        p->c[m] = cosl(a);
        p->s[m] = (long double)sign * sinl(a);
    }
    return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
    const int n = p->n;
    std::vector<long double> xr(n), xi(n);
    for (int j = 0; j < n; ++j) {
        xr[j] = in[j][0];
        xi[j] = in[j][1];
    }
    for (int k = 0; k < n; ++k) {
        long double re = 0.0L, im = 0.0L;
        long long m = 0;  // (j k) mod n
        for (int j = 0; j < n; ++j) {
            re += xr[j] * p->c[m] - xi[j] * p->s[m];
            im += xr[j] * p->s[m] + xi[j] * p->c[m];
            m += k;
            if (m >= n) m -= n;
        }
        out[k][0] = (double)re;
        out[k][1] = (double)im;
    }
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

void* fftw_malloc(size_t n) { return std::malloc(n); }

void fftw_free(void* p) { std::free(p); }
