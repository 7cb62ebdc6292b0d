// CPU ORACLE — test infrastructure, not the product.
//
// A plain-C++ FP64 restatement of Sassena's scattering-amplitude hot path, used
// only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg as the
// checker. Nothing in sassena_gb300/ links, loads or calls it.
//
// Parity status: PARITY UNPINNED. The reference ships no golden vectors for this
// path (its only test, tests/unit_broadcast.cpp, computes no numbers) and cannot
// be built here (MPI, Boost, FFTW3, HDF5, libxml2 and LAPACK are absent). This
// restatement is pinned instead by analytic known answers (static single atom,
// exact two-atom identity per direction, Gaussian self-diffusion), by the
// reference's own direct-vs-FFT correlation identity, and by an independent
// numpy restatement (oracle/numpy_oracle.py).
//
// Every function cites the reference file:line (paths inside the reference
// project) whose arithmetic it restates. FFTW (unpinned version, absent) is
// replaced by a self-written mixed-radix FP64 DFT of the SAME length 2*NF that
// the reference plans (all_vectors_scatter_device.cpp:52-53), so the transform
// sizes match even when NF is not a power of two.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off, no -march flags so x86
// and Arm hosts evaluate the same expressions).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

typedef std::complex<double> cd;

namespace {

// ---------------------------------------------------------------------------
// Mixed-radix FP64 DFT of arbitrary length (stand-in for fftw_execute_dft,
// smath.cpp:143,148). sign = -1 is FFTW_FORWARD, +1 is FFTW_BACKWARD; neither
// direction normalises, as in FFTW.
// ---------------------------------------------------------------------------
struct Dft {
    size_t n = 0;
    int sign = -1;
    std::vector<cd> w;  // w[k] = exp(sign*2*pi*i*k/n), k < n

    Dft(size_t n_, int sign_) : n(n_), sign(sign_), w(n_) {
        const long double two_pi = 6.283185307179586476925286766559L;
        for (size_t k = 0; k < n; ++k) {
            long double a = two_pi * (long double)k / (long double)n;
            w[k] = cd((double)cosl(a), (double)(sign * sinl(a)));
        }
    }

    static size_t smallest_factor(size_t m) {
        if (m % 4 == 0) return 4;
        if (m % 2 == 0) return 2;
        for (size_t p = 3; p * p <= m; p += 2)
            if (m % p == 0) return p;
        return m;
    }

    // out[k] = sum_j in[j*stride] * w^(j*k*(n/len)) for a sub-transform of length len.
    void rec(const cd* in, size_t len, size_t stride, cd* out, cd* scratch) const {
        if (len == 1) { out[0] = in[0]; return; }
        size_t p = smallest_factor(len);
        size_t m = len / p;
        // sub-transforms of the p interleaved sequences, into out[r*m .. r*m+m)
        for (size_t r = 0; r < p; ++r) rec(in + r * stride, m, stride * p, out + r * m, scratch);
        // combine: X[k + m*s] = sum_r w_len^{r(k+m*s)} Y_r[k]
        size_t step = n / len;  // w_len^e = w[(e*step) % n]
        for (size_t k = 0; k < m; ++k) {
            for (size_t s = 0; s < p; ++s) {
                cd acc = 0;
                size_t e = k + m * s;
                for (size_t r = 0; r < p; ++r) {
                    size_t idx = ((r * e) % len) * step;
                    acc += w[idx] * out[r * m + k];
                }
                scratch[k + m * s] = acc;
            }
        }
        for (size_t i = 0; i < len; ++i) out[i] = scratch[i];
    }

    void execute(cd* data) const {
        std::vector<cd> in(data, data + n), scratch(n);
        rec(in.data(), n, 1, data, scratch.data());
    }
};

// smath::auto_correlate_fftw(fftw_complex*, p1, p2, NF), smath.cpp:141-156.
// data holds 2*NF complex values, the upper NF already zero (alignpad,
// all_vectors_scatter_device.cpp:186-207).
void autocorrelate_fft(cd* data, size_t nf, const Dft& fwd, const Dft& bwd) {
    fwd.execute(data);
    for (size_t i = 0; i < 2 * nf; ++i) {
        double re = data[i].real() * data[i].real() + data[i].imag() * data[i].imag();
        data[i] = cd(re, 0.0);
    }
    bwd.execute(data);
    for (size_t i = 0; i < nf; ++i) {
        double factor = (1.0 / (2 * nf * (nf - i)));
        data[i] = cd(data[i].real() * factor, data[i].imag() * factor);
    }
}

// smath::auto_correlate_direct(fftw_complex*, N), smath.cpp:51-76. Note the sign
// of the imaginary part: the reference accumulates -a1r*a2i + a1i*a2r, i.e.
// sum_k a_k * conj(a_{k+tau}), the complex conjugate of the FFT method.
void autocorrelate_direct(cd* data, size_t nf) {
    std::vector<cd> local(data, data + nf);
    for (size_t tau = 0; tau < nf; ++tau) {
        double re = 0, im = 0;
        size_t last = nf - tau;
        for (size_t k = 0; k < last; ++k) {
            const cd& a1 = local[k];
            const cd& a2 = local[k + tau];
            re += a1.real() * a2.real() + a1.imag() * a2.imag();
            im += -a1.real() * a2.imag() + a1.imag() * a2.real();
        }
        data[tau] = cd(re / last, im / last);
    }
}

// smath::square_elements(fftw_complex*, N), smath.cpp:168-177.
void square_elements(cd* data, size_t nf) {
    for (size_t n = 0; n < nf; ++n) {
        double r = data[n].real() * data[n].real() + data[n].imag() * data[n].imag();
        data[n] = cd(r, 0.0);
    }
}

enum { DSP_AUTOCORRELATE = 0, DSP_SQUARE = 1, DSP_PLAIN = 2 };
enum { METHOD_FFTW = 0, METHOD_DIRECT = 1 };

// AllVectorsScatterDevice::dsp, all_vectors_scatter_device.cpp:209-229
// (SelfVectorsScatterDevice::dsp, self_vectors_scatter_device.cpp:115-135 is identical).
void dsp(cd* at, size_t nf, int type, int method, const Dft& fwd, const Dft& bwd) {
    if (type == DSP_AUTOCORRELATE) {
        if (method == METHOD_DIRECT) autocorrelate_direct(at, nf);
        else autocorrelate_fft(at, nf, fwd, bwd);
    } else if (type == DSP_SQUARE) {
        square_elements(at, nf);
    }
}

struct Accum {
    std::vector<cd> atfinal;
    cd afinal = 0, a2final = 0;
    explicit Accum(size_t nf) : atfinal(nf, 0.0) {}
    // AllVectorsScatterDevice::store, all_vectors_scatter_device.cpp:231-236
    // with smath::reduce (smath.cpp:239-247) and add_elements (smath.cpp:209-215).
    void store(const cd* at, size_t nf) {
        cd s = 0;
        for (size_t i = 0; i < nf; ++i) s += at[i];
        cd a = s * (1.0 / nf);
        afinal += a;
        a2final += a * std::conj(a);
        for (size_t n = 0; n < nf; ++n) atfinal[n] += at[n];
    }
    // normalisation, all_vectors_scatter_device.cpp:355-360 (smath.cpp:190-196)
    void finish(size_t nm, double* fqt, double* fq, double* fq2) {
        double factor = 1.0 / nm;
        for (size_t n = 0; n < atfinal.size(); ++n) {
            fqt[2 * n] = atfinal[n].real() * factor;
            fqt[2 * n + 1] = atfinal[n].imag() * factor;
        }
        cd a = afinal * factor, a2 = a2final * factor;
        fq[0] = a.real(); fq[1] = a.imag();
        fq2[0] = a2.real(); fq2[1] = a2.imag();
    }
};

template <class F>
void parallel_for(size_t n, int nthreads, F&& fn) {
    if (nthreads <= 1 || n <= 1) {
        for (size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<size_t> next(0);
    std::vector<std::thread> pool;
    int nt = (int)std::min<size_t>((size_t)nthreads, n);
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (size_t i = next++; i < n; i = next++) fn(i);
        });
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// Forward/backward FP64 DFT of length n in place (interleaved re,im).
void oracle_dft(double* data, size_t n, int sign) {
    Dft d(n, sign);
    d.execute(reinterpret_cast<cd*>(data));
}

// data: [2*nf][2] (upper half zero) -> first nf entries hold C(tau). smath.cpp:141-156.
void oracle_autocorrelate_fftw(double* data, size_t nf) {
    Dft fwd(2 * nf, -1), bwd(2 * nf, +1);
    autocorrelate_fft(reinterpret_cast<cd*>(data), nf, fwd, bwd);
}

// data: [nf][2]. smath.cpp:51-76.
void oracle_autocorrelate_direct(double* data, size_t nf) {
    autocorrelate_direct(reinterpret_cast<cd*>(data), nf);
}

// Coherent ("all") vectors device for a list of q-vectors.
//   coords      frame-major float32 [nf][na][3] (data_stager.cpp:110-114)
//   sub_offsets [nq+1] CSR offsets into subvectors (init_subvectors,
//               abstract_vectors_scatter_device.cpp:112-175)
//   subvectors  [nsub][3] double
//   factors     [nq][na] double, b_j(|q|) per q (scatter_factors.cpp:56-78)
//   outputs     fqt [nq][nf][2], fq [nq][2], fq2 [nq][2]
// Follows AllVectorsScatterDevice::compute (all_vectors_scatter_device.cpp:238-361,
// single-partition branch :259-285) and ::scatter (:388-439). Sub-vectors are
// scattered in parallel and then dsp+store run in sub-vector order, as the
// reference's main thread does (:270-279).
int oracle_all_vectors(const float* coords, size_t nf, size_t na, size_t nq,
                       const size_t* sub_offsets, const double* subvectors,
                       const double* factors, int dsp_type, int dsp_method,
                       int nthreads, double* fqt, double* fq, double* fq2) {
    if (nf == 0 || na == 0) return 1;
    Dft fwd(2 * nf, -1), bwd(2 * nf, +1);
    for (size_t iq = 0; iq < nq; ++iq) {
        size_t m0 = sub_offsets[iq], m1 = sub_offsets[iq + 1];
        size_t nm = m1 - m0;
        if (nm == 0) return 1;
        const double* sfs = factors + iq * na;
        Accum acc(nf);
        std::vector<cd> at(nm * 2 * nf);
        // scatter (:388-439): for each frame, sequential sum over atoms in FP64
        parallel_for(nm, nthreads, [&](size_t m) {
            const double* q = subvectors + 3 * (m0 + m);
            double qx = q[0], qy = q[1], qz = q[2];
            cd* p_a = &at[m * 2 * nf];
            for (size_t fi = 0; fi < nf; ++fi) {
                const float* p_data = coords + fi * na * 3;
                double Ar = 0, Ai = 0;
                for (size_t j = 0; j < na; ++j) {
                    double esf = sfs[j];
                    float x = p_data[3 * j], y = p_data[3 * j + 1], z = p_data[3 * j + 2];
                    double p = x * qx + y * qy + z * qz;
                    Ar += esf * cos(p);
                    Ai += esf * sin(p);
                }
                p_a[fi] = cd(Ar, Ai);
            }
            // alignpad (:186-207) zero-fills [nf, 2nf); dsp is per sub-vector
            for (size_t fi = nf; fi < 2 * nf; ++fi) p_a[fi] = 0;
            dsp(p_a, nf, dsp_type, dsp_method, fwd, bwd);
        });
        for (size_t m = 0; m < nm; ++m) acc.store(&at[m * 2 * nf], nf);
        acc.finish(nm, fqt + iq * nf * 2, fq + iq * 2, fq2 + iq * 2);
    }
    return 0;
}

// Incoherent ("self") vectors device. Follows SelfVectorsScatterDevice::compute
// (self_vectors_scatter_device.cpp:145-239): for each atom (outer) and each
// sub-vector (inner) the series s*(cos p, sin p) over all frames (:288-322),
// zero-padded to 2nf, dsp, store; the result is SUMMED over atoms and scaled by
// 1/NM (:233-238). Coordinates are read frame-major here; the reference first
// transposes them atom-major (DataStagerByAtom, data_stager.cpp:249-338), which
// changes no value.
int oracle_self_vectors(const float* coords, size_t nf, size_t na, size_t nq,
                        const size_t* sub_offsets, const double* subvectors,
                        const double* factors, int dsp_type, int dsp_method,
                        int nthreads, double* fqt, double* fq, double* fq2) {
    if (nf == 0 || na == 0) return 1;
    Dft fwd(2 * nf, -1), bwd(2 * nf, +1);
    for (size_t iq = 0; iq < nq; ++iq) {
        size_t m0 = sub_offsets[iq], m1 = sub_offsets[iq + 1];
        size_t nm = m1 - m0;
        if (nm == 0) return 1;
        const double* sfs = factors + iq * na;
        Accum acc(nf);
        std::vector<cd> at(nm * 2 * nf);
        for (size_t ai = 0; ai < na; ++ai) {
            double s = sfs[ai];
            parallel_for(nm, nthreads, [&](size_t mi) {
                const double* q = subvectors + 3 * (m0 + mi);
                double qx = q[0], qy = q[1], qz = q[2];
                cd* p = &at[mi * 2 * nf];
                for (size_t j = 0; j < nf; ++j) {
                    const float* r = coords + (j * na + ai) * 3;
                    float x1 = r[0], y1 = r[1], z1 = r[2];
                    double p1 = x1 * qx + y1 * qy + z1 * qz;
                    double sp1 = sin(p1);
                    double cp1 = cos(p1);
                    p[j] = cd(s * cp1, s * sp1);
                }
                for (size_t j = nf; j < 2 * nf; ++j) p[j] = 0;
                dsp(p, nf, dsp_type, dsp_method, fwd, bwd);
            });
            for (size_t mi = 0; mi < nm; ++mi) acc.store(&at[mi * 2 * nf], nf);
        }
        acc.finish(nm, fqt + iq * nf * 2, fq + iq * 2, fq2 + iq * 2);
    }
    return 0;
}

// Raw coherent amplitudes A[m][f] (AllVectorsScatterDevice::scatter,
// all_vectors_scatter_device.cpp:418-438) for the listed sub-vectors:
// out [nsub][nf][2]. Used to check the phase sum on its own.
int oracle_amplitudes(const float* coords, size_t nf, size_t na, size_t nsub,
                      const double* subvectors, const size_t* sub_shell,
                      const double* factors, int nthreads, double* out) {
    parallel_for(nsub, nthreads, [&](size_t m) {
        const double* q = subvectors + 3 * m;
        const double* sfs = factors + sub_shell[m] * na;
        for (size_t fi = 0; fi < nf; ++fi) {
            const float* p_data = coords + fi * na * 3;
            double Ar = 0, Ai = 0;
            for (size_t j = 0; j < na; ++j) {
                float x = p_data[3 * j], y = p_data[3 * j + 1], z = p_data[3 * j + 2];
                double p = x * q[0] + y * q[1] + z * q[2];
                Ar += sfs[j] * cos(p);
                Ai += sfs[j] * sin(p);
            }
            out[(m * nf + fi) * 2] = Ar;
            out[(m * nf + fi) * 2 + 1] = Ai;
        }
    });
    return 0;
}

// DatabaseSFactorsParameters::get, database.cpp:469-528 (types 0 and 2; type 1,
// Slater, is outside this path and returns NAN).
double oracle_sfactor(int type, const double* v, size_t nv, double q) {
    if (type == 0) return nv > 0 ? v[0] : NAN;
    if (type == 2) {
        if (nv < 9) return NAN;
        double den = 0.0;
        den += v[0] * exp(-v[1] * q * q);
        den += v[2] * exp(-v[3] * q * q);
        den += v[4] * exp(-v[5] * q * q);
        den += v[6] * exp(-v[7] * q * q);
        den += v[8];
        return den;
    }
    return NAN;
}

// DatabaseVolumesParameters::get, database.cpp:391-411. The reference evaluates
// powf (float) on the radius; that rounding is kept.
double oracle_volume(int type, const double* v, size_t nv) {
    if (nv < 1) return NAN;
    if (type == 0) return v[0];
    if (type == 1) return (4.0 / 3.0) * M_PI * powf((float)v[0], 3);
    if (type == 2) return sqrt(powf((float)M_PI, 3)) * powf((float)v[0], 3);
    return NAN;
}

// DatabaseExlusionParameters::get, database.cpp:430-450 (powf kept).
double oracle_exclusion(int type, const double* v, size_t nv, double effvolume, double q) {
    if (nv < 1) return NAN;
    if (type == 0) return v[0];
    if (type == 1) return effvolume * v[0];
    if (type == 2)
        return effvolume * exp(-1.0 * powf((float)effvolume, 2.0f / 3.0f) * powf((float)q, 2) / (4 * M_PI)) * v[0];
    return NAN;
}

// ScatteringVectorsParameters::create_from_scans for ONE scan,
// parameters.cpp:1125-1159: q_k = from + ((k/(points-1))^exponent)*(to-from)
// along base, with the reference's float powf. out must hold 3*points doubles.
// Returns the number of vectors written.
size_t oracle_scan(const double* base, double from, double to, size_t points,
                   double exponent, double* out) {
    size_t n = 0;
    auto push = [&](double s) {
        out[3 * n] = s * base[0]; out[3 * n + 1] = s * base[1]; out[3 * n + 2] = s * base[2];
        ++n;
    };
    if (points == 0) return 0;
    if (points == 1) { push((from + to) / 2); return n; }
    if (points == 2) { push(from); push(to); return n; }
    push(from);
    for (size_t j = 1; j < points - 1; ++j) {
        double scal = from + powf((float)(j * 1.0 / (points - 1)), (float)exponent) * (to - from);
        push(scal);
    }
    push(to);
    return n;
}

}  // extern "C"
