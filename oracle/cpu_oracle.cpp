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
#include <chrono>
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

// Seconds spent (summed over worker threads) in the phase sum and in dsp by the last
// vectors call: the correlation share of the CPU time. Two clock reads per series.
std::atomic<long long> g_scatter_ns(0), g_dsp_ns(0);
inline long long now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

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

// ---------------------------------------------------------------------------
// Multipole devices: coordinate representations and special functions.
// ---------------------------------------------------------------------------

// SphericalCoor3D(CartesianCoor3D), src/math/coor3d.cpp:168-215: r, theta = acos(z/r),
// phi in [0, 2 pi) from atan(y/x) with quadrant corrections; the staged values are
// rounded to float (coor_t, include/common.hpp:38; data_stager.cpp:110-114).
void to_spherical(float xf, float yf, float zf, float& r_out, float& phi_out, float& theta_out) {
    double x = xf, y = yf, z = zf;
    double r = sqrt(pow(x, 2) + pow(y, 2) + pow(z, 2));
    double theta = 0, phi = 0;
    if (r != 0) {
        theta = acos(z / r);
        if (x != 0.0) {
            phi = atan(y / x);
            if (x < 0.0) phi += M_PI;
            else if (y < 0.0) phi += 2 * M_PI;
        } else if (y != 0.0) {
            if (y > 0) phi = M_PI_2;
            if (y < 0) phi = 3 * M_PI_2;
        }
    }
    r_out = (float)r;
    phi_out = (float)phi;
    theta_out = (float)theta;
}

struct V3 {
    double x, y, z;
};
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double length(V3 a) { return sqrt(pow(a.x, 2) + pow(a.y, 2) + pow(a.z, 2)); }
V3 divide(V3 a, double l) { return {a.x / l, a.y / l, a.z / l}; }

// CartesianVectorBase(axis), coor3d.cpp:278-295: e_r, e_phi, e_z.
void axis_base(const double* axis, V3* base) {
    V3 ek{0, 0, 1}, ej{0, 1, 0};
    V3 a{axis[0], axis[1], axis[2]};
    V3 ez = divide(a, length(a));
    V3 ekez = cross(ek, ez);
    if (length(ekez) == 0) ekez = cross(ej, ez);
    V3 er = divide(ekez, length(ekez));
    V3 ezer = cross(ez, er);
    V3 ephi = divide(ezer, length(ezer));
    base[0] = er;
    base[1] = ephi;
    base[2] = ez;
}

// CylinderCoor3D(CartesianCoor3D), coor3d.cpp:116-141, with the reference's float
// sign(float, float) (include/math/coor3d.hpp:30) for the x < 0 branch.
void to_cylinder(V3 c, double& r, double& phi, double& z) {
    r = sqrt(pow(c.x, 2) + pow(c.y, 2));
    auto fsign = [](float a, float b) { return (b < 0.0) ? -a : a; };
    if (c.x != 0.0) {
        phi = atan(c.y / c.x);
        if (c.x < 0.0) phi = fsign((float)M_PI, (float)c.y) + phi;
    } else if (c.y != 0.0) {
        phi = fsign((float)M_PI_2, (float)c.y);
    } else {
        phi = 0.0;
    }
    phi = phi < 0 ? 2 * M_PI + phi : phi;
    z = c.z;
}

// Spherical Bessel functions j_0 .. j_L at x >= 0 (the reference calls
// boost::math::sph_bessel, multipole_scatter_device.cpp:484; Boost is absent here and
// this is an independent implementation): power series for x < 1/2, the upward
// recurrence j_{l+1} = (2l+1)/x j_l - j_{l-1} where it is stable (every l < x), and
// otherwise Miller's downward recurrence from order L + 32, normalised by j_0 or j_1.
void sph_bessel_all(int L, double x, double* j) {
    if (x == 0) {
        j[0] = 1;
        for (int l = 1; l <= L; ++l) j[l] = 0;
        return;
    }
    if (x < 0.5) {
        double xl = 1;  // x^l / (2l+1)!!
        for (int l = 0; l <= L; ++l) {
            if (l > 0) xl *= x / (2 * l + 1);
            double term = 1, sum = 1;
            for (int k = 1; k < 40; ++k) {
                term *= -x * x / (2.0 * k * (2 * l + 2 * k + 1));
                sum += term;
                if (fabs(term) < 1e-18 * fabs(sum)) break;
            }
            j[l] = xl * sum;
        }
        return;
    }
    const double j0 = sin(x) / x, j1 = sin(x) / (x * x) - cos(x) / x;
    if (x > L) {
        j[0] = j0;
        if (L >= 1) j[1] = j1;
        for (int l = 1; l < L; ++l) j[l + 1] = (2 * l + 1) / x * j[l] - j[l - 1];
        return;
    }
    const int N = L + 32;
    double fp = 0, f = 1e-250;  // f_{n+1}, f_n
    for (int n = N; n >= 1; --n) {
        double fm = (2 * n + 1) / x * f - fp;  // f_{n-1}
        fp = f;
        f = fm;
        if (n - 1 <= L) j[n - 1] = f;
        if (fabs(f) > 1e200) {
            for (int l = n - 1; l <= L; ++l) j[l] *= 1e-200;
            fp *= 1e-200;
            f *= 1e-200;
        }
    }
    const double scale = fabs(j0) >= fabs(j1) ? j0 / j[0] : j1 / j[1];
    for (int l = 0; l <= L; ++l) j[l] *= scale;
}

// Normalised associated Legendre functions with the Condon-Shortley phase,
// Pbar_l^m(x) = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!) P_l^m(x), 0 <= m <= l <= L, by the
// standard recurrences: Pbar_m^m = -sqrt((2m+1)/(2m)) sqrt(1-x^2) Pbar_{m-1}^{m-1},
// Pbar_{m+1}^m = sqrt(2m+3) x Pbar_m^m and
// Pbar_l^m = a_lm (x Pbar_{l-1}^m - b_lm Pbar_{l-2}^m). P is indexed l(l+1)/2 + m.
void legendre_norm(int L, double x, double* P) {
    auto at = [](int l, int m) { return l * (l + 1) / 2 + m; };
    const double s = sqrt((1 - x) * (1 + x));
    P[0] = sqrt(1.0 / (4 * M_PI));
    for (int m = 1; m <= L; ++m) P[at(m, m)] = -sqrt((2.0 * m + 1) / (2.0 * m)) * s * P[at(m - 1, m - 1)];
    for (int m = 0; m < L; ++m) P[at(m + 1, m)] = sqrt(2.0 * m + 3) * x * P[at(m, m)];
    for (int m = 0; m <= L; ++m)
        for (int l = m + 2; l <= L; ++l) {
            const double a = sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
            const double b = sqrt((((double)l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1));
            P[at(l, m)] = a * (x * P[at(l - 1, m)] - b * P[at(l - 2, m)]);
        }
}

// conj(Y_l^m(theta, phi)) with Y_l^{-m} = (-1)^m conj(Y_l^m) (the reference calls
// conj(boost::math::spherical_harmonic(l, m, theta, phi)), multipole_scatter_device.cpp:488).
cd conj_ylm(const double* P, int l, int m, double phi) {
    const int am = m < 0 ? -m : m;
    double v = P[l * (l + 1) / 2 + am];
    if (m < 0 && (am & 1)) v = -v;
    return cd(v * cos(m * phi), -v * sin(m * phi));
}

// J_0(x) and J_1(x) for x >= 25 from Hankel's asymptotic expansion,
// J_nu(x) = sqrt(2/(pi x)) (P cos chi - Q sin chi), chi = x - (nu/2 + 1/4) pi, with
// P, Q the alternating series in a_k(nu) = prod_{i<=k} (4 nu^2 - (2i-1)^2) / (k! 8^k x^k);
// cos chi and sin chi are formed from cos x and sin x so that no multiple of pi is
// subtracted from x.
void bessel01_asymptotic(double x, double& j0, double& j1) {
    double pq[2][2];
    for (int nu = 0; nu < 2; ++nu) {
        const double mu = 4.0 * nu * nu;
        double a = 1, P = 1, Q = 0;
        for (int k = 1; k < 60; ++k) {
            const double next = a * (mu - (2.0 * k - 1) * (2.0 * k - 1)) / (k * 8.0 * x);
            if (fabs(next) > fabs(a) && k > 2) break;  // the asymptotic series starts to diverge
            a = next;
            // k odd: into Q with sign (-1)^((k-1)/2); k even: into P with sign (-1)^(k/2)
            if (k & 1) Q += (((k - 1) / 2) & 1 ? -a : a);
            else P += ((k / 2) & 1 ? -a : a);
            if (fabs(a) < 1e-18) break;
        }
        pq[nu][0] = P;
        pq[nu][1] = Q;
    }
    const double c = cos(x), s = sin(x), h = sqrt(0.5), amp = sqrt(2.0 / (M_PI * x));
    const double c0 = h * (c + s), s0 = h * (s - c);   // cos, sin of x - pi/4
    const double c1 = h * (s - c), s1 = -h * (s + c);  // cos, sin of x - 3 pi/4
    j0 = amp * (pq[0][0] * c0 - pq[0][1] * s0);
    j1 = amp * (pq[1][0] * c1 - pq[1][1] * s1);
}

// Bessel functions of the first kind J_0 .. J_N at x >= 0 (the reference calls
// boost::math::cyl_bessel_j, multipole_scatter_device.cpp:956-975; independent
// implementation). For x >= 25 above every order needed: J_0, J_1 from the asymptotic
// expansion and the upward recurrence J_{n+1} = (2n/x) J_n - J_{n-1}, stable for n < x.
// Otherwise Miller's downward recurrence J_{n-1} = (2n/x) J_n - J_{n+1} from an even
// order M above max(N, x), normalised by J_0 + 2 sum_k J_2k = 1.
void cyl_bessel_all(int N, double x, double* J) {
    if (x == 0) {
        J[0] = 1;
        for (int n = 1; n <= N; ++n) J[n] = 0;
        return;
    }
    if (x >= 25 && x > N) {
        double j0, j1;
        bessel01_asymptotic(x, j0, j1);
        J[0] = j0;
        if (N >= 1) J[1] = j1;
        for (int n = 1; n < N; ++n) J[n + 1] = 2.0 * n / x * J[n] - J[n - 1];
        return;
    }
    const double top = std::max((double)N, x);
    int M = (int)(top + 20 + 2 * sqrt(top + 10));
    M += M & 1;
    double fp = 0, f = 1e-250, norm = 0;  // f_{n+1}, f_n
    if (M <= N) J[M] = f;
    for (int n = M; n >= 1; --n) {
        double fm = 2.0 * n / x * f - fp;  // f_{n-1}
        fp = f;
        f = fm;
        if (n - 1 <= N) J[n - 1] = f;
        if ((n - 1) % 2 == 0) norm += (n - 1 == 0 ? 1.0 : 2.0) * f;
        if (fabs(f) > 1e200) {
            for (int k = n - 1; k <= N && k <= M; ++k) J[k] *= 1e-200;
            fp *= 1e-200;
            f *= 1e-200;
            norm *= 1e-200;
        }
    }
    for (int n = 0; n <= N; ++n) J[n] /= norm;
}

void finish_factor(Accum& acc, double factor, double* fqt, double* fq, double* fq2) {
    for (size_t n = 0; n < acc.atfinal.size(); ++n) {
        fqt[2 * n] = acc.atfinal[n].real() * factor;
        fqt[2 * n + 1] = acc.atfinal[n].imag() * factor;
    }
    cd a = acc.afinal * factor, a2 = acc.a2final * factor;
    fq[0] = a.real();
    fq[1] = a.imag();
    fq2[0] = a2.real();
    fq2[1] = a2.imag();
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
// Thread-seconds of the last oracle_all_vectors / oracle_self_vectors call spent in the
// phase sum (scatter) and in dsp (correlation).
void oracle_last_split(double* scatter_s, double* dsp_s) {
    *scatter_s = g_scatter_ns.load() * 1e-9;
    *dsp_s = g_dsp_ns.load() * 1e-9;
}

int oracle_all_vectors(const float* coords, size_t nf, size_t na, size_t nq,
                       const size_t* sub_offsets, const double* subvectors,
                       const double* factors, int dsp_type, int dsp_method,
                       int nthreads, double* fqt, double* fq, double* fq2) {
    g_scatter_ns = 0;
    g_dsp_ns = 0;
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
            const long long t0 = now_ns();
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
            const long long t1 = now_ns();
            dsp(p_a, nf, dsp_type, dsp_method, fwd, bwd);
            g_scatter_ns += t1 - t0;
            g_dsp_ns += now_ns() - t1;
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
    g_scatter_ns = 0;
    g_dsp_ns = 0;
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
                const long long t0 = now_ns();
                for (size_t j = 0; j < nf; ++j) {
                    const float* r = coords + (j * na + ai) * 3;
                    float x1 = r[0], y1 = r[1], z1 = r[2];
                    double p1 = x1 * qx + y1 * qy + z1 * qz;
                    double sp1 = sin(p1);
                    double cp1 = cos(p1);
                    p[j] = cd(s * cp1, s * sp1);
                }
                for (size_t j = nf; j < 2 * nf; ++j) p[j] = 0;
                const long long t1 = now_ns();
                dsp(p, nf, dsp_type, dsp_method, fwd, bwd);
                g_scatter_ns += t1 - t0;
                g_dsp_ns += now_ns() - t1;
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
    // the reference's sqrt takes the float overload (std::sqrt after "using namespace std"), so the
    // whole product is a float
    if (type == 2) return (double)(std::sqrt(powf((float)M_PI, 3)) * powf((float)v[0], 3));
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

// ---------------------------------------------------------------------------
// Multipole devices (coherent). coords are Cartesian float32 frames [nf][na][3]
// as the stager delivers them; the representation the reference stages instead
// (SPHERICAL / CYLINDRICAL, multipole_scatter_device.cpp:53, :524, converted by
// coordinate_sets.cpp:359-363 and rounded to float) is formed here.
//   qvectors [nq][3], factors [nq][na], moments [nmom][2] (major, minor)
// ---------------------------------------------------------------------------

// MPSphereScatterDevice::compute / ::scatter, multipole_scatter_device.cpp:278-401,
// 428-497: A_lm(t) = sum_j 4 pi i^l b_j j_l(|q| r_j) conj(Y_l^m(theta_j, phi_j)), dsp
// and store per moment, all results times 1/(4 pi).
int oracle_mp_sphere(const float* coords, size_t nf, size_t na, size_t nq, const double* qvectors,
                     const double* factors, size_t nmom, const int* moments, int dsp_type,
                     int dsp_method, int nthreads, double* fqt, double* fq, double* fq2) {
    if (nf == 0 || na == 0 || nmom == 0) return 1;
    int L = 0;
    for (size_t k = 0; k < nmom; ++k) {
        if (moments[2 * k] < 0 || abs(moments[2 * k + 1]) > moments[2 * k]) return 1;
        L = std::max(L, moments[2 * k]);
    }
    std::vector<float> sph(nf * na * 3);  // r, phi, theta
    for (size_t i = 0; i < nf * na; ++i)
        to_spherical(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2], sph[3 * i], sph[3 * i + 1],
                     sph[3 * i + 2]);
    Dft fwd(2 * nf, -1), bwd(2 * nf, +1);
    const size_t np = (size_t)(L + 1) * (L + 2) / 2;
    for (size_t iq = 0; iq < nq; ++iq) {
        const double* q = qvectors + 3 * iq;
        const double ql = sqrt(pow(q[0], 2) + pow(q[1], 2) + pow(q[2], 2));
        const double* sfs = factors + iq * na;
        Accum acc(nf);
        std::vector<cd> at(nmom * 2 * nf);
        parallel_for(nf, nthreads, [&](size_t fi) {
            std::vector<double> jl(L + 1), P(np);
            std::vector<cd> A(nmom, 0.0);
            for (size_t j = 0; j < na; ++j) {
                const float* c = &sph[(fi * na + j) * 3];
                double r = c[0], phi = c[1], theta = c[2];
                sph_bessel_all(L, ql * r, jl.data());
                legendre_norm(L, cos(theta), P.data());
                for (size_t k = 0; k < nmom; ++k) {
                    int l = moments[2 * k], m = moments[2 * k + 1];
                    static const cd il[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
                    cd fmpiilesf = 4 * M_PI * il[l & 3] * sfs[j];
                    A[k] += fmpiilesf * jl[l] * conj_ylm(P.data(), l, m, phi);
                }
            }
            for (size_t k = 0; k < nmom; ++k) at[k * 2 * nf + fi] = A[k];
        });
        parallel_for(nmom, nthreads, [&](size_t k) {
            cd* p = &at[k * 2 * nf];
            for (size_t fi = nf; fi < 2 * nf; ++fi) p[fi] = 0;
            dsp(p, nf, dsp_type, dsp_method, fwd, bwd);
        });
        for (size_t k = 0; k < nmom; ++k) acc.store(&at[k * 2 * nf], nf);
        finish_factor(acc, 1.0 / (4 * M_PI), fqt + iq * nf * 2, fq + iq * 2, fq2 + iq * 2);
    }
    return 0;
}

// MPCylinderScatterDevice::compute / ::scatter, multipole_scatter_device.cpp:750-872,
// 900-986: coordinates and q in the cylinder frame of `axis`; per moment (l, m) with
// m in 0..3 a Bessel J_{2l} (m = 0, 1) or J_{2l-1} (m = 2, 3) term times cos / sin of the
// order times (phi - phi_q), the phase exp(i s z q_z) with s the sign of z q_z (the
// reference's parallel_sign), the factor sqrt(2 pi); all results times 1/(2 pi).
int oracle_mp_cylinder(const float* coords, size_t nf, size_t na, size_t nq, const double* qvectors,
                       const double* factors, size_t nmom, const int* moments, const double* axis,
                       int dsp_type, int dsp_method, int nthreads, double* fqt, double* fq, double* fq2) {
    if (nf == 0 || na == 0 || nmom == 0) return 1;
    int N = 0;
    for (size_t k = 0; k < nmom; ++k) {
        int l = moments[2 * k], m = moments[2 * k + 1];
        if (l < 0 || m < 0 || m > 3 || (l == 0 && m != 0)) return 1;
        N = std::max(N, 2 * l);
    }
    V3 base[3];
    axis_base(axis, base);
    std::vector<float> cyl(nf * na * 3);  // r, phi, z (float, as staged)
    for (size_t i = 0; i < nf * na; ++i) {
        V3 c{(double)coords[3 * i], (double)coords[3 * i + 1], (double)coords[3 * i + 2]};
        V3 pr{dot(c, base[0]), dot(c, base[1]), dot(c, base[2])};
        double r, phi, z;
        to_cylinder(pr, r, phi, z);
        cyl[3 * i] = (float)r;
        cyl[3 * i + 1] = (float)phi;
        cyl[3 * i + 2] = (float)z;
    }
    Dft fwd(2 * nf, -1), bwd(2 * nf, +1);
    for (size_t iq = 0; iq < nq; ++iq) {
        V3 qv{qvectors[3 * iq], qvectors[3 * iq + 1], qvectors[3 * iq + 2]};
        V3 qp{dot(qv, base[0]), dot(qv, base[1]), dot(qv, base[2])};
        double qr, qphi, qz;
        to_cylinder(qp, qr, qphi, qz);
        const double* sfs = factors + iq * na;
        Accum acc(nf);
        std::vector<cd> at(nmom * 2 * nf);
        parallel_for(nf, nthreads, [&](size_t fi) {
            std::vector<double> J(N + 1);
            std::vector<cd> A(nmom, 0.0);
            for (size_t j = 0; j < na; ++j) {
                const float* c = &cyl[(fi * na + j) * 3];
                double r = c[0], phi = c[1], z = c[2];
                double esf = sfs[j];
                double parallel_sign = 1.0;
                if ((z != 0) && (qz != 0)) parallel_sign = (z * qz) / (fabs(z) * fabs(qz));
                cd expi = std::exp(cd(0, parallel_sign * z * qz));
                double p = r * qr;
                double psiphi = phi - qphi;
                cyl_bessel_all(N, p, J.data());
                for (size_t k = 0; k < nmom; ++k) {
                    int l = moments[2 * k], m = moments[2 * k + 1];
                    if (m == 0 && l == 0) {
                        A[k] += expi * J[0] * esf;
                    } else if (m == 0 || m == 1) {
                        cd fac1 = 2.0 * ((l & 1) ? -1.0 : 1.0) * J[2 * l];
                        double t = m == 0 ? cos(2 * l * psiphi) : sin(2 * l * psiphi);
                        A[k] += sqrt(0.5) * fac1 * expi * t * esf;
                    } else {
                        cd fac2 = cd(0, 1.0) * (2.0 * (((l - 1) & 1) ? -1.0 : 1.0) * J[2 * l - 1]);
                        double t = m == 2 ? cos((2 * l - 1) * psiphi) : sin((2 * l - 1) * psiphi);
                        A[k] += sqrt(0.5) * fac2 * expi * t * esf;
                    }
                }
            }
            const double norm = sqrt(2 * M_PI);
            for (size_t k = 0; k < nmom; ++k) at[k * 2 * nf + fi] = norm * A[k];
        });
        parallel_for(nmom, nthreads, [&](size_t k) {
            cd* p = &at[k * 2 * nf];
            for (size_t fi = nf; fi < 2 * nf; ++fi) p[fi] = 0;
            dsp(p, nf, dsp_type, dsp_method, fwd, bwd);
        });
        for (size_t k = 0; k < nmom; ++k) acc.store(&at[k * 2 * nf], nf);
        finish_factor(acc, 1.0 / (2 * M_PI), fqt + iq * nf * 2, fq + iq * 2, fq2 + iq * 2);
    }
    return 0;
}

// Special functions and coordinate conversions on their own (for the tests).
void oracle_sph_bessel(int L, double x, double* out) { sph_bessel_all(L, x, out); }
void oracle_cyl_bessel(int N, double x, double* out) { cyl_bessel_all(N, x, out); }
// conj(Y_l^m(theta, phi)) for l <= L, m = -l..l in order (l, m): out [(L+1)^2][2]
void oracle_conj_ylm(int L, double theta, double phi, double* out) {
    std::vector<double> P((size_t)(L + 1) * (L + 2) / 2);
    legendre_norm(L, cos(theta), P.data());
    size_t k = 0;
    for (int l = 0; l <= L; ++l)
        for (int m = -l; m <= l; ++m, ++k) {
            cd v = conj_ylm(P.data(), l, m, phi);
            out[2 * k] = v.real();
            out[2 * k + 1] = v.imag();
        }
}
void oracle_to_spherical(const float* xyz, size_t n, float* out) {
    for (size_t i = 0; i < n; ++i) to_spherical(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], out[3 * i], out[3 * i + 1], out[3 * i + 2]);
}

}  // extern "C"
