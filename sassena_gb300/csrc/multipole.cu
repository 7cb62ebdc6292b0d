// Multipole orientational averages (coherent, FP64 form).
//
// Replaces MPSphereScatterDevice and MPCylinderScatterDevice
// (src/scatter_devices/multipole_scatter_device.cpp). Per q and per moment (l, m) the
// reference sums over atoms, for every frame:
//   sphere   A_lm(t) = sum_j 4 pi i^l b_j j_l(|q| r_j) conj(Y_l^m(theta_j, phi_j))   (:428-497)
//   cylinder A_lm(t) = sqrt(2 pi) sum_j b_j exp(i s z_j q_z) c_lm J_n(q_r r_j) T_m(n (phi_j - phi_q))
//            with n = 2l (m = 0, 1: T = cos, sin) or 2l - 1 (m = 2, 3), c = sqrt(1/2) 2 (-1)^l or
//            i sqrt(1/2) 2 (-1)^(l-1), (l, m) = (0, 0): J_0, and s the sign of z q_z  (:900-986)
// then correlates each moment like the vectors devices and scales the sum by 1/(4 pi)
// (sphere, :396-400) or 1/(2 pi) (cylinder, :865-870). Coordinates are in the spherical or
// cylindrical representation the reference stages (coordinate_sets.cpp:359-363), converted
// here on the device from the staged Cartesian frames in FP64 and rounded to float as the
// reference's float staging does (data_stager.cpp:110-114).
//
// GB300 layout.
//   sphere: the sum over atoms is, for one frame and one l, a product of the matrix
//     b_j(q) j_l(|q| r_j) [q x atom] with conj(Y_l^m(j)) [atom x m]. A basis kernel writes both
//     factors for a batch of frames to HBM (every Y_l^m once, not once per q); a tiled
//     contraction kernel stages atom tiles of both in shared memory and accumulates every
//     (q, m) output of one (frame, l) in FP64.
//   cylinder: one CTA per (q, frame) stages, for a tile of atoms, J_n(q_r r) for every
//     order n <= 2L, cos(n phi), sin(n phi) and b exp(i s z q_z) in shared memory; threads
//     then own orders n and accumulate sum_j X_j J_n cos(n phi_j) and ... sin(n phi_j);
//     each moment is formed from them with cos(n phi_q), sin(n phi_q).
// The special functions are this project's own FP64 implementations (Boost, which the
// reference calls, is not used): spherical Bessel functions by power series, upward
// recurrence where stable or Miller's downward recurrence; normalised associated Legendre
// functions by the standard three-term recurrences; cylinder Bessel functions by Hankel's
// asymptotic expansion plus upward recurrence for large arguments, Miller's algorithm
// otherwise. The amplitudes then go through the engine's correlation and average.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace sassgpu {

namespace {

constexpr int kMpMaxL = 40;  // largest major moment (sphere) / half order (cylinder)
constexpr int kMpTileAtoms = 32;

// ---------------------------------------------------------------------------------------
// coordinate representations
// ---------------------------------------------------------------------------------------
// SphericalCoor3D(CartesianCoor3D), coor3d.cpp:168-215 -> (r, phi, theta) as float.
__device__ float4 to_spherical(float xf, float yf, float zf) {
    const double x = xf, y = yf, z = zf;
    const double r = sqrt(x * x + y * y + z * z);  // squares of float values are exact
    double theta = 0, phi = 0;
    if (r != 0) {
        theta = acos(z / r);
        if (x != 0.0) {
            phi = atan(y / x);
            if (x < 0.0) phi += 3.14159265358979323846;
            else if (y < 0.0) phi += 2 * 3.14159265358979323846;
        } else if (y != 0.0) {
            if (y > 0) phi = 1.57079632679489661923;
            if (y < 0) phi = 3 * 1.57079632679489661923;
        }
    }
    return make_float4((float)r, (float)phi, (float)theta, 0.f);
}

// CylinderCoor3D(CartesianCoor3D) of the projected vector, coor3d.cpp:116-141, with the
// reference's float sign() for the x < 0 branch.
__host__ __device__ inline void to_cylinder(double x, double y, double z, double& r, double& phi, double& zz) {
    r = sqrt(x * x + y * y);
    const double kPi = 3.14159265358979323846, kPi2 = 1.57079632679489661923;
    if (x != 0.0) {
        phi = atan(y / x);
        if (x < 0.0) phi = (double)((float)y < 0.0f ? -(float)kPi : (float)kPi) + phi;
    } else if (y != 0.0) {
        phi = (double)((float)y < 0.0f ? -(float)kPi2 : (float)kPi2);
    } else {
        phi = 0.0;
    }
    phi = phi < 0 ? 2 * kPi + phi : phi;
    zz = z;
}

struct MpBase {
    double e[9];  // e_r, e_phi, e_z of CartesianVectorBase(axis), coor3d.cpp:278-295
};

// Spherical (r, phi, theta, class) or cylindrical (r, phi, z, class) of atom j at slot[j] of
// its frame row (padding slots: class -1).
__global__ void mp_convert_kernel(const float4* __restrict__ xyz, int na_pad, int na, int nf, int cylinder,
                                  MpBase b, const int* __restrict__ slot, const int* __restrict__ cls,
                                  float4* __restrict__ out) {
    const size_t n = (size_t)nf * na_pad;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(i % na_pad);
        if (j >= na) {
            out[i] = make_float4(0.f, 0.f, 0.f, -1.f);
            continue;
        }
        const float4 c = xyz[i];
        if (!cylinder) {
            float4 v = to_spherical(c.x, c.y, c.z);
            v.w = (float)cls[j];
            out[(i - j) + slot[j]] = v;
        } else {
            const double x = c.x, y = c.y, z = c.z;
            const double px = x * b.e[0] + y * b.e[1] + z * b.e[2];
            const double py = x * b.e[3] + y * b.e[4] + z * b.e[5];
            const double pz = x * b.e[6] + y * b.e[7] + z * b.e[8];
            double r, phi, zz;
            to_cylinder(px, py, pz, r, phi, zz);
            out[(i - j) + slot[j]] = make_float4((float)r, (float)phi, (float)zz, (float)cls[j]);
        }
    }
}

// ---------------------------------------------------------------------------------------
// special functions (FP64)
// ---------------------------------------------------------------------------------------
// b * j_l(x) for l = 0..L written to out[l * stride]. Divisions are hoisted (1/x once):
// GB300's FP64 pipe makes every division or square root a dozen FMAs.
__device__ void sph_bessel_row(int L, double x, double b, double* out, size_t stride) {
    if (x == 0) {
        out[0] = b;
        for (int l = 1; l <= L; ++l) out[l * stride] = 0;
        return;
    }
    if (x < 0.5) {  // power series
        double xl = 1;
        const double x2 = x * x;
        for (int l = 0; l <= L; ++l) {
            if (l > 0) xl *= x / (2 * l + 1);
            double term = 1, sum = 1;
            for (int k = 1; k < 40; ++k) {
                term *= -x2 / (2.0 * k * (2 * l + 2 * k + 1));
                sum += term;
                if (fabs(term) < 1e-18 * fabs(sum)) break;
            }
            out[l * stride] = b * xl * sum;
        }
        return;
    }
    const double ix = 1.0 / x;
    double sx, cx;
    sincos(x, &sx, &cx);
    const double j0 = sx * ix, j1 = (sx * ix - cx) * ix;
    if (x > L) {  // upward recurrence, stable for every l < x
        double jm = j0, jc = j1;
        out[0] = b * j0;
        if (L >= 1) out[stride] = b * j1;
        for (int l = 1; l < L; ++l) {
            const double jn = (2 * l + 1) * ix * jc - jm;
            out[(l + 1) * stride] = b * jn;
            jm = jc;
            jc = jn;
        }
        return;
    }
    // Miller's downward recurrence from order L + 32, normalised by j_0 or j_1
    const int N = L + 32;
    double fp = 0, f = 1e-250;
    for (int n = N; n >= 1; --n) {
        const double fm = (2 * n + 1) * ix * f - fp;
        fp = f;
        f = fm;
        if (n - 1 <= L) out[(n - 1) * stride] = f;
        if (fabs(f) > 1e200) {
            for (int l = n - 1; l <= L; ++l) out[l * stride] *= 1e-200;
            fp *= 1e-200;
            f *= 1e-200;
        }
    }
    const double scale = b * (fabs(j0) >= fabs(j1) ? j0 / out[0] : j1 / out[stride]);
    for (int l = 0; l <= L; ++l) out[l * stride] *= scale;
}

// Coefficients of the normalised associated Legendre recurrences, per (l, m) with m <= l:
//   cf[(l (l + 1)) / 2 + m] = (a_lm, b_lm), a = sqrt((4l^2 - 1)/(l^2 - m^2)),
//   b = sqrt(((l-1)^2 - m^2)/(4 (l-1)^2 - 1)) (l >= m + 2); the seeds per m:
//   sd[m] = (-sqrt((2m + 1)/(2m)), sqrt(2m + 3)).
__global__ void ylm_coeff_kernel(int L, double2* cf, double2* sd) {
    const int n = (L + 1) * (L + 2) / 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int l = 0;
        while ((l + 1) * (l + 2) / 2 <= i) ++l;
        const int m = i - l * (l + 1) / 2;
        double a = 0, bb = 0;
        if (l >= m + 2) {
            a = sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
            bb = sqrt((((double)l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1));
        }
        cf[i] = make_double2(a, bb);
        if (l == m) sd[m] = make_double2(m > 0 ? -sqrt((2.0 * m + 1) / (2.0 * m)) : 0.0, sqrt(2.0 * m + 3));
    }
}

// conj(Y_l^m(theta, phi)) for the requested moments (idx[l (2L+1) + L + m] -> moment, or -1)
// written to out[k * stride]; m outer, l inner, so the Legendre recurrence carries two values.
// e^{i m phi} by rotation (m multiplications of e^{i phi}).
__device__ void conj_ylm_row(int L, double theta, double phi, const int* __restrict__ idx, const double2* cf,
                             const double2* sd, double2* out, size_t stride) {
    const double x = cos(theta), s = sqrt((1 - x) * (1 + x));
    double pmm = sqrt(1.0 / (4 * 3.14159265358979323846));
    const int W = 2 * L + 1;
    double s1, c1;
    sincos(phi, &s1, &c1);
    double cm = 1.0, sm = 0.0;
    for (int m = 0; m <= L; ++m) {
        if (m > 0) {
            pmm = sd[m].x * s * pmm;
            const double cn = cm * c1 - sm * s1;
            sm = sm * c1 + cm * s1;
            cm = cn;
        }
        auto emit = [&](int l, double P) {
            const int kp = idx[l * W + L + m];
            if (kp >= 0) out[kp * stride] = make_double2(P * cm, -P * sm);
            if (m > 0) {
                const int kn = idx[l * W + L - m];
                const double v = (m & 1) ? -P : P;  // conj(Y_l^{-m}) = (-1)^m Pbar e^{i m phi}
                if (kn >= 0) out[kn * stride] = make_double2(v * cm, v * sm);
            }
        };
        emit(m, pmm);
        if (m < L) {
            double p2 = pmm, p1 = sd[m].y * x * pmm;
            emit(m + 1, p1);
            for (int l = m + 2; l <= L; ++l) {
                const double2 ab = cf[l * (l + 1) / 2 + m];
                const double p = ab.x * (x * p1 - ab.y * p2);
                emit(l, p);
                p2 = p1;
                p1 = p;
            }
        }
    }
}

// J_0(x), J_1(x) for x >= 25 by Hankel's asymptotic expansion (cos, sin of x - pi/4 and
// x - 3 pi/4 formed from cos x, sin x).
__device__ void bessel01_asymptotic(double x, double& j0, double& j1) {
    double P0 = 1, Q0 = 0, P1 = 1, Q1 = 0;
    for (int nu = 0; nu < 2; ++nu) {
        const double mu = 4.0 * nu * nu;
        double a = 1, P = 1, Q = 0;
        const double i8x = 1.0 / (8.0 * x);
        for (int k = 1; k < 60; ++k) {
            const double next = a * (mu - (2.0 * k - 1) * (2.0 * k - 1)) * i8x / k;
            if (fabs(next) > fabs(a) && k > 2) break;
            a = next;
            if (k & 1) Q += (((k - 1) / 2) & 1 ? -a : a);
            else P += ((k / 2) & 1 ? -a : a);
            if (fabs(a) < 1e-18) break;
        }
        if (nu == 0) {
            P0 = P;
            Q0 = Q;
        } else {
            P1 = P;
            Q1 = Q;
        }
    }
    double s, c;
    sincos(x, &s, &c);
    const double h = 0.70710678118654752440, amp = sqrt(2.0 / (3.14159265358979323846 * x));
    j0 = amp * (P0 * h * (c + s) - Q0 * h * (s - c));
    j1 = amp * (P1 * h * (s - c) + Q1 * h * (s + c));
}

// J_n(x), n = 0..N, written to out[n * stride].
__device__ void cyl_bessel_row(int N, double x, double* out, int stride) {
    if (x == 0) {
        out[0] = 1;
        for (int n = 1; n <= N; ++n) out[n * stride] = 0;
        return;
    }
    if (x >= 25 && x > N) {
        double j0, j1;
        bessel01_asymptotic(x, j0, j1);
        out[0] = j0;
        if (N >= 1) out[stride] = j1;
        double jm = j0, jc = j1;
        const double ix2 = 2.0 / x;
        for (int n = 1; n < N; ++n) {
            const double jn = n * ix2 * jc - jm;
            out[(n + 1) * stride] = jn;
            jm = jc;
            jc = jn;
        }
        return;
    }
    const double top = fmax((double)N, x);
    int M = (int)(top + 20 + 2 * sqrt(top + 10));
    M += M & 1;
    const double ix2 = 2.0 / x;
    double fp = 0, f = 1e-250, norm = 0;
    for (int n = M; n >= 1; --n) {
        const double fm = n * ix2 * f - fp;
        fp = f;
        f = fm;
        if (n - 1 <= N) out[(n - 1) * stride] = f;
        if (((n - 1) & 1) == 0) norm += (n - 1 == 0 ? 1.0 : 2.0) * f;
        if (fabs(f) > 1e200) {
            for (int k = n - 1; k <= N; ++k) out[k * stride] *= 1e-200;
            fp *= 1e-200;
            f *= 1e-200;
            norm *= 1e-200;
        }
    }
    const double inorm = 1.0 / norm;
    for (int n = 0; n <= N; ++n) out[n * stride] *= inorm;
}

// ---------------------------------------------------------------------------------------
// sphere: basis and contraction
// ---------------------------------------------------------------------------------------
struct MpSphereBasis {
    const float4* sph;  // [nf][na_pad] (r, phi, theta, class), atoms in order of frame-0 radius
    const int* cls;     // [na_pad] (-1 padding)
    const double* cf;   // [nq][nclass]
    const double* qlen; // [nq]
    const int* idx;     // [(L+1)(2L+1)]
    const double2* ycf; // Legendre coefficients [(L+1)(L+2)/2] and seeds [L+1] (ylm_coeff_kernel)
    const double2* ysd;
    double* Jb;         // [nfb][nq][L+1][na_pad]  b_j(q) j_l(|q| r_j)
    double2* Yc;        // [nfb][nmom][na_pad]     conj(Y_l^m(j))
    int na_pad, nclass, nq, L, nmom, f0, nfb;
};

// conj(Y_l^m) of every (frame, atom) of the batch; the coefficient tables live in shared memory.
__global__ void __launch_bounds__(128) mp_ylm_kernel(MpSphereBasis a) {
    extern __shared__ __align__(16) unsigned char smem[];
    double2* cf = reinterpret_cast<double2*>(smem);
    const int ncf = (a.L + 1) * (a.L + 2) / 2;
    double2* sd = cf + ncf;
    for (int i = threadIdx.x; i < ncf; i += blockDim.x) cf[i] = a.ycf[i];
    for (int i = threadIdx.x; i <= a.L; i += blockDim.x) sd[i] = a.ysd[i];
    __syncthreads();
    const size_t n = (size_t)a.nfb * a.na_pad;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int fl = (int)(i / a.na_pad), j = (int)(i - (size_t)fl * a.na_pad);
        const float4 c = a.sph[(size_t)(a.f0 + fl) * a.na_pad + j];
        conj_ylm_row(a.L, (double)c.z, (double)c.y, a.idx, cf, sd, a.Yc + (size_t)fl * a.nmom * a.na_pad + j,
                     a.na_pad);
    }
}

// b_j(q) j_l(|q| r_j) of every (frame, q, atom) of the batch.
__global__ void __launch_bounds__(128) mp_jl_kernel(MpSphereBasis a) {
    const size_t n = (size_t)a.nfb * a.nq * a.na_pad;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t fq = i / a.na_pad;
        const int j = (int)(i - fq * a.na_pad), fl = (int)(fq / a.nq), q = (int)(fq - (size_t)fl * a.nq);
        const float4 c = a.sph[(size_t)(a.f0 + fl) * a.na_pad + j];
        const int cl = (int)c.w;  // atoms sit in radius order; w carries the class (-1: padding)
        const double b = cl >= 0 ? a.cf[(size_t)q * a.nclass + cl] : 0.0;
        sph_bessel_row(a.L, a.qlen[q] * (double)c.x, b, a.Jb + (fq * (a.L + 1)) * a.na_pad + j, a.na_pad);
    }
}

struct MpSphereContract {
    const double* Jb;
    const double2* Yc;
    const int* perm;    // moments grouped by l
    const int* gl;      // [ngroups] l of the group
    const int* gstart;  // [ngroups] first entry in perm
    const int* gcount;  // [ngroups]
    double2* A;         // [nq][nmom][nf]
    int na_pad, na, nq, L, nmom, nf, f0;
};

constexpr int kContractThreads = 256, kContractOutputs = 4;

__global__ void __launch_bounds__(kContractThreads) mp_sphere_contract_kernel(MpSphereContract a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int g = blockIdx.x, fl = blockIdx.y;
    const int l = a.gl[g], k0 = a.gstart[g], cnt = a.gcount[g];
    const int nout = a.nq * cnt;
    const int obase = blockIdx.z * kContractThreads * kContractOutputs;
    if (obase >= nout) return;
    double* Js = reinterpret_cast<double*>(smem);                    // [nq][T]
    double2* Ys = reinterpret_cast<double2*>(Js + (size_t)a.nq * kMpTileAtoms);  // [cnt][T]
    double2 acc[kContractOutputs];
#pragma unroll
    for (int r = 0; r < kContractOutputs; ++r) acc[r] = make_double2(0.0, 0.0);
    const double* jrow = a.Jb + (size_t)fl * a.nq * (a.L + 1) * a.na_pad;
    const double2* yrow = a.Yc + (size_t)fl * a.nmom * a.na_pad;
    const int jend = (a.na + kMpTileAtoms - 1) / kMpTileAtoms * kMpTileAtoms;  // <= na_pad
    for (int j0 = 0; j0 < jend; j0 += kMpTileAtoms) {
        __syncthreads();
        for (int t = threadIdx.x; t < a.nq * kMpTileAtoms; t += kContractThreads) {
            const int q = t / kMpTileAtoms, jj = t - q * kMpTileAtoms;
            Js[t] = jrow[((size_t)q * (a.L + 1) + l) * a.na_pad + j0 + jj];
        }
        for (int t = threadIdx.x; t < cnt * kMpTileAtoms; t += kContractThreads) {
            const int kk = t / kMpTileAtoms, jj = t - kk * kMpTileAtoms;
            Ys[t] = yrow[(size_t)a.perm[k0 + kk] * a.na_pad + j0 + jj];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kContractOutputs; ++r) {
            const int o = obase + threadIdx.x + r * kContractThreads;
            if (o < nout) {
                const int q = o / cnt, kk = o - q * cnt;
                const double* jq = Js + q * kMpTileAtoms;
                const double2* yk = Ys + kk * kMpTileAtoms;
                double2 s = acc[r];
                for (int jj = 0; jj < kMpTileAtoms; ++jj) {
                    s.x = fma(jq[jj], yk[jj].x, s.x);
                    s.y = fma(jq[jj], yk[jj].y, s.y);
                }
                acc[r] = s;
            }
        }
    }
    // times 4 pi i^l
    const double f4 = 4 * 3.14159265358979323846;
#pragma unroll
    for (int r = 0; r < kContractOutputs; ++r) {
        const int o = obase + threadIdx.x + r * kContractThreads;
        if (o < nout) {
            const int q = o / cnt, kk = o - q * cnt, mom = a.perm[k0 + kk];
            double2 v = acc[r], w;
            switch (l & 3) {
                case 0: w = make_double2(v.x, v.y); break;
                case 1: w = make_double2(-v.y, v.x); break;
                case 2: w = make_double2(-v.x, -v.y); break;
                default: w = make_double2(v.y, -v.x); break;
            }
            a.A[((size_t)q * a.nmom + mom) * a.nf + a.f0 + fl] = make_double2(f4 * w.x, f4 * w.y);
        }
    }
}

// ---------------------------------------------------------------------------------------
// cylinder
// ---------------------------------------------------------------------------------------
struct MpCylinder {
    const float4* cyl;   // [nf][na_pad] (r, phi, z, class), atoms in order of frame-0 radius
    const int* cls;
    const double* cf;    // [nq][nclass]
    const double* qcyl;  // [nq][3] (q_r, phi_q, q_z)
    const int* mom;      // [nmom][2]
    double2* A;          // [nq][nmom][nf]
    int na_pad, na, nclass, nq, N, nmom, nf;
    int f0;              // first frame of the launch (blockIdx.y counts from it)
};

// One CTA per (frame, block of kCylQB q-vectors), kCylThreads threads, tiles of kCylTA atoms.
// Per tile, threads [0, QB TA) evaluate one (q, atom) pair each: the Bessel row J_n(q_r r) and
// X = b e^{i s z q_z}; threads [QB TA, QB TA + TA) evaluate cos(n phi), sin(n phi) of one atom
// (shared by the block's q-vectors). Then every thread owns (q, order, cos|sin) sums.
constexpr int kCylQB = 3, kCylTA = 32, kCylThreads = 128;
static_assert(kCylQB * kCylTA + kCylTA <= kCylThreads, "tile roles exceed the CTA");

__global__ void __launch_bounds__(kCylThreads) mp_cylinder_kernel(MpCylinder a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int f = a.f0 + blockIdx.y, q0 = blockIdx.x * kCylQB, nqb = min(kCylQB, a.nq - q0);
    const int N = a.N, W = N + 1, ntask = nqb * 2 * W;
    double* Jn = reinterpret_cast<double*>(smem);                         // [QB][W][TA]
    double* cn = Jn + (size_t)kCylQB * W * kCylTA;                          // [W][TA]
    double* sn = cn + (size_t)W * kCylTA;                                   // [W][TA]
    double2* X = reinterpret_cast<double2*>(sn + (size_t)W * kCylTA);      // [QB][TA]
    constexpr int NPT = (kCylQB * 2 * (2 * kMpMaxL + 1) + kCylThreads - 1) / kCylThreads;
    double2 acc[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k) acc[k] = make_double2(0.0, 0.0);
    const float4* row = a.cyl + (size_t)f * a.na_pad;
    const int tid = threadIdx.x;
    for (int j0 = 0; j0 < a.na; j0 += kCylTA) {
        __syncthreads();
        if (tid < kCylQB * kCylTA) {
            const int qq = tid / kCylTA, jj = tid - qq * kCylTA, j = j0 + jj;
            double* jrow = Jn + (size_t)qq * W * kCylTA + jj;
            if (qq < nqb && j < a.na) {
                const int q = q0 + qq;
                const double qr = a.qcyl[3 * q], qz = a.qcyl[3 * q + 2];
                const float4 c = row[j];
                const double r = c.x, z = c.z;
                const int cl = (int)c.w;  // atoms sit in radius order; w carries the class
                const double b = cl >= 0 ? a.cf[(size_t)q * a.nclass + cl] : 0.0;
                double sgn = 1.0;  // parallel_sign, multipole_scatter_device.cpp:944-948
                if (z != 0 && qz != 0) sgn = (z * qz) / (fabs(z) * fabs(qz));
                double es, ec;
                sincos(sgn * z * qz, &es, &ec);
                X[qq * kCylTA + jj] = make_double2(b * ec, b * es);
                cyl_bessel_row(N, r * qr, jrow, kCylTA);
            } else {
                X[qq * kCylTA + jj] = make_double2(0.0, 0.0);
                for (int n = 0; n <= N; ++n) jrow[n * kCylTA] = 0;
            }
        } else if (tid < kCylQB * kCylTA + kCylTA) {
            const int jj = tid - kCylQB * kCylTA, j = j0 + jj;
            double cp = 1, sp = 0, s1 = 0, c1 = 1;  // cos, sin of n phi by rotation
            if (j < a.na) sincos((double)row[j].y, &s1, &c1);
            for (int n = 0; n <= N; ++n) {
                cn[n * kCylTA + jj] = cp;
                sn[n * kCylTA + jj] = sp;
                const double cq = cp * c1 - sp * s1;
                sp = sp * c1 + cp * s1;
                cp = cq;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NPT; ++k) {
            const int t = tid + k * kCylThreads;
            if (t < ntask) {
                const int qq = t / (2 * W), rem = t - qq * 2 * W, n = rem >> 1;
                const double* jv = Jn + ((size_t)qq * W + n) * kCylTA;
                const double* tr = ((rem & 1) ? sn : cn) + (size_t)n * kCylTA;
                const double2* x = X + qq * kCylTA;
                double2 sacc = acc[k];
                for (int jj = 0; jj < kCylTA; ++jj) {
                    const double w = jv[jj] * tr[jj];
                    sacc.x = fma(x[jj].x, w, sacc.x);
                    sacc.y = fma(x[jj].y, w, sacc.y);
                }
                acc[k] = sacc;
            }
        }
    }
    __syncthreads();
    double2* Sv = reinterpret_cast<double2*>(smem);  // [QB][W][cos, sin]
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        const int t = tid + k * kCylThreads;
        if (t < ntask) Sv[t] = acc[k];
    }
    __syncthreads();
    const double norm = sqrt(2 * 3.14159265358979323846), h = 0.70710678118654752440;
    for (int idx = tid; idx < nqb * a.nmom; idx += kCylThreads) {
        const int qq = idx / a.nmom, k = idx - qq * a.nmom, q = q0 + qq;
        const double qphi = a.qcyl[3 * q + 1];
        const double2* S2 = Sv + (size_t)qq * 2 * W;
        const int l = a.mom[2 * k], m = a.mom[2 * k + 1];
        double2 v;
        if (l == 0 && m == 0) {
            v = S2[0];
        } else {
            const int n = m < 2 ? 2 * l : 2 * l - 1;
            double snq, cnq;
            sincos(n * qphi, &snq, &cnq);
            const double2 C = S2[2 * n], S = S2[2 * n + 1];
            double2 t;  // sum_j X_j J_n cos / sin (n (phi_j - phi_q))
            if (m == 0 || m == 2) t = make_double2(cnq * C.x + snq * S.x, cnq * C.y + snq * S.y);
            else t = make_double2(cnq * S.x - snq * C.x, cnq * S.y - snq * C.y);
            if (m < 2) {
                const double c = h * 2.0 * ((l & 1) ? -1.0 : 1.0);
                v = make_double2(c * t.x, c * t.y);
            } else {  // times i sqrt(1/2) 2 (-1)^(l-1)
                const double c = h * 2.0 * (((l - 1) & 1) ? -1.0 : 1.0);
                v = make_double2(-c * t.y, c * t.x);
            }
        }
        a.A[((size_t)q * a.nmom + k) * a.nf + f] = make_double2(norm * v.x, norm * v.y);
    }
}

size_t cylinder_smem(int N) {
    const size_t W = (size_t)N + 1;
    const size_t tiles = (size_t)(kCylQB + 2) * W * kCylTA * sizeof(double) + (size_t)kCylQB * kCylTA * sizeof(double2);
    return std::max(tiles, (size_t)kCylQB * 2 * W * sizeof(double2));
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
struct V3 {
    double x, y, z;
};
V3 cross3(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double len3(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
V3 div3(V3 a, double l) { return {a.x / l, a.y / l, a.z / l}; }

// CartesianVectorBase(axis), coor3d.cpp:278-295
bool axis_base(const double* axis, MpBase& b) {
    V3 a{axis[0], axis[1], axis[2]};
    if (!(len3(a) > 0)) return false;
    V3 ez = div3(a, len3(a));
    V3 ekez = cross3(V3{0, 0, 1}, ez);
    if (len3(ekez) == 0) ekez = cross3(V3{0, 1, 0}, ez);
    V3 er = div3(ekez, len3(ekez));
    V3 ezer = cross3(ez, er);
    V3 ephi = div3(ezer, len3(ezer));
    const V3 e[3] = {er, ephi, ez};
    for (int k = 0; k < 3; ++k) {
        b.e[3 * k] = e[k].x;
        b.e[3 * k + 1] = e[k].y;
        b.e[3 * k + 2] = e[k].z;
    }
    return true;
}

int fail(std::string& m, int code, const std::string& what) {
    m = what;
    return code;
}

}  // namespace

}  // namespace sassgpu

using namespace sassgpu;

extern "C" int sass_multipole_compute(sass_plan* p, int type, size_t nq, const double* qvectors,
                                      const double* class_factors, size_t nmom, const int32_t* moments,
                                      const double* axis, double* fqt, double* fq, double* fq2) {
    if (!p) return SASS_ERR_ARG;
    if (nq == 0) return SASS_OK;
    if (!qvectors || !class_factors || !moments || !fqt || !fq || !fq2 || nmom == 0)
        return fail(p->msg, SASS_ERR_ARG, "NULL argument or no moments");
    if (type != SASS_MULTIPOLE_SPHERE && type != SASS_MULTIPOLE_CYLINDER)
        return fail(p->msg, SASS_ERR_ARG, "multipole type must be sphere or cylinder");
    if (p->d.precision != SASS_PRECISION_FP64 || p->d.scattering != SASS_SCATTERING_ALL)
        return fail(p->msg, SASS_ERR_UNSUPPORTED, "multipole devices need a coherent FP64 plan");
    if (!p->sys.staged || !p->sys.classes_set) return fail(p->msg, SASS_ERR_STATE, "plan not staged");
    const bool cyl = type == SASS_MULTIPOLE_CYLINDER;
    int L = 0;  // largest major moment
    for (size_t k = 0; k < nmom; ++k) {
        const int l = moments[2 * k], m = moments[2 * k + 1];
        // the reference's checks, parameters.cpp:1076-1114
        if (l < 0) return fail(p->msg, SASS_ERR_ARG, "major multipole moment must be >= 0");
        if (!cyl && std::abs(m) > l) return fail(p->msg, SASS_ERR_ARG, "minor multipole moment must be within -major..major");
        if (cyl && (m < 0 || m > 3)) return fail(p->msg, SASS_ERR_ARG, "minor multipole moment must be between 0 and 3");
        if (cyl && l == 0 && m != 0) return fail(p->msg, SASS_ERR_ARG, "minor multipole moment must be 0 for major 0");
        L = std::max(L, l);
    }
    if (L > kMpMaxL) return fail(p->msg, SASS_ERR_UNSUPPORTED, "major multipole moments above 40 are not supported");
    MpBase base{};
    if (cyl && (!axis || !axis_base(axis, base))) return fail(p->msg, SASS_ERR_ARG, "cylinder axis must be a nonzero vector");

    std::string& m = p->msg;
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        cudaGetLastError();
        m = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? SASS_ERR_OOM : SASS_ERR_CUDA;
    };
#define MCK(expr)                                  \
    do {                                           \
        cudaError_t e_ = (expr);                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
    } while (0)
    MCK(cudaSetDevice(p->d.device));
    memset(&p->timing, 0, sizeof(p->timing));
    SystemState& s = p->sys;
    const size_t nf = s.nf, na_pad = s.na_pad, nclass = s.nclass;
    cudaStream_t st = p->st;
    size_t launches = 0;

    // per-q inputs: |q| (sphere) or the projected q in cylinder coordinates
    std::vector<double> qin(cyl ? 3 * nq : nq);
    for (size_t i = 0; i < nq; ++i) {
        const double* qv = qvectors + 3 * i;
        if (!cyl) {
            qin[i] = sqrt(qv[0] * qv[0] + qv[1] * qv[1] + qv[2] * qv[2]);  // q.length()
        } else {
            const double px = qv[0] * base.e[0] + qv[1] * base.e[1] + qv[2] * base.e[2];
            const double py = qv[0] * base.e[3] + qv[1] * base.e[4] + qv[2] * base.e[5];
            const double pz = qv[0] * base.e[6] + qv[1] * base.e[7] + qv[2] * base.e[8];
            to_cylinder(px, py, pz, qin[3 * i], qin[3 * i + 1], qin[3 * i + 2]);
        }
    }
    // sphere: lookup (l, m) -> moment and moments grouped by l
    const int W = 2 * L + 1;
    std::vector<int> idx((size_t)(L + 1) * W, -1), perm, gl, gstart, gcount;
    if (!cyl) {
        for (size_t k = 0; k < nmom; ++k) idx[moments[2 * k] * W + L + moments[2 * k + 1]] = (int)k;
        for (int l = 0; l <= L; ++l) {
            const int start = (int)perm.size();
            for (size_t k = 0; k < nmom; ++k)
                if (moments[2 * k] == l) perm.push_back((int)k);
            if ((int)perm.size() > start) {
                gl.push_back(l);
                gstart.push_back(start);
                gcount.push_back((int)perm.size() - start);
            }
        }
    }
    // one packed upload of every small input (16-byte aligned pieces)
    std::vector<unsigned char> blob;
    auto put = [&](const void* h, size_t bytes) {
        const size_t off = (blob.size() + 15) / 16 * 16;
        blob.resize(off + bytes);
        if (bytes) memcpy(blob.data() + off, h, bytes);
        return off;
    };
    const size_t o_qin = put(qin.data(), qin.size() * sizeof(double));
    const size_t o_cf = put(class_factors, nq * nclass * sizeof(double));
    const size_t o_mom = put(moments, nmom * 2 * sizeof(int32_t));
    const size_t o_idx = put(idx.data(), idx.size() * sizeof(int));
    const size_t o_perm = put(perm.data(), perm.size() * sizeof(int));
    const size_t o_gl = put(gl.data(), gl.size() * sizeof(int));
    const size_t o_gs = put(gstart.data(), gstart.size() * sizeof(int));
    const size_t o_gc = put(gcount.data(), gcount.size() * sizeof(int));
    MCK(p->mp_in.ensure(blob.size()));
    MCK(p->mp_amp.ensure(nq * nmom * nf * sizeof(double2)));
    MCK(p->mp_out.ensure(nq * (nf + 2) * sizeof(double2)));
    unsigned char* din = p->mp_in.as<unsigned char>();
    auto dptr = [&](size_t off) { return din + off; };
    MCK(cudaEventRecord(p->ev[4], st));
    MCK(cudaMemcpyAsync(din, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
    MCK(cudaEventRecord(p->ev[0], st));

    // representation cache (rebuilt after staging or for another device type / axis)
    if (s.mp_type != type || !s.mp_valid || (cyl && memcmp(s.mp_axis, axis, sizeof(s.mp_axis)) != 0)) {
        MCK(s.mp_xyz.ensure(nf * na_pad * sizeof(float4)));
        // Atoms sorted by their frame-0 distance from the axis (cylinder) or the origin
        // (sphere): consecutive atoms then have similar Bessel arguments, so a warp's 32
        // Bessel rows take one branch (Miller's recurrence, Hankel's expansion, the power
        // series, the upward recurrence) with similar trip counts. A warp-wide FP64
        // instruction holds the narrow FP64 pipe whatever its active lanes.
        std::vector<float4> f0(na_pad);
        MCK(cudaMemcpyAsync(f0.data(), s.xyz.p, na_pad * sizeof(float4), cudaMemcpyDeviceToHost, st));
        MCK(cudaStreamSynchronize(st));
        std::vector<double> r2(s.na);
        for (size_t j = 0; j < s.na; ++j) {
            const double x = f0[j].x, y = f0[j].y, z = f0[j].z;
            if (cyl) {
                const double px = x * base.e[0] + y * base.e[1] + z * base.e[2];
                const double py = x * base.e[3] + y * base.e[4] + z * base.e[5];
                r2[j] = px * px + py * py;
            } else {
                r2[j] = x * x + y * y + z * z;
            }
        }
        std::vector<int> order(s.na), pos(s.na);
        for (size_t j = 0; j < s.na; ++j) order[j] = (int)j;
        std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return r2[u] < r2[v]; });
        for (size_t k = 0; k < s.na; ++k) pos[order[k]] = (int)k;
        MCK(p->mp_slot.ensure(s.na * sizeof(int)));
        MCK(cudaMemcpyAsync(p->mp_slot.p, pos.data(), s.na * sizeof(int), cudaMemcpyHostToDevice, st));
        MCK(cudaStreamSynchronize(st));
        const int* slot = p->mp_slot.as<int>();
        const size_t n = nf * na_pad;
        const int blocks = (int)grid_blocks(n, 256, 16);
        mp_convert_kernel<<<std::max(blocks, 1), 256, 0, st>>>(s.xyz.as<float4>(), (int)na_pad, (int)s.na, (int)nf, cyl,
                                                                base, slot, s.cls.as<int>(), s.mp_xyz.as<float4>());
        MCK(cudaGetLastError());
        ++launches;
        s.mp_type = type;
        s.mp_valid = true;
        if (cyl) memcpy(s.mp_axis, axis, sizeof(s.mp_axis));
    }
    const double* d_cf = reinterpret_cast<const double*>(dptr(o_cf));
    if (!cyl) {
        // frame batches: basis of up to a quarter of the free memory (at most 16 GB), so that
        // one contraction launch has thousands of CTAs
        size_t free_b = 0, total_b = 0;
        MCK(cudaMemGetInfo(&free_b, &total_b));
        const size_t budget = std::max<size_t>((size_t)1 << 28, std::min<size_t>((size_t)16 << 30, free_b / 4));
        const size_t per_frame = na_pad * (nq * (L + 1) * sizeof(double) + nmom * sizeof(double2));
        const size_t nfb = std::max<size_t>(1, std::min<size_t>({nf, budget / per_frame, (size_t)65535}));  // grid y
        const int ncf = (L + 1) * (L + 2) / 2;
        MCK(p->mp_ycf.ensure((size_t)(ncf + L + 1) * sizeof(double2)));
        ylm_coeff_kernel<<<(ncf + 127) / 128, 128, 0, st>>>(L, p->mp_ycf.as<double2>(), p->mp_ycf.as<double2>() + ncf);
        MCK(cudaGetLastError());
        ++launches;
        const size_t ysm = (size_t)(ncf + L + 1) * sizeof(double2);
        MCK(p->mp_Jb.ensure(nfb * nq * (L + 1) * na_pad * sizeof(double)));
        MCK(p->mp_Yc.ensure(nfb * nmom * na_pad * sizeof(double2)));
        int maxcnt = 0;
        for (int c : gcount) maxcnt = std::max(maxcnt, c);
        const size_t csm = nq * kMpTileAtoms * sizeof(double) + (size_t)maxcnt * kMpTileAtoms * sizeof(double2);
        if (csm > 48 * 1024)
            MCK(cudaFuncSetAttribute(mp_sphere_contract_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
        const int zchunks = (int)((nq * maxcnt + kContractThreads * kContractOutputs - 1) /
                                  (kContractThreads * kContractOutputs));
        for (size_t f0 = 0; f0 < nf; f0 += nfb) {
            const int nb = (int)std::min(nfb, nf - f0);
            MpSphereBasis ba{};
            ba.sph = s.mp_xyz.as<float4>();
            ba.cls = s.cls.as<int>();
            ba.cf = d_cf;
            ba.qlen = reinterpret_cast<const double*>(dptr(o_qin));
            ba.idx = reinterpret_cast<const int*>(dptr(o_idx));
            ba.ycf = p->mp_ycf.as<double2>();
            ba.ysd = p->mp_ycf.as<double2>() + ncf;
            ba.Jb = p->mp_Jb.as<double>();
            ba.Yc = p->mp_Yc.as<double2>();
            ba.na_pad = (int)na_pad;
            ba.nclass = (int)nclass;
            ba.nq = (int)nq;
            ba.L = L;
            ba.nmom = (int)nmom;
            ba.f0 = (int)f0;
            ba.nfb = nb;
            const size_t ny = (size_t)nb * na_pad, nj = ny * nq;
            mp_ylm_kernel<<<grid_blocks(ny, 128, 64), 128, ysm, st>>>(ba);
            MCK(cudaGetLastError());
            mp_jl_kernel<<<grid_blocks(nj, 128, 64), 128, 0, st>>>(ba);
            MCK(cudaGetLastError());
            ++launches;
            MpSphereContract ca{};
            ca.Jb = p->mp_Jb.as<double>();
            ca.Yc = p->mp_Yc.as<double2>();
            ca.perm = reinterpret_cast<const int*>(dptr(o_perm));
            ca.gl = reinterpret_cast<const int*>(dptr(o_gl));
            ca.gstart = reinterpret_cast<const int*>(dptr(o_gs));
            ca.gcount = reinterpret_cast<const int*>(dptr(o_gc));
            ca.A = p->mp_amp.as<double2>();
            ca.na_pad = (int)na_pad;
            ca.na = (int)s.na;
            ca.nq = (int)nq;
            ca.L = L;
            ca.nmom = (int)nmom;
            ca.nf = (int)nf;
            ca.f0 = (int)f0;
            dim3 grid((unsigned)gl.size(), (unsigned)nb, (unsigned)zchunks);
            mp_sphere_contract_kernel<<<grid, kContractThreads, csm, st>>>(ca);
            MCK(cudaGetLastError());
            launches += 2;
        }
    } else {
        MpCylinder ca{};
        ca.cyl = s.mp_xyz.as<float4>();
        ca.cls = s.cls.as<int>();
        ca.cf = d_cf;
        ca.qcyl = reinterpret_cast<const double*>(dptr(o_qin));
        ca.mom = reinterpret_cast<const int*>(dptr(o_mom));
        ca.A = p->mp_amp.as<double2>();
        ca.na_pad = (int)na_pad;
        ca.na = (int)s.na;
        ca.nclass = (int)nclass;
        ca.nq = (int)nq;
        ca.N = 2 * L;
        ca.nmom = (int)nmom;
        ca.nf = (int)nf;
        const size_t sm = cylinder_smem(2 * L);
        if (sm > 48 * 1024) MCK(cudaFuncSetAttribute(mp_cylinder_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        for (size_t f0 = 0; f0 < nf; f0 += 65535) {  // frames in grid y, at most 65,535 per launch
            ca.f0 = (int)f0;
            const unsigned nfl = (unsigned)std::min<size_t>(65535, nf - f0);
            mp_cylinder_kernel<<<dim3((unsigned)((nq + kCylQB - 1) / kCylQB), nfl), kCylThreads, sm, st>>>(ca);
            MCK(cudaGetLastError());
            ++launches;
        }
    }
    const size_t phase_launches = launches;
    // correlation and average of the amplitudes: moments play the sub-vectors
    EngineConfig cfg;
    cfg.scattering = p->d.scattering;
    cfg.dsp = p->d.dsp_type;
    cfg.method = p->d.dsp_method;
    cfg.precision = p->d.precision;
    cfg.device = p->d.device;
    std::vector<WorkItem> items(1);
    WorkItem& it = items[0];
    it.sys = &s;
    for (size_t i = 0; i <= nq; ++i) it.offs.push_back(i * nmom);
    it.d_cf = d_cf;
    double2* o = p->mp_out.as<double2>();
    it.d_fqt = o;
    it.d_fq = o + nq * nf;
    it.d_fq2 = o + nq * (nf + 1);
    it.d_amp_given = p->mp_amp.as<double2>();
    it.norm = cyl ? 1.0 / (2 * 3.14159265358979323846) : 1.0 / (4 * 3.14159265358979323846);
    int rc = p->eng.prepare(cfg, items, p->msg);
    if (rc) return rc;
    MCK(cudaEventRecord(p->ev[1], st));
    cudaEvent_t ev[4] = {p->ev[8], p->ev[9], p->ev[2], p->ev[3]};
    rc = p->eng.enqueue(st, p->msg, ev);
    if (rc) return rc;
    launches += p->eng.stats().launches;
    std::vector<double2> host(nq * (nf + 2));
    MCK(cudaEventRecord(p->ev[6], st));
    MCK(cudaMemcpyAsync(host.data(), o, host.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
    MCK(cudaEventRecord(p->ev[7], st));
    MCK(cudaStreamSynchronize(st));
    unsigned flag = 0;
    MCK(cudaMemcpy(&flag, p->eng.err_word(), sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (flag) return fail(p->msg, SASS_ERR_TIMEOUT, "device error flag " + std::to_string(flag));
    memcpy(fqt, host.data(), nq * nf * sizeof(double2));
    memcpy(fq, host.data() + nq * nf, nq * sizeof(double2));
    memcpy(fq2, host.data() + nq * (nf + 1), nq * sizeof(double2));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p->ev[0], p->ev[1]) == cudaSuccess) p->timing.phase_ms = ms;
    if (cudaEventElapsedTime(&ms, p->ev[9], p->ev[2]) == cudaSuccess) p->timing.corr_ms = ms;
    if (cudaEventElapsedTime(&ms, p->ev[2], p->ev[3]) == cudaSuccess) p->timing.finalize_ms = ms;
    if (cudaEventElapsedTime(&ms, p->ev[4], p->ev[0]) == cudaSuccess) p->timing.h2d_ms = ms;
    if (cudaEventElapsedTime(&ms, p->ev[6], p->ev[7]) == cudaSuccess) p->timing.d2h_ms = ms;
    if (cudaEventElapsedTime(&ms, p->ev[4], p->ev[7]) == cudaSuccess) p->timing.total_ms = ms;
    p->timing.kernel_launches = launches;
    p->timing.phase_launches = phase_launches;
    p->timing.h2d_bytes = blob.size();
    p->timing.d2h_bytes = host.size() * sizeof(double2);
    cudaGetLastError();
    p->msg.clear();
    return SASS_OK;
#undef MCK
}
