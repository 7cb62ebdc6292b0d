"""CPU oracle for Sassena's scattering-amplitude hot path (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this package, and only as the checker. The product package
``sassena_gb300`` never imports it.

Parity status: pinned to the reference's own code. The reference has no golden
vectors for this path and cannot be built whole here (MPI, Boost, FFTW3, HDF5 and
libxml2 are absent), but its hot path compiles from its own sources against small
stand-in headers (``ref_build/``, output in ``_ref/``): the coherent and incoherent
vectors devices, smath, scatter factors, database getters and q-vector scans.
``tests/golden/reference.npz`` holds that code's outputs, and the C++ restatement
(``cpu_oracle.cpp``) reproduces them (bit for bit where the sums are sequential,
within FFT rounding where FFTW is involved; ``tests/test_reference_pin.py``). The
analytic known answers and the independent numpy restatement (``numpy_oracle.py``)
remain as further checks.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_TIMING_PATH = os.path.join(_HERE, "_build", "liboracle_timing.so")
_lib = None
_timing = None

DSP_AUTOCORRELATE, DSP_SQUARE, DSP_PLAIN = 0, 1, 2
METHOD_FFTW, METHOD_DIRECT = 0, 1

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_sp = ctypes.POINTER(ctypes.c_size_t)


def build() -> str:
    """Compile the oracle library with its Makefile (idempotent), and the reference's own
    compiled hot path (oracle/_ref) where the reference tree is present."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "ref_build")], check=True)
    return _LIB_PATH


def lib(timing=False):
    """The parity build of the oracle, or (timing=True) its CPU-baseline build."""
    global _lib, _timing
    if timing and _timing is not None:
        return _timing
    if not timing and _lib is not None:
        return _lib
    path = _TIMING_PATH if timing else _LIB_PATH
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(
        os.path.join(_HERE, "cpu_oracle.cpp")
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    L = ctypes.CDLL(path)
    L.oracle_last_split.argtypes = [_dp, _dp]
    for name in ("oracle_all_vectors", "oracle_self_vectors"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = [_fp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, _sp, _dp, _dp,
                      ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
    L.oracle_amplitudes.restype = ctypes.c_int
    L.oracle_amplitudes.argtypes = [_fp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                                    _dp, _sp, _dp, ctypes.c_int, _dp]
    L.oracle_dft.argtypes = [_dp, ctypes.c_size_t, ctypes.c_int]
    L.oracle_autocorrelate_fftw.argtypes = [_dp, ctypes.c_size_t]
    L.oracle_autocorrelate_direct.argtypes = [_dp, ctypes.c_size_t]
    L.oracle_sfactor.restype = ctypes.c_double
    L.oracle_sfactor.argtypes = [ctypes.c_int, _dp, ctypes.c_size_t, ctypes.c_double]
    L.oracle_volume.restype = ctypes.c_double
    L.oracle_volume.argtypes = [ctypes.c_int, _dp, ctypes.c_size_t]
    L.oracle_exclusion.restype = ctypes.c_double
    L.oracle_exclusion.argtypes = [ctypes.c_int, _dp, ctypes.c_size_t, ctypes.c_double,
                                   ctypes.c_double]
    _ip = ctypes.POINTER(ctypes.c_int)
    L.oracle_mp_sphere.restype = ctypes.c_int
    L.oracle_mp_sphere.argtypes = [_fp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, _dp,
                                   _dp, ctypes.c_size_t, _ip, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, _dp, _dp, _dp]
    L.oracle_mp_cylinder.restype = ctypes.c_int
    L.oracle_mp_cylinder.argtypes = [_fp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                                     _dp, _dp, ctypes.c_size_t, _ip, _dp, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
    L.oracle_sph_bessel.argtypes = [ctypes.c_int, ctypes.c_double, _dp]
    L.oracle_cyl_bessel.argtypes = [ctypes.c_int, ctypes.c_double, _dp]
    L.oracle_conj_ylm.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp]
    L.oracle_to_spherical.argtypes = [_fp, ctypes.c_size_t, _fp]
    L.oracle_scan.restype = ctypes.c_size_t
    L.oracle_scan.argtypes = [_dp, ctypes.c_double, ctypes.c_double, ctypes.c_size_t,
                              ctypes.c_double, _dp]
    if timing:
        _timing = L
    else:
        _lib = L
    return L


def _ptr(a, t):
    return a.ctypes.data_as(t)


def _vectors(kind, coords, sub_offsets, subvectors, factors, dsp_type, dsp_method, nthreads, timing=False):
    coords = np.ascontiguousarray(coords, dtype=np.float32)
    nf, na = coords.shape[0], coords.shape[1]
    sub_offsets = np.ascontiguousarray(sub_offsets, dtype=np.uintp)
    subvectors = np.ascontiguousarray(subvectors, dtype=np.float64).reshape(-1, 3)
    nq = len(sub_offsets) - 1
    factors = np.ascontiguousarray(factors, dtype=np.float64).reshape(nq, na)
    fqt = np.zeros((nq, nf, 2))
    fq = np.zeros((nq, 2))
    fq2 = np.zeros((nq, 2))
    fn = getattr(lib(timing), "oracle_%s_vectors" % kind)
    rc = fn(_ptr(coords, _fp), nf, na, nq, _ptr(sub_offsets, _sp), _ptr(subvectors, _dp),
            _ptr(factors, _dp), dsp_type, dsp_method, nthreads, _ptr(fqt, _dp), _ptr(fq, _dp),
            _ptr(fq2, _dp))
    if rc != 0:
        raise ValueError("oracle_%s_vectors rejected its arguments" % kind)
    return fqt, fq, fq2


def all_vectors(coords, sub_offsets, subvectors, factors, dsp_type=DSP_AUTOCORRELATE,
                dsp_method=METHOD_FFTW, nthreads=None, timing=False):
    """Coherent S(q,t) per q: returns (fqt [nq,nf,2], fq [nq,2], fq2 [nq,2]).
    timing=True runs the CPU-baseline build (for timings only)."""
    return _vectors("all", coords, sub_offsets, subvectors, factors, dsp_type, dsp_method,
                    nthreads or os.cpu_count(), timing)


def self_vectors(coords, sub_offsets, subvectors, factors, dsp_type=DSP_AUTOCORRELATE,
                 dsp_method=METHOD_FFTW, nthreads=None, timing=False):
    """Incoherent F(q,t) per q: returns (fqt [nq,nf,2], fq [nq,2], fq2 [nq,2])."""
    return _vectors("self", coords, sub_offsets, subvectors, factors, dsp_type, dsp_method,
                    nthreads or os.cpu_count(), timing)


def last_split(timing=False):
    """(scatter_s, dsp_s): thread-seconds of the last vectors call of that build spent in
    the phase sum and in the correlation (dsp)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    lib(timing).oracle_last_split(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def amplitudes(coords, subvectors, sub_shell, factors, nthreads=None):
    """A[m, f] = sum_j b_j(shell(m)) exp(i q_m . r_j(f)) as complex128 [nsub, nf]."""
    coords = np.ascontiguousarray(coords, dtype=np.float32)
    nf, na = coords.shape[0], coords.shape[1]
    subvectors = np.ascontiguousarray(subvectors, dtype=np.float64).reshape(-1, 3)
    sub_shell = np.ascontiguousarray(sub_shell, dtype=np.uintp)
    factors = np.ascontiguousarray(factors, dtype=np.float64).reshape(-1, na)
    out = np.zeros((len(subvectors), nf, 2))
    lib().oracle_amplitudes(_ptr(coords, _fp), nf, na, len(subvectors), _ptr(subvectors, _dp),
                            _ptr(sub_shell, _sp), _ptr(factors, _dp), nthreads or os.cpu_count(),
                            _ptr(out, _dp))
    return out[..., 0] + 1j * out[..., 1]


def autocorrelate_fftw(a):
    nf = len(a)
    buf = np.zeros((2 * nf, 2))
    buf[:nf, 0] = np.real(a)
    buf[:nf, 1] = np.imag(a)
    lib().oracle_autocorrelate_fftw(_ptr(buf, _dp), nf)
    return buf[:nf, 0] + 1j * buf[:nf, 1]


def autocorrelate_direct(a):
    nf = len(a)
    buf = np.stack([np.real(a), np.imag(a)], axis=1).astype(np.float64).copy()
    lib().oracle_autocorrelate_direct(_ptr(buf, _dp), nf)
    return buf[:, 0] + 1j * buf[:, 1]


def dft(a, sign=-1):
    n = len(a)
    buf = np.stack([np.real(a), np.imag(a)], axis=1).astype(np.float64).copy()
    lib().oracle_dft(_ptr(buf, _dp), n, sign)
    return buf[:, 0] + 1j * buf[:, 1]


def sfactor(ftype, params, q):
    p = np.ascontiguousarray(params, dtype=np.float64)
    return lib().oracle_sfactor(ftype, _ptr(p, _dp), len(p), q)


def volume(ftype, params):
    p = np.ascontiguousarray(params, dtype=np.float64)
    return lib().oracle_volume(ftype, _ptr(p, _dp), len(p))


def exclusion(ftype, params, effvolume, q):
    p = np.ascontiguousarray(params, dtype=np.float64)
    return lib().oracle_exclusion(ftype, _ptr(p, _dp), len(p), effvolume, q)


def scan(base, frm, to, points, exponent=1.0):
    base = np.ascontiguousarray(base, dtype=np.float64)
    out = np.zeros((max(points, 1), 3))
    n = lib().oracle_scan(_ptr(base, _dp), frm, to, points, exponent, _ptr(out, _dp))
    return out[:n]


def _mp(kind, coords, qvectors, factors, moments, axis, dsp_type, dsp_method, nthreads):
    coords = np.ascontiguousarray(coords, dtype=np.float32)
    nf, na = coords.shape[0], coords.shape[1]
    q = np.ascontiguousarray(qvectors, dtype=np.float64).reshape(-1, 3)
    nq = len(q)
    factors = np.ascontiguousarray(factors, dtype=np.float64).reshape(nq, na)
    mom = np.ascontiguousarray(moments, dtype=np.int32).reshape(-1, 2)
    fqt, fq, fq2 = np.zeros((nq, nf, 2)), np.zeros((nq, 2)), np.zeros((nq, 2))
    ip = ctypes.POINTER(ctypes.c_int)
    args = [_ptr(coords, _fp), nf, na, nq, _ptr(q, _dp), _ptr(factors, _dp), len(mom), _ptr(mom, ip)]
    if kind == "cylinder":
        args.append(_ptr(np.ascontiguousarray(axis, np.float64), _dp))
    args += [dsp_type, dsp_method, nthreads or os.cpu_count(), _ptr(fqt, _dp), _ptr(fq, _dp),
             _ptr(fq2, _dp)]
    rc = getattr(lib(), "oracle_mp_" + kind)(*args)
    if rc != 0:
        raise ValueError("oracle_mp_%s rejected its arguments" % kind)
    return fqt, fq, fq2


def mp_sphere(coords, qvectors, factors, moments, dsp_type=DSP_AUTOCORRELATE,
              dsp_method=METHOD_FFTW, nthreads=None):
    """Multipole sphere device: (fqt [nq,nf,2], fq [nq,2], fq2 [nq,2])."""
    return _mp("sphere", coords, qvectors, factors, moments, None, dsp_type, dsp_method, nthreads)


def mp_cylinder(coords, qvectors, factors, moments, axis, dsp_type=DSP_AUTOCORRELATE,
                dsp_method=METHOD_FFTW, nthreads=None):
    """Multipole cylinder device around `axis`: (fqt, fq, fq2)."""
    return _mp("cylinder", coords, qvectors, factors, moments, axis, dsp_type, dsp_method,
               nthreads)


def sph_bessel(L, x):
    out = np.zeros(L + 1)
    lib().oracle_sph_bessel(L, float(x), _ptr(out, _dp))
    return out


def cyl_bessel(N, x):
    out = np.zeros(N + 1)
    lib().oracle_cyl_bessel(N, float(x), _ptr(out, _dp))
    return out


def conj_ylm(L, theta, phi):
    """conj(Y_l^m(theta, phi)) for (l, m) = (0,0), (1,-1), (1,0), (1,1), ... as complex."""
    out = np.zeros(((L + 1) ** 2, 2))
    lib().oracle_conj_ylm(L, float(theta), float(phi), _ptr(out, _dp))
    return out[:, 0] + 1j * out[:, 1]


def to_spherical(xyz):
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    out = np.zeros_like(xyz)
    lib().oracle_to_spherical(_ptr(xyz, _fp), len(xyz), _ptr(out, _fp))
    return out


def sphere_moments(resolution):
    """Moments (0,0), (1,-1..1), ..., (L,-L..L) (parameters.cpp:1049-1058)."""
    return [(0, 0)] + [(l, m) for l in range(1, resolution + 1) for m in range(-l, l + 1)]


def cylinder_moments(resolution):
    """Moments (0,0), (l,0..3) for l = 1..L (parameters.cpp:1060-1068)."""
    return [(0, 0)] + [(l, m) for l in range(1, resolution + 1) for m in range(4)]
