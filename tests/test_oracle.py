"""CPU tests of the oracle: cross-check of the two restatements and analytic pins.

The reference ships no golden vectors for this path and cannot be built here, so the
oracle is pinned by: (1) the independent numpy restatement, (2) the reference's own
direct-vs-FFT correlation identity (smath.cpp:51-76 vs :141-156, which differ by a
complex conjugate), (3) analytic known answers.
"""
import numpy as np
import pytest

import oracle
import oracle.numpy_oracle as npo
from sassena_gb300 import synth

from helpers import cplx, rel_err_sqt


@pytest.mark.parametrize("scattering", ["all", "self"])
@pytest.mark.parametrize("dsp", [0, 1, 2])
@pytest.mark.parametrize("method", [0, 1])
def test_cpp_matches_numpy(scattering, dsp, method):
    w = synth.small(scattering, seed=5, na=13, nf=10, nq=2, nm=3)
    fn_c = oracle.all_vectors if scattering == "all" else oracle.self_vectors
    fn_n = npo.all_vectors if scattering == "all" else npo.self_vectors
    a = fn_c(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), dsp, method, nthreads=3)
    b = fn_n(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), dsp, method)
    assert rel_err_sqt(b[0], a[0]).max() < 1e-13
    assert np.allclose(cplx(a[1]), b[1], rtol=1e-12, atol=1e-13 * np.abs(b[1]).max())
    assert np.allclose(cplx(a[2]), b[2], rtol=1e-12, atol=1e-13 * np.abs(b[2]).max())


@pytest.mark.parametrize("n", [1, 2, 7, 12, 30, 64, 97])
def test_dft_any_length(n):
    rng = np.random.default_rng(n)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    assert np.allclose(oracle.dft(x, -1), np.fft.fft(x), atol=1e-12 * n)
    assert np.allclose(oracle.dft(x, +1), np.fft.ifft(x) * n, atol=1e-12 * n)


@pytest.mark.parametrize("nf", [1, 5, 16, 33])
def test_direct_is_conjugate_of_fft(nf):
    rng = np.random.default_rng(nf)
    a = rng.normal(size=nf) + 1j * rng.normal(size=nf)
    d = oracle.autocorrelate_direct(a)
    f = oracle.autocorrelate_fftw(a)
    assert np.allclose(d, np.conj(f), atol=1e-13 * np.abs(f).max())
    # and the FFT form is (1/(NF-tau)) sum_k conj(a_k) a_{k+tau}
    ref = np.array([np.sum(np.conj(a[:nf - t]) * a[t:]) / (nf - t) for t in range(nf)])
    assert np.allclose(f, ref, atol=1e-13 * np.abs(ref).max())


def test_static_single_atom_known_answer():
    nf = 8
    coords = np.tile(np.array([[[0.3, 1.0, -2.0]]], np.float32), (nf, 1, 1))
    offs = np.array([0, 4], np.uintp)
    sv = synth.sphere_directions(4, 1) * 2.0
    fqt, fq, fq2 = oracle.all_vectors(coords, offs, sv, np.array([[1.7]]), 0, 0)
    assert np.allclose(cplx(fqt), 1.7 ** 2, atol=1e-14)
    assert np.allclose(cplx(fq), 1.7 ** 2) and np.allclose(cplx(fq2), 1.7 ** 4)


def test_two_atom_exact_identity():
    r = np.array([[0.0, 0.0, 0.0], [1.0, 2.0, -0.5]], np.float32)
    coords = np.tile(r[None], (3, 1, 1))
    dirs = synth.fibonacci_sphere(50)
    q = 0.9
    b = np.array([[1.5, -0.4]])
    fqt, fq, _ = oracle.all_vectors(coords, np.array([0, 50], np.uintp), q * dirs, b, 1, 0)
    d = (r[1] - r[0]).astype(float)
    expect = np.mean(1.5 ** 2 + 0.4 ** 2 - 2 * 1.5 * 0.4 * np.cos(q * dirs @ d))
    assert abs(fq[0, 0] - expect) < 1e-13


def test_debye_limit_dense_directions():
    # Orientational average of two atoms tends to b1^2 + b2^2 + 2 b1 b2 sin(qd)/(qd).
    r = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 3.0]], np.float32)
    coords = r[None]
    dirs = synth.fibonacci_sphere(4000)
    q = 1.3
    fqt, fq, _ = oracle.all_vectors(coords, np.array([0, 4000], np.uintp), q * dirs,
                                    np.array([[1.0, 1.0]]), 1, 0)
    qd = q * 3.0
    assert abs(fq[0, 0] - (2 + 2 * np.sin(qd) / qd)) < 2e-3


def test_incoherent_gaussian_diffusion():
    # Gaussian steps (per-axis sigma) give F_s(q,tau) -> b^2 exp(-q^2 sigma^2 tau / 2).
    w = synth.incoherent_fqt(seed=4, na=300, nf=16, nq=1, qmin=0.8, qmax=0.8, nm=20)
    w.class_factors[:] = 1.0
    fqt, _, _ = oracle.self_vectors(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), 0, 0)
    tau = np.arange(w.nf)
    expect = w.na * np.exp(-0.8 ** 2 * 0.1 ** 2 * tau / 2)
    got = cplx(fqt)[0].real
    assert np.allclose(got[:8], expect[:8], rtol=0.02)


def test_scan_and_factors():
    q = oracle.scan([1.0, 0.0, 0.0], 0.1, 2.0, 10, 1.0)
    assert q.shape == (10, 3)
    assert np.allclose(q[:, 0], np.linspace(0.1, 2.0, 10), atol=2e-7)
    assert q[0, 0] == 0.1 and q[-1, 0] == 2.0  # endpoints exact, interior via float powf
    v = np.array([1.0, 0.1, 2.0, 0.2, 0.5, 0.3, 0.25, 0.4, 0.1])
    for qq in (0.0, 0.3, 1.7):
        assert abs(oracle.sfactor(2, v, qq) - synth.sfactor_type2(v, qq)) < 1e-14
    assert oracle.sfactor(0, [3.5], 9.0) == 3.5
    assert np.isnan(oracle.sfactor(1, [1.0] * 15, 1.0))  # Slater: outside this path
