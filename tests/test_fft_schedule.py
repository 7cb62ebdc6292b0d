"""CPU emulation of the GPU correlation algorithm (index arithmetic of correlate.cu).

The device kernels use a radix-2 DIF forward transform (natural in, bit-reversed out)
whose first stage is folded into the load of the zero-padded series, a power spectrum
accumulated per shell, mean_tau C = sum_w P(w) K(w) with a bit-reversed kernel K, and a
radix-2 DIT inverse (bit-reversed in, natural out). These tests replay exactly those
loops in numpy and compare with the oracle's restatement of smath.cpp:141-156.
"""
import numpy as np
import pytest

import oracle


def bitrev(x, lg):
    r = 0
    for _ in range(lg):
        r = (r << 1) | (x & 1)
        x >>= 1
    return r


def twiddles(L):
    k = np.arange(L // 2)
    return np.exp(-2j * np.pi * k / L)


def dif_forward(x_nat, nf, lg):
    """Folded first stage + dif_tail, as in correlate.cu (x beyond nf is zero)."""
    L = 1 << lg
    half = L // 2
    tw = twiddles(L)
    buf = np.zeros(L, dtype=np.complex128)
    for p in range(half):
        x = x_nat[p] if p < nf else 0.0
        buf[p] = x
        buf[p + half] = x * tw[p]
    for lh in range(lg - 2, -1, -1):
        h = 1 << lh
        sh = lg - 1 - lh
        for b in range(half):
            p = b & (h - 1)
            i0 = ((b >> lh) << (lh + 1)) + p
            u, w = buf[i0], buf[i0 + h]
            buf[i0] = u + w
            buf[i0 + h] = (u - w) * tw[p << sh]
    return buf


def dit_inverse(buf, lg):
    L = 1 << lg
    half = L // 2
    tw = twiddles(L)
    buf = buf.copy()
    for lh in range(lg):
        h = 1 << lh
        sh = lg - 1 - lh
        for b in range(half):
            p = b & (h - 1)
            i0 = ((b >> lh) << (lh + 1)) + p
            u = buf[i0]
            w = buf[i0 + h] * np.conj(tw[p << sh])
            buf[i0] = u + w
            buf[i0 + h] = u - w
    return buf


def kernel_br(nf, lg):
    L = 1 << lg
    tau = np.arange(nf)
    wt = 1.0 / (nf * L * (nf - tau))
    K = np.array([np.sum(wt * np.exp(2j * np.pi * w * tau / L)) for w in range(L)])
    out = np.zeros(L, dtype=np.complex128)
    for w in range(L):
        out[bitrev(w, lg)] = K[w]
    return out


@pytest.mark.parametrize("nf", [1, 2, 3, 5, 8, 13, 16])
def test_dif_is_bitreversed_fft(nf):
    rng = np.random.default_rng(nf)
    lg = max(2, int(np.ceil(np.log2(2 * nf))))
    L = 1 << lg
    x = rng.normal(size=nf) + 1j * rng.normal(size=nf)
    y = dif_forward(x, nf, lg)
    ref = np.fft.fft(np.concatenate([x, np.zeros(L - nf)]))
    br = np.array([bitrev(i, lg) for i in range(L)])
    assert np.allclose(y, ref[br], atol=1e-12)


@pytest.mark.parametrize("lg", [2, 3, 5, 7])
def test_dit_inverse_of_bitreversed(lg):
    rng = np.random.default_rng(lg)
    L = 1 << lg
    X = rng.normal(size=L) + 1j * rng.normal(size=L)
    br = np.array([bitrev(i, lg) for i in range(L)])
    y = dit_inverse(X[br], lg)
    assert np.allclose(y, np.fft.ifft(X) * L, atol=1e-10)


@pytest.mark.parametrize("nf,nm", [(1, 1), (3, 2), (7, 3), (12, 4), (16, 1)])
def test_shell_pipeline_matches_oracle(nf, nm):
    """sum_v P_v -> one inverse; a_v = sum P K; equals per-series smath + store."""
    rng = np.random.default_rng(100 + nf)
    lg = max(2, int(np.ceil(np.log2(2 * nf))))
    L = 1 << lg
    series = rng.normal(size=(nm, nf)) + 1j * rng.normal(size=(nm, nf))
    K = kernel_br(nf, lg)
    P = np.zeros(L)
    asum = 0j
    a2 = 0.0
    for v in range(nm):
        X = dif_forward(series[v], nf, lg)
        Pv = np.abs(X) ** 2
        P += Pv
        av = np.sum(Pv * K)
        asum += av
        a2 += abs(av) ** 2
    y = dit_inverse(P.astype(np.complex128), lg)
    fqt = y[:nf] / (L * (nf - np.arange(nf))) / nm
    # reference semantics through the C++ oracle's smath restatement
    at = np.zeros(nf, dtype=np.complex128)
    ra = 0j
    ra2 = 0j
    for v in range(nm):
        c = oracle.autocorrelate_fftw(series[v])
        a = c.sum() / nf
        ra += a
        ra2 += a * np.conj(a)
        at += c
    assert np.allclose(fqt, at / nm, rtol=1e-12, atol=1e-12 * np.abs(at[0]))
    assert np.allclose(asum / nm, ra / nm, rtol=1e-12, atol=1e-13)
    assert np.allclose(a2 / nm, (ra2 / nm).real, rtol=1e-12)
