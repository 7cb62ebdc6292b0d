"""Independent numpy FP64 restatement of the scattering-amplitude path (test infrastructure).

A second oracle, written separately from ``cpu_oracle.cpp`` so that the two cross-check
each other. Vectorised over atoms and frames; meant for small shapes only.

References (paths inside the reference project):
  phase sum          src/scatter_devices/all_vectors_scatter_device.cpp:418-438
  self series        src/scatter_devices/self_vectors_scatter_device.cpp:306-317
  FFT correlation    src/math/smath.cpp:141-156 (forward, |X|^2, backward, 1/(2NF(NF-tau)))
  direct correlation src/math/smath.cpp:51-76 (conjugate sign convention)
  store              src/scatter_devices/all_vectors_scatter_device.cpp:231-236
  normalisation      src/scatter_devices/all_vectors_scatter_device.cpp:355-360
"""
from __future__ import annotations

import numpy as np


def amplitude(coords, q, b):
    """A(t) = sum_j b_j exp(i q.r_j(t)); coords float32 [nf, na, 3] promoted to float64."""
    r = np.asarray(coords, dtype=np.float32).astype(np.float64)
    p = r @ np.asarray(q, dtype=np.float64)  # [nf, na]
    return (np.asarray(b, dtype=np.float64)[None, :] * np.exp(1j * p)).sum(axis=1)


def correlate(a, dsp_type=0, dsp_method=0):
    """dsp of one series (smath.cpp): autocorrelate (fftw/direct), square, plain."""
    a = np.asarray(a, dtype=np.complex128)
    nf = len(a)
    if dsp_type == 0:
        x = np.zeros(2 * nf, dtype=np.complex128)
        x[:nf] = a
        X = np.fft.fft(x)
        c = np.fft.ifft(np.abs(X) ** 2) * (2 * nf)  # unnormalised backward transform
        c = c[:nf] / (2 * nf * (nf - np.arange(nf)))
        return np.conj(c) if dsp_method == 1 else c
    if dsp_type == 1:
        return (np.abs(a) ** 2).astype(np.complex128)
    return a.copy()


def _accumulate(series_list, nf):
    at = np.zeros(nf, dtype=np.complex128)
    a1 = 0j
    a2 = 0j
    for c in series_list:
        a = c.sum() / nf
        a1 += a
        a2 += a * np.conj(a)
        at += c
    return at, a1, a2


def all_vectors(coords, sub_offsets, subvectors, factors, dsp_type=0, dsp_method=0):
    coords = np.asarray(coords, dtype=np.float32)
    nf = coords.shape[0]
    nq = len(sub_offsets) - 1
    fqt = np.zeros((nq, nf), dtype=np.complex128)
    fq = np.zeros(nq, dtype=np.complex128)
    fq2 = np.zeros(nq, dtype=np.complex128)
    for iq in range(nq):
        m0, m1 = sub_offsets[iq], sub_offsets[iq + 1]
        cs = [correlate(amplitude(coords, subvectors[m], factors[iq]), dsp_type, dsp_method)
              for m in range(m0, m1)]
        at, a1, a2 = _accumulate(cs, nf)
        nm = m1 - m0
        fqt[iq], fq[iq], fq2[iq] = at / nm, a1 / nm, a2 / nm
    return fqt, fq, fq2


def self_vectors(coords, sub_offsets, subvectors, factors, dsp_type=0, dsp_method=0):
    r = np.asarray(coords, dtype=np.float32).astype(np.float64)
    nf, na = r.shape[0], r.shape[1]
    nq = len(sub_offsets) - 1
    fqt = np.zeros((nq, nf), dtype=np.complex128)
    fq = np.zeros(nq, dtype=np.complex128)
    fq2 = np.zeros(nq, dtype=np.complex128)
    for iq in range(nq):
        m0, m1 = sub_offsets[iq], sub_offsets[iq + 1]
        cs = []
        for j in range(na):
            for m in range(m0, m1):
                p = r[:, j, :] @ np.asarray(subvectors[m], dtype=np.float64)
                cs.append(correlate(factors[iq][j] * np.exp(1j * p), dsp_type, dsp_method))
        at, a1, a2 = _accumulate(cs, nf)
        nm = m1 - m0
        fqt[iq], fq[iq], fq2[iq] = at / nm, a1 / nm, a2 / nm
    return fqt, fq, fq2
