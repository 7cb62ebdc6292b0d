"""Shared helpers for the parity tests."""
import numpy as np


def rel_err_sqt(fqt, ref):
    """max_t |S - S_ref| / |S_ref(q,0)| per q (the path's error metric)."""
    ref = np.asarray(ref)
    fqt = np.asarray(fqt)
    if ref.ndim == 3:  # [nq, nf, 2] from the oracle
        ref = ref[..., 0] + 1j * ref[..., 1]
    den = np.maximum(np.abs(ref[:, 0]), 1e-300)
    return np.max(np.abs(fqt - ref), axis=1) / den


def cplx(a):
    a = np.asarray(a)
    return a[..., 0] + 1j * a[..., 1]


def rel_err_vec(x, ref):
    """|x - ref| / max(|ref|) over a vector of complex values."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    scale = max(np.max(np.abs(ref)), 1e-300)
    return np.max(np.abs(x - ref)) / scale
