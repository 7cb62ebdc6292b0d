"""The benchmark configurations at full size, through properties that do not need the CPU
oracle at that size:
  * incoherent F(q, 0) = sum_j b_j^2 exactly (|exp(i q.r)| = 1), per shell;
  * fq2 >= |fq|^2 (the mean of |mean_v|^2 against the square of the mean; incoherent:
    n fq2 >= |fq|^2 with n the atoms summed per direction);
  * fqt(q, 0) real and non-negative, fq0 = fqt(q, 0);
  * the FP32 form against the plain FP64 form on a subset of shells (same GPU), bar 1e-3;
  * the kernel the schedule reports (the shell recurrence for the scans).
The FP64 form itself is pinned against the oracle at small sizes (test_gpu_parity.py)."""
import numpy as np
import pytest

from sassena_gb300 import abi, synth

from helpers import rel_err_sqt

pytestmark = pytest.mark.gpu


def run(w, precision, shells=None, schedule=None):
    idx = np.arange(w.nq) if shells is None else np.asarray(shells)
    offs = np.arange(len(idx) + 1, dtype=np.uintp) * w.nm
    sv = (w.shells[idx, None, None] * w.directions[None]).reshape(-1, 3)
    with abi.Plan(w.na, w.nf, len(w.class_names), w.scattering, w.dsp, "fftw", precision) as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        out = p.compute(offs, sv, w.class_factors[idx])
        if schedule is not None:
            schedule.update(p.schedule())
    return out


def common_properties(fqt, fq, fq2, n=1):
    # n: series summed (not averaged) per direction, i.e. the atoms of the incoherent device
    # (Cauchy-Schwarz: |sum of n means|^2 <= n sum |mean|^2)
    s0 = fqt[:, 0]
    assert np.all(s0.real >= 0)
    assert np.abs(s0.imag).max() <= 1e-6 * np.abs(s0.real).max()
    assert np.all(n * fq2.real >= np.abs(fq) ** 2 * (1 - 1e-6))


def test_coherent_sqt_full_size(native_lib):
    w = synth.coherent_sqt()  # 10,000 atoms, 1,024 frames, 20 shells x 500 directions
    sch = {}
    fqt, fq, fq2 = run(w, "fp32", schedule=sch)
    assert sch["rec_tiles"] > 0 and sch["direct_tiles"] == 0  # the scan takes the recurrence
    common_properties(fqt, fq, fq2)
    sub = [0, w.nq // 2, w.nq - 1]
    ref = run(w, "fp64", shells=sub)
    assert rel_err_sqt(fqt[sub], ref[0]).max() <= 1e-3


def test_incoherent_fqt_full_size(native_lib):
    w = synth.incoherent_fqt()  # 1,000 atoms, 128 frames, 10 shells x 100 directions
    b2 = (w.factors() ** 2).sum(axis=1)  # F_s(q, 0) = sum_j b_j^2
    for precision, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        fqt, fq, fq2 = run(w, precision)
        np.testing.assert_allclose(fqt[:, 0].real, b2, rtol=tol, atol=0)
        common_properties(fqt, fq, fq2, n=w.na)
    ref = run(w, "fp64")
    assert rel_err_sqt(run(w, "fp32")[0], ref[0]).max() <= 1e-3


def test_static_xray_full_size(native_lib):
    w = synth.static_xray()  # 100,000 atoms, 64 frames, 200 shells x 2,000 directions, square
    fqt, fq, fq2 = run(w, "fp32")
    assert np.all(fqt.real >= 0) and np.abs(fqt.imag).max() == 0.0  # |A|^2 averaged
    common_properties(fqt, fq, fq2)
    ref = run(w, "fp64", shells=[w.nq // 3])
    assert rel_err_sqt(fqt[[w.nq // 3]], ref[0]).max() <= 1e-3
