"""Long trajectories (NF > 4096): the four-step autocorrelation through HBM (padded length
2^14 .. 2^20) and the frame-looped square/plain kernels, against the oracle. The reference
has no frame limit; these sizes take the paths that the short-series tests never reach.
Bars as everywhere: FP64 <= 1e-12, FP32 <= 1e-3 (max_t |S - S_ref| / |S_ref(q,0)|)."""
import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

from helpers import cplx, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}
TOL = {"fp64": 1e-12, "fp32": 1e-3}


def check(w, precision, method="fftw", tol=None):
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    ref = fn(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), DSP_ID[w.dsp], METHOD_ID[method],
             nthreads=8)
    fqt, fq, fq2 = abi.compute_workload(w, precision=precision, method=method)
    tol = tol or TOL[precision]
    e = (rel_err_sqt(fqt, ref[0]).max(), rel_err_vec(fq, cplx(ref[1])), rel_err_vec(fq2, cplx(ref[2])))
    assert max(e) <= tol, "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e
    return e


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nf", [4097, 5000, 9000, 30000])
def test_coherent_long_autocorrelation(native_lib, precision, nf):
    # padded lengths 2^14, 2^14, 2^15, 2^16: R = 4, 4, 8, 16 rows of 4,096
    w = synth.small("all", "autocorrelate", seed=71, na=23, nf=nf, nq=2, nm=3, box=10.0)
    check(w, precision)


def test_coherent_long_direct_method(native_lib):
    # dsp.method = direct: the conjugate convention of smath.cpp:51-76 at long length
    w = synth.small("all", "autocorrelate", seed=72, na=17, nf=4500, nq=2, nm=2, box=10.0)
    check(w, "fp64", method="direct")


def test_coherent_long_many_series(native_lib):
    # enough series per shell for several chunks per row
    w = synth.small("all", "autocorrelate", seed=73, na=11, nf=4200, nq=3, nm=40, box=10.0)
    check(w, "fp64")


@pytest.mark.parametrize("scattering", ["all", "self"])
@pytest.mark.parametrize("dsp", ["square", "plain"])
def test_long_square_plain(native_lib, scattering, dsp):
    w = synth.small(scattering, dsp, seed=74, na=13, nf=6000, nq=2, nm=3, box=10.0)
    check(w, "fp64")
    check(w, "fp32")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nf", [4100, 8300])
def test_incoherent_long_autocorrelation(native_lib, precision, nf):
    # (atom, direction) series generated per batch, then the same four-step passes
    w = synth.small("self", "autocorrelate", seed=76, na=13, nf=nf, nq=2, nm=3, box=10.0)
    check(w, precision)


def test_incoherent_long_direct_method(native_lib):
    w = synth.small("self", "autocorrelate", seed=77, na=7, nf=4400, nq=2, nm=2, box=10.0)
    check(w, "fp64", method="direct")


def test_longest_series_refused(native_lib):
    with pytest.raises(abi.SassError) as e:
        abi.Plan(10, 600000, 1, "all", "autocorrelate", "fftw", "fp64")
    assert e.value.code == 3


def test_multipole_long(native_lib):
    # given amplitudes (the multipole devices) through the long correlation
    w = synth.small("all", "autocorrelate", seed=75, na=15, nf=4300, nq=2, nm=3, box=10.0)
    rng = np.random.default_rng(75)
    q = rng.normal(size=(2, 3))
    q *= (w.shells / np.linalg.norm(q, axis=1))[:, None]
    moments = oracle.sphere_moments(3)
    ref = oracle.mp_sphere(w.coords, q, w.factors(), moments)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", "autocorrelate", "fftw", "fp64") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        fqt, fq, fq2 = p.multipole("sphere", q, w.class_factors, moments)
    assert rel_err_sqt(fqt, ref[0]).max() <= 1e-12
    assert rel_err_vec(fq, cplx(ref[1])) <= 1e-12
