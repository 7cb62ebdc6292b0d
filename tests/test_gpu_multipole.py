"""GPU parity of the multipole devices (sass_multipole_compute) against the FP64 oracle:
MPSphereScatterDevice and MPCylinderScatterDevice (multipole_scatter_device.cpp), bar
1e-12 with the error metric max_t |S - S_ref| / |S_ref(q,0)| (FP64 form)."""
import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

from helpers import cplx, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}


def case(seed, na, nf, nq, box=12.0, dsp="autocorrelate"):
    w = synth.small("all", dsp, seed=seed, na=na, nf=nf, nq=nq, nm=3, box=box)
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(nq, 3))
    q *= (w.shells / np.linalg.norm(q, axis=1))[:, None]
    return w, q


def check(w, q, kind, moments, axis=(0.0, 0.0, 1.0), method="fftw", tol=1e-12):
    if kind == "sphere":
        ref = oracle.mp_sphere(w.coords, q, w.factors(), moments, DSP_ID[w.dsp], METHOD_ID[method])
    else:
        ref = oracle.mp_cylinder(w.coords, q, w.factors(), moments, axis, DSP_ID[w.dsp],
                                 METHOD_ID[method])
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", w.dsp, method, "fp64") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        fqt, fq, fq2 = p.multipole(kind, q, w.class_factors, moments, axis)
    e = (rel_err_sqt(fqt, ref[0]).max(), rel_err_vec(fq, cplx(ref[1])), rel_err_vec(fq2, cplx(ref[2])))
    assert max(e) <= tol, "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e
    return e


@pytest.mark.parametrize("dsp,method", [("autocorrelate", "fftw"), ("autocorrelate", "direct"),
                                        ("square", "fftw"), ("plain", "fftw")])
def test_sphere_parity(native_lib, dsp, method):
    w, q = case(51, na=37, nf=24, nq=3, dsp=dsp)
    check(w, q, "sphere", oracle.sphere_moments(8), method=method)


@pytest.mark.parametrize("dsp,method", [("autocorrelate", "fftw"), ("autocorrelate", "direct"),
                                        ("square", "fftw"), ("plain", "fftw")])
def test_cylinder_parity(native_lib, dsp, method):
    w, q = case(52, na=41, nf=20, nq=3, dsp=dsp)
    check(w, q, "cylinder", oracle.cylinder_moments(8), axis=(1.0, 1.0, 0.3), method=method)


def test_sphere_moment_file_and_ragged_sizes(native_lib):
    # a moment list as a file gives it: any order, any subset (parameters.cpp:1039-1047)
    w, q = case(53, na=300, nf=37, nq=4, box=30.0)
    moments = [(3, -2), (0, 0), (12, 5), (12, -12), (1, 1), (7, 0), (3, 2)]
    check(w, q, "sphere", moments)


def test_large_arguments(native_lib):
    # |q| r up to ~100: the asymptotic / upward Bessel paths and the sphere's upward recurrence
    w, q = case(54, na=150, nf=16, nq=2, box=60.0)
    q *= 3.0 / np.linalg.norm(q, axis=1)[:, None]
    check(w, q, "sphere", oracle.sphere_moments(20))
    check(w, q, "cylinder", oracle.cylinder_moments(20), axis=(0.2, -0.5, 1.0))


def test_sphere_cached_representation_follows_classes_and_frames(native_lib):
    # the sphere's representation (atoms in radius order, classes carried along) is cached
    # between calls: new classes or a new staging rebuild it
    w, q = case(59, na=70, nf=10, nq=2, box=30.0)
    mom = oracle.sphere_moments(6)
    cls2 = w.atom_class[::-1].copy()
    w2 = synth.small("all", "autocorrelate", seed=60, na=70, nf=10, nq=2, nm=3, box=30.0)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", "autocorrelate", "fftw", "fp64") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        for coords, cls in ((w.coords, w.atom_class), (w.coords, cls2), (w2.coords, cls2)):
            if coords is not w.coords:
                p.stage(coords)
            p.set_classes(cls)
            fqt, fq, fq2 = p.multipole("sphere", q, w.class_factors, mom)
            ref = oracle.mp_sphere(coords, q, w.class_factors[:, cls], mom)
            assert rel_err_sqt(fqt, ref[0]).max() <= 1e-12
            assert rel_err_vec(fq, cplx(ref[1])) <= 1e-12


def test_cylinder_cached_representation_follows_classes_and_frames(native_lib):
    # the cylinder representation (atoms in radius order, classes carried along) is cached
    # between calls: new classes or a new staging rebuild it, another axis too
    w, q = case(57, na=70, nf=10, nq=2, box=30.0)
    mom = oracle.cylinder_moments(6)
    cls2 = w.atom_class[::-1].copy()
    w2 = synth.small("all", "autocorrelate", seed=58, na=70, nf=10, nq=2, nm=3, box=30.0)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", "autocorrelate", "fftw", "fp64") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        for coords, cls, axis in ((w.coords, w.atom_class, (0.0, 0.0, 1.0)), (w.coords, cls2, (0.0, 0.0, 1.0)),
                                  (w2.coords, cls2, (0.0, 0.0, 1.0)), (w2.coords, cls2, (1.0, 0.5, 0.2))):
            if coords is not w.coords:
                p.stage(coords)
            p.set_classes(cls)
            fqt, fq, fq2 = p.multipole("cylinder", q, w.class_factors, mom, axis)
            ref = oracle.mp_cylinder(coords, q, w.class_factors[:, cls], mom, axis)
            assert rel_err_sqt(fqt, ref[0]).max() <= 1e-12
            assert rel_err_vec(fq, cplx(ref[1])) <= 1e-12


def test_cylinder_axis_along_reference_axes(native_lib):
    w, q = case(55, na=64, nf=12, nq=2)
    for axis in [(0, 0, 1.0), (0, 0, -2.0), (1.0, 0, 0), (0, 3.0, 0)]:
        check(w, q, "cylinder", oracle.cylinder_moments(5), axis=axis)


def test_errors(native_lib):
    w, q = case(56, na=20, nf=8, nq=1)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", precision="fp32") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        with pytest.raises(abi.SassError) as e:
            p.multipole("sphere", q, w.class_factors, [(0, 0)])
        assert e.value.code == 3  # SASS_ERR_UNSUPPORTED
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", precision="fp64") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        for kind, mom in [("sphere", [(2, 3)]), ("cylinder", [(1, 4)]), ("cylinder", [(0, 1)])]:
            with pytest.raises(abi.SassError) as e:
                p.multipole(kind, q, w.class_factors, mom)
            assert e.value.code == 1  # SASS_ERR_ARG


@pytest.mark.parametrize("kind", ["sphere", "cylinder"])
def test_more_frames_than_one_grid_dimension(native_lib, kind):
    # 70,000 frames: the cylinder launches frames in chunks of 65,535 (grid y), the sphere
    # batches at most 65,535 frames per basis, and the correlation takes the long path
    w, q = case(56, na=5, nf=70000, nq=1, box=6.0)
    moments = oracle.sphere_moments(1) if kind == "sphere" else oracle.cylinder_moments(1)
    # at the largest lags an FFT-based correlation (the oracle's, the reference's FFTW, this
    # one) recovers a single product from transforms of the whole series: rounding relative to
    # S(q,0) grows with NF, so the FP64 bar scales as NF / 16,384 beyond that length
    check(w, q, kind, moments, axis=(0.2, 0.1, 1.0), tol=1e-12 * 70000 / 16384)
