"""The drop-in binding (sassena_gb300/integration: GpuVectorsScatterDevice) against the
reference itself, on the CPU.

The binding is compiled against the reference's own headers and driven by the reference's
own AbstractScatterDevice::run() in oracle/_ref (oracle/ref_build), with a C ABI that
records its calls instead of running them. tests/golden/reference.npz keeps, for every
device case, the reference device's rows and the binding's recorded calls on the same
inputs. Here:
  - the oracle run on exactly the recorded calls (sub-vectors, per-atom classes, class
    factors) reproduces the reference device's rows, so the binding hands the library the
    reference's sub-vectors and scattering lengths;
  - every class groups atoms of one database type, and its factors are the reference's
    ScatterFactors values for that type;
  - where the reference tree is present, the binding is rebuilt against it and rerun.
The recorded calls are replayed through the real library on the GPU in
test_gpu_binding.py.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle

from helpers import cplx, reference_cases, reference_fixture, rel_err_sqt, rel_err_vec

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = reference_cases()
DSP = {0: 0, 1: 1, 2: 2}
TYPE = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD = {"fftw": 0, "direct": 1}


def tolerance(case):
    if case.dsp == "autocorrelate" and case.method == "fftw":
        return 1e-13 * max(1.0, case.nf / 256.0)
    return 1e-15


@pytest.mark.parametrize("name", sorted(CASES))
def test_binding_calls_reproduce_reference_rows(name):
    c = CASES[name]
    scattering, dsp, method, precision, na, nf, nclass = (int(v) for v in c.bind_desc)
    assert (scattering, dsp, method, precision) == (c.scattering == "self", TYPE[c.dsp], METHOD[c.method], 0)
    assert (na, nf, nclass) == (c.na, c.nf, c.bind_class_factors.shape[1])
    factors = c.bind_class_factors[:, c.bind_classes]  # [nq][na]
    fn = oracle.all_vectors if c.scattering == "all" else oracle.self_vectors
    fqt, fq, fq2 = fn(c.coords, c.bind_offs, c.bind_subvectors, factors, TYPE[c.dsp], METHOD[c.method], nthreads=4)
    e = (rel_err_sqt(cplx(fqt), c.fqt).max(), rel_err_vec(cplx(fq), cplx(c.fq)), rel_err_vec(cplx(fq2), cplx(c.fq2)))
    assert max(e) <= tolerance(c), "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e


@pytest.mark.parametrize("name", sorted(CASES))
def test_binding_classes_follow_scatter_factors(name):
    """One class per database type present (kappa 1 everywhere in these cases), with the
    factors the reference's ScatterFactors gives that type at every |q|."""
    c = CASES[name]
    types = c.atom_class  # the database type of every target atom
    for k in np.unique(c.bind_classes):
        members = types[c.bind_classes == k]
        assert np.all(members == members[0])
        np.testing.assert_array_equal(c.bind_class_factors[:, k], c.class_factors[:, members[0]])
    assert len(np.unique(c.bind_classes)) == len(np.unique(types))


def test_binding_builds_against_reference_and_reruns():
    """Rebuild oracle/_ref (the reference's sources and the binding against its headers) and
    rerun the binding on one case: the recorded calls must equal the fixture's. Skipped
    where the reference tree is absent (the GPU machine)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "make_reference_golden", os.path.join(ROOT, "tests", "golden", "make_reference_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    try:
        L = mk.load()
    except (subprocess.CalledProcessError, OSError) as e:
        pytest.skip("reference tree not available: %s" % e)
    z = reference_fixture()
    name = "coh_square_xray_background"
    g = lambda k: z[name + "." + k]  # noqa: E731
    self_, dsp, method = str(g("kind")).split("/")
    tables = (g("sf_type"), g("sf_const"), g("vol"), g("ex_type"), g("ex_const"))
    q_out, _, _, _ = mk.run_case(L, self_ == "self", dsp, method, g("coords"), g("atom_type"), tables,
                                 float(g("background")), g("qvectors"), g("orient"), binding=True)
    assert np.array_equal(q_out, g("q_out"))
    calls = mk.binding_calls(L, g("coords"))
    for k, v in calls.items():
        assert np.array_equal(v, g(k)), k
