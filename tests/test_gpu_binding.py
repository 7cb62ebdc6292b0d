"""The drop-in binding's calls, replayed through the real library on the GPU.

GpuVectorsScatterDevice (sassena_gb300/integration), compiled against the reference's
headers and driven by the reference's own run(), recorded the C ABI calls it makes on every
device case of tests/golden/reference.npz (see test_binding.py). Here the same calls go
through the real library: sass_plan_create with the recorded description, then
sass_stage_frames, sass_set_atom_classes and one sass_compute with the recorded sub-vectors
and class factors. The rows must equal the reference device's own rows: FP64 <= 1e-12,
FP32 <= 1e-3 (max_t |S - S_ref| / |S_ref(q,0)|; fq, fq2 relative to their largest value).
"""
import pytest

from sassena_gb300 import abi

from helpers import cplx, reference_cases, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-3}
CASES = reference_cases()
SCATTERING = {0: "all", 1: "self"}
DSP = {0: "autocorrelate", 1: "square", 2: "plain"}
METHOD = {0: "fftw", 1: "direct"}


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_binding_calls_on_gpu_match_reference_device(native_lib, name, precision):
    c = CASES[name]
    scattering, dsp, method, _, na, nf, nclass = (int(v) for v in c.bind_desc)
    with abi.Plan(na, nf, nclass, SCATTERING[scattering], DSP[dsp], METHOD[method], precision) as p:
        p.stage(c.coords)
        p.set_classes(c.bind_classes)
        fqt, fq, fq2 = p.compute(c.bind_offs, c.bind_subvectors, c.bind_class_factors)
    e = (rel_err_sqt(fqt, c.fqt).max(), rel_err_vec(fq, cplx(c.fq)), rel_err_vec(fq2, cplx(c.fq2)))
    assert max(e) <= TOL[precision], "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e
