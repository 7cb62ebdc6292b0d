"""The CUDA path through the C ABI against the reference's own compiled code.

tests/golden/reference.npz holds outputs of the reference's scatter devices compiled from
its sources (see tests/golden/make_reference_golden.py). The GPU computes the same runs
from the fixture's inputs: the sub-vectors as the reference forms them and the class
factors of the reference's ScatterFactors. Bars: FP64 <= 1e-12, FP32 <= 1e-3, on
max_t |S - S_ref| / |S_ref(q,0)| per q and on fq, fq2 relative to their largest value.
"""
import numpy as np
import pytest

from sassena_gb300 import abi

from helpers import cplx, reference_cases, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-3}
CASES = reference_cases()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_devices(native_lib, name, precision):
    c = CASES[name]
    with abi.Plan(c.na, c.nf, c.class_factors.shape[1], c.scattering, c.dsp, c.method, precision) as p:
        p.stage(c.coords)
        p.set_classes(c.atom_class)
        fqt, fq, fq2 = p.compute(c.sub_offsets(), c.subvectors(), c.class_factors)
    e = (rel_err_sqt(fqt, c.fqt).max(), rel_err_vec(fq, cplx(c.fq)), rel_err_vec(fq2, cplx(c.fq2)))
    assert max(e) <= TOL[precision], "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e
