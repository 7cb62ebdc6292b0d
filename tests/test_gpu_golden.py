"""The CUDA path through the C ABI against the committed golden fixtures (tests/golden, the FP64
oracle's outputs on seeded inputs kept in the fixture). Bars as in the other parity tests:
FP64 <= 1e-12, FP32 <= 1e-3 (max_t |S - S_ref| / |S_ref(q,0)|; fq, fq2 relative to their
largest value); the staged frames of the device pre-pass equal the fixture's (fits within
one float32 ulp)."""
import os

import numpy as np
import pytest

from sassena_gb300 import abi

from helpers import GOLDEN, cplx, golden, rel_err_sqt, rel_err_vec
import prepass_cases as pc

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-3}
SCATTER = golden("scatter")
MULTIPOLE = golden("multipole")
FITS = {"fitrottrans", "fitrot_file", "fit_instant", "pre_post"}


def errors(fx, fqt, fq, fq2):
    return (rel_err_sqt(fqt, fx.fqt).max(), rel_err_vec(fq, cplx(fx.fq)), rel_err_vec(fq2, cplx(fx.fq2)))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(SCATTER))
def test_scatter_matches_fixture(native_lib, name, precision):
    fx = SCATTER[name]
    with abi.Plan(fx.na, fx.nf, fx.class_factors.shape[1], fx.scattering, fx.dsp, fx.method, precision) as p:
        p.stage(fx.coords)
        p.set_classes(fx.atom_class)
        out = p.compute(fx.sub_offsets(), fx.subvectors(), fx.class_factors)
    e = errors(fx, *out)
    assert max(e) <= TOL[precision], "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e


@pytest.mark.parametrize("name", sorted(MULTIPOLE))
def test_multipole_matches_fixture(native_lib, name):
    fx = MULTIPOLE[name]
    moments = [tuple(int(v) for v in m) for m in fx.extra["moments"]]
    with abi.Plan(fx.na, fx.nf, fx.class_factors.shape[1], "all", fx.dsp, fx.method, "fp64") as p:
        p.stage(fx.coords)
        p.set_classes(fx.atom_class)
        out = p.multipole(str(fx.extra["mp"]), fx.extra["q"], fx.class_factors, moments,
                          tuple(fx.extra["axis"]))
    e = errors(fx, *out)
    assert max(e) <= 1e-12, "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e


@pytest.mark.parametrize("name", pc.CASES)
def test_prepass_matches_fixture(native_lib, tmp_path, name):
    z = np.load(os.path.join(GOLDEN, "prepass.npz"))
    w, cfg, o = pc.build(name, str(tmp_path / "run"))
    steps, masses = pc.host_steps(cfg, str(tmp_path / "dry.json"))
    target = o["target"] if o["target"] is not None else list(range(pc.NA))
    want = z[name + ".staged"]
    with abi.Plan(len(target), pc.NF, 4, "all", "autocorrelate", "fftw", "fp64") as p:
        got = p.stage_prepass(z["coords"], masses, steps, target)
    if name in FITS:
        assert (np.abs(got - want) <= np.spacing(np.abs(want).astype(np.float32))).all()
    else:
        np.testing.assert_array_equal(got, want)
