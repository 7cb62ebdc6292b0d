"""The oracle against the committed golden fixtures (tests/golden, made by make_golden.py).

The fixtures hold seeded inputs with the FP64 oracle's outputs; these CPU tests keep both
restatements (the C++ oracle and the numpy oracle) on them, so a change to either shows up
here. The GPU path is held to the same fixtures in test_gpu_golden.py."""
import os

import numpy as np
import pytest

import oracle
import oracle.numpy_oracle as npo
from oracle import alignment as al

from helpers import GOLDEN, cplx, golden, rel_err_sqt, rel_err_vec
import prepass_cases as pc

DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}
SCATTER = golden("scatter")
MULTIPOLE = golden("multipole")


def errors(fx, out):
    return (rel_err_sqt(cplx(out[0]), fx.fqt).max(), rel_err_vec(cplx(out[1]), cplx(fx.fq)),
            rel_err_vec(cplx(out[2]), cplx(fx.fq2)))


def test_fixture_inventory():
    # every dsp type and method on both devices, the three workload shapes and a long series
    assert len(SCATTER) == 13 and set(MULTIPOLE) == {"mp_sphere", "mp_cylinder"}
    kinds = {(f.scattering, f.dsp, f.method) for f in SCATTER.values()}
    for s in ("all", "self"):
        for d, m in (("autocorrelate", "fftw"), ("autocorrelate", "direct"), ("square", "fftw"),
                     ("plain", "fftw")):
            assert (s, d, m) in kinds
    assert SCATTER["long_series"].nf > 4096 and SCATTER["coherent_sqt_shape"].nf == 1024
    assert SCATTER["incoherent_blocks"].nf == 600 and SCATTER["incoherent_blocks"].scattering == "self"


@pytest.mark.parametrize("name", sorted(SCATTER))
def test_cpp_oracle_reproduces_fixture(name):
    fx = SCATTER[name]
    fn = oracle.all_vectors if fx.scattering == "all" else oracle.self_vectors
    out = fn(fx.coords, fx.sub_offsets(), fx.subvectors(), fx.factors(), DSP_ID[fx.dsp], METHOD_ID[fx.method],
             nthreads=4)
    assert max(errors(fx, out)) <= 1e-13


@pytest.mark.parametrize("name", sorted(n for n in SCATTER if n != "long_series"))
def test_numpy_oracle_reproduces_fixture(name):
    fx = SCATTER[name]
    fn = npo.all_vectors if fx.scattering == "all" else npo.self_vectors
    fqt, fq, fq2 = fn(fx.coords, fx.sub_offsets(), fx.subvectors(), fx.factors(), DSP_ID[fx.dsp],
                      METHOD_ID[fx.method])
    assert rel_err_sqt(fqt, fx.fqt).max() <= 1e-12
    assert rel_err_vec(fq, cplx(fx.fq)) <= 1e-12 and rel_err_vec(fq2, cplx(fx.fq2)) <= 1e-12


@pytest.mark.parametrize("name", sorted(MULTIPOLE))
def test_multipole_oracle_reproduces_fixture(name):
    fx = MULTIPOLE[name]
    mom = [tuple(int(v) for v in m) for m in fx.extra["moments"]]
    if str(fx.extra["mp"]) == "sphere":
        out = oracle.mp_sphere(fx.coords, fx.extra["q"], fx.factors(), mom)
    else:
        out = oracle.mp_cylinder(fx.coords, fx.extra["q"], fx.factors(), mom, tuple(fx.extra["axis"]))
    assert max(errors(fx, out)) <= 1e-13


@pytest.mark.parametrize("name", pc.CASES)
def test_alignment_oracle_reproduces_fixture(tmp_path, name):
    z = np.load(os.path.join(GOLDEN, "prepass.npz"))
    w, _, o = pc.build(name, str(tmp_path / "run"))
    np.testing.assert_array_equal(w.coords, z["coords"])  # the case's inputs are the fixture's
    got = al.load(w.coords, o["masses"], o["alignments"], o["motions"], o["target"])
    want = z[name + ".staged"]
    # fits go through LAPACK's SVD, whose last bits may differ between builds
    assert (np.abs(got - want) <= np.spacing(np.abs(want).astype(np.float32))).all()

