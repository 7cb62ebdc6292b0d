"""The batched form: many systems of uneven size in one graph-captured launch sequence
(one persistent phase-sum launch over all systems' tiles), checked per system against
the oracle, replayed, and autotuned."""
import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

from helpers import cplx, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-3}


def workloads(scattering="all"):
    return synth.batched_uneven(seed=9, nsys=5, na_range=(40, 300), nf_range=(9, 60),
                                nq_range=(1, 4), nm_range=(3, 70), scattering=scattering)


def ref(w):
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    return fn(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), 0, 0, nthreads=8)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("scattering", ["all", "self"])
def test_batch_matches_oracle_per_system(native_lib, precision, scattering):
    ws = workloads(scattering)
    refs = [ref(w) for w in ws]
    with abi.Batch(ws, precision=precision) as b:
        for replay in range(2):  # the graph is captured once and replayed
            b.run()
            b.sync()
            for w, r in zip(ws, refs):
                fqt, fq, fq2 = b.results(ws.index(w))
                assert rel_err_sqt(fqt, r[0]).max() <= TOL[precision]
                assert rel_err_vec(fq, cplx(r[1])) <= TOL[precision]
                assert rel_err_vec(fq2, cplx(r[2])) <= TOL[precision]
        info = b.info()
        assert info["terms"] == sum(w.terms() for w in ws)


def test_batch_autotune_keeps_results(native_lib):
    ws = workloads("all")
    refs = [ref(w) for w in ws]
    with abi.Batch(ws, precision="fp32") as b:
        best = b.autotune(repeats=1)
        assert best["q_per_lane"] in (0, 1, 2, 4, 8) and best["ms"] > 0
        b.run()
        b.sync()
        for i, r in enumerate(refs):
            assert rel_err_sqt(b.results(i)[0], r[0]).max() <= 1e-3


def test_plan_autotune(native_lib):
    w = synth.small("all", "autocorrelate", seed=61, na=500, nf=40, nq=3, nm=70)
    r = ref(w)
    with abi.Plan(w.na, w.nf, len(w.class_names), precision="fp32") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        shape = p.autotune(w.sub_offsets(), w.subvectors(), w.class_factors, repeats=1)
        fqt, _, _ = p.compute(w.sub_offsets(), w.subvectors(), w.class_factors)
        # q_per_lane 0: the automatic tile shape won (or the recurrence covers every shell)
        assert shape["q_per_lane"] in (0, 1, 2, 4, 8)
    assert rel_err_sqt(fqt, r[0]).max() <= 1e-3


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("scattering", ["all", "self"])
def test_batch_mixes_long_and_short_series(native_lib, precision, scattering):
    # one captured launch sequence with a long system (four-step transform through HBM,
    # NF > 4096) next to short ones (shared-memory transforms)
    ws = [synth.small(scattering, "autocorrelate", seed=81, na=9, nf=4500, nq=2, nm=3, box=10.0),
          synth.small(scattering, "autocorrelate", seed=82, na=31, nf=40, nq=3, nm=5),
          synth.small(scattering, "autocorrelate", seed=83, na=12, nf=9000, nq=1, nm=2, box=10.0)]
    refs = [ref(w) for w in ws]
    with abi.Batch(ws, precision=precision) as b:
        for replay in range(2):
            b.run()
            b.sync()
            for i, r in enumerate(refs):
                fqt, fq, fq2 = b.results(i)
                assert rel_err_sqt(fqt, r[0]).max() <= TOL[precision]
                assert rel_err_vec(fq, cplx(r[1])) <= TOL[precision]
