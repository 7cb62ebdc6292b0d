"""The oracle pinned to the reference's own compiled code (CPU).

tests/golden/reference.npz holds the outputs of the reference's scatter devices, signal
math, scatter factors, database getters and q-vector scans, compiled from the reference's
sources by oracle/ref_build (FFTW replaced by an extended-precision DFT with FFTW's
definition) on seeded inputs kept in the fixture. The C++ oracle must reproduce them:
  - dsp square and plain, and the direct autocorrelation: the same FP64 sums in the same
    order, so the same bits (checked to 1e-15);
  - the FFT autocorrelation: within FFT rounding, 1e-13 of |S(q,0)| per 256 frames;
  - database getters and scans: bit for bit (the scans' float powf included).
The GPU path is held to the same fixture in test_gpu_reference_pin.py.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

from helpers import cplx, reference_cases, reference_fixture, rel_err_sqt, rel_err_vec

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}
CASES = reference_cases()


def tolerance(case):
    if case.dsp == "autocorrelate" and case.method == "fftw":
        return 1e-13 * max(1.0, case.nf / 256.0)
    return 1e-15


def test_fixture_inventory():
    kinds = {(c.scattering, c.dsp, c.method) for c in CASES.values()}
    for s in ("all", "self"):
        for d, m in (("autocorrelate", "fftw"), ("autocorrelate", "direct"), ("square", "fftw"),
                     ("plain", "fftw")):
            assert (s, d, m) in kinds
    nfs = {c.nf for c in CASES.values()}
    assert {37, 128, 1024} <= nfs
    assert any(len(c.orient) == 0 for c in CASES.values())
    for c in CASES.values():
        assert np.array_equal(c.q_out, c.qvectors)  # rows written in q order, one rank


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference_devices(name):
    c = CASES[name]
    fn = oracle.all_vectors if c.scattering == "all" else oracle.self_vectors
    fqt, fq, fq2 = fn(c.coords, c.sub_offsets(), c.subvectors(), c.factors(), DSP_ID[c.dsp], METHOD_ID[c.method],
                      nthreads=4)
    e = (rel_err_sqt(cplx(fqt), c.fqt).max(), rel_err_vec(cplx(fq), cplx(c.fq)), rel_err_vec(cplx(fq2), cplx(c.fq2)))
    assert max(e) <= tolerance(c), "rel err fqt/fq/fq2 = %.2e/%.2e/%.2e" % e


def test_oracle_database_getters_match_reference():
    z = reference_fixture()
    for row in z["db.sfactor"]:
        ft, q, c = int(row[0]), row[1], row[2:11]
        assert oracle.sfactor(ft, c, q) == row[11]
    for ft, r, want in z["db.volume"]:
        assert oracle.volume(int(ft), [r]) == want
    for ft, c, v, q, want in z["db.exclusion"]:
        assert oracle.exclusion(int(ft), [c], v, q) == want


def test_class_factors_follow_reference_scatter_factors():
    """b = sf - background * exclusion(kappa * volume, |q|) per type and |q| (the reference's
    ScatterFactors::update) against the oracle's database restatement."""
    z = reference_fixture()
    c = CASES["coh_square_xray_background"]
    bg = float(z[c.name + ".background"])
    sf_type, sf_const = z[c.name + ".sf_type"], z[c.name + ".sf_const"]
    vol, ex_type, ex_const = z[c.name + ".vol"], z[c.name + ".ex_type"], z[c.name + ".ex_const"]
    q = c.qvectors
    for i, ql in enumerate(np.sqrt(q[:, 0] ** 2 + q[:, 1] ** 2 + q[:, 2] ** 2)):
        for t in range(len(sf_type)):
            v = oracle.volume(0, [vol[t]])
            want = oracle.sfactor(int(sf_type[t]), sf_const[t], ql) - bg * oracle.exclusion(
                int(ex_type[t]), [ex_const[t]], 1.0 * v, ql)
            assert want == c.class_factors[i, t]


def _scan_names():
    z = reference_fixture()
    return sorted({k.split(".", 1)[0] for k in z.files if k.startswith("scans_")})


@pytest.mark.parametrize("name", _scan_names())
def test_oracle_and_host_scans_match_reference(name, tmp_path):
    z = reference_fixture()
    g = lambda k: z[name + "." + k]  # noqa: E731
    want = g("qvectors")
    frm, to, pts, ex, base = g("scan_from"), g("scan_to"), g("scan_points"), g("scan_exponent"), g("scan_base")
    if len(frm) == 1:
        got = oracle.scan(base[0], frm[0], to[0], int(pts[0]), ex[0])
        assert np.array_equal(got.reshape(-1, 3), want)
    # the host layer's configuration reader (sassena-gpu) for every case
    w = synth.small("all", seed=2, na=5, nf=3, nq=1, nm=1)
    cfg = synth.write_files(str(tmp_path / "s"), w)
    scans = "".join(
        "<scan><base><x>%r</x><y>%r</y><z>%r</z></base><from>%r</from><to>%r</to><points>%d</points>"
        "<exponent>%r</exponent></scan>" % (float(b[0]), float(b[1]), float(b[2]), float(f), float(t), int(p),
                                            float(e))
        for f, t, p, e, b in zip(frm, to, pts, ex, base))
    txt = open(cfg).read().replace(
        "<vectors><type>file</type><file>qvectors.txt</file></vectors>",
        "<vectors><type>scans</type><scans>%s</scans></vectors>" % scans)
    open(cfg, "w").write(txt)
    got = abi.config_qvectors(cfg)
    assert np.array_equal(np.asarray(got).reshape(-1, 3), want)


def test_reference_build_reproduces_fixture():
    """Rebuild the reference library from the reference tree and rerun two cases: the
    committed fixture must be what the reference's code gives. Skipped where the reference
    tree is absent (the GPU machine)."""
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
    for name in ("coh_acf_fftw", "inc_acf_direct"):
        g = lambda k: z[name + "." + k]  # noqa: E731
        self_, dsp, method = str(g("kind")).split("/")
        tables = (g("sf_type"), g("sf_const"), g("vol"), g("ex_type"), g("ex_const"))
        q_out, fqt, fq, fq2 = mk.run_case(L, self_ == "self", dsp, method, g("coords"), g("atom_type"), tables,
                                          float(g("background")), g("qvectors"), g("orient"))
        assert np.array_equal(fqt, g("fqt")) and np.array_equal(fq, g("fq")) and np.array_equal(fq2, g("fq2"))
