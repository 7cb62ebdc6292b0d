"""End to end on the GPU through the drop-in boundary: scatter.xml + db.xml + PDB + DCD ->
sassena-gpu (C++ host devices -> C ABI -> kernels) -> signal.h5, checked against the
oracle, and the resume contract (sassena.cpp:270-308: already computed q are skipped,
new rows are appended)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

import h5lite

pytestmark = pytest.mark.gpu


def run(cfg, *extra):
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg] + list(extra), capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    return r


def small(*a, **k):
    """A small workload with |q|-independent factors (database type 0 constants)."""
    w = synth.small(*a, **k)
    w.class_factors[:] = w.class_factors[:1]
    return w


def reference(w, method=0):
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    dsp = {"autocorrelate": 0, "square": 1, "plain": 2}[w.dsp]
    sv = (w.shells[:, None, None] * w.directions[None]).reshape(-1, 3)
    return fn(w.coords, w.sub_offsets(), sv, w.factors(), dsp, method, nthreads=8)


def read_rows(path):
    f = h5lite.File(path)
    c = lambda a: a[..., 0] + 1j * a[..., 1]  # noqa: E731
    return (f.read("qvectors"), c(f.read("fqt")), c(f.read("fq0")), c(f.read("fq")),
            c(f.read("fq2")))


@pytest.mark.parametrize("scattering,dsp", [("all", "autocorrelate"), ("self", "autocorrelate"),
                                            ("all", "square")])
def test_driver_fp64_matches_oracle(native_lib, tmp_path, scattering, dsp):
    w = small(scattering, dsp, seed=51, na=41, nf=18, nq=3, nm=6)
    cfg = synth.write_files(str(tmp_path / "run"), w, precision="fp64")
    run(cfg)
    q, fqt, fq0, fq, fq2 = read_rows(str(tmp_path / "run" / "signal.h5"))
    ref = reference(w)
    rfqt = ref[0][..., 0] + 1j * ref[0][..., 1]
    assert np.allclose(q[:, 0], w.shells, rtol=0, atol=0)
    err = (np.abs(fqt - rfqt).max(axis=1) / np.abs(rfqt[:, 0])).max()
    assert err <= 1e-12, err
    assert np.array_equal(fq0, fqt[:, 0])
    assert np.allclose(fq, ref[1][:, 0] + 1j * ref[1][:, 1], rtol=1e-12, atol=1e-14)
    assert np.allclose(fq2, ref[2][:, 0] + 1j * ref[2][:, 1], rtol=1e-12, atol=1e-14)


def test_driver_fp32_form(native_lib, tmp_path):
    w = small("all", "autocorrelate", seed=52, na=60, nf=30, nq=2, nm=8)
    cfg = synth.write_files(str(tmp_path / "run"), w, precision="fp32")
    run(cfg)
    q, fqt, *_ = read_rows(str(tmp_path / "run" / "signal.h5"))
    ref = reference(w)
    rfqt = ref[0][..., 0] + 1j * ref[0][..., 1]
    assert (np.abs(fqt - rfqt).max(axis=1) / np.abs(rfqt[:, 0])).max() <= 1e-3


def test_driver_resume_appends(native_lib, tmp_path):
    w = small("all", "autocorrelate", seed=53, na=30, nf=12, nq=4, nm=5)
    d = str(tmp_path / "run")
    cfg = synth.write_files(d, w, precision="fp64")
    full = open(os.path.join(d, "qvectors.txt")).read().splitlines()
    # first run: q-vectors 2 and 0 only
    with open(os.path.join(d, "qvectors.txt"), "w") as f:
        f.write(full[2] + "\n" + full[0] + "\n")
    run(cfg)
    q1, fqt1, *_ = read_rows(os.path.join(d, "signal.h5"))
    assert np.allclose(q1[:, 0], w.shells[[2, 0]])
    # second run with all four: only 1 and 3 are computed and appended after the old rows
    with open(os.path.join(d, "qvectors.txt"), "w") as f:
        f.write("\n".join(full) + "\n")
    r = run(cfg)
    assert "Found 2 old qvectors" in r.stderr
    q2, fqt2, fq02, fq2_, f22 = read_rows(os.path.join(d, "signal.h5"))
    assert np.allclose(q2[:, 0], w.shells[[2, 0, 1, 3]])
    assert np.array_equal(fqt2[:2], fqt1)
    ref = reference(w)
    rfqt = ref[0][..., 0] + 1j * ref[0][..., 1]
    err = (np.abs(fqt2 - rfqt[[2, 0, 1, 3]]).max(axis=1) / np.abs(rfqt[[2, 0, 1, 3], 0])).max()
    assert err <= 1e-12
    # third run: nothing left
    r = run(cfg)
    assert "No qvectors left" in r.stderr


def test_driver_rejects_nf_mismatch_on_resume(native_lib, tmp_path):
    w = small("all", "autocorrelate", seed=54, na=10, nf=8, nq=2, nm=2)
    d = str(tmp_path / "run")
    cfg = synth.write_files(d, w)
    run(cfg)
    synth.write_dcd(os.path.join(d, "sample.dcd"), w.coords[:5])
    os.remove(os.path.join(d, "qvectors.txt"))
    with open(os.path.join(d, "qvectors.txt"), "w") as f:
        f.write("0.77 0 0\n")
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg], capture_output=True, text=True)
    assert r.returncode == 1 and "NF=" in r.stderr
