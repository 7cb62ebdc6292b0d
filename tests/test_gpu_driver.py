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


@pytest.mark.parametrize("kind,resolution,axis", [("sphere", 6, None), ("cylinder", 5, (1.0, -0.5, 0.7))])
def test_driver_multipole_matches_oracle(native_lib, tmp_path, kind, resolution, axis):
    # scattering.average.orientation.type = multipole (scatter_device_factory.cpp:145-201):
    # the q-vectors themselves enter, so the file gets general 3-vectors of the scan's lengths
    w = small("all", "autocorrelate", seed=54, na=37, nf=16, nq=3, nm=4)
    rng = np.random.default_rng(54)
    q = rng.normal(size=(len(w.shells), 3))
    q *= (w.shells / np.linalg.norm(q, axis=1))[:, None]
    ax = "" if axis is None else "<axis><x>%r</x><y>%r</y><z>%r</z></axis>" % axis
    average = ("<average><orientation><type>multipole</type><multipole><type>%s</type><moments>"
               "<type>resolution</type><resolution>%d</resolution></moments></multipole>%s"
               "</orientation></average>" % (kind, resolution, ax))
    d = str(tmp_path / "run")
    cfg = synth.write_files(d, w, precision="fp64", average=average)
    with open(os.path.join(d, "qvectors.txt"), "w") as f:
        for v in q:
            f.write("%.17g %.17g %.17g\n" % tuple(v))
    run(cfg)
    qo, fqt, fq0, fq, _ = read_rows(os.path.join(d, "signal.h5"))
    if kind == "sphere":
        ref = oracle.mp_sphere(w.coords, q, w.factors(), oracle.sphere_moments(resolution))
    else:
        ref = oracle.mp_cylinder(w.coords, q, w.factors(), oracle.cylinder_moments(resolution), axis)
    # rows in completion order: match them to the q-vectors
    order = [int(np.argmin(np.abs(q - v).sum(axis=1))) for v in qo]
    assert sorted(order) == list(range(len(q)))
    rfqt = (ref[0][..., 0] + 1j * ref[0][..., 1])[order]
    err = (np.abs(fqt - rfqt).max(axis=1) / np.abs(rfqt[:, 0])).max()
    assert err <= 1e-12, err
    assert np.array_equal(fq0, fqt[:, 0])
    assert np.allclose(fq, (ref[1][:, 0] + 1j * ref[1][:, 1])[order], rtol=1e-12, atol=1e-14)


def test_driver_fp32_linear_scan(native_lib, tmp_path):
    # a linear scan with a file orientation set: every |q| shares the direction set, so the
    # FP32 form takes the shell-recurrence kernel through the driver (no caller-side change)
    w = small("all", "autocorrelate", seed=55, na=120, nf=24, nq=1, nm=12)
    d = str(tmp_path / "run")
    cfg = synth.write_files(d, w, precision="fp32")
    txt = open(cfg).read().replace(
        "<vectors><type>file</type><file>qvectors.txt</file></vectors>",
        "<vectors><type>scans</type><scans><scan><base><x>1</x><y>0</y><z>0</z></base>"
        "<from>0.2</from><to>2.2</to><points>9</points></scan></scans></vectors>")
    open(cfg, "w").write(txt)
    r = run(cfg)
    q, fqt, *_ = read_rows(os.path.join(d, "signal.h5"))
    lengths = np.linalg.norm(q, axis=1)
    sv = (lengths[:, None, None] * w.directions[None]).reshape(-1, 3)
    offs = np.arange(len(q) + 1, dtype=np.uintp) * w.nm
    fac = np.repeat(w.factors()[:1], len(q), axis=0)
    ref = oracle.all_vectors(w.coords, offs, sv, fac, 0, 0, nthreads=8)
    rfqt = ref[0][..., 0] + 1j * ref[0][..., 1]
    assert (np.abs(fqt - rfqt).max(axis=1) / np.abs(rfqt[:, 0])).max() <= 1e-3
    assert "recurrence" in r.stderr
