"""Staging pre-pass on the GPU (sass_stage_frames_prepass) against oracle.alignment: the
steps sassena-gpu builds for each configuration are applied on the device and the staged
float32 frames compared with the oracle's CoordinateSets::load. Centres of mass,
translations and motions are summed in the reference's order, so those frames are equal
bit for bit; fits go through an SVD (LAPACK in the oracle, Jacobi here), so they may differ
by one float32 ulp. End to end, the driver's S(q,t) for aligned configurations matches the
FP64 oracle run on the oracle's aligned frames (bar 1e-12)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from oracle import alignment as al
from sassena_gb300 import abi

import h5lite
import prepass_cases as pc

pytestmark = pytest.mark.gpu

FITS = {"fitrottrans", "fitrot_file", "fit_instant", "pre_post"}


def host_steps(cfg, tmp_path):
    return pc.host_steps(cfg, str(tmp_path / "dry.json"))


@pytest.mark.parametrize("name", pc.CASES)
def test_prepass_matches_oracle(native_lib, tmp_path, name):
    w, cfg, o = pc.build(name, str(tmp_path / "run"))
    steps, masses = host_steps(cfg, tmp_path)
    want = al.load(w.coords, o["masses"], o["alignments"], o["motions"], o["target"])
    target = o["target"] if o["target"] is not None else list(range(pc.NA))
    for precision in ("fp64", "fp32"):
        with abi.Plan(len(target), pc.NF, 4, "all", "autocorrelate", "fftw", precision) as p:
            got = p.stage_prepass(w.coords, masses, steps, target)
        if name in FITS:
            ulp = np.spacing(np.abs(want).astype(np.float32))
            assert (np.abs(got - want) <= ulp).all(), np.abs(got - want).max()
        else:
            np.testing.assert_array_equal(got, want)


def test_prepass_empty_and_errors(native_lib):
    w = pc.workload()
    m = np.ones(pc.NA)
    with abi.Plan(pc.NA, pc.NF, 4, "all") as p:
        # no steps: the target atoms staged unchanged
        np.testing.assert_array_equal(p.stage_prepass(w.coords, m, [], list(range(pc.NA))), w.coords)
        # empty lists are allowed (a centre of nothing is 0)
        got = p.stage_prepass(w.coords, m, [{"type": "center", "selection": list(range(5)),
                                             "reference_selection": []}], list(range(pc.NA)))
        np.testing.assert_array_equal(got, w.coords)
        with pytest.raises(abi.SassError):
            p.stage_prepass(w.coords, m, [{"type": "center", "selection": [pc.NA], "reference_selection": []}],
                            list(range(pc.NA)))
        with pytest.raises(abi.SassError):
            p.stage_prepass(w.coords, m, [{"type": "fitrottrans", "selection": [], "reference_selection": [0, 1],
                                           "fit_target": [0], "fit_source": [2]}], list(range(pc.NA)))
        with pytest.raises(abi.SassError):
            p.stage_prepass(w.coords, m, [{"type": "motion", "selection": [0], "reference_selection": [0]}],
                            list(range(pc.NA)))


@pytest.mark.parametrize("name", ["pre_post", "motions", "fittrans"])
def test_driver_with_alignments_matches_oracle(native_lib, tmp_path, name):
    d = str(tmp_path / "run")
    w, cfg, o = pc.build(name, d)
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    aligned = al.load(w.coords, o["masses"], o["alignments"], o["motions"], o["target"])
    target = o["target"] if o["target"] is not None else list(range(pc.NA))
    cls = w.atom_class[target]
    sv = (w.shells[:, None, None] * w.directions[None]).reshape(-1, 3)
    ref = oracle.all_vectors(aligned, w.sub_offsets(), sv, w.class_factors[:, cls], 0, 0, nthreads=8)
    f = h5lite.File(os.path.join(d, "signal.h5"))
    fqt = f.read("fqt")
    fqt = fqt[..., 0] + 1j * fqt[..., 1]
    rfqt = ref[0][..., 0] + 1j * ref[0][..., 1]
    err = (np.abs(fqt - rfqt).max(axis=1) / np.abs(rfqt[:, 0])).max()
    assert err <= 1e-12, err


def read_dcd(path, nf, na):
    """Frames [nf, na, 3] of a DCD in the reference writer's layout (unit-cell block on)."""
    raw = open(path, "rb").read()
    off = 4 + 84 + 4 + 12 + 12  # header record, title record, atom-count record
    out = np.zeros((nf, na, 3), dtype=np.float32)
    for f in range(nf):
        off += 4 + 48 + 4
        for k in range(3):
            out[f, :, k] = np.frombuffer(raw, dtype=np.float32, count=na, offset=off + 4)
            off += 8 + 4 * na
    return out


@pytest.mark.parametrize("name", ["motions", "pre_post"])
def test_driver_dumps_the_aligned_frames(native_lib, tmp_path, name):
    # stager.dump after the device pre-pass: the file holds the oracle's aligned frames
    d = str(tmp_path / "run")
    w, cfg, o = pc.build(name, d)
    with open(cfg) as f:
        xml = f.read()
    with open(cfg, "w") as f:
        f.write(xml.replace("<stager>", "<stager><dump>true</dump>") if "<stager>" in xml
                else xml.replace("</root>", "<stager><dump>true</dump></stager></root>"))
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want = al.load(w.coords, o["masses"], o["alignments"], o["motions"], o["target"])
    got = read_dcd(os.path.join(d, "dump.dcd"), want.shape[0], want.shape[1])
    if name in FITS:
        assert (np.abs(got - want) <= np.spacing(np.abs(want).astype(np.float32))).all()
    else:
        np.testing.assert_array_equal(got, want)
