"""Staging pre-pass, host side (no GPU): the steps sassena-gpu builds from sample
alignments and motions (selection walks, reference structures, walker translations,
masses) against the reference's rules restated in oracle.alignment, plus the oracle's own
pins (centre of mass at the origin, a fit that undoes a rigid motion) and the error paths."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import alignment as al
from sassena_gb300 import abi, synth

import prepass_cases as pc


def dry(cfg, tmp_path):
    out = str(tmp_path / "dry.json")
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg, "--dry-run", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.load(open(out))


def test_merge_walk_restatement():
    # coordinate_set.cpp:48-64: an unsorted sub-selection loses the atoms it walks past
    assert al.walk(list(range(6)), [3, 1, 4]) == [(3, 0), (4, 2)]
    assert al.walk([1, 4, 7], [1, 7]) == [(0, 0), (2, 1)]
    assert al.walk([], [1]) == []


@pytest.mark.parametrize("name", pc.CASES)
def test_host_steps_match_the_reference_rules(tmp_path, name):
    w, cfg, o = pc.build(name, str(tmp_path / "run"))
    j = dry(cfg, tmp_path)
    steps = j["prepass"]
    np.testing.assert_array_equal(np.array(j["masses"]), o["masses"])
    sysl = list(range(pc.NA))
    walked = lambda s: [s[k] for _, k in al.walk(sysl, s)]  # noqa: E731
    pre = [a for a in o["alignments"] if a["order"] == "pre"]
    post = [a for a in o["alignments"] if a["order"] == "post"]
    expect = [("a", a) for a in pre] + [("m", m) for m in o["motions"]] + [("a", a) for a in post]
    assert len(steps) == len(expect)
    for st, (kind, e) in zip(steps, expect):
        ref = e["reference"]
        if kind == "m":
            assert st["type"] == 4
            assert st["selection"] == walked(e["selection"])
            if ref is None:
                assert st["reference_selection"] == walked(e["reference_selection"]) and st["reference"] == []
            else:
                assert st["reference_selection"] == e["reference_selection"]
                np.testing.assert_array_equal(np.reshape(st["reference"], (-1, 3)), ref[e["reference_selection"]])
            tr = np.reshape(st["translations"], (-1, 3))
            for f in range(pc.NF):  # the walker's translation, bit for bit
                np.testing.assert_array_equal(tr[f], al.motion_translation(e, f))
            continue
        t = {"center": 0, "fittrans": 1, "fitrottrans": 2, "fitrot": 3}[e["type"]]
        assert st["type"] == t
        if t == 0:
            assert st["selection"] == walked(e["selection"])
            assert st["reference_selection"] == walked(e["reference_selection"])
            continue
        if ref is None:
            assert st["reference_selection"] == sysl and st["reference"] == []
        else:
            assert st["reference_selection"] == e["reference_selection"]
            np.testing.assert_array_equal(np.reshape(st["reference"], (-1, 3)), ref[e["reference_selection"]])
        if t == 1:
            assert st["selection"] == walked(e["selection"])
        else:
            fsel = sysl if ref is None else e["reference_selection"]
            pairs = al.walk(e["selection"], fsel)
            assert st["fit_target"] == [e["selection"][c] for c, _ in pairs]
            assert st["fit_source"] == [fsel[k] for _, k in pairs]
            assert st["selection"] == (walked(e["selection"]) if t == 3 else [])


def test_oracle_center_and_fit_pins():
    w = pc.workload()
    masses = np.array(pc.MASSES)[w.atom_class]
    sysl = list(range(pc.NA))
    out = al.load(w.coords, masses, [{"type": "center", "selection": sysl, "reference_selection": sysl,
                                      "reference": None}]).astype(np.float64)
    com = (out * masses[None, :, None]).sum(axis=1) / masses.sum()
    assert np.abs(com).max() < 1e-5  # float32 storage of centred coordinates
    # frames 1.. are rigid motions of a random walk: fitting on frame 0 removes the motion
    core = pc.SELECTIONS["core"]
    ref0 = w.coords[0].astype(np.float64)
    fitted = al.load(w.coords, masses, [{"type": "fitrottrans", "selection": sysl, "reference_selection": sysl,
                                         "reference": ref0}])
    rmsd_before = np.sqrt(((w.coords[1:] - w.coords[:1]) ** 2).sum(axis=2).mean())
    rmsd_after = np.sqrt(((fitted[1:] - fitted[:1]) ** 2).sum(axis=2).mean())
    assert rmsd_after < 0.5 * rmsd_before
    # a frame that is an exact rigid copy of the reference fits back onto it
    R = pc.rotation(np.random.default_rng(3))
    frames = np.stack([ref0, ref0 @ R.T + np.array([3.0, -1.0, 2.0])]).astype(np.float32)
    back = al.load(frames, masses, [{"type": "fitrottrans", "selection": sysl, "reference_selection": core,
                                     "reference": frames[0].astype(np.float64)}])
    assert np.abs(back[1, :20] - frames[0, :20]).max() < 1e-4
    np.testing.assert_array_equal(back[1, 20:], frames[1, 20:])  # not in the fit selection: unmoved


@pytest.mark.parametrize("xml,needle", [
    (pc.alignment_xml("spin"), "Fitting routine not understood"),
    (pc.alignment_xml("center", order="mid"), "Ordering of alignment not understood"),
    (pc.alignment_xml("fitrottrans", selection="shell", ref=dict(type="frame", selection="odd")),
     "read its reduced copy"),
    (pc.alignment_xml("fittrans", ref=dict(type="nowhere")), "Reference type not understood"),
    (pc.alignment_xml("center", selection="nosuch"), "unknown selection"),
    ("</alignments><motions>" + pc.motion_xml("brownian", "core", 0.1, (1.0, 0.0, 0.0)) + "</motions><alignments>",
     "does not reproduce"),
    ("</alignments><motions>" + pc.motion_xml("wobble", "core", 0.1, (1.0, 0.0, 0.0)) + "</motions><alignments>",
     "Motion type not understood"),
])
def test_prepass_configuration_errors(tmp_path, xml, needle):
    w = pc.workload()
    d = str(tmp_path / "run")
    cfg = synth.write_files(d, w, sample_extra=pc.SELECTIONS_XML + "<alignments>" + xml + "</alignments>",
                            masses=pc.MASSES)
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg, "--dry-run", str(tmp_path / "x.json")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and needle in r.stderr, r.stderr


def test_pdb_reference_frames(tmp_path):
    # PDBFrameset::generate_index: frames end at END lines; past the end -> last frame
    p = str(tmp_path / "ref.pdb")
    rec = "ATOM  %5d C1   MOL A   1    %8.3f%8.3f%8.3f  1.00  0.00\n"
    with open(p, "w") as f:
        f.write(rec % (1, 1.0, 2.0, 3.0) + rec % (2, 4.0, 5.0, 6.0) + "END\n")
        f.write(rec % (1, -1.5, 0.25, 9.125) + rec % (2, 7.0, 8.0, 9.0) + "ENDMDL\n")
    w = pc.workload()
    d = str(tmp_path / "run")
    import shutil
    os.makedirs(d, exist_ok=True)
    shutil.copy(p, os.path.join(d, "ref.pdb"))
    for frame, want in ((1, [-1.5, 0.25, 9.125, 7.0, 8.0, 9.0]), (5, [-1.5, 0.25, 9.125, 7.0, 8.0, 9.0]),
                        (0, [1.0, 2.0, 3.0, 4.0, 5.0, 6.0])):
        xml = pc.alignment_xml("fittrans", ref={"type": "file", "file": "ref.pdb", "frame": frame,
                                                "selection": "two"})
        extra = pc.SELECTIONS_XML.replace("</selections>", "<selection><name>two</name><type>range</type>"
                                          "<from>0</from><to>1</to></selection></selections>")
        cfg = synth.write_files(d, w, sample_extra=extra + "<alignments>" + xml + "</alignments>",
                                masses=pc.MASSES)
        assert dry(cfg, tmp_path)["prepass"][0]["reference"] == want
