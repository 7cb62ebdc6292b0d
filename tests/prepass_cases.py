"""Configurations with sample alignments and motions, shared by the CPU tests of the host
pre-pass setup and the GPU tests of the device pre-pass.

Each case writes a small system (40 atoms, 7 frames of a random walk that also rotates and
drifts, so fits have work to do) with the driver's files, and describes the same steps in
the terms of oracle.alignment.load (selections as index lists, references as full frames).
"""
import json
import os
import subprocess

import numpy as np

from sassena_gb300 import abi, synth

NA, NF = 40, 7
MASSES = [1.008, 12.011, 14.007, 15.999]  # per class H, C, N, O

SELECTIONS = {
    "core": list(range(0, 20)),
    "shell": list(range(20, 40)),
    "odd": list(range(1, 40, 2)),
    "mixed": [5, 2, 9, 30],  # not ascending: the reference's walks drop atom 2
}

SELECTIONS_XML = """<selections>
  <selection><name>core</name><type>range</type><from>0</from><to>19</to></selection>
  <selection><name>shell</name><type>range</type><from>20</from><to>39</to></selection>
  <selection><name>odd</name><type>index</type>%s</selection>
  <selection><name>mixed</name><type>index</type><index>5</index><index>2</index><index>9</index><index>30</index></selection>
</selections>""" % "".join("<index>%d</index>" % i for i in range(1, 40, 2))


def rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def workload(seed=61):
    w = synth.small("all", "autocorrelate", seed=seed, na=NA, nf=NF, nq=2, nm=4, box=14.0)
    w.class_factors[:] = w.class_factors[:1]
    rng = np.random.default_rng(seed)
    c = w.coords.astype(np.float64)
    for f in range(1, NF):  # frame f: rotated about the centre and shifted
        R = rotation(rng)
        ctr = c[f].mean(axis=0)
        c[f] = (c[f] - ctr) @ R.T + ctr + rng.normal(scale=2.0, size=3)
    w.coords = c.astype(np.float32)
    return w


def alignment_xml(type_, selection="system", order=None, ref=None):
    """<alignment>; ref = dict(type=..., frame=..., file=..., selection=...)."""
    x = "<alignment><type>%s</type><selection>%s</selection>" % (type_, selection)
    if order:
        x += "<order>%s</order>" % order
    if ref:
        x += "<reference>" + "".join("<%s>%s</%s>" % (k, v, k) for k, v in ref.items()) + "</reference>"
    return x + "</alignment>"


def motion_xml(type_, selection, displace, direction, ref=None, **kw):
    x = "<motion><type>%s</type><selection>%s</selection><displace>%r</displace>" % (type_, selection, displace)
    x += "<direction><x>%r</x><y>%r</y><z>%r</z></direction>" % tuple(direction)
    for k, v in kw.items():
        x += "<%s>%r</%s>" % (k, v, k)
    if ref:
        x += "<reference>" + "".join("<%s>%s</%s>" % (k, v, k) for k, v in ref.items()) + "</reference>"
    return x + "</motion>"


def pdb_coords(path):
    xyz = []
    for line in open(path):
        if line.startswith("ATOM  "):
            xyz.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
    return np.array(xyz)


# name -> (alignments [(xml kwargs, oracle dict)], motions [(xml kwargs, oracle dict)], target)
def _cases():
    core, shell, odd, mixed = (SELECTIONS[k] for k in ("core", "shell", "odd", "mixed"))
    allat = list(range(NA))
    F = lambda k: ("frame", k)  # noqa: E731
    return {
        "center": ([dict(type_="center")], [], None),
        "center_sel": ([dict(type_="center", selection="shell", ref=dict(selection="core"))], [], None),
        "fittrans": ([dict(type_="fittrans", ref=dict(type="frame", frame=3, selection="core"))], [], None),
        "fitrottrans": ([dict(type_="fitrottrans", ref=dict(type="frame", frame=0, selection="core"))], [], None),
        "fitrot_file": ([dict(type_="fitrot", selection="core", ref=dict(type="file", file="sample.pdb"))], [], None),
        "fit_instant": ([dict(type_="fitrottrans", selection="odd", ref=dict(type="instant"))], [], None),
        "motions": ([], [dict(type_="linear", selection="core", displace=0.25, direction=(1.0, 2.0, 0.5)),
                         dict(type_="oscillation", selection="odd", displace=0.7, direction=(0.0, 1.0, 1.0),
                              frequency=0.05, sampling=2, ref=dict(type="frame", frame=2)),
                         dict(type_="fixed", selection="mixed", displace=1.5, direction=(0.3, -0.2, 0.9))], None),
        "pre_post": ([dict(type_="center"),
                      dict(type_="fitrottrans", order="post", ref=dict(type="frame", frame=1, selection="core"))],
                     [dict(type_="linear", selection="shell", displace=0.1, direction=(0.0, 0.0, 1.0))], "shell"),
    }


CASES = sorted(_cases())


def _oracle_ref(ref, default_type, sel_name, w, pdb):
    """reference structure of an alignment/motion for oracle.alignment.load (full frame)."""
    t = (ref or {}).get("type", default_type)
    if t == "instant":
        return None
    if t == "frame":
        k = min(int((ref or {}).get("frame", 0)), NF - 1)
        return w.coords[k].astype(np.float64)
    return pdb


def build(name, directory):
    """Files for case `name` in `directory`; returns (w, scatter.xml path, oracle kwargs)."""
    als, mos, target = _cases()[name]
    w = workload()
    extra = "<stager><target>%s</target></stager>" % target if target else ""
    sample_extra = SELECTIONS_XML
    if als:
        sample_extra += "<alignments>" + "".join(alignment_xml(**a) for a in als) + "</alignments>"
    if mos:
        sample_extra += "<motions>" + "".join(motion_xml(**m) for m in mos) + "</motions>"
    cfg = synth.write_files(directory, w, precision="fp64", sample_extra=sample_extra, extra=extra,
                            masses=MASSES)
    pdb = pdb_coords(os.path.join(directory, "sample.pdb"))
    sel = dict(SELECTIONS, system=list(range(NA)))
    o_al = []
    for a in als:
        ref = a.get("ref") or {}
        s = a.get("selection", "system")
        o_al.append({"type": a["type_"], "order": a.get("order", "pre"), "selection": sel[s],
                     "reference_selection": sel[ref.get("selection", s)],
                     "reference": _oracle_ref(ref, "frame", s, w, pdb)})
    o_mo = []
    for m in mos:
        ref = m.get("ref") or {}
        s = m["selection"]
        o_mo.append({"type": m["type_"], "displace": m["displace"], "direction": m["direction"],
                     "sampling": m.get("sampling", 1), "frequency": m.get("frequency", 0.001),
                     "selection": sel[s], "reference_selection": sel[ref.get("selection", s)],
                     "reference": _oracle_ref(ref, "instant", s, w, pdb)})
    masses = np.array(MASSES)[w.atom_class]
    return w, cfg, dict(alignments=o_al, motions=o_mo, target=sel[target] if target else None,
                        masses=masses)


STEP_TYPES = {0: "center", 1: "fittrans", 2: "fitrottrans", 3: "fitrot", 4: "motion"}


def host_steps(cfg, out_json):
    """The pre-pass steps and masses sassena-gpu builds for `cfg` (its --dry-run JSON), in the
    terms of abi.Plan.stage_prepass."""
    r = subprocess.run([abi.DRIVER_PATH, "--config", cfg, "--dry-run", out_json], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    j = json.load(open(out_json))
    steps = []
    for s in j["prepass"]:
        d = {"type": STEP_TYPES[s["type"]], "selection": s["selection"],
             "reference_selection": s["reference_selection"], "fit_target": s["fit_target"],
             "fit_source": s["fit_source"]}
        if s["reference"]:
            d["reference"] = np.reshape(s["reference"], (-1, 3))
        if s["translations"]:
            d["translations"] = np.reshape(s["translations"], (-1, 3))
        steps.append(d)
    return steps, np.array(j["masses"])
