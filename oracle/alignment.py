"""numpy FP64 restatement of the per-frame alignments and translation motions that the
reference applies before staging (test infrastructure).

It restates, at the level of the reference's own data structures:
  CoordinateSets::load            src/sample/coordinate_sets.cpp:244-368
  CenterOfMass (both forms)       src/sample/center_of_mass.cpp:160-264
  Fit                             src/sample/center_of_mass.cpp:53-157 (LAPACK SVD: numpy's)
  CoordinateSet reduction         src/sample/coordinate_set.cpp:32-67
  translate / transform           src/sample/coordinate_set.cpp:107-188
  Linear/Fixed/Oscillation walkers src/sample/motion_walker.cpp (translation in row 3 of a 4x4)
  alignment / motion defaults     src/control/parameters.cpp:234-340

Selections are index lists in selection order. Every loop over two selections replays the
reference's merge walk (`walk`), and every sum runs in list order with separately rounded
products and sums (numpy elementwise operations, np.cumsum), as the reference's loops do.
"""
from __future__ import annotations

import math

import numpy as np


def walk(csel, ssel):
    """The reference's merge of a coordinate-set selection with a sub-selection: pairs
    (csel_iter, ssel_iter) where csel[csel_iter] == ssel[ssel_iter] (coordinate_set.cpp:48-64)."""
    out = []
    i = k = 0
    while i < len(csel) and k < len(ssel):
        a, b = csel[i], ssel[k]
        if a == b:
            out.append((i, k))
            i += 1
            k += 1
        elif a > b:
            k += 1
        else:
            i += 1
    return out


def _seq(a):
    """Sequential sum along axis 0 (the reference's accumulation order)."""
    a = np.asarray(a, dtype=np.float64)
    if len(a) == 0:
        return np.zeros(a.shape[1:])
    return np.cumsum(a, axis=0)[-1]


def com_walk(cs, csel, sel, masses):
    """CenterOfMass(atoms, cs, cs_selection, cofm_selection) (center_of_mass.cpp:160-216)."""
    if len(sel) < 1 or len(csel) < 1:
        return np.zeros(3)
    pairs = walk(csel, sel)
    ci = np.array([p[0] for p in pairs], dtype=np.int64)
    m = np.asarray(masses, dtype=np.float64)[np.asarray(csel, dtype=np.int64)[ci]]
    r = cs[ci]
    return _seq(r * m[:, None]) / _seq(m)


def com_list(cs, sel, masses):
    """CenterOfMass(atoms, cset, selection): coordinate i belongs to atom sel[i]
    (center_of_mass.cpp:247-264)."""
    if len(sel) == 0:
        return np.zeros(3)
    m = np.asarray(masses, dtype=np.float64)[np.asarray(sel, dtype=np.int64)]
    r = cs[: len(sel)]
    return _seq(r * m[:, None]) / _seq(m)


def translate(cs, t, csel, sel):
    for i, _ in walk(csel, sel):
        cs[i] = cs[i] + t


def fit(cs, system, manip, cs_ref, ref_sel, masses):
    """Fit::Fit (center_of_mass.cpp:53-157); cs is modified in place."""
    pairs = walk(system, ref_sel)
    red = np.array([cs[i] for i, _ in pairs], dtype=np.float64).reshape(-1, 3)
    if len(red) != len(cs_ref):
        raise ValueError("Fitting requires the reference and the target to contain the same number of atoms")
    ref = com_list(cs_ref, ref_sel, masses)
    pos = com_list(red, ref_sel, masses)
    m = np.asarray(masses, dtype=np.float64)[np.asarray(ref_sel, dtype=np.int64)]
    v = red - pos
    u = cs_ref - ref
    K = _seq(m[:, None, None] * (u[:, :, None] * v[:, None, :]))
    U, S, Vt = np.linalg.svd(K)
    d = np.linalg.det(U @ Vt)
    R = U @ (np.diag([1.0, 1.0, d]) @ Vt)
    b = red - pos
    after = (R[None, :, 0] * b[:, 0:1] + R[None, :, 1] * b[:, 1:2]) + R[None, :, 2] * b[:, 2:3]
    red = after + ref
    for ci, si in walk(manip, ref_sel):
        a = manip[ci]
        if ref_sel[si] >= len(red):
            raise IndexError("the reference reads outside its fit copy here")
        cs[a] = red[ref_sel[si]]


def motion_translation(motion, frame):
    """translation(timepos) of the deterministic walkers (motion_walker.cpp)."""
    d = np.asarray(motion["direction"], dtype=np.float64)
    length = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    kind = motion["type"]
    if kind == "linear":
        tr = (motion["displace"] * motion.get("sampling", 1)) * d / length
        return float(frame) * tr
    if kind == "fixed":
        return motion["displace"] * d / length
    if kind == "oscillation":
        tr = motion["displace"] * d / length
        arg = 2 * math.pi * float(frame) * motion.get("frequency", 0.001) * motion.get("sampling", 1)
        return tr * math.sin(arg)
    raise ValueError("motion type not restated: " + kind)


def load(frames, masses, alignments=(), motions=(), target=None):
    """CoordinateSets::load for every frame, then the stager's float32 store.

    frames: float32 [nf, N, 3]. alignments: dicts with "type" (center, fittrans,
    fitrottrans, fitrot), "order" ("pre"/"post"), "selection" and "reference_selection"
    (index lists) and "reference": None for "instant", else the reference frame's full
    coordinates [N', 3] (a trajectory frame or a PDB frame), reduced here by
    reference_selection. motions: dicts with "type" (linear, fixed, oscillation),
    "displace", "direction", "sampling", "frequency", "selection",
    "reference_selection" and "reference" as above. target: index list (None: all).
    Returns float32 [nf, len(target), 3]."""
    nf, N = frames.shape[0], frames.shape[1]
    system = list(range(N))
    target = system if target is None else list(target)

    def ref_coords(a):
        if a.get("reference") is None:
            return None
        full = np.asarray(a["reference"], dtype=np.float64)
        return full[np.asarray(a["reference_selection"], dtype=np.int64)]

    def align(cs, a):
        sel, rsel = list(a["selection"]), list(a["reference_selection"])
        rc = ref_coords(a)
        if rc is None:  # instant: the current coordinates and the whole system
            rc_cs, rc_sel = cs, system
        else:
            rc_cs, rc_sel = rc, rsel
        t = a["type"]
        if t == "center":
            origin = com_walk(cs, system, rsel, masses)
            translate(cs, -1.0 * origin, system, sel)
        elif t == "fittrans":
            ref = com_list(rc_cs, rc_sel, masses)
            pos = com_walk(cs, system, sel, masses)
            translate(cs, ref - pos, system, sel)
        elif t == "fitrottrans":
            fit(cs, system, sel, rc_cs.copy() if rc is None else rc_cs, rc_sel, masses)
        elif t == "fitrot":
            pos = com_walk(cs, system, sel, masses)
            fit(cs, system, sel, rc_cs.copy() if rc is None else rc_cs, rc_sel, masses)
            translate(cs, pos, system, sel)
        else:
            raise ValueError("Fitting routine not understood: " + t)

    out = np.zeros((nf, len(walk(system, target)), 3), dtype=np.float32)
    for f in range(nf):
        cs = frames[f].astype(np.float64)
        for a in alignments:
            if a.get("order", "pre") == "pre":
                align(cs, a)
        for mo in motions:
            sel, rsel = list(mo["selection"]), list(mo["reference_selection"])
            rc = ref_coords(mo)
            ref = com_list(rc, rsel, masses) if rc is not None else com_walk(cs, system, rsel, masses)
            translate(cs, -1.0 * ref, system, sel)
            t = motion_translation(mo, f)
            for i, _ in walk(system, sel):  # prod(pos, T): ((x*1 + y*0) + z*0) + 1*t
                x, y, z = cs[i]
                cs[i] = np.array([((x * 1.0 + y * 0.0) + z * 0.0) + t[0],
                                  ((x * 0.0 + y * 1.0) + z * 0.0) + t[1],
                                  ((x * 0.0 + y * 0.0) + z * 1.0) + t[2]])
            translate(cs, ref, system, sel)
        for a in alignments:
            if a.get("order", "pre") == "post":
                align(cs, a)
        red = np.array([cs[i] for i, _ in walk(system, target)], dtype=np.float64).reshape(-1, 3)
        out[f] = red.astype(np.float32)
    return out
