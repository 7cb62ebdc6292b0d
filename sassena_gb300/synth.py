"""Seeded synthetic trajectories and scattering set-ups for the benchmark workloads.

No public dataset is involved: every workload is generated from a seed with numpy's
PCG64. Coordinates are float32 frame-major ``[nf, na, 3]``, the layout the reference's
``DataStagerByFrame`` produces (src/stager/data_stager.cpp:110-114).

Workloads (sizes as named in the benchmark definitions):
  * ``incoherent_fqt``   1,000 atoms, 30 A box, 128 frames, Gaussian steps sigma=0.1 A per
                         axis, H/C/N/O 50/30/10/10 with incoherent lengths, 10 shells
                         0.1-2.0 1/A, 100 directions per shell.
  * ``coherent_sqt``     10,000 atoms, 50 A box, 1,024 frames, sigma=0.05 A steps plus a
                         harmonic pull (3-D RMSD saturating near 1 A), H/C/N/O/S coherent
                         lengths, 20 shells 0.05-3.0 1/A, 500 directions per shell.
  * ``static_xray``      20,000-bead random coil (bond 1.5 A) + 80,000 solvent atoms in a
                         110 A box, 64 frames, four-Gaussian form factors with seeded
                         coefficients, 200 shells 0.01-0.5 1/A, 2,000 directions.
Directions on the sphere come from normalised Gaussian triples (the project's own
generator; the reference's Boost mt19937/uniform_on_sphere stream is not reproduced).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Neutron scattering lengths in fm. Coherent: NIST b_c. Incoherent: sqrt(sigma_inc/4pi).
COHERENT_FM = {"H": -3.7390, "C": 6.6460, "N": 9.3600, "O": 5.8030, "S": 2.8470}
INCOHERENT_FM = {"H": 25.274, "C": 0.089, "N": 1.990, "O": 0.080, "S": 0.236}


@dataclass
class Workload:
    """One scattering calculation: trajectory, atom classes, shells and directions."""

    name: str
    coords: np.ndarray            # float32 [nf, na, 3]
    atom_class: np.ndarray        # int32 [na]; class c has factor class_factors[s, c]
    class_names: list
    class_factors: np.ndarray     # float64 [nq, nclass], b_c(|q_s|)
    shells: np.ndarray            # float64 [nq], |q|
    directions: np.ndarray        # float64 [nm, 3], unit vectors shared by all shells
    scattering: str = "all"       # "all" (coherent) or "self" (incoherent)
    dsp: str = "autocorrelate"    # autocorrelate | square | plain
    meta: dict = field(default_factory=dict)

    @property
    def nf(self):
        return self.coords.shape[0]

    @property
    def na(self):
        return self.coords.shape[1]

    @property
    def nq(self):
        return len(self.shells)

    @property
    def nm(self):
        return len(self.directions)

    def terms(self):
        """atom x q-vector x frame terms of the phase sum."""
        return self.na * self.nq * self.nm * self.nf

    def sub_offsets(self):
        return np.arange(self.nq + 1, dtype=np.uintp) * self.nm

    def subvectors(self):
        """[nq*nm, 3]: |q_s| * u_m, shell-major (init_subvectors order)."""
        return (self.shells[:, None, None] * self.directions[None, :, :]).reshape(-1, 3)

    def factors(self):
        """Per-atom factors [nq, na] expanded from the classes."""
        return self.class_factors[:, self.atom_class]


def sphere_directions(n, seed):
    rng = np.random.default_rng(np.random.PCG64(seed))
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def fibonacci_sphere(n):
    """Deterministic near-uniform points (spherical Fibonacci lattice)."""
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * math.pi * (3.0 - math.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def _types(rng, na, names, ratios):
    counts = np.floor(np.asarray(ratios, dtype=float) / sum(ratios) * na).astype(int)
    counts[0] += na - counts.sum()
    t = np.repeat(np.arange(len(names)), counts)
    rng.shuffle(t)
    return t.astype(np.int32)


def random_walk(rng, r0, nf, sigma, k=0.0, chunk=64):
    """Frames r_{t+1} = r_t + sigma*xi - k (r_t - r_0); float32 [nf, na, 3]."""
    na = r0.shape[0]
    out = np.empty((nf, na, 3), dtype=np.float32)
    r = r0.astype(np.float64).copy()
    out[0] = r
    t = 1
    while t < nf:
        m = min(chunk, nf - t)
        steps = rng.standard_normal((m, na, 3)) * sigma
        for i in range(m):
            r += steps[i]
            if k:
                r -= k * (r - r0)
            out[t + i] = r
        t += m
    return out


def incoherent_fqt(seed=1, na=1000, nf=128, box=30.0, sigma=0.1, nq=10, qmin=0.1, qmax=2.0,
                   nm=100):
    rng = np.random.default_rng(np.random.PCG64(seed))
    names = ["H", "C", "N", "O"]
    cls = _types(rng, na, names, [50, 30, 10, 10])
    r0 = rng.uniform(0.0, box, (na, 3))
    coords = random_walk(rng, r0, nf, sigma)
    shells = np.linspace(qmin, qmax, nq)
    b = np.array([INCOHERENT_FM[n] for n in names])
    return Workload("incoherent_fqt", coords, cls, names, np.tile(b, (nq, 1)), shells,
                    sphere_directions(nm, seed + 1000), scattering="self",
                    meta=dict(box=box, sigma=sigma, seed=seed))


def coherent_sqt(seed=2, na=10000, nf=1024, box=50.0, sigma=0.05, rmsd=1.0, nq=20, qmin=0.05,
                 qmax=3.0, nm=500):
    rng = np.random.default_rng(np.random.PCG64(seed))
    names = ["H", "C", "N", "O", "S"]
    cls = _types(rng, na, names, [50, 30, 8, 10, 2])
    r0 = rng.uniform(0.0, box, (na, 3))
    # OU stationary per-axis variance sigma^2/(2k-k^2); 3-D MSD = rmsd^2.
    c = 3.0 * sigma * sigma / (rmsd * rmsd)
    k = 1.0 - math.sqrt(1.0 - c)
    coords = random_walk(rng, r0, nf, sigma, k=k)
    shells = np.linspace(qmin, qmax, nq)
    b = np.array([COHERENT_FM[n] for n in names])
    return Workload("coherent_sqt", coords, cls, names, np.tile(b, (nq, 1)), shells,
                    sphere_directions(nm, seed + 1000), scattering="all",
                    meta=dict(box=box, sigma=sigma, k=k, seed=seed))


def xray_form_factor_params(rng, ntypes):
    """Four-Gaussian + constant coefficients: a_k in [0.5,3], b_k in [0.5,50], c in [0,1].

    Returned as the database's sfactor type-2 parameter vector
    v = (a1, b1/16pi^2, a2, b2/16pi^2, a3, b3/16pi^2, a4, b4/16pi^2, c), because the
    reference evaluates v0*exp(-v1 q^2)+... (database.cpp:513-523) while the
    form factor is a_k exp(-b_k q^2/16pi^2).
    """
    out = []
    for _ in range(ntypes):
        a = rng.uniform(0.5, 3.0, 4)
        bb = rng.uniform(0.5, 50.0, 4) / (16.0 * math.pi ** 2)
        c = rng.uniform(0.0, 1.0)
        v = np.empty(9)
        v[0:8:2] = a
        v[1:8:2] = bb
        v[8] = c
        out.append(v)
    return np.array(out)


def sfactor_type2(v, q):
    return (v[0] * np.exp(-v[1] * q * q) + v[2] * np.exp(-v[3] * q * q)
            + v[4] * np.exp(-v[5] * q * q) + v[6] * np.exp(-v[7] * q * q) + v[8])


def static_xray(seed=3, nbeads=20000, nsolvent=80000, nf=64, box=110.0, bond=1.5, sigma=0.05,
                nq=200, qmin=0.01, qmax=0.5, nm=2000):
    rng = np.random.default_rng(np.random.PCG64(seed))
    steps = rng.standard_normal((nbeads, 3))
    steps *= bond / np.linalg.norm(steps, axis=1, keepdims=True)
    chain = np.cumsum(steps, axis=0)
    chain += box / 2.0 - chain.mean(axis=0)
    solvent = rng.uniform(0.0, box, (nsolvent, 3))
    r0 = np.concatenate([chain, solvent])
    coords = random_walk(rng, r0, nf, sigma)
    names = ["C", "O"]  # coil beads / solvent
    cls = np.concatenate([np.zeros(nbeads, np.int32), np.ones(nsolvent, np.int32)])
    params = xray_form_factor_params(rng, len(names))
    shells = np.linspace(qmin, qmax, nq)
    cf = np.stack([sfactor_type2(params[c], shells) for c in range(len(names))], axis=1)
    return Workload("static_xray", coords, cls, names, cf, shells,
                    sphere_directions(nm, seed + 1000), scattering="all", dsp="square",
                    meta=dict(box=box, seed=seed, sfactor_params=params))


def small(scattering="all", dsp="autocorrelate", seed=7, na=37, nf=24, nq=3, nm=5, box=12.0):
    """A tiny random case for parity tests (ragged sizes on purpose)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    names = ["H", "C", "N", "O"]
    cls = rng.integers(0, len(names), na).astype(np.int32)
    r0 = rng.uniform(0.0, box, (na, 3))
    coords = random_walk(rng, r0, nf, 0.2)
    shells = np.linspace(0.3, 2.5, nq)
    table = COHERENT_FM if scattering == "all" else INCOHERENT_FM
    b = np.array([table[n] for n in names])
    cf = np.tile(b, (nq, 1)) * (1.0 + 0.1 * np.arange(nq))[:, None]
    return Workload("small", coords, cls, names, cf, shells, sphere_directions(nm, seed + 1),
                    scattering=scattering, dsp=dsp)


WORKLOADS = {
    "incoherent_fqt": incoherent_fqt,
    "coherent_sqt": coherent_sqt,
    "static_xray": static_xray,
}


# ----------------------------------------------------------------------------------------
# Files for the sassena-gpu driver: PDB + DCD + db.xml + scatter.xml (+ orientation file)
# ----------------------------------------------------------------------------------------
PDB_NAMES = {"H": "H1", "C": "C1", "N": "N1", "O": "O1", "S": "S1"}


def write_pdb(path, w):
    """ATOM records whose names map through db.xml's names/pdb regexes (atoms.cpp:64-86)."""
    with open(path, "w") as f:
        r0 = w.coords[0]
        for j in range(w.na):
            nm = PDB_NAMES.get(w.class_names[w.atom_class[j]], w.class_names[w.atom_class[j]])
            f.write("ATOM  %5d %-4s MOL A   1    %8.3f%8.3f%8.3f  1.00  0.00\n"
                    % ((j + 1) % 100000, nm, r0[j, 0], r0[j, 1], r0[j, 2]))
        f.write("END\n")


def write_dcd(path, coords):
    """CHARMM DCD as the reference's DCDCoordinateWriter lays it out (coordinate_writer.cpp:37-144):
    84-byte header (unit-cell block flag set), empty title, natoms, then per frame a 48-byte
    unit cell and the X, Y, Z records."""
    import struct
    coords = np.asarray(coords, dtype=np.float32)
    nf, na = coords.shape[0], coords.shape[1]
    with open(path, "wb") as f:
        hdr = struct.pack("<i4s9if13i", 84, b"CORD", nf, 0, 1, 0, 0, 0, 0, 0, 0, 1.0,
                          1, 0, 0, 0, 0, 0, 0, 0, 0, 24, 84, 4, 0)
        # 84 | CORD | nf 0 1 0*6 | dt | ext1=1 ext2=0 0*7 24 | 84, then title record 4 0 4
        f.write(hdr)
        f.write(struct.pack("<i", 4))
        f.write(struct.pack("<3i", 4, na, 4))
        cell = struct.pack("<i6di", 48, 0, 0, 0, 0, 0, 0, 48)
        rec = struct.pack("<i", 4 * na)
        for t in range(nf):
            f.write(cell)
            for k in range(3):
                f.write(rec)
                f.write(np.ascontiguousarray(coords[t, :, k]).tobytes())
                f.write(rec)


def write_database(path, w, sfactor_params=None, masses=None):
    """db.xml: names/pdb regexes, masses (1.0, or `masses` per class), sizes, exclusion
    factors and scattering factors (type 0 constants from the workload's class factors, or
    type 2 parameter vectors)."""
    lines = ["<?xml version=\"1.0\"?>", "<root>", "<names><pdb>"]
    for c in w.class_names:
        lines.append("<element><name>%s</name><param>%s[0-9]*</param></element>" % (c, c))
    lines.append("</pdb></names><masses>")
    for i, c in enumerate(w.class_names):
        m = 1.0 if masses is None else masses[i]
        lines.append("<element><name>%s</name><param>%.17g</param></element>" % (c, m))
    lines.append("</masses><sizes>")
    for c in w.class_names:
        lines.append("<element><name>%s</name><type>0</type><param>1.0</param></element>" % c)
    lines.append("</sizes><exclusionfactors>")
    for c in w.class_names:
        lines.append("<element><name>%s</name><type>0</type><param>0.0</param></element>" % c)
    lines.append("</exclusionfactors><scatterfactors>")
    for i, c in enumerate(w.class_names):
        if sfactor_params is not None:
            ps = "".join("<param>%.17g</param>" % v for v in sfactor_params[i])
            lines.append("<element><name>%s</name><type>2</type>%s</element>" % (c, ps))
        else:
            lines.append("<element><name>%s</name><type>0</type><param>%.17g</param></element>"
                         % (c, w.class_factors[0, i]))
    lines.append("</scatterfactors></root>")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_files(directory, w, precision="fp64", method="fftw", qvectors_file=True,
                signal="signal.h5", sfactor_params=None, extra="", average=None, sample_extra="",
                masses=None):
    """Write sample.pdb, sample.dcd, db.xml, qvectors.txt, orientations.txt and scatter.xml
    for workload `w` into `directory`; returns the scatter.xml path.

    q-vectors are |q_s| along x (the orientation set ignores the q direction,
    abstract_vectors_scatter_device.cpp:123-129) and the directions come from a file
    (vectors.type=file, parameters.cpp:932-943). `average` replaces the <average> element
    (e.g. a multipole orientation); `sample_extra` goes inside <sample> (alignments,
    motions, selections); `masses` are the database masses per class."""
    import os
    if sfactor_params is None and not np.all(w.class_factors == w.class_factors[:1]):
        raise ValueError("type-0 database factors cannot vary with |q|; pass sfactor_params")
    os.makedirs(directory, exist_ok=True)
    write_pdb(os.path.join(directory, "sample.pdb"), w)
    write_dcd(os.path.join(directory, "sample.dcd"), w.coords)
    write_database(os.path.join(directory, "db.xml"), w, sfactor_params, masses)
    with open(os.path.join(directory, "qvectors.txt"), "w") as f:
        for q in w.shells:
            f.write("%.17g 0 0\n" % q)
    with open(os.path.join(directory, "orientations.txt"), "w") as f:
        for d in w.directions:
            f.write("%.17g %.17g %.17g\n" % tuple(d))
    xml = """<?xml version="1.0"?>
<root>
  <sample>
    <structure><file>sample.pdb</file><format>pdb</format></structure>
    <framesets><frameset><file>sample.dcd</file><format>dcd</format></frameset></framesets>
    %(sample_extra)s
  </sample>
  <database><type>file</type><file>db.xml</file></database>
  <scattering>
    <type>%(type)s</type>
    <vectors><type>file</type><file>qvectors.txt</file></vectors>
    <dsp><type>%(dsp)s</type><method>%(method)s</method></dsp>
    %(average)s
    <signal><file>%(signal)s</file></signal>
  </scattering>
  <gpu><precision>%(precision)s</precision></gpu>
  %(extra)s
</root>
""" % dict(type=w.scattering, dsp=w.dsp, method=method, signal=signal, precision=precision,
           extra=extra, sample_extra=sample_extra, average=average or """<average><orientation><type>vectors</type>
      <vectors><type>file</type><file>orientations.txt</file></vectors>
    </orientation></average>""")
    path = os.path.join(directory, "scatter.xml")
    with open(path, "w") as f:
        f.write(xml)
    return path


def batched_uneven(seed=4, nsys=64, na_range=(500, 50000), nf_range=(256, 4096), nq_range=(5, 40),
                   nm_range=(100, 1000), qrange=(0.1, 2.5), density=0.1, sigma=0.1,
                   scattering="all"):
    """Many independent systems of uneven size for the batched launch.

    Atom and frame counts are log-uniform in their ranges, each system is built as the
    1,000-atom workload (uniform positions at `density` atoms/A^3, Gaussian random walk,
    H/C/N/O 50/30/10/10) with its own shells (uniform in `qrange`, sorted) and its own
    direction set (size uniform in `nm_range`)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    names = ["H", "C", "N", "O"]
    table = COHERENT_FM if scattering == "all" else INCOHERENT_FM
    b = np.array([table[n] for n in names])
    out = []
    for i in range(nsys):
        na = int(round(math.exp(rng.uniform(math.log(na_range[0]), math.log(na_range[1])))))
        nf = int(round(math.exp(rng.uniform(math.log(nf_range[0]), math.log(nf_range[1])))))
        nq = int(rng.integers(nq_range[0], nq_range[1] + 1))
        nm = int(rng.integers(nm_range[0], nm_range[1] + 1))
        box = (na / density) ** (1.0 / 3.0)
        cls = _types(rng, na, names, [50, 30, 10, 10])
        r0 = rng.uniform(0.0, box, (na, 3))
        coords = random_walk(rng, r0, nf, sigma)
        shells = np.sort(rng.uniform(qrange[0], qrange[1], nq))
        out.append(Workload("batched_%d" % i, coords, cls, names, np.tile(b, (nq, 1)), shells,
                            sphere_directions(nm, seed * 1000 + i), scattering=scattering,
                            meta=dict(box=box, seed=seed)))
    return out


def layered(seed=5, na=50000, nf=2048, box=80.0, period=8.0, amplitude=0.3, sigma=0.05, nq=100,
            qmin=0.1, qmax=1.5, nm=64):
    """Anisotropic layered system: density along z modulated as 1 + amplitude*cos(2 pi z/period)
    (rejection sampling), uniform in x and y, Gaussian random walk; coherent H/C/N/O lengths."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    z = np.empty(0)
    while len(z) < na:
        c = rng.uniform(0.0, box, 2 * na)
        keep = rng.uniform(0.0, 1.0 + amplitude, 2 * na) < 1.0 + amplitude * np.cos(2 * math.pi * c / period)
        z = np.concatenate([z, c[keep]])
    r0 = np.stack([rng.uniform(0.0, box, na), rng.uniform(0.0, box, na), z[:na]], axis=1)
    names = ["H", "C", "N", "O"]
    cls = _types(rng, na, names, [50, 30, 10, 10])
    coords = random_walk(rng, r0, nf, sigma)
    shells = np.linspace(qmin, qmax, nq)
    b = np.array([COHERENT_FM[n] for n in names])
    return Workload("layered", coords, cls, names, np.tile(b, (nq, 1)), shells,
                    sphere_directions(nm, seed + 1000), scattering="all",
                    meta=dict(box=box, period=period, amplitude=amplitude, seed=seed))


def aligned_rods(seed=6, nmol=300, per_mol=8, spacing=1.5, box=40.0, nf=32, sigma=2.0, nq=3,
                 qmin=0.5, qmax=1.5, nm=32):
    """Rigid rod-like molecules aligned along z (per_mol atoms, `spacing` apart) whose centres
    diffuse fast (Gaussian steps sigma per frame): intermolecular interference averages out over
    the frames while the intramolecular form factor |sum_k exp(i q_z k d)|^2 leaves a smooth,
    strongly anisotropic orientational dependence."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    centres = rng.uniform(0.0, box, (nmol, 3))
    offs = np.zeros((per_mol, 3))
    offs[:, 2] = (np.arange(per_mol) - 0.5 * (per_mol - 1)) * spacing
    coords = np.empty((nf, nmol * per_mol, 3), dtype=np.float32)
    c = centres.copy()
    for t in range(nf):
        coords[t] = (c[:, None, :] + offs[None, :, :]).reshape(-1, 3)
        c += rng.standard_normal(c.shape) * sigma
    na = nmol * per_mol
    names = ["C"]
    cls = np.zeros(na, np.int32)
    shells = np.linspace(qmin, qmax, nq)
    return Workload("aligned_rods", coords, cls, names, np.full((nq, 1), COHERENT_FM["C"]), shells,
                    sphere_directions(nm, seed + 1000), scattering="all",
                    meta=dict(box=box, spacing=spacing, per_mol=per_mol, seed=seed))
