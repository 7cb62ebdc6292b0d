"""Shared helpers for the parity tests."""
import os

import numpy as np


def rel_err_sqt(fqt, ref):
    """max_t |S - S_ref| / |S_ref(q,0)| per q (the path's error metric)."""
    ref = np.asarray(ref)
    fqt = np.asarray(fqt)
    if ref.ndim == 3:  # [nq, nf, 2] from the oracle
        ref = ref[..., 0] + 1j * ref[..., 1]
    den = np.maximum(np.abs(ref[:, 0]), 1e-300)
    return np.max(np.abs(fqt - ref), axis=1) / den


def cplx(a):
    a = np.asarray(a)
    return a[..., 0] + 1j * a[..., 1]


def rel_err_vec(x, ref):
    """|x - ref| / max(|ref|) over a vector of complex values."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    scale = max(np.max(np.abs(ref)), 1e-300)
    return np.max(np.abs(x - ref)) / scale


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class Fixture:
    """One case of a golden .npz (arrays named "<case>.<field>"), with the workload rebuilt."""

    def __init__(self, z, name):
        self.name = name
        g = lambda k: z[name + "." + k]  # noqa: E731
        self.scattering, self.dsp, self.method = str(g("kind")).split("/")
        self.coords = g("coords")
        self.atom_class = g("atom_class")
        self.class_factors = g("class_factors")
        self.shells = g("shells")
        self.directions = g("directions")
        self.fqt, self.fq, self.fq2 = g("fqt"), g("fq"), g("fq2")
        self.extra = {k.split(".", 1)[1]: z[k] for k in z.files if k.startswith(name + ".")}

    @property
    def na(self):
        return self.coords.shape[1]

    @property
    def nf(self):
        return self.coords.shape[0]

    def sub_offsets(self):
        return np.arange(len(self.shells) + 1, dtype=np.uintp) * len(self.directions)

    def subvectors(self):
        return (self.shells[:, None, None] * self.directions[None]).reshape(-1, 3)

    def factors(self):
        return self.class_factors[:, self.atom_class]


def golden(family):
    """{case: Fixture} of tests/golden/<family>.npz."""
    z = np.load(os.path.join(GOLDEN, family + ".npz"))
    names = sorted({k.split(".", 1)[0] for k in z.files if k.endswith(".fqt")})
    return {n: Fixture(z, n) for n in names}


class ReferenceCase:
    """One device run of tests/golden/reference.npz (outputs of the reference's own compiled
    scatter devices, made by make_reference_golden.py), with the q-vectors expanded into
    sub-vectors the way the reference does it: file orientations normalised by 1/|v|
    (parameters.cpp:936-941) and scaled by |q| (abstract_vectors_scatter_device.cpp:116-122);
    no orientations means the q-vector itself (:172)."""

    def __init__(self, z, name):
        g = lambda k: z[name + "." + k]  # noqa: E731
        self.name = name
        self.scattering, self.dsp, self.method = str(g("kind")).split("/")
        self.coords = g("coords")
        self.atom_class = g("atom_type")
        self.class_factors = g("class_factors")
        self.qvectors, self.orient = g("qvectors"), g("orient")
        self.fqt, self.fq, self.fq2 = g("fqt"), g("fq"), g("fq2")
        self.q_out = g("q_out")
        # what GpuVectorsScatterDevice (sassena_gb300/integration), driven by the reference's
        # own run(), passed to the C ABI on the same case (make_reference_golden.py)
        self.bind_desc = g("bind_desc")  # scattering, dsp type, method, precision, na, nf, nclass
        self.bind_offs = g("bind_offs").astype(np.uintp)
        self.bind_subvectors = g("bind_subvectors")
        self.bind_class_factors = g("bind_class_factors")
        self.bind_classes = g("bind_classes")

    @property
    def na(self):
        return self.coords.shape[1]

    @property
    def nf(self):
        return self.coords.shape[0]

    def sub_offsets(self):
        per = max(len(self.orient), 1)
        return np.arange(len(self.qvectors) + 1, dtype=np.uintp) * per

    def subvectors(self):
        q = self.qvectors
        if len(self.orient) == 0:
            return q.copy()
        ql = np.sqrt(q[:, 0] ** 2 + q[:, 1] ** 2 + q[:, 2] ** 2)
        ol = np.sqrt(self.orient[:, 0] ** 2 + self.orient[:, 1] ** 2 + self.orient[:, 2] ** 2)
        u = (1.0 / ol)[:, None] * self.orient
        return (ql[:, None, None] * u[None]).reshape(-1, 3)

    def factors(self):
        return self.class_factors[:, self.atom_class]


def reference_cases():
    """{case: ReferenceCase} of the device runs in tests/golden/reference.npz."""
    z = np.load(os.path.join(GOLDEN, "reference.npz"))
    names = sorted({k.split(".", 1)[0] for k in z.files if k.endswith(".fqt")})
    return {n: ReferenceCase(z, n) for n in names}


def reference_fixture():
    return np.load(os.path.join(GOLDEN, "reference.npz"))
