"""Writes the golden fixtures of this directory: seeded inputs with the FP64 oracle's outputs.

The reference ships no golden vectors for the scattering path and cannot be built here (it
needs MPI, Boost, FFTW3, HDF5, libxml2 and LAPACK), so these fixtures hold the outputs of the
oracle (oracle/cpu_oracle.cpp, itself cross-checked against the numpy restatement and the
analytic known answers in test_oracle.py). Each fixture keeps its inputs, so it does not depend
on the random streams of numpy staying the same across versions.

    python tests/golden/make_golden.py      # from the repository root; rewrites *.npz

Families (one .npz each, arrays prefixed by the case name):
  scatter_*   coherent / incoherent devices, every dsp type and method, the three benchmark
              workload shapes shrunk (incoherent F(q,t) at 128 frames, coherent S(q,t) at 1,024
              frames, the static X-ray square with sfactor type-2 factors), an incoherent series
              of 600 frames and one long series;
  multipole   the sphere and cylinder multipole devices;
  prepass     the staged frames after the alignments and motions of tests/prepass_cases.py.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import alignment as al  # noqa: E402
from sassena_gb300 import synth  # noqa: E402

DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}


def scatter_cases():
    """name -> (workload, method)."""
    out = {}
    for dsp, method in (("autocorrelate", "fftw"), ("autocorrelate", "direct"), ("square", "fftw"),
                        ("plain", "fftw")):
        tag = dsp if dsp != "autocorrelate" else "acf_" + method
        out["coh_" + tag] = (synth.small("all", dsp, seed=101, na=23, nf=17, nq=3, nm=4), method)
        out["inc_" + tag] = (synth.small("self", dsp, seed=102, na=19, nf=13, nq=2, nm=3), method)
    out["incoherent_fqt_shape"] = (synth.incoherent_fqt(seed=103, na=40, nf=128, nq=3, nm=8), "fftw")
    out["coherent_sqt_shape"] = (synth.coherent_sqt(seed=104, na=12, nf=1024, box=10.0, nq=2, nm=4),
                                 "fftw")
    out["static_xray_shape"] = (synth.static_xray(seed=105, nbeads=30, nsolvent=90, nf=8, box=20.0,
                                                  nq=3, qmin=0.05, qmax=0.5, nm=6), "fftw")
    out["long_series"] = (synth.small("all", "autocorrelate", seed=106, na=3, nf=4200, nq=1, nm=2,
                                      box=10.0), "fftw")
    out["incoherent_blocks"] = (synth.small("self", "autocorrelate", seed=107, na=5, nf=600, nq=2, nm=3,
                                            box=10.0), "fftw")  # padded length 2,048: 4 blocks of 512
    return out


def run_scatter(w, method):
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    return fn(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), DSP_ID[w.dsp], METHOD_ID[method],
              nthreads=4)


def multipole_cases():
    """name -> (workload, q [nq, 3], kind, moments, axis)."""
    out = {}
    for kind, seed, moments, axis in (("sphere", 111, oracle.sphere_moments(4), (0.0, 0.0, 1.0)),
                                      ("cylinder", 112, oracle.cylinder_moments(4), (1.0, 1.0, 0.3))):
        w = synth.small("all", "autocorrelate", seed=seed, na=17, nf=12, nq=2, nm=3, box=12.0)
        rng = np.random.default_rng(seed)
        q = rng.normal(size=(2, 3))
        q *= (w.shells / np.linalg.norm(q, axis=1))[:, None]
        out["mp_" + kind] = (w, q, kind, np.array(moments, dtype=np.int64), np.array(axis))
    return out


def run_multipole(w, q, kind, moments, axis):
    mom = [tuple(int(v) for v in m) for m in moments]
    if kind == "sphere":
        return oracle.mp_sphere(w.coords, q, w.factors(), mom)
    return oracle.mp_cylinder(w.coords, q, w.factors(), mom, tuple(axis))


def save_workload(d, name, w, method):
    d[name + ".coords"] = w.coords
    d[name + ".atom_class"] = w.atom_class
    d[name + ".class_factors"] = w.class_factors
    d[name + ".shells"] = w.shells
    d[name + ".directions"] = w.directions
    d[name + ".kind"] = np.array("%s/%s/%s" % (w.scattering, w.dsp, method))


def main():
    d = {}
    for name, (w, method) in scatter_cases().items():
        save_workload(d, name, w, method)
        fqt, fq, fq2 = run_scatter(w, method)
        d[name + ".fqt"], d[name + ".fq"], d[name + ".fq2"] = fqt, fq, fq2
    np.savez_compressed(os.path.join(HERE, "scatter.npz"), **d)

    d = {}
    for name, (w, q, kind, moments, axis) in multipole_cases().items():
        save_workload(d, name, w, "fftw")
        d[name + ".q"], d[name + ".moments"], d[name + ".axis"] = q, moments, axis
        d[name + ".mp"] = np.array(kind)
        fqt, fq, fq2 = run_multipole(w, q, kind, moments, axis)
        d[name + ".fqt"], d[name + ".fq"], d[name + ".fq2"] = fqt, fq, fq2
    np.savez_compressed(os.path.join(HERE, "multipole.npz"), **d)

    import prepass_cases as pc
    d = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name in pc.CASES:
            w, _, o = pc.build(name, os.path.join(tmp, name))
            if name == pc.CASES[0]:
                d["coords"] = w.coords
            d[name + ".staged"] = al.load(w.coords, o["masses"], o["alignments"], o["motions"], o["target"])
    np.savez_compressed(os.path.join(HERE, "prepass.npz"), **d)


if __name__ == "__main__":
    main()
