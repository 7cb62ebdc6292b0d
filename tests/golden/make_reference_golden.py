"""Writes tests/golden/reference.npz: outputs of the reference's own compiled code.

The reference's scatter devices, signal math, scatter factors, database getters and
q-vector scans are compiled from their sources (read in place, never copied into this
repository) against small stand-in headers by oracle/ref_build/Makefile into
oracle/_ref/libsassena_ref.so. FFTW is replaced there by an extended-precision direct
DFT with FFTW's definition. This script runs that library on seeded synthetic inputs and
stores the inputs together with the outputs, so the tests can pin the FP64 oracle and the
GPU path to the reference's arithmetic without the reference tree (which the GPU machine does
not have).

    python tests/golden/make_reference_golden.py    # from the repository root

Cases (arrays prefixed by the case name):
  coh_* / inc_*      the coherent and incoherent vectors devices, every dsp type and method,
                     file orientations (vectors.type = file) and orientation-free q-vectors;
                     frame counts 37 (padded transform length 74, not a power of two), 48,
                     128 and 1,024; one case with the type-2 (four-Gaussian) form factors, a
                     background factor and exclusion factors; one run with one worker thread
  scans_*            ScatteringVectorsParameters::create_from_scans for 1, 2 and 3 scans
  db_*               DatabaseSFactorsParameters / Volumes / Exclusion getters
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libsassena_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_sp = ctypes.POINTER(ctypes.c_size_t)


def load(ref_tree=None):
    """Build (if needed) and load oracle/_ref/libsassena_ref.so."""
    cmd = ["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_build")]
    if ref_tree:
        cmd.append("REF=" + ref_tree)
    subprocess.run(cmd, check=True)
    L = ctypes.CDLL(LIB, mode=os.RTLD_NOW)
    L.ref_run_vectors.restype = ctypes.c_long
    L.ref_run_vectors.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t, _fp,
                                  ctypes.c_size_t, ctypes.c_size_t, _ip, ctypes.c_size_t, _ip, _dp, _dp, _ip,
                                  _dp, ctypes.c_double, ctypes.c_size_t, _dp, ctypes.c_size_t, _dp, _dp, _dp,
                                  _dp, _dp]
    L.bind_run_vectors.restype = ctypes.c_long
    L.bind_run_vectors.argtypes = L.ref_run_vectors.argtypes
    L.bind_last_sizes.argtypes = [ctypes.POINTER(ctypes.c_long), _sp]
    L.bind_last_calls.argtypes = [_sp, _dp, _dp, _ip, _fp]
    L.ref_scans.restype = ctypes.c_long
    L.ref_scans.argtypes = [ctypes.c_size_t, _dp, _dp, _sp, _dp, _dp, ctypes.c_size_t, _dp]
    L.ref_sfactor.restype = ctypes.c_double
    L.ref_sfactor.argtypes = [ctypes.c_int, _dp, ctypes.c_size_t, ctypes.c_double]
    L.ref_volume.restype = ctypes.c_double
    L.ref_volume.argtypes = [ctypes.c_int, _dp, ctypes.c_size_t]
    L.ref_exclusion.restype = ctypes.c_double
    L.ref_exclusion.argtypes = [ctypes.c_int, _dp, ctypes.c_size_t, ctypes.c_double, ctypes.c_double]
    L.ref_last_error.restype = ctypes.c_char_p
    return L


def _p(a, t):
    return a.ctypes.data_as(t)


# Per-type database tables: H, C, N, O, S with coherent neutron lengths (fm, sfactor type 0),
# volumes in A^3 (volume type 0) and exclusion type 2 (Gaussian) with factor 1.
COHERENT = np.array([-3.7390, 6.6460, 9.3600, 5.8030, 2.8470])
INCOHERENT = np.array([25.274, 0.089, 1.990, 0.080, 0.236])
VOLUMES = np.array([5.15, 16.44, 2.49, 9.13, 25.23])


def type_tables(kind, rng=None, ntype=5):
    """(sf_type [ntype], sf_const [ntype, 9], vol [ntype], ex_type [ntype], ex_const [ntype])."""
    sf_const = np.zeros((ntype, 9))
    if kind == "xray":  # four Gaussians + c with b_k / 16 pi^2 folded in (database type 2)
        sf_type = np.full(ntype, 2, dtype=np.int32)
        a = rng.uniform(0.5, 3.0, (ntype, 4))
        b = rng.uniform(0.5, 50.0, (ntype, 4)) / (16 * np.pi ** 2)
        sf_const[:, 0:8:2] = a
        sf_const[:, 1:8:2] = b
        sf_const[:, 8] = rng.uniform(0.0, 1.0, ntype)
    else:
        sf_type = np.zeros(ntype, dtype=np.int32)
        sf_const[:, 0] = (COHERENT if kind == "coherent" else INCOHERENT)[:ntype]
    return (sf_type, sf_const, VOLUMES[:ntype].copy(), np.full(ntype, 2, dtype=np.int32), np.ones(ntype))


def trajectory(rng, na, nf, box, sigma):
    r = rng.uniform(0.0, box, (na, 3))
    out = np.empty((nf, na, 3), dtype=np.float32)
    for t in range(nf):
        out[t] = r
        r = r + rng.normal(0.0, sigma, (na, 3))
    return out


def directions(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True) * rng.uniform(0.5, 2.0, (n, 1))  # unnormalised on purpose


def run_case(L, self_, dsp, method, coords, atom_type, tables, background, qvectors, orient, nthreads=3,
             binding=False):
    sf_type, sf_const, vol, ex_type, ex_const = tables
    nf, na = coords.shape[0], coords.shape[1]
    nq, nm = len(qvectors), len(orient)
    q_out = np.zeros((nq, 3))
    fqt = np.zeros((nq, nf, 2))
    fq = np.zeros((nq, 2))
    fq2 = np.zeros((nq, 2))
    orient_arr = np.ascontiguousarray(orient if nm else np.zeros((1, 3)))
    fn = L.bind_run_vectors if binding else L.ref_run_vectors
    rows = fn(int(self_), dsp.encode(), method.encode(), nthreads,
                             _p(np.ascontiguousarray(coords), _fp), nf, na,
                             _p(np.ascontiguousarray(atom_type, dtype=np.int32), _ip), len(sf_type),
                             _p(sf_type, _ip), _p(sf_const, _dp), _p(vol, _dp), _p(ex_type, _ip), _p(ex_const, _dp),
                             background, nq, _p(np.ascontiguousarray(qvectors), _dp), nm, _p(orient_arr, _dp),
                             _p(q_out, _dp), _p(fqt, _dp), _p(fq, _dp), _p(fq2, _dp))
    if rows != nq:
        raise RuntimeError("reference run failed (%d rows): %s" % (rows, L.ref_last_error().decode()))
    return q_out, fqt, fq, fq2


def binding_calls(L, coords):
    """What GpuVectorsScatterDevice passed to the C ABI in the last bind_run_vectors."""
    ints = (ctypes.c_long * 8)()
    sizes = (ctypes.c_size_t * 4)()
    L.bind_last_sizes(ints, sizes)
    offs = np.zeros(sizes[0], dtype=np.uintp)
    sv = np.zeros(sizes[1])
    cf = np.zeros(sizes[2])
    classes = np.zeros(ints[4], dtype=np.int32)
    frames = np.zeros(sizes[3], dtype=np.float32)
    L.bind_last_calls(_p(offs, _sp), _p(sv, _dp), _p(cf, _dp), _p(classes, _ip), _p(frames, _fp))
    if not np.array_equal(frames.reshape(coords.shape), coords):
        raise RuntimeError("the binding staged other frames than the stager's")
    if ints[7] != 1:
        raise RuntimeError("the binding made %d sass_compute calls, expected one" % ints[7])
    return dict(bind_desc=np.array(list(ints)[:7], dtype=np.int64), bind_offs=offs.astype(np.int64),
                bind_subvectors=sv.reshape(-1, 3), bind_class_factors=cf.reshape(len(offs) - 1, ints[6]),
                bind_classes=classes)


def class_factors(L, tables, background, qlen):
    """b(type, |q|) = sf - background * exclusion(kappa = 1 times volume) as
    ScatterFactors::update forms it (scatter_factors.cpp:56-78), per |q| and type."""
    sf_type, sf_const, vol, ex_type, ex_const = tables
    out = np.zeros((len(qlen), len(sf_type)))
    for i, ql in enumerate(qlen):
        for t in range(len(sf_type)):
            sf = L.ref_sfactor(int(sf_type[t]), _p(np.ascontiguousarray(sf_const[t]), _dp), 9, ql)
            if background != 0.0:
                v = L.ref_volume(0, _p(np.array([vol[t]]), _dp), 1)
                ef = L.ref_exclusion(int(ex_type[t]), _p(np.array([ex_const[t]]), _dp), 1, 1.0 * v, ql)
                sf = sf - background * ef
            out[i, t] = sf
    return out


def vector_cases(L):
    rng = np.random.default_rng(20261204)
    cases = {}

    def add(name, self_, dsp, method, na, nf, nq, nm, box=15.0, sigma=0.2, kind=None, background=0.0,
            nthreads=3):
        kind = kind or ("incoherent" if self_ else "coherent")
        ntype = 5 if kind != "incoherent" else 4
        tables = type_tables(kind, rng, ntype)
        coords = trajectory(rng, na, nf, box, sigma)
        atom_type = rng.integers(0, ntype, na).astype(np.int32)
        base = rng.normal(size=(nq, 3))
        qlen = np.linspace(0.3, 2.4, nq)
        qvectors = base / np.linalg.norm(base, axis=1, keepdims=True) * qlen[:, None]
        orient = directions(rng, nm) if nm else np.zeros((0, 3))
        q_out, fqt, fq, fq2 = run_case(L, self_, dsp, method, coords, atom_type, tables, background, qvectors,
                                       orient, nthreads)
        qref = np.sqrt(qvectors[:, 0] ** 2 + qvectors[:, 1] ** 2 + qvectors[:, 2] ** 2)
        # the binding device on the same case: the rows it writes (zero: its C ABI only
        # records) must come in the reference's order, and its recorded calls are kept
        bq_out, _, _, _ = run_case(L, self_, dsp, method, coords, atom_type, tables, background, qvectors,
                                   orient, nthreads, binding=True)
        if not np.array_equal(bq_out, q_out):
            raise RuntimeError("binding rows out of order in " + name)
        calls = binding_calls(L, coords)
        cases[name] = dict(**calls,kind=np.array("%s/%s/%s" % ("self" if self_ else "all", dsp, method)),
                           coords=coords, atom_type=atom_type, sf_type=tables[0], sf_const=tables[1],
                           vol=tables[2], ex_type=tables[3], ex_const=tables[4], background=np.array(background),
                           qvectors=qvectors, orient=orient, q_out=q_out, fqt=fqt, fq=fq, fq2=fq2,
                           class_factors=class_factors(L, tables, background, qref))

    for dsp, method in (("autocorrelate", "fftw"), ("autocorrelate", "direct"), ("square", "fftw"),
                        ("plain", "fftw")):
        tag = dsp if dsp != "autocorrelate" else "acf_" + method
        add("coh_" + tag, False, dsp, method, na=64, nf=48, nq=4, nm=9)
        add("inc_" + tag, True, dsp, method, na=24, nf=32, nq=3, nm=5)
    add("coh_acf_nf37", False, "autocorrelate", "fftw", na=40, nf=37, nq=3, nm=6)
    add("inc_acf_nf37", True, "autocorrelate", "fftw", na=15, nf=37, nq=2, nm=4)
    add("coh_acf_no_orientation", False, "autocorrelate", "fftw", na=50, nf=20, nq=5, nm=0)
    add("coh_acf_one_thread", False, "autocorrelate", "fftw", na=30, nf=24, nq=2, nm=7, nthreads=1)
    add("inc_acf_nf128", True, "autocorrelate", "fftw", na=30, nf=128, nq=2, nm=4, sigma=0.1)
    add("coh_acf_nf1024", False, "autocorrelate", "fftw", na=64, nf=1024, nq=2, nm=3, box=10.0, sigma=0.05)
    add("coh_square_xray_background", False, "square", "fftw", na=80, nf=16, nq=5, nm=11, box=20.0,
        kind="xray", background=0.35)
    return cases


def scan_cases(L):
    specs = {
        "scans_one_linear": [(0.1, 2.0, 10, 1.0, (1.0, 0.0, 0.0))],
        "scans_one_power": [(0.05, 3.0, 20, 1.7, (0.3, -0.4, 0.866))],
        "scans_one_point": [(0.5, 1.5, 1, 1.0, (0.0, 0.0, 1.0))],
        "scans_two_points": [(0.5, 1.5, 2, 1.0, (0.0, 1.0, 0.0))],
        "scans_two": [(0.1, 1.0, 4, 1.0, (1.0, 0.0, 0.0)), (0.2, 0.6, 3, 0.5, (0.0, 1.0, 0.0))],
        "scans_three": [(0.0, 1.0, 3, 1.0, (1.0, 0.0, 0.0)), (0.0, 1.0, 3, 2.0, (0.0, 1.0, 0.0)),
                        (-0.5, 0.5, 5, 1.0, (0.0, 0.0, 1.0))],
    }
    cases = {}
    for name, scans in specs.items():
        f = np.array([s[0] for s in scans])
        t = np.array([s[1] for s in scans])
        p = np.array([s[2] for s in scans], dtype=np.uintp)
        e = np.array([s[3] for s in scans])
        b = np.ascontiguousarray(np.array([s[4] for s in scans], dtype=np.float64))
        out = np.zeros((4096, 3))
        n = L.ref_scans(len(scans), _p(f, _dp), _p(t, _dp), _p(p, _sp), _p(e, _dp), _p(b, _dp), 4096,
                        _p(out, _dp))
        cases[name] = dict(scan_from=f, scan_to=t, scan_points=p.astype(np.int64), scan_exponent=e, scan_base=b,
                           qvectors=out[:n].copy())
    return cases


def database_cases(L):
    rng = np.random.default_rng(5)
    sf_rows, vol_rows, ex_rows = [], [], []
    for ft in (0, 2):
        for _ in range(6):
            c = np.concatenate([rng.uniform(0.5, 3.0, 8) * np.array([1, 0.01] * 4), [rng.uniform(0, 1)]])
            for q in (0.0, 0.01, 0.37, 1.5, 3.0):
                sf_rows.append([ft, q, *c, L.ref_sfactor(ft, _p(np.ascontiguousarray(c), _dp), 9, q)])
    for ft in (0, 1, 2):
        for r in (0.7, 1.3, 2.2):
            vol_rows.append([ft, r, L.ref_volume(ft, _p(np.array([r]), _dp), 1)])
    for ft in (0, 1, 2):
        for c in (0.4, 1.0):
            for v in (3.0, 17.5):
                for q in (0.0, 0.5, 2.5):
                    ex_rows.append([ft, c, v, q, L.ref_exclusion(ft, _p(np.array([c]), _dp), 1, v, q)])
    return {"db": dict(sfactor=np.array(sf_rows), volume=np.array(vol_rows), exclusion=np.array(ex_rows))}


def main():
    L = load(sys.argv[1] if len(sys.argv) > 1 else None)
    arrays = {}
    for group in (vector_cases(L), scan_cases(L), database_cases(L)):
        for case, fields in group.items():
            for k, v in fields.items():
                arrays["%s.%s" % (case, k)] = v
    path = os.path.join(HERE, "reference.npz")
    np.savez_compressed(path, **arrays)
    print("wrote %s (%d arrays, %.0f kB)" % (path, len(arrays), os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()
