"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bars (error metric rel_err = max_t |S - S_ref| / |S_ref(q,0)| per q):
  * FP64 plain path: <= 1e-12 (the reference's FP64 results, oracle restatement);
  * FP32 fast path:  <= 1e-3 (the accuracy target of the precision form).
"""
import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

from helpers import cplx, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

DSPS = [("autocorrelate", "fftw"), ("autocorrelate", "direct"), ("square", "fftw"),
        ("plain", "fftw")]
DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}
TOL = {"fp64": 1e-12, "fp32": 1e-3}


def run_oracle(w, dsp, method):
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    return fn(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), DSP_ID[dsp],
              METHOD_ID[method], nthreads=8)


def run_gpu(w, precision, method, tile=None):
    return abi.compute_workload(w, precision=precision, method=method, tile=tile)


def check(w, precision, method, tile=None):
    ref_fqt, ref_fq, ref_fq2 = run_oracle(w, w.dsp, method)
    fqt, fq, fq2 = run_gpu(w, precision, method, tile)
    tol = TOL[precision]
    e_t = rel_err_sqt(fqt, ref_fqt).max()
    e_q = rel_err_vec(fq, cplx(ref_fq))
    e_q2 = rel_err_vec(fq2, cplx(ref_fq2))
    assert e_t <= tol, "fqt rel err %.3e > %.1e" % (e_t, tol)
    assert e_q <= tol, "fq rel err %.3e > %.1e" % (e_q, tol)
    assert e_q2 <= tol, "fq2 rel err %.3e > %.1e" % (e_q2, tol)
    return e_t, e_q, e_q2


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("dsp,method", DSPS)
def test_coherent_small(native_lib, precision, dsp, method):
    w = synth.small("all", dsp, seed=11, na=37, nf=24, nq=3, nm=5)
    check(w, precision, method)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("dsp,method", DSPS)
def test_incoherent_small(native_lib, precision, dsp, method):
    w = synth.small("self", dsp, seed=12, na=29, nf=21, nq=2, nm=4)
    check(w, precision, method)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_coherent_ragged_medium(native_lib, precision):
    # NA not a multiple of the 128-atom granule, NF not a power of two, NM not a
    # multiple of 32 and shells of different sizes (CSR offsets).
    w = synth.small("all", "autocorrelate", seed=13, na=301, nf=77, nq=4, nm=45)
    check(w, precision, "fftw")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_incoherent_ragged_medium(native_lib, precision):
    w = synth.small("self", "autocorrelate", seed=14, na=150, nf=100, nq=2, nm=7)
    check(w, precision, "fftw")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_uneven_shells(native_lib, precision):
    w = synth.small("all", "autocorrelate", seed=15, na=64, nf=33, nq=3, nm=40)
    offs = np.array([0, 3, 40, 41, 120], dtype=np.uintp)  # 4 q-vectors, uneven sub-vector sets
    rng = np.random.default_rng(5)
    sv = rng.normal(size=(120, 3))
    cf = np.tile(w.class_factors[:1], (4, 1))
    fac = cf[:, w.atom_class]
    ref = oracle.all_vectors(w.coords, offs, sv, fac, 0, 0, nthreads=8)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", "autocorrelate", "fftw", precision) as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        fqt, fq, fq2 = p.compute(offs, sv, cf)
    assert rel_err_sqt(fqt, ref[0]).max() <= TOL[precision]
    assert rel_err_vec(fq2, cplx(ref[2])) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("splits", [1, 3])
def test_amplitudes_and_atom_splits(native_lib, precision, splits):
    w = synth.small("all", "autocorrelate", seed=16, na=700, nf=19, nq=2, nm=9)
    sv = w.subvectors()
    shell = np.repeat(np.arange(w.nq), w.nm).astype(np.int32)
    ref = oracle.amplitudes(w.coords, sv, shell.astype(np.uintp), w.factors(), nthreads=8)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", precision=precision) as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        q = 1
        tile = (q, 8, 128) if precision == "fp32" else (q, 4, 64)
        p.set_tile(*tile, atom_splits=splits)
        amp = p.amplitudes(sv, shell, w.class_factors)
    scale = np.abs(w.factors()).sum(axis=1).max()
    err = np.abs(amp - ref).max() / scale
    assert err <= (1e-13 if precision == "fp64" else 2e-5), err


FP32_SHAPES = [(1, 8, 128, 0), (2, 8, 128, 0), (4, 8, 128, 0), (8, 8, 128, 0), (8, 8, 128, 1),
               (4, 4, 128, 0), (8, 4, 128, 0), (8, 4, 128, 1), (2, 8, 64, 0), (4, 8, 64, 0)]


@pytest.mark.parametrize("shape", FP32_SHAPES)
def test_fp32_direct_shapes(native_lib, shape):
    # every instantiated FP32 tile of the direct kernel: scalar (Q=1), paired SFU, and paired
    # with one pair of polynomial sin/cos per lane, on ragged sizes
    w = synth.small("all", "autocorrelate", seed=17, na=450, nf=21, nq=3, nm=70, box=25.0)
    sv = w.subvectors()
    shell = np.repeat(np.arange(w.nq), w.nm).astype(np.int32)
    ref = oracle.amplitudes(w.coords, sv, shell.astype(np.uintp), w.factors(), nthreads=8)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", precision="fp32") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        p.set_tile(*shape[:3])
        p.set_poly(shape[3])
        amp = p.amplitudes(sv, shell, w.class_factors)
        assert p.schedule()["poly_pairs"] == shape[3]
    scale = np.abs(w.factors()).sum(axis=1).max()
    err = np.abs(amp - ref).max() / scale
    assert err <= 2e-6, err


def test_static_single_atom(native_lib):
    # One static atom: |A|^2 = b^2 for every q and t (known answer).
    nf = 16
    coords = np.tile(np.array([[[1.5, -2.0, 0.25]]], dtype=np.float32), (nf, 1, 1))
    b = 3.7
    offs = np.array([0, 6], dtype=np.uintp)
    sv = synth.sphere_directions(6, 3) * 1.3
    for precision in ("fp64", "fp32"):
        with abi.Plan(1, nf, 1, "all", "autocorrelate", "fftw", precision) as p:
            p.stage(coords)
            p.set_classes(np.zeros(1, np.int32))
            fqt, fq, fq2 = p.compute(offs, sv, np.array([[b]]))
        assert np.allclose(fqt.real, b * b, rtol=1e-12 if precision == "fp64" else 1e-5)
        assert np.abs(fqt.imag).max() <= 1e-12 * b * b if precision == "fp64" else 1e-5 * b * b


def test_two_atom_identity(native_lib):
    # Two static atoms: |A(q u)|^2 = b1^2 + b2^2 + 2 b1 b2 cos(q u.d) per direction, exact.
    nf = 4
    r = np.array([[0.0, 0.0, 0.0], [1.2, -0.7, 2.1]], dtype=np.float32)
    coords = np.tile(r[None], (nf, 1, 1))
    b = np.array([2.0, -1.3])
    dirs = synth.fibonacci_sphere(64)
    q = 1.7
    offs = np.array([0, 64], dtype=np.uintp)
    with abi.Plan(2, nf, 2, "all", "square", "fftw", "fp64") as p:
        p.stage(coords)
        p.set_classes(np.array([0, 1], np.int32))
        fqt, fq, fq2 = p.compute(offs, q * dirs, b[None, :])
    d = (r[1] - r[0]).astype(np.float64)
    expect = np.mean(b[0] ** 2 + b[1] ** 2 + 2 * b[0] * b[1] * np.cos(q * dirs @ d))
    assert abs(fq[0].real - expect) <= 1e-12 * abs(expect)
    assert np.allclose(fqt[0].real, expect, rtol=1e-12)


def test_error_paths(native_lib):
    with pytest.raises(abi.SassError) as e:
        abi.Plan(10, 0, 1)
    assert e.value.code == 1
    with pytest.raises(abi.SassError) as e:  # beyond the long-series transform (NF <= 524,288)
        abi.Plan(10, 600000, 1, "all", "autocorrelate")
    assert e.value.code == 3
    with abi.Plan(4, 4, 2) as p:
        with pytest.raises(abi.SassError) as e:
            p.compute(np.array([0, 1], np.uintp), np.ones((1, 3)), np.ones((1, 2)))
        assert e.value.code == 6  # compute before staging
        p.stage(np.zeros((4, 4, 3), np.float32))
        with pytest.raises(abi.SassError) as e:
            p.set_classes(np.array([0, 1, 2, 0], np.int32))  # class 2 >= nclass
        assert e.value.code == 1
        p.set_classes(np.array([0, 1, 1, 0], np.int32))
        with pytest.raises(abi.SassError) as e:
            p.compute(np.array([0, 0], np.uintp), np.ones((1, 3)), np.ones((1, 2)))
        assert e.value.code == 1  # a q-vector with no sub-vectors
        with pytest.raises(abi.SassError) as e:
            p.set_tile(3, 8, 128)
        assert e.value.code == 3
        # the plan stays usable after rejected calls
        fqt, fq, fq2 = p.compute(np.array([0, 1], np.uintp), np.ones((1, 3)), np.ones((1, 2)))
        assert np.isfinite(fqt).all()


def test_single_frame(native_lib):
    w = synth.small("all", "autocorrelate", seed=17, na=20, nf=1, nq=2, nm=3)
    check(w, "fp64", "fftw")


@pytest.mark.parametrize("nf", [128, 1024])
def test_coherent_fp32_error_at_length(native_lib, nf):
    """FP32 form at realistic trajectory lengths stays well inside 1e-3."""
    rng = np.random.default_rng(nf)
    w = synth.coherent_sqt(seed=21, na=500, nf=nf, nq=3, nm=8, box=20.0)
    check(w, "fp32", "fftw")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nf", [300, 600, 1500])
def test_coherent_block_fft_lengths(native_lib, precision, nf):
    # padded lengths 1,024, 2,048 and 4,096: the block-register FFT with 2, 4 and 8 blocks
    # of 512 points; 7 directions per shell leave warps without a series in a chunk's last round
    w = synth.small("all", "autocorrelate", seed=23, na=19, nf=nf, nq=3, nm=7)
    check(w, precision, "fftw")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_coherent_block_fft_direct_method_and_many_series(native_lib, precision):
    # the conjugate convention of the direct method, and enough series per shell for
    # several chunks and rounds
    w = synth.small("all", "autocorrelate", seed=24, na=11, nf=700, nq=2, nm=150)
    check(w, precision, "direct")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nf", [300, 600, 1500])
def test_incoherent_block_fft_lengths(native_lib, precision, nf):
    # the incoherent block-register FFT at padded lengths 1,024, 2,048 and 4,096; 5 directions
    # per shell leave warps without a series in each atom's last round
    w = synth.small("self", "autocorrelate", seed=25, na=9, nf=nf, nq=2, nm=5)
    check(w, precision, "fftw")


def test_incoherent_block_fft_direct_method_and_chunks(native_lib):
    # the direct method's conjugate, and enough atoms for several chunks per shell
    w = synth.small("self", "autocorrelate", seed=26, na=150, nf=520, nq=2, nm=3)
    check(w, "fp64", "direct")
    check(w, "fp32", "direct")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("dsp", ["square", "plain"])
@pytest.mark.parametrize("nf", [50, 100, 230, 500])
def test_coherent_square_plain_warp_kernel(native_lib, precision, dsp, nf):
    # warp per series with 2, 4, 8 and 16 frames per lane; 45 directions per shell give every
    # warp of a chunk a different number of series
    w = synth.small("all", dsp, seed=27, na=13, nf=nf, nq=3, nm=45)
    check(w, precision, "fftw")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("dsp", ["square", "plain"])
@pytest.mark.parametrize("nf", [40, 100, 300, 500])
def test_incoherent_square_plain_warp_kernel(native_lib, precision, dsp, nf):
    # the incoherent warp-per-series form: 4 atoms staged per barrier, 150 atoms give several
    # chunks per shell and a last group of fewer atoms; 7 directions leave warps idle
    w = synth.small("self", dsp, seed=28, na=150, nf=nf, nq=2, nm=7)
    check(w, precision, "fftw")


def test_out_of_memory_is_a_status(native_lib):
    # a trajectory far beyond HBM (16.7M atoms x 131,072 frames = 35 TB staged): the device
    # allocation fails first, staging returns SASS_ERR_OOM with a message, nothing is read
    # from the host buffer, and the process keeps working
    import ctypes
    with abi.Plan(1 << 24, 1 << 17, 1, "all", "autocorrelate", "fftw", "fp32") as p:
        dummy = np.zeros(3, dtype=np.float32)
        rc = p.lib.sass_stage_frames(p._h, dummy.ctypes.data_as(ctypes.c_void_p), 0)
        assert rc == 2, rc
        assert p.lib.sass_plan_error(p._h)
    w = synth.small("all", "autocorrelate", seed=18, na=20, nf=9, nq=2, nm=3)
    check(w, "fp64", "fftw")


@pytest.mark.parametrize("scattering", ["all", "self"])
def test_repeated_calls_follow_new_inputs(native_lib, scattering):
    # A call with the same q-vector layout as the previous one reuses the engine's
    # descriptors; new class factors, new sub-vector values, a new staging or new classes
    # must still reach the result. Each call is compared bit for bit with a fresh plan.
    import dataclasses

    w1 = synth.small(scattering, "autocorrelate", seed=61, na=200, nf=30, nq=4, nm=12)
    w2 = dataclasses.replace(w1, class_factors=w1.class_factors * 1.5 + 0.25)
    w3 = dataclasses.replace(w1, directions=synth.sphere_directions(w1.nm, 62))
    w4 = dataclasses.replace(synth.small(scattering, "autocorrelate", seed=63, na=200, nf=30, nq=4, nm=12),
                             shells=w1.shells, directions=w1.directions, class_factors=w1.class_factors,
                             atom_class=w1.atom_class)
    w5 = dataclasses.replace(w4, atom_class=np.roll(w4.atom_class, 7))

    def fresh(w, precision):
        return abi.compute_workload(w, precision)

    for precision in ("fp64", "fp32"):
        with abi.Plan(w1.na, w1.nf, len(w1.class_names), scattering, "autocorrelate", "fftw", precision) as p:
            p.stage(w1.coords)
            p.set_classes(w1.atom_class)
            for w, restage, reclass in ((w1, False, False), (w1, False, False), (w2, False, False),
                                        (w3, False, False), (w4, True, False), (w5, False, True)):
                if restage:
                    p.stage(w.coords)
                if reclass:
                    p.set_classes(w.atom_class)
                got = p.compute(w.sub_offsets(), w.subvectors(), np.ascontiguousarray(w.class_factors))
                for a, b in zip(got, fresh(w, precision)):
                    np.testing.assert_array_equal(a, b)
