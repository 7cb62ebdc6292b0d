"""GPU parity of the FP32 shell-recurrence kernel (shells along one direction set).

The reference's sphere/file orientation types give every |q| the same direction set
(abstract_vectors_scatter_device.cpp:112-130) and linear scans give equally spaced |q|;
the library then evaluates runs of shells with a three-term recurrence. Every case is
checked against the FP64 oracle with the FP32 form's bar (1e-3, error metric
max_t |S - S_ref| / |S_ref(q,0)|), and the schedule shows which kernel ran.
"""
import dataclasses

import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

from helpers import cplx, rel_err_sqt, rel_err_vec

pytestmark = pytest.mark.gpu

DSP_ID = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD_ID = {"fftw": 0, "direct": 1}
TOL = 1e-3


def reference(w, method="fftw"):
    return oracle.all_vectors(w.coords, w.sub_offsets(), w.subvectors(), w.factors(),
                              DSP_ID[w.dsp], METHOD_ID[method], nthreads=8)


def errors(got, ref):
    fqt, fq, fq2 = got
    r_fqt, r_fq, r_fq2 = ref
    return (rel_err_sqt(fqt, r_fqt).max(), rel_err_vec(fq, cplx(r_fq)),
            rel_err_vec(fq2, cplx(r_fq2)))


def assert_close(got, ref, tol=TOL):
    e = errors(got, ref)
    assert max(e) <= tol, "rel err fqt/fq/fq2 = %.3e/%.3e/%.3e > %.1e" % (e + (tol,))
    return e


def with_shells(w, shells):
    shells = np.asarray(shells, dtype=np.float64)
    cf = np.tile(w.class_factors[0], (len(shells), 1)) * (1.0 + 0.05 * np.arange(len(shells)))[:, None]
    return dataclasses.replace(w, shells=shells, class_factors=cf)


@pytest.fixture(scope="module")
def linear_case():
    w = synth.small("all", "autocorrelate", seed=31, na=301, nf=40, nq=17, nm=45, box=20.0)
    return w, reference(w)


@pytest.mark.parametrize("k", [4, 8, 12, 16, 20, 24, 32])
def test_every_width(native_lib, linear_case, k):
    w, ref = linear_case
    sch = {}
    got = abi.compute_workload(w, "fp32", recurrence=k, schedule=sch)
    assert sch["rec_shells_per_lane"] == k and sch["rec_shells"] == w.nq and sch["direct_tiles"] == 0
    e = assert_close(got, ref)
    print("K=%d rel err %.2e %.2e %.2e" % ((k,) + e))


def test_long_run_several_groups(native_lib):
    # 45 equally spaced shells: several groups per lane at every width
    w = synth.small("all", "autocorrelate", seed=38, na=211, nf=24, nq=45, nm=21, box=18.0)
    ref = reference(w)
    for k in (8, 20, 32):
        sch = {}
        got = abi.compute_workload(w, "fp32", recurrence=k, schedule=sch)
        assert sch["rec_shells"] == 45 and sch["rec_shells_per_lane"] == k
        assert_close(got, ref)


def test_automatic_width_and_off(native_lib, linear_case):
    w, ref = linear_case
    sch = {}
    on = abi.compute_workload(w, "fp32", schedule=sch)
    assert sch["rec_shells"] == w.nq and sch["rec_shells_per_lane"] > 0
    sch_off = {}
    off = abi.compute_workload(w, "fp32", recurrence=-1, schedule=sch_off)
    assert sch_off["rec_tiles"] == 0 and sch_off["direct_tiles"] > 0
    assert_close(on, ref)
    assert_close(off, ref)
    # FP64 plans never take the FP32 recurrence
    sch64 = {}
    abi.compute_workload(w, "fp64", schedule=sch64)
    assert sch64["rec_tiles"] == 0


@pytest.mark.parametrize("dsp,method", [("square", "fftw"), ("plain", "fftw"),
                                        ("autocorrelate", "direct")])
def test_dsp_variants(native_lib, dsp, method):
    w = synth.small("all", dsp, seed=32, na=97, nf=30, nq=6, nm=33)
    sch = {}
    got = abi.compute_workload(w, "fp32", method=method, schedule=sch)
    assert sch["rec_shells"] == 6
    assert_close(got, reference(w, method))


def test_mixed_runs_and_zero_shell(native_lib):
    w = synth.small("all", "autocorrelate", seed=33, na=130, nf=26, nq=10, nm=20)
    # runs: [0.3..0.9] (4 shells), 1.37 / 2.0 / 2.1 alone, [3.5..3.7] (3 shells)
    w = with_shells(w, [0.3, 0.5, 0.7, 0.9, 1.37, 2.0, 2.1, 3.5, 3.6, 3.7])
    sch = {}
    got = abi.compute_workload(w, "fp32", schedule=sch)
    assert sch["rec_shells"] == 7 and sch["direct_tiles"] > 0
    assert_close(got, reference(w))
    # |q| = 0 opens a run (all its sub-vectors are zero multiples of the base set)
    w0 = with_shells(w, np.linspace(0.0, 1.5, 7))
    sch = {}
    got = abi.compute_workload(w0, "fp32", schedule=sch)
    assert sch["rec_shells"] == 7
    assert_close(got, reference(w0))


def test_float_rounded_scan(native_lib):
    # |q| computed in float32 as a linear scan would be: still one run
    w = synth.small("all", "autocorrelate", seed=34, na=77, nf=20, nq=12, nm=17)
    q = (np.float32(0.1) + np.arange(12, dtype=np.float32) * np.float32(0.23)).astype(np.float64)
    w = with_shells(w, q)
    sch = {}
    got = abi.compute_workload(w, "fp32", schedule=sch)
    assert sch["rec_shells"] == 12
    assert_close(got, reference(w))


def test_atom_splits(native_lib):
    w = synth.small("all", "autocorrelate", seed=35, na=1000, nf=24, nq=8, nm=40, box=25.0)
    ref = reference(w)
    for splits in (3, 5, 8):
        sch = {}
        got = abi.compute_workload(w, "fp32", tile=(0, 0, 0, splits), schedule=sch)
        assert sch["rec_shells"] == 8 and sch["atom_splits"] > 1
        assert_close(got, ref)


def test_class_layouts(native_lib):
    base = synth.small("all", "autocorrelate", seed=36, na=203, nf=22, nq=5, nm=31)
    rng = np.random.default_rng(9)
    # six classes, two of them without atoms, segments not multiples of 32
    cls = rng.choice([0, 2, 3, 5], size=base.na, p=[0.5, 0.3, 0.15, 0.05]).astype(np.int32)
    b = np.array([-3.739, 6.646, 9.36, 5.803, 2.847, 4.1])
    cf = np.tile(b, (base.nq, 1)) * (1.0 + 0.1 * np.arange(base.nq))[:, None]
    w6 = dataclasses.replace(base, atom_class=cls, class_names=list("ABCDEF"), class_factors=cf)
    # one class
    w1 = dataclasses.replace(base, atom_class=np.zeros(base.na, np.int32), class_names=["A"],
                             class_factors=np.full((base.nq, 1), 2.5))
    for w in (w6, w1):
        sch = {}
        got = abi.compute_workload(w, "fp32", schedule=sch)
        assert sch["rec_shells"] == base.nq
        assert_close(got, reference(w))


def test_general_subvectors_use_direct_kernel(native_lib):
    w = synth.small("all", "autocorrelate", seed=37, na=90, nf=18, nq=4, nm=12)
    rng = np.random.default_rng(3)
    sv = rng.normal(size=(w.nq * w.nm, 3))
    offs = w.sub_offsets()
    with abi.Plan(w.na, w.nf, len(w.class_names), precision="fp32") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        got = p.compute(offs, sv, w.class_factors)
        sch = p.schedule()
    assert sch["rec_tiles"] == 0
    ref = oracle.all_vectors(w.coords, offs, sv, w.factors(), 0, 0, nthreads=8)
    assert_close(got, ref)


def test_batch_uses_recurrence(native_lib):
    ws = [synth.small("all", "autocorrelate", seed=40 + i, na=na, nf=nf, nq=nq, nm=nm)
          for i, (na, nf, nq, nm) in enumerate([(150, 20, 5, 33), (61, 31, 3, 8), (400, 16, 9, 70)])]
    with abi.Batch(ws, precision="fp32") as b:
        b.run()
        b.sync()
        sch = b.schedule()
        assert sch["rec_shells"] == 5 + 3 + 9
        for i, w in enumerate(ws):
            assert_close(b.results(i), reference(w))
        # forcing the recurrence off gives the same results within the FP32 bar
        b.set_recurrence(-1)
        b.run()
        b.sync()
        assert b.schedule()["rec_tiles"] == 0
        for i, w in enumerate(ws):
            assert_close(b.results(i), reference(w))


def test_autotune_considers_recurrence(native_lib):
    w = synth.small("all", "autocorrelate", seed=45, na=500, nf=32, nq=12, nm=64)
    with abi.Plan(w.na, w.nf, len(w.class_names), precision="fp32") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        p.autotune(w.sub_offsets(), w.subvectors(), w.class_factors, repeats=1)
        got = p.compute(w.sub_offsets(), w.subvectors(), w.class_factors)
    assert_close(got, reference(w))


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_split_slices_never_empty(native_lib, precision):
    # 10,000 atoms, one shell of 32 directions, 160 frames: few tiles, so the automatic
    # atom split is large and does not divide the stage count evenly. Every slice must
    # be written, also after the plan's partial buffer held other values.
    rng = np.random.default_rng(46)
    na, nf = 10000, 160
    w = synth.coherent_sqt(seed=46, na=na, nf=nf, nq=1, nm=32, qmin=1.1, qmax=1.1)
    with abi.Plan(na, nf, len(w.class_names), precision=precision) as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        dirs = rng.normal(size=(128, 3))
        p.compute(np.array([0, 64, 128], np.uintp), dirs, w.class_factors[[0, 0]])  # dirties buffers
        got = p.compute(w.sub_offsets(), w.subvectors(), w.class_factors)
        sch = p.schedule()
    assert sch["atom_splits"] > 1
    ref = reference(w)
    assert_close(got, ref, 1e-12 if precision == "fp64" else TOL)


def test_restaging_refreshes_the_class_sorted_copy(native_lib):
    # Once the class-sorted copy exists, each staging fills it in the same pass as the padded
    # frames, from host memory read in place (pageable or pinned) or from device memory; new
    # classes rebuild it. Every staging form gives the same bits, and each result matches
    # the oracle on the frames and classes of that moment.
    import torch

    w1 = synth.small("all", "autocorrelate", seed=47, na=300, nf=40, nq=6, nm=24)
    w2 = dataclasses.replace(synth.small("all", "autocorrelate", seed=48, na=300, nf=40, nq=6, nm=24),
                             shells=w1.shells, directions=w1.directions, class_factors=w1.class_factors)
    w2b = dataclasses.replace(w2, atom_class=w1.atom_class)
    args = (w1.sub_offsets(), w1.subvectors(), w1.class_factors)
    lib = abi.load()
    with abi.Plan(w1.na, w1.nf, len(w1.class_names), precision="fp32") as p:
        p.stage(w1.coords)
        p.set_classes(w1.atom_class)
        assert_close(p.compute(*args), reference(w1))
        assert p.schedule()["rec_tiles"] > 0
        p.stage(w2.coords)  # pageable numpy memory; classes of w1
        pageable = p.compute(*args)
        assert_close(pageable, reference(w2b))
        hp = lib.sass_host_alloc(w2.coords.nbytes)
        try:
            pinned = np.ctypeslib.as_array((np.ctypeslib.ctypes.c_float * w2.coords.size).from_address(hp))
            pinned[:] = w2.coords.reshape(-1)
            p.stage(pinned.reshape(w2.coords.shape))
            for a, b in zip(p.compute(*args), pageable):
                np.testing.assert_array_equal(a, b)
        finally:
            lib.sass_host_free(hp)
        d = torch.from_numpy(w2.coords).cuda()
        p.stage(d.data_ptr(), on_device=True)
        for a, b in zip(p.compute(*args), pageable):
            np.testing.assert_array_equal(a, b)
        p.set_classes(w2.atom_class)  # new classes: a new slot map
        assert_close(p.compute(*args), reference(w2))
        p.stage(w1.coords)
        p.set_classes(w1.atom_class)
        assert_close(p.compute(*args), reference(w1))


def test_staging_of_pageable_memory_locked_elsewhere(native_lib):
    # Pageable host memory is page-locked for the staging call and read through its device
    # mapping. Where part of the buffer is already locked by someone else, locking fails and
    # the device reads the pages in place: the same bits either way, and the caller's own
    # registration is left as it was.
    import torch

    import os

    w = synth.small("all", "autocorrelate", seed=49, na=300, nf=400, nq=6, nm=24)
    args = (w.sub_offsets(), w.subvectors(), w.class_factors)
    cr = torch.cuda.cudart()
    with abi.Plan(w.na, w.nf, len(w.class_names), precision="fp32") as p:
        p.set_classes(w.atom_class)
        p.stage(w.coords)
        first = p.compute(*args)
        assert_close(first, reference(w))
        p.stage(w.coords)  # the same buffer again
        for a, b in zip(p.compute(*args), first):
            np.testing.assert_array_equal(a, b)
        # whole pages inside the buffer's middle half (1.4 MB of coordinates)
        page = os.sysconf("SC_PAGE_SIZE")
        lo = -(-(w.coords.ctypes.data + w.coords.nbytes // 4) // page) * page
        hi = (w.coords.ctypes.data + 3 * w.coords.nbytes // 4) // page * page
        assert hi > lo
        assert int(cr.cudaHostRegister(lo, hi - lo, 0)) == 0
        try:
            p.stage(w.coords)
            for a, b in zip(p.compute(*args), first):
                np.testing.assert_array_equal(a, b)
        finally:
            assert int(cr.cudaHostUnregister(lo)) == 0


def test_prefetched_frames_stage_the_same_bits(native_lib):
    # sass_prefetch_frames has the next compute copy a buffer ahead on the plan's copy stream
    # while its kernels run; the next staging of that buffer converts from the copy. Pageable
    # and pinned buffers, a copy discarded by staging another buffer, and a request replaced
    # by a second one (staged with no compute in between) all give the bits of a plain
    # staging.
    w1 = synth.small("all", "autocorrelate", seed=51, na=300, nf=40, nq=6, nm=24)
    w2 = dataclasses.replace(synth.small("all", "autocorrelate", seed=52, na=300, nf=40, nq=6, nm=24),
                             atom_class=w1.atom_class)
    args = (w1.sub_offsets(), w1.subvectors(), w1.class_factors)
    lib = abi.load()
    with abi.Plan(w1.na, w1.nf, len(w1.class_names), precision="fp32") as p:
        p.set_classes(w1.atom_class)
        p.stage(w1.coords)
        plain1 = p.compute(*args)
        assert_close(plain1, reference(w1))
        p.stage(w2.coords)
        plain2 = p.compute(*args)

        def same(got, want):
            for a, b in zip(got, want):
                np.testing.assert_array_equal(a, b)

        p.prefetch(w1.coords)  # pageable numpy memory
        p.compute(*args)  # work the copy overlaps (frames of w2)
        p.stage(w1.coords)
        same(p.compute(*args), plain1)
        p.prefetch(w2.coords)  # copied during the compute, then discarded: another buffer is staged
        p.compute(*args)
        p.stage(w1.coords)
        same(p.compute(*args), plain1)
        p.prefetch(w1.coords)  # replaced by the second prefetch
        p.prefetch(w2.coords)
        p.stage(w2.coords)
        same(p.compute(*args), plain2)
        hp = lib.sass_host_alloc(w1.coords.nbytes)
        try:
            pinned = np.ctypeslib.as_array((np.ctypeslib.ctypes.c_float * w1.coords.size)
                                           .from_address(hp)).reshape(w1.coords.shape)
            pinned[...] = w1.coords
            p.prefetch(pinned)
            p.compute(*args)
            p.stage(pinned)
            same(p.compute(*args), plain1)
            p.prefetch(pinned)  # pending when the plan is destroyed
            arg_error = {name: code for code, name in abi.STATUS.items()}["SASS_ERR_ARG"]
            assert lib.sass_prefetch_frames(p._h, None) == arg_error
            assert lib.sass_prefetch_frames(None, pinned.ctypes.data) == arg_error
        finally:
            p.close()
            lib.sass_host_free(hp)
