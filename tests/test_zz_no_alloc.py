"""sass_correlate_noalloc: the allocation-free entry point for callers that must not
allocate GPU memory while they run (a fixed, pre-reserved device memory budget, code
inside a memory-pool callback, services that cannot risk out-of-memory mid-run).

It must give the same S(q,t), fq and fq2 as the allocating path (sass_compute) on the
same amplitudes, call after call, although every call reuses the same fixed device
array. Collected last on purpose, so that a run stopping at the first failure has run
every other test already.
"""
import ctypes

import numpy as np
import pytest

from sassena_gb300 import abi, synth

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 parity bar used by the other GPU tests


def _reference(w, method):
    offs = w.sub_offsets()
    sv = w.subvectors()
    shell = np.repeat(np.arange(w.nq), w.nm).astype(np.int32)
    with abi.Plan(w.na, w.nf, len(w.class_names), "all", "autocorrelate", method, "fp64") as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        fqt, fq, fq2 = p.compute(offs, sv, w.class_factors)
        amp = p.amplitudes(sv, shell, w.class_factors)
    return amp, (fqt, fq, fq2)


def _rel(x, ref):
    return np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300)


@pytest.mark.parametrize("method", ["fftw", "direct"])
def test_noalloc_matches_allocating_path_twice(native_lib, method):
    import torch

    w = synth.small("all", "autocorrelate", seed=41, na=130, nf=57, nq=3, nm=19)
    amp, (fqt_ref, fq_ref, fq2_ref) = _reference(w, method)
    d_amp = torch.from_numpy(np.stack([amp.real, amp.imag], axis=-1).copy()).cuda()
    d_offs = torch.from_numpy(w.sub_offsets().astype(np.int64)).cuda()
    d_fqt = torch.empty((w.nq, w.nf, 2), dtype=torch.float64, device="cuda")
    d_fq = torch.empty((w.nq, 2), dtype=torch.float64, device="cuda")
    d_fq2 = torch.empty((w.nq, 2), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    lib = abi.load()
    for call in range(2):
        d_fqt.fill_(float("nan"))
        d_fq.fill_(float("nan"))
        d_fq2.fill_(float("nan"))
        rc = lib.sass_correlate_noalloc(0, ctypes.c_void_p(stream), d_amp.data_ptr(), w.nf, w.nq,
                                        d_offs.data_ptr(), abi.METHOD[method], d_fqt.data_ptr(),
                                        d_fq.data_ptr(), d_fq2.data_ptr())
        assert rc == 0, abi.STATUS.get(rc, rc)
        torch.cuda.synchronize()
        fqt = d_fqt.cpu().numpy()
        fq = d_fq.cpu().numpy()
        fq2 = d_fq2.cpu().numpy()
        fqt = fqt[..., 0] + 1j * fqt[..., 1]
        den = np.abs(fqt_ref[:, 0])
        err_t = (np.abs(fqt - fqt_ref).max(axis=1) / den).max()
        assert err_t <= TOL, "call %d: fqt rel err %.3e" % (call, err_t)
        assert _rel(fq[:, 0] + 1j * fq[:, 1], fq_ref) <= TOL, call
        assert _rel(fq2[:, 0] + 1j * fq2[:, 1], fq2_ref) <= TOL, call


def test_noalloc_rejects_sizes_beyond_its_array(native_lib):
    import torch

    lib = abi.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    offs = torch.zeros(300, dtype=torch.int64, device="cuda")
    p = buf.data_ptr()
    # NF = 5000 needs a padded length of 16384 > 8192
    assert lib.sass_correlate_noalloc(0, None, p, 5000, 1, offs.data_ptr(), 0, p, p, p) == 3
    # 200 q-vectors > 128
    assert lib.sass_correlate_noalloc(0, None, p, 10, 200, offs.data_ptr(), 0, p, p, p) == 3
    assert lib.sass_correlate_noalloc(0, None, p, 10, 1, None, 0, p, p, p) == 1
