"""sass_correlate_noalloc: the allocation-free entry point for callers that must not
allocate GPU memory while they run (a fixed, pre-reserved device memory budget, code
inside a memory-pool callback, services that cannot risk out-of-memory mid-run).

It must give the same S(q,t), fq and fq2 as the allocating path (sass_compute) on the
same amplitudes, call after call, although every call reuses the same fixed device
array. The cases cover every transform form the fixed array serves (padded lengths 8
to 8,192), one q with 128 partial slots and 128 q with one slot each, and calls whose
NF changes from one call to the next, which rebuilds the array's FFT tables. Collected
last on purpose, so that a run stopping at the first failure has run every other test
already.
"""
import ctypes

import numpy as np
import pytest

import oracle
from sassena_gb300 import abi, synth

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 parity bar used by the other GPU tests


def _reference(w, method):
    """Amplitudes of w and the allocating path's (fqt, fq, fq2) computed from them."""
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


class _Case:
    """Device inputs and outputs of one workload, and the allocating path's results."""

    def __init__(self, w, method):
        import torch

        self.w, self.method = w, method
        amp, self.ref = _reference(w, method)
        self.d_amp = torch.from_numpy(np.stack([amp.real, amp.imag], axis=-1).copy()).cuda()
        self.d_offs = torch.from_numpy(w.sub_offsets().astype(np.int64)).cuda()
        self.d_fqt = torch.empty((w.nq, w.nf, 2), dtype=torch.float64, device="cuda")
        self.d_fq = torch.empty((w.nq, 2), dtype=torch.float64, device="cuda")
        self.d_fq2 = torch.empty((w.nq, 2), dtype=torch.float64, device="cuda")

    def call(self):
        """One call of the entry point; returns (fqt, fq, fq2) as complex host arrays."""
        import torch

        for t in (self.d_fqt, self.d_fq, self.d_fq2):
            t.fill_(float("nan"))
        lib = abi.load()
        stream = torch.cuda.current_stream().cuda_stream
        w = self.w
        rc = lib.sass_correlate_noalloc(0, ctypes.c_void_p(stream), self.d_amp.data_ptr(), w.nf, w.nq,
                                        self.d_offs.data_ptr(), abi.METHOD[self.method],
                                        self.d_fqt.data_ptr(), self.d_fq.data_ptr(), self.d_fq2.data_ptr())
        assert rc == 0, abi.STATUS.get(rc, rc)
        torch.cuda.synchronize()
        c = lambda t: (lambda a: a[..., 0] + 1j * a[..., 1])(t.cpu().numpy())  # noqa: E731
        return c(self.d_fqt), c(self.d_fq), c(self.d_fq2)

    def check(self, out, label):
        fqt, fq, fq2 = out
        fqt_ref, fq_ref, fq2_ref = self.ref
        err_t = (np.abs(fqt - fqt_ref).max(axis=1) / np.abs(fqt_ref[:, 0])).max()
        assert err_t <= TOL, "%s: fqt rel err %.3e" % (label, err_t)
        assert _rel(fq, fq_ref) <= TOL, label
        assert _rel(fq2, fq2_ref) <= TOL, label


def _workload(nf, nq, nm, seed, na=24):
    return synth.small("all", "autocorrelate", seed=seed, na=na, nf=nf, nq=nq, nm=nm)


@pytest.mark.parametrize("method", ["fftw", "direct"])
def test_noalloc_matches_allocating_path_and_oracle_twice(native_lib, method):
    w = _workload(57, 3, 19, seed=41, na=130)
    case = _Case(w, method)
    ref_fqt, _, _ = oracle.all_vectors(w.coords, w.sub_offsets(), w.subvectors(), w.factors(), 0,
                                       abi.METHOD[method], nthreads=4)
    ref = ref_fqt[..., 0] + 1j * ref_fqt[..., 1]
    for call in range(2):
        out = case.call()
        case.check(out, "call %d" % call)
        err = (np.abs(out[0] - ref).max(axis=1) / np.abs(ref[:, 0])).max()
        assert err <= TOL, "call %d: fqt rel err vs oracle %.3e" % (call, err)


# NF 3, 57, 1,000 and 4,096 pad to 8, 128, 2,048 and 8,192 points: the shared-memory warp
# transform, the register-resident warp transform, the block-register transform and the
# CTA transform at the array's size limit. One q uses all 128 partial slots; 128 q use one
# slot each and fill every finalisation entry.
@pytest.mark.parametrize("nf", [3, 57, 1000, 4096])
@pytest.mark.parametrize("nq,nm", [(1, 300), (128, 2)])
def test_noalloc_transform_forms_and_slot_layouts(native_lib, nf, nq, nm):
    case = _Case(_workload(nf, nq, nm, seed=nf + nq), "fftw")
    for call in range(2):
        case.check(case.call(), "nf %d nq %d call %d" % (nf, nq, call))


def test_noalloc_nf_changes_between_calls(native_lib):
    """Alternating NF rebuilds the tables in the array on every change; a repeated NF
    reuses them. Each call must still equal the allocating path."""
    cases = {nf: _Case(_workload(nf, 4, 5, seed=7 * nf), "fftw") for nf in (57, 1000, 4096, 3)}
    for i, nf in enumerate((57, 1000, 57, 57, 4096, 3, 1000, 1000, 57)):
        cases[nf].check(cases[nf].call(), "call %d (nf %d)" % (i, nf))


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
