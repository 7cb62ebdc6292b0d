"""ctypes binding of the C ABI in include/sassena_gb300.h.

The library is loaded from the package's in-tree build directory. There is no
fallback: if the shared library is missing or a CUDA device is absent, the calls
raise. Numpy arrays are passed as plain pointers; results come back as numpy arrays.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libsassena_gb300.so")

SASS_OK = 0
STATUS = {0: "SASS_OK", 1: "SASS_ERR_ARG", 2: "SASS_ERR_OOM", 3: "SASS_ERR_UNSUPPORTED",
          4: "SASS_ERR_CUDA", 5: "SASS_ERR_TIMEOUT", 6: "SASS_ERR_STATE"}

SCATTERING = {"all": 0, "self": 1}
DSP = {"autocorrelate": 0, "square": 1, "plain": 2}
METHOD = {"fftw": 0, "direct": 1}
PRECISION = {"fp64": 0, "fp32": 1}

# Every symbol the header declares (checked by the CPU tests).
EXPORTS = [
    "sass_plan_create", "sass_plan_destroy", "sass_plan_error", "sass_status_name",
    "sass_stage_frames", "sass_prefetch_frames", "sass_set_atom_classes", "sass_compute", "sass_amplitudes",
    "sass_last_timing", "sass_set_phase_tile", "sass_frame_center", "sass_host_alloc",
    "sass_host_free", "sass_probe_pipes", "sass_probe_fp64", "sass_correlate_noalloc", "sass_version",
    "sass_autotune", "sass_batch_create", "sass_batch_autotune", "sass_batch_run",
    "sass_batch_sync", "sass_batch_results", "sass_batch_timing", "sass_batch_info",
    "sass_batch_error", "sass_batch_destroy", "sass_batch_set_tile",
    "sass_mlp_create", "sass_mlp_destroy", "sass_mlp_error", "sass_mlp_param_count",
    "sass_mlp_set_scaling", "sass_mlp_get_params", "sass_mlp_set_params", "sass_mlp_gradient",
    "sass_mlp_train", "sass_mlp_predict", "sass_mlp_sphere_mean", "sass_compute_cv",
    "sass_set_shell_recurrence", "sass_plan_schedule", "sass_batch_set_shell_recurrence",
    "sass_batch_schedule", "sass_set_phase_poly", "sass_batch_set_phase_poly",
    "sass_multipole_compute", "sass_stage_frames_prepass",
]


class SassError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class PlanDesc(ctypes.Structure):
    _fields_ = [("scattering", ctypes.c_int), ("dsp_type", ctypes.c_int),
                ("dsp_method", ctypes.c_int), ("precision", ctypes.c_int),
                ("na", ctypes.c_size_t), ("nf", ctypes.c_size_t), ("nclass", ctypes.c_size_t),
                ("device", ctypes.c_int), ("stream", ctypes.c_void_p),
                ("amplitude_budget_bytes", ctypes.c_size_t)]


class System(ctypes.Structure):
    _fields_ = [("na", ctypes.c_size_t), ("nf", ctypes.c_size_t), ("nclass", ctypes.c_size_t),
                ("coords", ctypes.c_void_p), ("atom_class", ctypes.c_void_p),
                ("nq", ctypes.c_size_t), ("sub_offsets", ctypes.c_void_p),
                ("subvectors", ctypes.c_void_p), ("class_factors", ctypes.c_void_p)]


STEP = {"center": 0, "fittrans": 1, "fitrottrans": 2, "fitrot": 3, "motion": 4}


class PrepassStep(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("reserved", ctypes.c_int),
                ("selection", ctypes.c_void_p), ("nselection", ctypes.c_size_t),
                ("reference_selection", ctypes.c_void_p), ("nreference", ctypes.c_size_t),
                ("reference", ctypes.c_void_p),
                ("fit_target", ctypes.c_void_p), ("fit_source", ctypes.c_void_p),
                ("nfit", ctypes.c_size_t), ("translations", ctypes.c_void_p)]


class Timing(ctypes.Structure):
    _fields_ = [("phase_ms", ctypes.c_double), ("corr_ms", ctypes.c_double),
                ("finalize_ms", ctypes.c_double), ("h2d_ms", ctypes.c_double),
                ("d2h_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_uint64), ("phase_launches", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Schedule(ctypes.Structure):
    _fields_ = [("terms", ctypes.c_double), ("direct_tiles", ctypes.c_uint64),
                ("rec_tiles", ctypes.c_uint64), ("rec_shells", ctypes.c_uint64),
                ("rec_shells_per_lane", ctypes.c_int), ("q_per_lane", ctypes.c_int),
                ("warps", ctypes.c_int), ("atoms", ctypes.c_int), ("atom_splits", ctypes.c_int),
                ("poly_pairs", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_sz = ctypes.c_size_t


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("sassena_gb300 native library not built: %s (run __graft_entry__.build())"
                      % path)
    L = ctypes.CDLL(path)
    L.sass_plan_create.argtypes = [ctypes.POINTER(PlanDesc), ctypes.POINTER(_vp)]
    L.sass_plan_destroy.argtypes = [_vp]
    L.sass_plan_destroy.restype = None
    L.sass_plan_error.argtypes = [_vp]
    L.sass_plan_error.restype = ctypes.c_char_p
    L.sass_status_name.argtypes = [ctypes.c_int]
    L.sass_status_name.restype = ctypes.c_char_p
    L.sass_stage_frames.argtypes = [_vp, _vp, ctypes.c_int]
    L.sass_prefetch_frames.argtypes = [_vp, _vp]
    L.sass_stage_frames_prepass.argtypes = [_vp, _vp, ctypes.c_size_t, _vp, ctypes.POINTER(PrepassStep),
                                            ctypes.c_size_t, _vp, _vp]
    L.sass_set_atom_classes.argtypes = [_vp, _vp, ctypes.c_int]
    L.sass_compute.argtypes = [_vp, _sz, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int]
    L.sass_amplitudes.argtypes = [_vp, _sz, _vp, _vp, _sz, _vp, _vp]
    L.sass_last_timing.argtypes = [_vp, ctypes.POINTER(Timing)]
    L.sass_set_phase_tile.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.sass_frame_center.argtypes = [_vp, _dp]
    L.sass_host_alloc.argtypes = [_sz]
    L.sass_host_alloc.restype = _vp
    L.sass_host_free.argtypes = [_vp]
    L.sass_host_free.restype = None
    L.sass_version.restype = ctypes.c_char_p
    L.sass_probe_pipes.argtypes = [ctypes.c_int, _dp, _dp]
    L.sass_probe_fp64.argtypes = [ctypes.c_int, _dp]
    _ip = ctypes.POINTER(ctypes.c_int)
    L.sass_autotune.argtypes = [_vp, _sz, _vp, _vp, _vp, ctypes.c_int, _ip, _ip, _ip, _ip]
    L.sass_batch_create.argtypes = [ctypes.POINTER(PlanDesc), _sz, ctypes.POINTER(System),
                                    ctypes.POINTER(_vp)]
    L.sass_batch_autotune.argtypes = [_vp, ctypes.c_int, _ip, _ip, _ip, _ip, _dp]
    L.sass_batch_run.argtypes = [_vp]
    L.sass_batch_set_tile.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.sass_batch_sync.argtypes = [_vp]
    L.sass_batch_results.argtypes = [_vp, _sz, _vp, _vp, _vp]
    L.sass_batch_timing.argtypes = [_vp, ctypes.POINTER(Timing)]
    L.sass_batch_info.argtypes = [_vp, _dp, ctypes.POINTER(ctypes.c_uint64), _ip, _ip, _ip, _ip]
    L.sass_batch_error.argtypes = [_vp]
    L.sass_batch_error.restype = ctypes.c_char_p
    L.sass_batch_destroy.argtypes = [_vp]
    L.sass_batch_destroy.restype = None
    L.sass_mlp_create.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.sass_mlp_destroy.argtypes = [_vp]
    L.sass_mlp_destroy.restype = None
    L.sass_mlp_error.argtypes = [_vp]
    L.sass_mlp_error.restype = ctypes.c_char_p
    L.sass_mlp_set_scaling.argtypes = [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double]
    L.sass_mlp_get_params.argtypes = [_vp, _vp, _vp]
    L.sass_mlp_set_params.argtypes = [_vp, _vp]
    L.sass_mlp_gradient.argtypes = [_vp, _vp, _vp, _sz, _vp, _dp]
    L.sass_mlp_train.argtypes = [_vp, _vp, _vp, _sz, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 _dp]
    L.sass_mlp_predict.argtypes = [_vp, _vp, _sz, _vp]
    L.sass_mlp_sphere_mean.argtypes = [_vp, _vp, _sz, _sz, _vp]
    L.sass_compute_cv.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _vp, _sz, _vp, _vp, _vp, _vp, _vp]
    L.sass_correlate_noalloc.argtypes = [ctypes.c_int, _vp, _vp, _sz, _sz, _vp, ctypes.c_int, _vp,
                                         _vp, _vp]
    L.sass_set_shell_recurrence.argtypes = [_vp, ctypes.c_int]
    L.sass_plan_schedule.argtypes = [_vp, ctypes.POINTER(Schedule)]
    L.sass_batch_set_shell_recurrence.argtypes = [_vp, ctypes.c_int]
    L.sass_batch_schedule.argtypes = [_vp, ctypes.POINTER(Schedule)]
    L.sass_set_phase_poly.argtypes = [_vp, ctypes.c_int]
    L.sass_multipole_compute.argtypes = [_vp, ctypes.c_int, _sz, _vp, _vp, _sz, _vp, _vp, _vp, _vp,
                                         _vp]
    L.sass_batch_set_phase_poly.argtypes = [_vp, ctypes.c_int]
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(_vp) if isinstance(a, np.ndarray) else _vp(a)


class Plan:
    """One scatter-device computation (a sass_plan) for fixed NA, NF and settings."""

    def __init__(self, na, nf, nclass, scattering="all", dsp="autocorrelate", method="fftw",
                 precision="fp64", device=0, stream=None, amplitude_budget_bytes=0):
        self.lib = load()
        self.na, self.nf, self.nclass = int(na), int(nf), int(nclass)
        d = PlanDesc(SCATTERING[scattering], DSP[dsp], METHOD[method], PRECISION[precision],
                     self.na, self.nf, self.nclass, device, stream or 0, amplitude_budget_bytes)
        h = _vp()
        rc = self.lib.sass_plan_create(ctypes.byref(d), ctypes.byref(h))
        self._h = h
        if rc != SASS_OK:
            msg = self.error()
            self.close()
            raise SassError(rc, msg)

    def error(self):
        if not self._h:
            return ""
        return self.lib.sass_plan_error(self._h).decode()

    def _check(self, rc):
        if rc != SASS_OK:
            raise SassError(rc, self.error())

    def close(self):
        if getattr(self, "_h", None):
            self.lib.sass_plan_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def stage(self, coords, on_device=False):
        """coords: float32 [nf, na, 3] numpy array, or a device pointer (int)."""
        if on_device:
            return self._check(self.lib.sass_stage_frames(self._h, _vp(coords), 1))
        c = np.ascontiguousarray(coords, dtype=np.float32)
        if c.shape != (self.nf, self.na, 3):
            raise ValueError("coords must be [nf, na, 3]")
        self._check(self.lib.sass_stage_frames(self._h, _ptr(c), 0))

    def prefetch(self, coords):
        """Have the next compute() copy these host frames ahead for the next stage() of the same
        array (sass_prefetch_frames). The array is kept alive here and must not change until
        that stage()."""
        c = np.ascontiguousarray(coords, dtype=np.float32)
        if c.shape != (self.nf, self.na, 3):
            raise ValueError("coords must be [nf, na, 3]")
        self._prefetched = c
        self._check(self.lib.sass_prefetch_frames(self._h, _ptr(c)))

    def stage_prepass(self, frames, masses, steps, target, return_staged=True):
        """Alignments / motions on the whole system, then staging of the target atoms.

        frames: float32 [nf, nsys, 3]; masses [nsys]; target [na] system indices;
        steps: dicts with "type" (center, fittrans, fitrottrans, fitrot, motion),
        "selection", "reference_selection", optional "reference" ([nref, 3]),
        "fit_target" and "fit_source" (fits) and "translations" ([nf, 3], motions).
        Returns the staged float32 frames [nf, na, 3] (None with return_staged=False)."""
        fr = np.ascontiguousarray(frames, dtype=np.float32)
        nsys = fr.shape[1]
        if fr.shape != (self.nf, nsys, 3):
            raise ValueError("frames must be [nf, nsys, 3]")
        ms = np.ascontiguousarray(masses, dtype=np.float64)
        tg = np.ascontiguousarray(target, dtype=np.uintp)
        keep = []
        arr = (PrepassStep * max(1, len(steps)))()
        for k, st in enumerate(steps):
            def lst(key, dtype=np.uintp, shape=None):
                v = st.get(key)
                if v is None:
                    return None, 0
                a = np.ascontiguousarray(v, dtype=dtype)
                if shape is not None:
                    a = a.reshape(shape)
                keep.append(a)
                return a.ctypes.data, len(a)
            e = arr[k]
            e.type = STEP[st["type"]]
            e.selection, e.nselection = lst("selection")
            e.reference_selection, e.nreference = lst("reference_selection")
            e.reference, _ = lst("reference", np.float64, (-1, 3))
            e.fit_target, e.nfit = lst("fit_target")
            e.fit_source, _ = lst("fit_source")
            e.translations, _ = lst("translations", np.float64, (-1, 3))
        out = np.zeros((self.nf, self.na, 3), dtype=np.float32) if return_staged else None
        self._check(self.lib.sass_stage_frames_prepass(self._h, _ptr(fr), nsys, _ptr(ms), arr, len(steps),
                                                       _ptr(tg), _ptr(out) if return_staged else None))
        return out

    def set_classes(self, atom_class):
        c = np.ascontiguousarray(atom_class, dtype=np.int32)
        if c.shape != (self.na,):
            raise ValueError("atom_class must be [na]")
        self._check(self.lib.sass_set_atom_classes(self._h, _ptr(c), 0))

    def set_tile(self, q_per_lane=0, warps=0, atoms=0, atom_splits=0):
        self._check(self.lib.sass_set_phase_tile(self._h, q_per_lane, warps, atoms, atom_splits))

    def multipole(self, kind, qvectors, class_factors, moments, axis=(0.0, 0.0, 1.0)):
        """Multipole orientational average ("sphere" or "cylinder"): (fqt, fq, fq2) per q."""
        q = np.ascontiguousarray(qvectors, dtype=np.float64).reshape(-1, 3)
        nq = len(q)
        cf = np.ascontiguousarray(class_factors, dtype=np.float64).reshape(nq, self.nclass)
        mom = np.ascontiguousarray(moments, dtype=np.int32).reshape(-1, 2)
        ax = np.ascontiguousarray(axis, dtype=np.float64)
        fqt = np.zeros((nq, self.nf, 2))
        fq = np.zeros((nq, 2))
        fq2 = np.zeros((nq, 2))
        t = {"sphere": 0, "cylinder": 1}[kind]
        self._check(self.lib.sass_multipole_compute(self._h, t, nq, _ptr(q), _ptr(cf), len(mom),
                                                    _ptr(mom), _ptr(ax), _ptr(fqt), _ptr(fq),
                                                    _ptr(fq2)))
        return (fqt[..., 0] + 1j * fqt[..., 1], fq[:, 0] + 1j * fq[:, 1],
                fq2[:, 0] + 1j * fq2[:, 1])

    def set_poly(self, poly_pairs):
        """Pairs of each lane's q-vectors whose sin/cos use the FP32 pipe (direct kernel)."""
        self._check(self.lib.sass_set_phase_poly(self._h, poly_pairs))

    def set_recurrence(self, shells_per_lane=0):
        """Shell recurrence of the FP32 form: 0 automatic, -1 off, else 4/8/12/16/20/24/32."""
        self._check(self.lib.sass_set_shell_recurrence(self._h, shells_per_lane))

    def schedule(self):
        s = Schedule()
        self._check(self.lib.sass_plan_schedule(self._h, ctypes.byref(s)))
        return s.as_dict()

    def compute(self, sub_offsets, subvectors, class_factors):
        """Host in/out: returns (fqt [nq, nf] complex, fq [nq] complex, fq2 [nq] complex)."""
        offs = np.ascontiguousarray(sub_offsets, dtype=np.uintp)
        nq = len(offs) - 1
        sv = np.ascontiguousarray(subvectors, dtype=np.float64).reshape(-1, 3)
        cf = np.ascontiguousarray(class_factors, dtype=np.float64).reshape(nq, self.nclass)
        fqt = np.zeros((nq, self.nf, 2))
        fq = np.zeros((nq, 2))
        fq2 = np.zeros((nq, 2))
        self._check(self.lib.sass_compute(self._h, nq, _ptr(offs), _ptr(sv), _ptr(cf), _ptr(fqt),
                                          _ptr(fq), _ptr(fq2), 0))
        return (fqt[..., 0] + 1j * fqt[..., 1], fq[:, 0] + 1j * fq[:, 1],
                fq2[:, 0] + 1j * fq2[:, 1])

    def compute_device(self, sub_offsets, d_subvectors, d_class_factors, d_fqt, d_fq, d_fq2):
        """All array arguments except sub_offsets are device pointers (ints)."""
        offs = np.ascontiguousarray(sub_offsets, dtype=np.uintp)
        self._check(self.lib.sass_compute(self._h, len(offs) - 1, _ptr(offs), _vp(d_subvectors),
                                          _vp(d_class_factors), _vp(d_fqt), _vp(d_fq), _vp(d_fq2),
                                          1))

    def amplitudes(self, subvectors, sub_shell, class_factors):
        sv = np.ascontiguousarray(subvectors, dtype=np.float64).reshape(-1, 3)
        sh = np.ascontiguousarray(sub_shell, dtype=np.int32)
        cf = np.ascontiguousarray(class_factors, dtype=np.float64).reshape(-1, self.nclass)
        out = np.zeros((len(sv), self.nf, 2))
        self._check(self.lib.sass_amplitudes(self._h, len(sv), _ptr(sv), _ptr(sh), len(cf),
                                             _ptr(cf), _ptr(out)))
        return out[..., 0] + 1j * out[..., 1]

    def timing(self):
        t = Timing()
        self._check(self.lib.sass_last_timing(self._h, ctypes.byref(t)))
        return t.as_dict()

    def autotune(self, sub_offsets, subvectors, class_factors, repeats=2):
        """Time every tile shape on this workload; the plan keeps the fastest."""
        offs = np.ascontiguousarray(sub_offsets, dtype=np.uintp)
        nq = len(offs) - 1
        sv = np.ascontiguousarray(subvectors, dtype=np.float64).reshape(-1, 3)
        cf = np.ascontiguousarray(class_factors, dtype=np.float64).reshape(nq, self.nclass)
        out = [ctypes.c_int() for _ in range(4)]
        self._check(self.lib.sass_autotune(self._h, nq, _ptr(offs), _ptr(sv), _ptr(cf), repeats,
                                           *[ctypes.byref(o) for o in out]))
        r = dict(zip(("q_per_lane", "warps", "atoms", "split_atoms"), [o.value for o in out]))
        r["rec_shells_per_lane"] = self.schedule()["rec_shells_per_lane"]
        return r

    def center(self):
        c = np.zeros(3)
        self._check(self.lib.sass_frame_center(self._h, c.ctypes.data_as(_dp)))
        return c


class Batch:
    """Many systems in one graph-captured launch sequence (sass_batch_*)."""

    def __init__(self, workloads, precision="fp32", method="fftw", device=0, stream=None):
        self.lib = load()
        w0 = workloads[0]
        d = PlanDesc(SCATTERING[w0.scattering], DSP[w0.dsp], METHOD[method], PRECISION[precision],
                     0, 0, 0, device, stream or 0, 0)
        self._keep = []
        sys = (System * len(workloads))()
        for i, w in enumerate(workloads):
            c = np.ascontiguousarray(w.coords, dtype=np.float32)
            cls = np.ascontiguousarray(w.atom_class, dtype=np.int32)
            offs = np.ascontiguousarray(w.sub_offsets(), dtype=np.uintp)
            sv = np.ascontiguousarray(w.subvectors(), dtype=np.float64)
            cf = np.ascontiguousarray(w.class_factors, dtype=np.float64)
            self._keep += [c, cls, offs, sv, cf]
            sys[i] = System(w.na, w.nf, len(w.class_names), c.ctypes.data, cls.ctypes.data, w.nq,
                            offs.ctypes.data, sv.ctypes.data, cf.ctypes.data)
        self.shapes = [(w.nq, w.nf) for w in workloads]
        h = _vp()
        rc = self.lib.sass_batch_create(ctypes.byref(d), len(workloads), sys, ctypes.byref(h))
        self._h = h
        if rc != SASS_OK:
            msg = self.error()
            self.close()
            raise SassError(rc, msg)

    def error(self):
        return self.lib.sass_batch_error(self._h).decode() if self._h else ""

    def _check(self, rc):
        if rc != SASS_OK:
            raise SassError(rc, self.error())

    def close(self):
        if getattr(self, "_h", None):
            self.lib.sass_batch_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def autotune(self, repeats=1):
        out = [ctypes.c_int() for _ in range(4)]
        ms = ctypes.c_double()
        self._check(self.lib.sass_batch_autotune(self._h, repeats, *[ctypes.byref(o) for o in out],
                                                 ctypes.byref(ms)))
        r = dict(zip(("q_per_lane", "warps", "atoms", "split_atoms"), [o.value for o in out]))
        r["ms"] = ms.value
        r["rec_shells_per_lane"] = self.schedule()["rec_shells_per_lane"]
        return r

    def set_tile(self, q_per_lane=0, warps=0, atoms=0, split_atoms=0):
        self._check(self.lib.sass_batch_set_tile(self._h, q_per_lane, warps, atoms, split_atoms))

    def set_recurrence(self, shells_per_lane=0):
        self._check(self.lib.sass_batch_set_shell_recurrence(self._h, shells_per_lane))

    def set_poly(self, poly_pairs):
        self._check(self.lib.sass_batch_set_phase_poly(self._h, poly_pairs))

    def schedule(self):
        s = Schedule()
        self._check(self.lib.sass_batch_schedule(self._h, ctypes.byref(s)))
        return s.as_dict()

    def run(self):
        self._check(self.lib.sass_batch_run(self._h))

    def sync(self):
        self._check(self.lib.sass_batch_sync(self._h))

    def results(self, i):
        nq, nf = self.shapes[i]
        fqt = np.zeros((nq, nf, 2))
        fq = np.zeros((nq, 2))
        fq2 = np.zeros((nq, 2))
        self._check(self.lib.sass_batch_results(self._h, i, _ptr(fqt), _ptr(fq), _ptr(fq2)))
        return (fqt[..., 0] + 1j * fqt[..., 1], fq[:, 0] + 1j * fq[:, 1], fq2[:, 0] + 1j * fq2[:, 1])

    def timing(self):
        t = Timing()
        self._check(self.lib.sass_batch_timing(self._h, ctypes.byref(t)))
        return t.as_dict()

    def info(self):
        terms = ctypes.c_double()
        tiles = ctypes.c_uint64()
        out = [ctypes.c_int() for _ in range(4)]
        self._check(self.lib.sass_batch_info(self._h, ctypes.byref(terms), ctypes.byref(tiles),
                                             *[ctypes.byref(o) for o in out]))
        r = dict(zip(("q_per_lane", "warps", "atoms", "split_atoms"), [o.value for o in out]))
        r.update(terms=terms.value, phase_tiles=tiles.value)
        return r


class MLP:
    """The control-variate network (sass_mlp_*)."""

    def __init__(self, device=0, seed=0):
        self.lib = load()
        self.nparams = self.lib.sass_mlp_param_count()
        h = _vp()
        rc = self.lib.sass_mlp_create(device, seed, ctypes.byref(h))
        self._h = h
        if rc != SASS_OK:
            raise SassError(rc, self.error())

    def error(self):
        return self.lib.sass_mlp_error(self._h).decode() if self._h else ""

    def _check(self, rc):
        if rc != SASS_OK:
            raise SassError(rc, self.error())

    def close(self):
        if getattr(self, "_h", None):
            self.lib.sass_mlp_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scaling(self, q_mid, q_half, y_mean, y_std):
        self._check(self.lib.sass_mlp_set_scaling(self._h, q_mid, q_half, y_mean, y_std))

    def params(self):
        m = np.zeros(self.nparams, np.float32)
        b = np.zeros(self.nparams, np.uint16)
        self._check(self.lib.sass_mlp_get_params(self._h, _ptr(m), _ptr(b)))
        bf = (b.astype(np.uint32) << 16).view(np.float32)
        return m, bf

    def set_params(self, master):
        m = np.ascontiguousarray(master, np.float32)
        self._check(self.lib.sass_mlp_set_params(self._h, _ptr(m)))

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.sass_mlp_gradient(self._h, _ptr(x), _ptr(t), len(t), _ptr(g),
                                               ctypes.byref(loss)))
        return g, loss.value

    def train(self, x, t, steps, batch=4096, lr=1e-3):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.sass_mlp_train(self._h, _ptr(x), _ptr(t), len(t), steps, batch, lr,
                                            ctypes.byref(loss)))
        return loss.value

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(len(x), np.float32)
        self._check(self.lib.sass_mlp_predict(self._h, _ptr(x), len(x), _ptr(y)))
        return y

    def sphere_mean(self, qlen, npoints=32768):
        q = np.ascontiguousarray(qlen, np.float64)
        out = np.zeros(len(q))
        self._check(self.lib.sass_mlp_sphere_mean(self._h, _ptr(q), len(q), npoints, _ptr(out)))
        return out


def compute_cv(plan, net, qlen, dirs, class_factors, nquad=32768):
    """Control-variate and plain MC estimates on the same directions (see sass_compute_cv)."""
    q = np.ascontiguousarray(qlen, np.float64)
    d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    cf = np.ascontiguousarray(class_factors, np.float64).reshape(len(q), plan.nclass)
    nq, nf = len(q), plan.nf
    a, b = np.zeros((nq, nf, 2)), np.zeros((nq, nf, 2))
    c, e = np.zeros((nq, 2)), np.zeros((nq, 2))
    diag = np.zeros((nq, 3))
    plan._check(plan.lib.sass_compute_cv(plan._h, net._h, nq, _ptr(q), len(d), _ptr(d), _ptr(cf),
                                         nquad, _ptr(a), _ptr(b), _ptr(c), _ptr(e), _ptr(diag)))
    z = lambda v: v[..., 0] + 1j * v[..., 1]  # noqa: E731
    return z(a), z(b), z(c), z(e), diag


def probe_pipes(device=0):
    """Measured (sfu_ops_per_s, fp32_fma_per_s) of the device."""
    L = load()
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = L.sass_probe_pipes(device, ctypes.byref(a), ctypes.byref(b))
    if rc != SASS_OK:
        raise SassError(rc, "sass_probe_pipes failed")
    return a.value, b.value


def probe_fp64(device=0):
    """Measured FP64 FMA/s of the device."""
    L = load()
    a = ctypes.c_double()
    rc = L.sass_probe_fp64(device, ctypes.byref(a))
    if rc != SASS_OK:
        raise SassError(rc, "sass_probe_fp64 failed")
    return a.value


def compute_workload(w, precision="fp64", method="fftw", device=0, tile=None, recurrence=None,
                     schedule=None):
    """Run a synth.Workload through the C ABI; returns (fqt, fq, fq2).

    recurrence: shells per lane of the FP32 shell recurrence (None: automatic, -1: off);
    schedule: a dict that receives the plan's schedule of the call."""
    with Plan(w.na, w.nf, len(w.class_names), w.scattering, w.dsp, method, precision,
              device) as p:
        p.stage(w.coords)
        p.set_classes(w.atom_class)
        if tile:
            p.set_tile(*tile)
        if recurrence is not None:
            p.set_recurrence(recurrence)
        out = p.compute(w.sub_offsets(), w.subvectors(), w.class_factors)
        if schedule is not None:
            schedule.update(p.schedule())
        return out


# ----------------------------------------------------------------------------------------
# Host layer (no GPU): signal-file writer/reader and configuration parsing
# ----------------------------------------------------------------------------------------
HOST_LIB_PATH = os.path.join(_PKG, "_lib", "libsassena_host.so")
DRIVER_PATH = os.path.join(_PKG, "_lib", "sassena-gpu")
_host = None


def host():
    global _host
    if _host is None:
        if not os.path.exists(HOST_LIB_PATH):
            raise OSError("host library not built: %s" % HOST_LIB_PATH)
        H = ctypes.CDLL(HOST_LIB_PATH)
        H.sass_host_error.restype = ctypes.c_char_p
        H.sass_host_signal_write.argtypes = [ctypes.c_char_p, _sz, _sz, _vp, _vp, _vp, _vp, _vp,
                                             ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, _sz]
        H.sass_host_signal_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(_sz),
                                            ctypes.POINTER(_sz), ctypes.POINTER(ctypes.c_int),
                                            _vp, _vp, _vp, _vp, _vp]
        H.sass_host_config_qvectors.argtypes = [ctypes.c_char_p, _vp, _sz, ctypes.POINTER(_sz)]
        _host = H
    return _host


def write_signal(path, qvectors, fqt=None, fq0=None, fq=None, fq2=None, rawconfig="",
                 database="", chunksize=0):
    """Write a signal.h5 (complex arrays; None = dataset not written; chunksize: rows per
    chunk, 0 = the reference's default 10000)."""
    H = host()
    q = np.ascontiguousarray(qvectors, dtype=np.float64).reshape(-1, 3)
    nq = len(q)
    nf = 0 if fqt is None else np.asarray(fqt).shape[1]

    def ri(a, shape):
        if a is None:
            return None
        a = np.asarray(a, dtype=np.complex128).reshape(shape)
        return np.ascontiguousarray(np.stack([a.real, a.imag], axis=-1))

    arrs = [ri(fqt, (nq, nf)), ri(fq0, (nq,)), ri(fq, (nq,)), ri(fq2, (nq,))]
    flags = sum(1 << i for i, a in enumerate(arrs) if a is not None)
    ptrs = [a.ctypes.data_as(_vp) if a is not None else None for a in arrs]
    rc = H.sass_host_signal_write(path.encode(), nq, nf, q.ctypes.data_as(_vp), *ptrs, flags,
                                  rawconfig.encode(), database.encode(), chunksize)
    if rc:
        raise RuntimeError(H.sass_host_error().decode())


def read_signal(path):
    """Read a signal.h5 with the host library: dict of complex arrays + qvectors."""
    H = host()
    nq, nf, flags = _sz(), _sz(), ctypes.c_int()
    rc = H.sass_host_signal_read(path.encode(), ctypes.byref(nq), ctypes.byref(nf),
                                 ctypes.byref(flags), None, None, None, None, None)
    if rc:
        raise RuntimeError(H.sass_host_error().decode())
    q = np.zeros((nq.value, 3))
    fqt = np.zeros((nq.value, nf.value, 2))
    f0, f1, f2 = (np.zeros((nq.value, 2)) for _ in range(3))
    rc = H.sass_host_signal_read(path.encode(), ctypes.byref(nq), ctypes.byref(nf),
                                 ctypes.byref(flags), q.ctypes.data_as(_vp),
                                 fqt.ctypes.data_as(_vp), f0.ctypes.data_as(_vp),
                                 f1.ctypes.data_as(_vp), f2.ctypes.data_as(_vp))
    if rc:
        raise RuntimeError(H.sass_host_error().decode())
    c = lambda a: a[..., 0] + 1j * a[..., 1]  # noqa: E731
    out = {"qvectors": q}
    for bit, name, arr in ((1, "fqt", fqt), (2, "fq0", f0), (4, "fq", f1), (8, "fq2", f2)):
        if flags.value & bit:
            out[name] = c(arr)
    return out


def config_qvectors(config_path):
    H = host()
    n = _sz()
    rc = H.sass_host_config_qvectors(config_path.encode(), None, 0, ctypes.byref(n))
    if rc:
        raise RuntimeError(H.sass_host_error().decode())
    out = np.zeros((n.value, 3))
    H.sass_host_config_qvectors(config_path.encode(), out.ctypes.data_as(_vp), n.value,
                                ctypes.byref(n))
    return out
