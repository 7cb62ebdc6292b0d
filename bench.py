#!/usr/bin/env python3
"""Benchmark of the GB300 scattering-amplitude hot path (one JSON line on rank 0).

Workload (default): coherent dynamic S(q,t) — 10,000 atoms in a 50 A box, 1,024 frames of
Gaussian random walk (sigma 0.05 A) with a harmonic pull (RMSD ~1 A), H/C/N/O/S coherent
lengths, 20 shells 0.05-3.0 1/A x 500 directions, FFT autocorrelation (padded length
2,048). Seeded synthetic data. A "step" is the whole computation: phase sum over
1.024e11 atom.q.frame terms, correlation, orientational average.

  value      terms/s of the chosen (FP32) path, inputs resident in HBM, CUDA events on
             the plan's stream (coordinates 164 MB > 129 MB L2: inputs larger than L2).
  e2e        the same through the C ABI with host buffers: pinned host coordinates,
             sub-vectors and factors copied in and S(q,t)/fq/fq2 copied out every step (the
             next step's coordinates copied during the compute: sass_prefetch_frames).
  roofline   phase-sum kernel: terms/s against the SFU ceiling measured live by
             sass_probe_pipes (2 SFU results per term), and FP32 FMA rate for reference.
  plain      the plain FP64 path on the same GPU (same terms), its time, and the FP32
             path's max relative error in S(q,t) against it (time-to-1e-3 comparison).
  cpu_baseline  the CPU oracle (FP64 restatement of the reference, all host threads) on
             a bounded sample of the same workload.

Other workloads (--workload): incoherent_fqt, static_xray, batched_uneven, layered_cv, and
multipole_sphere / multipole_cylinder (the multipole devices on the coherent trajectory, FP64,
terms = atoms x q-vectors x moments x frames), prepass (sample alignments on the device).

--impl reference times that CPU restatement (the reference itself cannot be built:
MPI, Boost, FFTW3, HDF5 and libxml2 are absent) and prints its own line.
Multi-GPU: replicas only — every rank runs the full workload on its own GPU (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "atom*q*frame terms/s; time to 1e-3 rel err in S(q,t), chosen vs plain, same GPU"
UNIT = "terms/s"
MP_METRIC = "atom*q*moment*frame terms/s of the multipole orientational average (FP64)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="coherent_sqt")
    ap.add_argument("--plain-shells", type=int, default=0,
                    help="shells of the plain FP64 comparison run (0: every shell when the whole "
                         "workload takes at most --plain-budget seconds, else 3, time scaled by terms)")
    ap.add_argument("--plain-budget", type=float, default=30.0)
    ap.add_argument("--oracle-terms", type=float, default=6e8,
                    help="atom*q*frame terms of the oracle sample of the FP64/FP32 accuracy check")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-step-seconds", type=float, default=5.0,
                    help="CPU time of each timed step of --impl reference (a bounded sample)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"],
                    help="form timed by the scatter workloads (fp64: the plain FP64 path itself)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--nq", type=int, default=0, help="override the number of shells (profiling)")
    ap.add_argument("--nf", type=int, default=0, help="override the number of frames (profiling)")
    ap.add_argument("--nsys", type=int, default=0, help="systems of the batched workload")
    ap.add_argument("--na", type=int, default=0, help="override the number of atoms (layered_cv)")
    ap.add_argument("--budgets", default="64,256,1024,4096",
                    help="direction budgets M of the layered_cv workload")
    ap.add_argument("--draws", type=int, default=16,
                    help="independent direction draws per budget of the layered_cv workload")
    ap.add_argument("--cv-samples", type=int, default=100000,
                    help="exact |A|^2 training samples of the control variate (layered_cv)")
    ap.add_argument("--resolution", type=int, default=20,
                    help="largest major moment (multipole_sphere / multipole_cylinder)")
    ap.add_argument("--cv-steps", type=int, default=2500, help="training steps (layered_cv)")
    return ap.parse_args()


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region (median SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(name, nq=0, nf=0):
    from sassena_gb300 import synth
    kw = {}
    if nq:
        kw["nq"] = nq
    if nf:
        kw["nf"] = nf
    return synth.WORKLOADS[name](**kw)


def cpu_sample(w, seconds, nthreads):
    """Time the oracle's CPU-baseline build (-O3, tuned for the host CPU) on one shell x m
    directions, m grown until the sample takes about `seconds`. The oracle runs one direction
    per worker thread, so m stays a multiple of the thread count (or all of the shell's
    directions): a partial last round would understate the CPU's rate. Also reports the
    share of the CPU time spent in the correlation (dsp) rather than the phase sum."""
    import oracle
    s = w.nq // 2
    m = min(w.nm, nthreads)
    fac = w.factors()[s:s + 1]
    dsp = {"autocorrelate": 0, "square": 1, "plain": 2}[w.dsp]
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    while True:
        sv = w.shells[s] * w.directions[:m]
        offs = np.array([0, m], dtype=np.uintp)
        t0 = time.perf_counter()
        fn(w.coords, offs, sv, fac, dsp, 0, nthreads, timing=True)
        dt = time.perf_counter() - t0
        terms = w.na * m * w.nf
        if dt >= seconds * 0.6 or m >= w.nm:
            sc, ds = oracle.last_split(timing=True)
            return {"value": terms / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
                    "seconds": dt, "terms": terms, "correlation_share": ds / max(sc + ds, 1e-12),
                    "sample": "oracle (FP64 restatement, pinned to the reference's compiled devices; "
                              "-O3 CPU-baseline build) on shell %d/%d x %d of %d directions, all %d atoms "
                              "x %d frames (%.3g terms, %.1f s)" % (s, w.nq, m, w.nm, w.na, w.nf, terms, dt)}
        m = max(m * 2, int(m * seconds * 0.8 / max(dt, 1e-3)))
        m = min(w.nm, (m + nthreads - 1) // nthreads * nthreads)


def workload_config(w, world):
    """The config object both arms print for a scatter workload."""
    return {"workload": w.name, "na": w.na, "nf": w.nf, "nq": w.nq, "nm": w.nm,
            "terms_per_step": w.terms(), "dsp": w.dsp, "scattering": w.scattering,
            "fft_length": 1 << max(2, int(np.ceil(np.log2(2 * w.nf)))),
            "l2": "inputs larger than L2 (coordinates %.0f MB)" % (w.na * w.nf * 16 / 1e6),
            "parallelism": "replicas x%d" % world}


MP_WORKLOADS = ("multipole_sphere", "multipole_cylinder")
MP_AXIS = (0.0, 0.0, 1.0)


def multipole_workload(args):
    """The coherent_sqt trajectory (10,000 atoms, 1,024 frames) with one q-vector per shell
    in a seeded random direction, and the moments of `--resolution` (default 20, the
    reference's default)."""
    import oracle
    w = make_workload("coherent_sqt", args.nq, args.nf)
    rng = np.random.default_rng(7)
    d = rng.normal(size=(w.nq, 3))
    qv = w.shells[:, None] * d / np.linalg.norm(d, axis=1)[:, None]
    kind = args.workload.split("_")[1]
    res = args.resolution
    moments = oracle.sphere_moments(res) if kind == "sphere" else oracle.cylinder_moments(res)
    return w, qv, kind, moments


def mp_terms(w, moments):
    return float(w.na) * w.nq * len(moments) * w.nf


def cpu_sample_mp(w, qv, kind, moments, seconds, nthreads):
    """Time the oracle's multipole device on one q-vector, all atoms and moments, over a
    growing prefix of the frames (~`seconds`)."""
    import oracle
    s = w.nq // 2
    fac = w.factors()[s:s + 1]
    nf = min(w.nf, 2 * nthreads)
    while True:
        t0 = time.perf_counter()
        if kind == "sphere":
            oracle.mp_sphere(w.coords[:nf], qv[s:s + 1], fac, moments, nthreads=nthreads)
        else:
            oracle.mp_cylinder(w.coords[:nf], qv[s:s + 1], fac, moments, MP_AXIS, nthreads=nthreads)
        dt = time.perf_counter() - t0
        terms = float(w.na) * len(moments) * nf
        if dt >= seconds * 0.4 or nf >= w.nf:
            return {"value": terms / dt, "unit": "terms/s", "cores": nthreads, "kind": "port",
                    "sample": "oracle multipole %s (FP64 restatement) on q-vector %d/%d, all %d "
                              "atoms x %d moments x %d of %d frames (%.3g terms, %.1f s)"
                              % (kind, s, w.nq, w.na, len(moments), nf, w.nf, terms, dt)}
        nf = max(nf * 2, int(nf * seconds * 0.6 / max(dt, 1e-3)))
        nf = min(w.nf, (nf + nthreads - 1) // nthreads * nthreads)  # whole rounds of frames per thread


def run_reference(args, dist):
    if dist.rank != 0:
        return
    if args.workload == "prepass":
        from oracle import alignment as al
        w = make_workload("coherent_sqt", args.nq, args.nf)
        masses, _ = prepass_case(w)
        allat = list(range(w.na))
        al_steps = [{"type": "center", "selection": allat, "reference_selection": allat, "reference": None},
                    {"type": "fitrottrans", "selection": allat, "reference_selection": allat,
                     "reference": w.coords[0].astype(np.float64)}]
        vals, nfs = [], 2
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            al.load(w.coords[:nfs], masses, al_steps)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                vals.append(w.na * nfs / dt)
        v = statistics.median(vals)
        units = float(w.na) * w.nf
        print(json.dumps({"impl": "reference", "metric": "atom*frame/s through the staging pre-pass "
                          "(center + fitrottrans onto frame 0)", "value": v, "unit": "atom-frames/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": units / v * 1e3, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                          "config": {"workload": "prepass", "na": w.na, "nf": w.nf},
                          "cpu_baseline": {"value": v, "unit": "atom-frames/s", "cores": 1, "kind": "port",
                                           "sample": "oracle.alignment.load on %d of %d frames" % (nfs, w.nf)},
                          "e2e": {"value": v, "unit": "atom-frames/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0},
                          "note": "reference unbuildable here; timed the numpy restatement of "
                                  "CoordinateSets::load (one core), ms_per_step extrapolated by frames"}))
        return
    if args.workload in MP_WORKLOADS:
        w, qv, kind, moments = multipole_workload(args)
        nthreads = os.cpu_count() or 1
        vals = []
        for i in range(args.warmup + args.steps):
            r = cpu_sample_mp(w, qv, kind, moments, args.cpu_seconds / max(1, args.steps), nthreads)
            if i >= args.warmup:
                vals.append(r["value"])
        v = statistics.median(vals)
        terms = mp_terms(w, moments)
        print(json.dumps({"impl": "reference", "metric": MP_METRIC, "value": v, "unit": "terms/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": terms / v * 1e3, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded)",
                          "config": {"workload": args.workload, "na": w.na, "nf": w.nf, "nq": w.nq,
                                     "moments": len(moments), "resolution": args.resolution,
                                     "terms_per_step": terms},
                          "cpu_baseline": {"value": v, "unit": "terms/s", "cores": nthreads,
                                           "kind": "port", "sample": r["sample"]},
                          "e2e": {"value": v, "unit": "terms/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0},
                          "note": "reference unbuildable here (MPI/Boost/FFTW3/HDF5/libxml2 "
                                  "absent); timed its CPU restatement, ms_per_step extrapolated "
                                  "by terms"}))
        return
    if args.workload == "batched_uneven":  # the CPU rate per term: one system of the batch
        from sassena_gb300 import synth
        w = synth.batched_uneven(seed=4, nsys=args.nsys or 64)[0]
    elif args.workload == "layered_cv":
        from sassena_gb300 import synth
        w = synth.layered()
    else:
        w = make_workload(args.workload, args.nq, args.nf)
    nthreads = os.cpu_count() or 1
    vals, secs, shares = [], [], []
    for i in range(args.warmup + args.steps):
        # each step is a bounded sample of the workload: one shell x as many directions as
        # take about --ref-step-seconds on every host thread (warm-up samples are shorter)
        r = cpu_sample(w, args.ref_step_seconds if i >= args.warmup else 1.0, nthreads)
        if i >= args.warmup:
            vals.append(r["value"])
            secs.append(r["seconds"])
            shares.append(r["correlation_share"])
    v = statistics.median(vals)
    cfg = workload_config(w, dist.world)
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": statistics.median(secs) * 1e3,
                      "ms_per_full_step_extrapolated": w.terms() / v * 1e3, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic (seeded)", "config": cfg,
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                                       "sample": r["sample"],
                                       "correlation_share": statistics.median(shares)},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0},
                      "note": "the reference's whole program cannot be built here (MPI/Boost/FFTW3/HDF5/"
                              "libxml2 absent); timed the CPU oracle, which reproduces the reference's "
                              "compiled scatter devices (tests/test_reference_pin.py). A step is a bounded "
                              "sample of the workload; ms_per_full_step_extrapolated scales it by terms"}))


def hbm_peak():
    """HBM GB/s for the correlation's roofline: the measured copy bandwidth in
    MEASURED_PEAKS.json where the file is present, else 6,800 GB/s (an earlier GB300
    measurement, reported as the fallback)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            v = json.load(f).get("hbm_gbs")
        if v:
            return float(v), "of measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    return 6800.0, "of fallback (6.8 TB/s)"


def profile_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` on `workload` from its ncu capture
    (profiles/<kernel>_<workload>.json), or None where none was taken."""
    prof = os.path.join(ROOT, "profiles", "%s_%s.json" % (kernel, workload))
    if not os.path.exists(prof):
        return None
    with open(prof) as f:
        return json.load(f).get("dram_bytes_per_launch")


def phase_roofline(w, sch, phase_ms, corr_ms, sfu, fma):
    """Roofline of the step's dominant kernel against its live-measured ceiling.

    Coherent: the shell-recurrence kernel (>= 2 FMA + 2 FADD per term on the FP32 pipe) or the
    direct kernel (sin + cos per term on the SFU). Incoherent: the fused series + FFT kernel,
    bound by its FP32 FFT work (5 L log2 L flops per series of NF frames) or the SFU."""
    terms = w.terms()
    if w.scattering == "self":
        L = 1 << max(2, int(np.ceil(np.log2(2 * w.nf))))
        flops_per_term = 5.0 * L * np.log2(L) / w.nf
        peak = min(2.0 * fma / flops_per_term, sfu / 2.0)
        # FP32 form: the transposed register FFT at L = 64 .. 256, the lane-strided one to 512
        kernel = ("reg2_fft_kernel" if 64 <= L <= 256 else "reg_fft_kernel") if L <= 512 else \
            ("self_blk_fft_kernel" if L <= 4096 else "self_fft_kernel")
        achieved = terms / (corr_ms * 1e-3)
        return {"bound": "fp32" if 2.0 * fma / flops_per_term < sfu / 2.0 else "sfu",
                "achieved": achieved, "peak": peak, "unit": "terms/s", "frac": achieved / peak,
                "traffic": profile_traffic(kernel, w.name), "kernel": kernel, "kernel_ms": corr_ms,
                "peak_source": "measured live: sass_probe_pipes FP32 %.4g FMA/s x 2 / %.1f FFT "
                               "flops per term; SFU %.4g results/s / 2" % (fma, flops_per_term, sfu),
                "schedule": sch}
    achieved = terms / (phase_ms * 1e-3)
    rec_only = sch["rec_tiles"] > 0 and sch["direct_tiles"] == 0
    kernel = "phase_rec_kernel" if rec_only else "phase_sum_kernel"
    traffic = profile_traffic(kernel, w.name)
    if rec_only:
        # per term at least one FMA per component (recurrence) and one FADD per component
        # (accumulation) on the FP32 pipe: 4 lane operations
        peak = fma / 4.0
        roof = {"bound": "fp32", "peak_source": "measured live: sass_probe_pipes FP32 %.4g "
                "lane-ops/s / 4 per term (2 FMA recurrence + 2 FADD accumulate)" % fma,
                "sfu_results_per_s": sfu,
                "direct_evaluation_ceiling": sfu / 2.0}
    else:
        peak = sfu / 2.0
        roof = {"bound": "sfu", "peak_source": "measured live: sass_probe_pipes SFU %.4g "
                "results/s / 2 per term" % sfu, "fp32_fma_per_s": fma}
    roof.update({"achieved": achieved, "peak": peak, "unit": "terms/s",
                 "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
                 "kernel_ms": phase_ms, "schedule": sch})
    return roof


def shell_errors(got, ref):
    """Per shell: S(q,t) as max_t |S - S_ref| / |S_ref(q,0)|; I(q) as fq (the time-averaged
    correlation), fq0 = S(q,0) and fq2, each relative to its reference value."""
    (f, a, a2), (rf, ra, ra2) = got, ref
    den = np.abs(rf[:, 0])
    return {"sqt": np.abs(f - rf).max(axis=1) / den, "fq": np.abs(a - ra) / np.abs(ra),
            "fq0": np.abs(f[:, 0] - rf[:, 0]) / den, "fq2": np.abs(a2 - ra2) / np.abs(ra2)}


def _cplx(a):
    return a[..., 0] + 1j * a[..., 1]


def fp64_roofline(w, t64, terms, dev):
    """The plain FP64 form's phase-sum kernel against the FP64 pipe rate measured live
    (sass_probe_fp64). Its FP64 pipe instructions per term (products, sums and the
    software sin/cos) come from the ncu capture in profiles/phase_sum_kernel_fp64_<workload>.json."""
    from sassena_gb300 import abi
    fma = abi.probe_fp64(dev)
    prof = os.path.join(ROOT, "profiles", "phase_sum_kernel_fp64_%s.json" % w.name)
    per_term = None
    if os.path.exists(prof):
        with open(prof) as f:
            per_term = json.load(f).get("fp64_pipe_inst_per_term")
    achieved = terms / (t64["phase_ms"] * 1e-3)
    roof = {"bound": "fp64", "kernel": "phase_sum_kernel<double>", "kernel_ms": t64["phase_ms"],
            "fp64_fma_per_s": fma, "achieved": achieved, "unit": "terms/s"}
    if per_term:
        roof.update({"fp64_pipe_inst_per_term": per_term, "peak": fma / per_term,
                     "frac": achieved * per_term / fma,
                     "peak_source": "measured live: sass_probe_fp64 %.4g FP64 FMA/s / %.1f FP64-pipe "
                                    "instructions per term (ncu)" % (fma, per_term)})
    return roof


def plain_fp64_audit(args, w, plan, ms, dev):
    """The plain FP64 form on the same GPU: its time on the whole workload (a subset of
    shells, scaled by terms, only where the whole would exceed --plain-budget seconds), the
    FP32 path's error against it for every shell it ran, and both forms against the CPU
    oracle on a seeded sample of directions per shell (all atoms and frames)."""
    import oracle
    from sassena_gb300 import abi

    terms = w.terms()
    nclass = len(w.class_names)
    cf_all = np.ascontiguousarray(w.class_factors)
    full32 = plan.compute(w.sub_offsets(), w.subvectors(), cf_all)  # the measured FP32 output

    def subset(idx, dirs):
        offs = np.arange(len(idx) + 1, dtype=np.uintp) * len(dirs)
        return offs, (w.shells[idx, None, None] * dirs[None]).reshape(-1, 3), cf_all[idx]

    with abi.Plan(w.na, w.nf, nclass, w.scattering, w.dsp, "fftw", "fp64", device=dev) as p64:
        p64.stage(w.coords)
        p64.set_classes(w.atom_class)
        mid = np.array([w.nq // 2])
        p64.compute(*subset(mid, w.directions))
        est_ms = p64.timing()["total_ms"] * w.nq
        if args.plain_shells == 0 and est_ms <= args.plain_budget * 1e3:
            idx = np.arange(w.nq)
        else:
            ns = max(1, min(args.plain_shells or 3, w.nq))
            idx = np.linspace(0, w.nq - 1, ns).round().astype(int)
        ref = p64.compute(*subset(idx, w.directions))
        t64 = p64.timing()
        sch64 = p64.schedule()
        # the oracle sample: D seeded directions per shell (at least 8, so that each shell's
        # value is an orientational average and not one direction's intensity, which can sit
        # in a deep minimum), all atoms and frames, on every step_q-th shell within the budget
        d = min(w.nm, max(8, int(args.oracle_terms // (w.nq * w.na * w.nf))))
        step_q = max(1, int(np.ceil(w.nq * w.na * w.nf * d / args.oracle_terms)))
        oidx = np.arange(0, w.nq, step_q)
        rng = np.random.default_rng(2026)
        odirs = w.directions[np.sort(rng.choice(w.nm, d, replace=False))]
        o_offs, o_sv, o_cf = subset(oidx, odirs)
        g64 = p64.compute(o_offs, o_sv, o_cf)
    g32 = plan.compute(o_offs, o_sv, o_cf)
    dsp = {"autocorrelate": 0, "square": 1, "plain": 2}[w.dsp]
    fn = oracle.all_vectors if w.scattering == "all" else oracle.self_vectors
    t0 = time.perf_counter()
    orc = [_cplx(a) for a in fn(w.coords, o_offs, o_sv, o_cf[:, w.atom_class], dsp, 0, os.cpu_count())]
    oracle_s = time.perf_counter() - t0

    e32 = shell_errors([x[idx] for x in full32], ref)
    eo32 = shell_errors(g32, orc)
    eo64 = shell_errors(g64, orc)
    run_terms = w.na * w.nf * w.nm * len(idx)
    plain_tps = run_terms / (t64["total_ms"] * 1e-3)
    full_ms = terms / plain_tps * 1e3
    lst = lambda v: [float(x) for x in v]  # noqa: E731
    res = {"value": plain_tps, "unit": UNIT, "shells_run": int(len(idx)),
           "whole_workload": bool(len(idx) == w.nq),
           ("ms_full_workload" if len(idx) == w.nq else "ms_full_workload_extrapolated"): full_ms,
           "speedup_same_gpu": full_ms / ms,
           "schedule": sch64,
           "fp32_max_rel_err_vs_fp64": float(e32["sqt"].max()),
           "fp32_rel_err_per_shell": {"q": lst(w.shells[idx]), "sqt": lst(e32["sqt"]),
                                      "sqt_median": float(np.median(e32["sqt"])), "iq_fq": lst(e32["fq"]),
                                      "fq0": lst(e32["fq0"]), "fq2": lst(e32["fq2"])},
           "vs_oracle": {"directions_per_shell": int(d), "shells": int(len(oidx)),
                         "sample": "oracle FP64 on %d shells x %d seeded directions, all %d atoms x %d "
                                   "frames (%.1f s on %d threads)" % (len(oidx), d, w.na, w.nf, oracle_s,
                                                                       os.cpu_count()),
                         "fp32_sqt_per_shell": lst(eo32["sqt"]), "fp32_sqt_max": float(eo32["sqt"].max()),
                         "fp32_fq_max": float(eo32["fq"].max()), "fp32_fq0_max": float(eo32["fq0"].max()),
                         "fp32_fq2_max": float(eo32["fq2"].max()),
                         "fp64_sqt_max": float(eo64["sqt"].max()), "fp64_fq_max": float(eo64["fq"].max()),
                         "fp64_fq2_max": float(eo64["fq2"].max())}}
    # the FP64 phase-sum kernel's roofline, where it ran (self scattering has no phase sum:
    # its FP64 series go straight into the correlation)
    if sch64.get("direct_tiles", 0) > 0:
        res["roofline"] = fp64_roofline(w, t64, run_terms, dev)
    return res


def run_ours(args, dist):
    import torch

    from sassena_gb300 import abi

    dev = dist.local
    torch.cuda.set_device(dev)
    w = make_workload(args.workload, args.nq, args.nf)
    # a dedicated stream: the library's work and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    nclass = len(w.class_names)
    terms = w.terms()
    plan = abi.Plan(w.na, w.nf, nclass, w.scattering, w.dsp, "fftw", args.precision, device=dev,
                    stream=stream.cuda_stream)
    plan.stage(w.coords)
    plan.set_classes(w.atom_class)
    offs = w.sub_offsets()
    sv = torch.from_numpy(w.subvectors()).cuda()
    cf = torch.from_numpy(np.ascontiguousarray(w.class_factors)).cuda()
    fqt = torch.zeros((w.nq, w.nf, 2), dtype=torch.float64, device="cuda")
    fq = torch.zeros((w.nq, 2), dtype=torch.float64, device="cuda")
    fq2 = torch.zeros((w.nq, 2), dtype=torch.float64, device="cuda")

    def step():
        plan.compute_device(offs, sv.data_ptr(), cf.data_ptr(), fqt.data_ptr(), fq.data_ptr(),
                            fq2.data_ptr())
        return plan.timing()

    for _ in range(max(3, args.warmup)):
        step()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phase_ms, corr_ms, launches = [], [], 0
    e0.record(stream)
    for _ in range(args.steps):
        t = step()
        phase_ms.append(t["phase_ms"])
        corr_ms.append(t["corr_ms"] + t["finalize_ms"])
        launches += t["kernel_launches"]
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dist.barrier()
    ms = dist.max(e0.elapsed_time(e1) / args.steps)
    value = terms * dist.world / (ms * 1e-3)

    # ---- end to end through the C ABI with host buffers ------------------------------
    lib = abi.load()
    nbytes = w.coords.nbytes
    hp = lib.sass_host_alloc(nbytes)
    host_coords = np.ctypeslib.as_array((np.ctypeslib.ctypes.c_float * w.coords.size)
                                        .from_address(hp)).reshape(w.coords.shape)
    host_coords[...] = w.coords
    sv_h = w.subvectors()
    cf_h = np.ascontiguousarray(w.class_factors)
    # Each step stages its frames and computes; while it computes, the plan's copy stream
    # brings the next step's frames over (sass_prefetch_frames), so every step still moves
    # one step's coordinates host -> device inside its timed region. The first step's copy
    # is made inside the first (warm-up) step's region.
    e2e_ms = []
    n_e2e = 0 if args.no_e2e else args.warmup + args.steps
    for i in range(n_e2e):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if i == 0:
            plan.prefetch(host_coords)
        plan.stage(host_coords)
        plan.prefetch(host_coords)  # the next step's frames
        res = plan.compute(offs, sv_h, cf_h)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if n_e2e:
        plan.stage(host_coords)  # consume the last copy before the buffer is freed
    lib.sass_host_free(hp)
    e2e_step = dist.max(statistics.median(e2e_ms) if e2e_ms else float("nan"))
    h2d = nbytes + sv_h.nbytes + cf_h.nbytes
    d2h = w.nq * (w.nf + 2) * 16

    # ---- roofline of the dominant kernel ---------------------------------------------------
    sch = plan.schedule()
    sfu, fma = abi.probe_pipes(dev)
    if args.precision == "fp64":
        roof = fp64_roofline(w, {"phase_ms": statistics.median(phase_ms)}, terms, dev)
        roof["schedule"] = sch
    else:
        roof = phase_roofline(w, sch, statistics.median(phase_ms), statistics.median(corr_ms), sfu, fma)
    corr = statistics.median(corr_ms)
    # algorithmic bytes: the FP32 amplitudes read once (float2, 8 B) and the FP64 row written
    # per shell
    corr_bytes = (w.nq * w.nm * w.nf * 8) + (w.nq * w.nf * 16)
    lg = max(2, int(np.ceil(np.log2(2 * w.nf))))
    if w.dsp != "autocorrelate":
        if w.scattering == "all":
            corr_kernel = "corr_sq_warp_kernel" if w.nf <= 512 else "corr_direct_kernel"
        else:
            corr_kernel = "self_direct_kernel"
    elif lg <= 9:
        corr_kernel = "reg2_fft_kernel" if args.precision == "fp32" and 6 <= lg <= 8 else "reg_fft_kernel"
    elif lg <= 12 and w.scattering == "all":
        corr_kernel = "blk_fft_kernel"
    else:
        corr_kernel = "corr_fft_kernel" if w.scattering == "all" else "self_fft_kernel"
    hbm, hbm_src = hbm_peak()
    roof_corr = {"bound": "hbm", "kernel": corr_kernel + "+finalize_kernel", "ms": corr,
                 "achieved": corr_bytes / (corr * 1e-3) / 1e9, "unit": "GB/s", "peak": hbm,
                 "frac": corr_bytes / (corr * 1e-3) / 1e9 / hbm, "peak_source": hbm_src,
                 "algorithmic_bytes": corr_bytes}
    if w.scattering == "self":  # series generated inside the FFT kernel: no amplitudes in HBM
        roof_corr = {"kernel": roof["kernel"] + "+finalize_kernel", "ms": corr,
                     "note": "fused with the series generation; its roofline is `roofline`"}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
           "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if args.precision == "fp32" else "f64",
           "data": "synthetic (seeded random walk, %s)" % w.name,
           "config": workload_config(w, dist.world),
           "e2e": {"value": terms * dist.world / (e2e_step * 1e-3), "unit": UNIT,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_step,
                   "note": "per step: stage + compute through the C ABI from pinned host memory, "
                           "results read back; the coordinates of the next step are copied on the "
                           "plan's copy stream during the compute (sass_prefetch_frames)"},
           "roofline": roof, "roofline_correlation": roof_corr,
           "gpu_launches": int(launches), "clocks": clk}

    # ---- plain FP64 path on the same GPU, and the FP32 error against it -------------------
    if not args.no_plain and args.precision == "fp32":
        out["plain_fp64"] = plain_fp64_audit(args, w, plan, ms, dev)

    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_sample(w, args.cpu_seconds, os.cpu_count() or 1)
    if dist.rank == 0:
        print(json.dumps(out))
    plan.close()


def run_multipole(args, dist):
    """Multipole sphere / cylinder devices (FP64): terms = atoms x q-vectors x moments x
    frames. `value`: sass_multipole_compute with the frames resident in HBM (q-vectors,
    factors and moments are host inputs of that call, a few KB); `e2e`: staging from pinned
    host memory plus the same call."""
    import torch

    from sassena_gb300 import abi

    dev = dist.local
    torch.cuda.set_device(dev)
    w, qv, kind, moments = multipole_workload(args)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    nclass = len(w.class_names)
    terms = mp_terms(w, moments)
    cf = np.ascontiguousarray(w.class_factors)
    plan = abi.Plan(w.na, w.nf, nclass, "all", w.dsp, "fftw", "fp64", device=dev,
                    stream=stream.cuda_stream)
    plan.stage(w.coords)
    plan.set_classes(w.atom_class)

    def step():
        plan.multipole(kind, qv, cf, moments, MP_AXIS)
        return plan.timing()

    for _ in range(max(3, args.warmup)):
        step()
    steps = max(1, min(args.steps, 5))
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phase_ms, corr_ms, launches = [], [], 0
    e0.record(stream)
    for _ in range(steps):
        t = step()
        phase_ms.append(t["phase_ms"])
        corr_ms.append(t["corr_ms"] + t["finalize_ms"])
        launches += t["kernel_launches"]
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dist.barrier()
    ms = dist.max(e0.elapsed_time(e1) / steps)
    value = terms * dist.world / (ms * 1e-3)

    lib = abi.load()
    nbytes = w.coords.nbytes
    hp = lib.sass_host_alloc(nbytes)
    host_coords = np.ctypeslib.as_array((np.ctypeslib.ctypes.c_float * w.coords.size)
                                        .from_address(hp)).reshape(w.coords.shape)
    host_coords[...] = w.coords
    e2e_ms = []
    for i in range(0 if args.no_e2e else 1 + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan.stage(host_coords)
        plan.multipole(kind, qv, cf, moments, MP_AXIS)
        torch.cuda.synchronize()
        if i >= 1:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    lib.sass_host_free(hp)
    e2e_step = dist.max(statistics.median(e2e_ms) if e2e_ms else float("nan"))
    t = plan.timing()

    fp64 = abi.probe_fp64(dev)
    ph = statistics.median(phase_ms)
    # algorithmic FP64 work of the moment sums: sphere 2 FMA per term (real j_l b times a
    # complex Y); cylinder 6 operations per atom, q, frame and order (J cos, J sin, 4 FMA)
    if kind == "sphere":
        ops = 2.0 * terms
        per = "2 FMA per term (sum_j b j_l(qr) conj(Y_lm))"
    else:
        ops = 6.0 * w.na * w.nq * w.nf * (2 * args.resolution + 1)
        per = "6 FP64 operations per atom, q, frame and order n <= 2L"
    achieved = ops / (ph * 1e-3)
    roof = {"bound": "fp64", "achieved": achieved, "peak": fp64, "unit": "FP64 op/s",
            "frac": achieved / fp64, "traffic": None,
            "kernel": "mp_sphere_basis+contract" if kind == "sphere" else "mp_cylinder_kernel",
            "kernel_ms": ph, "peak_source": "measured live: sass_probe_fp64 %.4g FMA/s; "
                                            "algorithmic work %s" % (fp64, per)}
    out = {"metric": MP_METRIC, "value": value, "unit": "terms/s", "n_gpus": dist.world,
           "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded random walk, coherent_sqt trajectory)",
           "config": {"workload": args.workload, "na": w.na, "nf": w.nf, "nq": w.nq,
                      "moments": len(moments), "resolution": args.resolution,
                      "axis": list(MP_AXIS) if kind == "cylinder" else None,
                      "terms_per_step": terms, "dsp": w.dsp,
                      "l2": "inputs larger than L2 (coordinates %.0f MB)" % (w.na * w.nf * 16 / 1e6),
                      "parallelism": "replicas x%d" % dist.world},
           "e2e": {"value": terms * dist.world / (e2e_step * 1e-3), "unit": "terms/s",
                   "h2d_bytes_per_step": nbytes + t["h2d_bytes"],
                   "d2h_bytes_per_step": t["d2h_bytes"], "ms_per_step": e2e_step},
           "roofline": roof, "phase_ms": ph, "correlation_ms": statistics.median(corr_ms),
           "gpu_launches": int(launches), "clocks": clk}
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_sample_mp(w, qv, kind, moments, args.cpu_seconds,
                                            os.cpu_count() or 1)
    if dist.rank == 0:
        print(json.dumps(out))
    plan.close()


def prepass_case(w, nframes=None):
    """Steps of the prepass workload: centre the system, then fit every frame onto frame 0
    (all atoms); masses by class."""
    na = w.na
    allat = np.arange(na, dtype=np.uintp)
    masses = np.array([1.008, 12.011, 14.007, 15.999, 32.06])[w.atom_class % 5]
    steps = [{"type": "center", "selection": allat, "reference_selection": allat},
             {"type": "fitrottrans", "selection": allat, "reference_selection": allat,
              "reference": w.coords[0].astype(np.float64), "fit_target": allat, "fit_source": allat}]
    return masses, steps


def run_prepass(args, dist):
    """Staging pre-pass (sample alignments): the coherent_sqt trajectory (10,000 atoms x
    1,024 frames) centred and fitted onto frame 0 on the device, then staged. value =
    atom-frames per second through sass_stage_frames_prepass from host frames (the host
    copy is part of the call)."""
    import torch

    from sassena_gb300 import abi

    dev = dist.local
    torch.cuda.set_device(dev)
    w = make_workload("coherent_sqt", args.nq, args.nf)
    masses, steps = prepass_case(w)
    lib = abi.load()
    nbytes = w.coords.nbytes
    hp = lib.sass_host_alloc(nbytes)
    frames = np.ctypeslib.as_array((np.ctypeslib.ctypes.c_float * w.coords.size)
                                   .from_address(hp)).reshape(w.coords.shape)
    frames[...] = w.coords
    target = np.arange(w.na, dtype=np.uintp)
    plan = abi.Plan(w.na, w.nf, len(w.class_names), "all", w.dsp, "fftw", "fp32", device=dev)
    for _ in range(max(3, args.warmup)):
        plan.stage_prepass(frames, masses, steps, target, return_staged=False)
    steps_n = max(1, min(args.steps, 10))
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(steps_n):
        plan.stage_prepass(frames, masses, steps, target, return_staged=False)
    torch.cuda.synchronize()
    ms = dist.max((time.perf_counter() - t0) * 1e3 / steps_n)
    clk = clocks.stop()
    units = float(w.na) * w.nf
    out = {"metric": "atom*frame/s through the staging pre-pass (center + fitrottrans onto frame 0)",
           "value": units * dist.world / (ms * 1e-3), "unit": "atom-frames/s", "n_gpus": dist.world,
           "steps": steps_n, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded random walk, coherent_sqt trajectory)",
           "config": {"workload": "prepass", "na": w.na, "nf": w.nf,
                      "steps": ["center", "fitrottrans"], "timing": "host clock around the C-ABI call "
                      "(host frames in page-locked memory; upload, pre-pass, staging, synchronised)"},
           "e2e": {"value": units * dist.world / (ms * 1e-3), "unit": "atom-frames/s",
                   "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": w.nf * 9 * 8 * 2,
                   "ms_per_step": ms},
           "gpu_launches": None, "clocks": clk}
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        from oracle import alignment as al
        nfs = 2
        t0 = time.perf_counter()
        al.load(w.coords[:nfs], masses,
                [{"type": "center", "selection": list(range(w.na)), "reference_selection": list(range(w.na)),
                  "reference": None},
                 {"type": "fitrottrans", "selection": list(range(w.na)),
                  "reference_selection": list(range(w.na)), "reference": w.coords[0].astype(np.float64)}])
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": w.na * nfs / dt, "unit": "atom-frames/s", "cores": 1, "kind": "port",
                               "sample": "oracle.alignment.load (numpy restatement) on %d frames x %d atoms, "
                                         "%.2f s" % (nfs, w.na, dt)}
    if dist.rank == 0:
        print(json.dumps(out))
    lib.sass_host_free(hp)
    plan.close()


def run_batched(args, dist):
    """The batched form: 64 systems of uneven size in one graph-captured launch sequence."""
    import torch

    from sassena_gb300 import abi, synth

    dev = dist.local
    torch.cuda.set_device(dev)
    nsys = args.nsys or 64
    ws = synth.batched_uneven(seed=4, nsys=nsys)
    terms = sum(w.terms() for w in ws)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    # autotune on a representative subset (every 8th system), apply to the full batch
    t0 = time.perf_counter()
    with abi.Batch(ws[::8], precision="fp32", device=dev, stream=stream.cuda_stream) as sub:
        tuned = sub.autotune(repeats=1)
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    rec = tuned["rec_shells_per_lane"] or -1  # the subset's choice: a width, or off
    b = abi.Batch(ws, precision="fp32", device=dev, stream=stream.cuda_stream)
    b.set_tile(tuned["q_per_lane"], tuned["warps"], tuned["atoms"], tuned["split_atoms"])
    b.set_recurrence(rec)
    create_s = time.perf_counter() - t0
    steps = min(args.steps, 5)  # one replay is seconds long: keep the timed region short
    for _ in range(max(3, args.warmup)):
        b.run()
    b.sync()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.run()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    b.sync()
    ms = dist.max(e0.elapsed_time(e1) / steps)
    info = b.info()
    sched = b.schedule()
    launches = b.timing()["kernel_launches"] * steps
    # end to end: stage every system from host memory, one run, copy all results back
    e2e = []
    for i in range(0 if args.no_e2e else 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with abi.Batch(ws, precision="fp32", device=dev, stream=stream.cuda_stream) as bb:
            bb.set_tile(tuned["q_per_lane"], tuned["warps"], tuned["atoms"], tuned["split_atoms"])
            bb.set_recurrence(rec)
            bb.run()
            for k in range(len(ws)):
                bb.results(k)
            # every result is on the host: the step ends here; releasing the batch's device
            # memory (cudaFree of every system's buffers) is not part of it
            e2e.append((time.perf_counter() - t0) * 1e3)
    b.close()
    h2d = sum(w.coords.nbytes + w.subvectors().nbytes for w in ws)
    d2h = sum(w.nq * (w.nf + 2) * 16 for w in ws)
    out = {"metric": METRIC, "value": terms * dist.world / (ms * 1e-3), "unit": UNIT,
           "n_gpus": dist.world, "steps": steps, "warmup": max(3, args.warmup),
           "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded, %d systems)" % len(ws),
           "config": {"workload": "batched_uneven", "systems": len(ws),
                      "na_range": [min(w.na for w in ws), max(w.na for w in ws)],
                      "nf_range": [min(w.nf for w in ws), max(w.nf for w in ws)],
                      "terms_per_step": terms, "phase_tiles": info["phase_tiles"],
                      "schedule": sched,
                      "tile": tuned, "autotune_s": tune_s, "create_s": create_s,
                      "l2": "inputs larger than L2"},
           "e2e": {"value": terms / (min(e2e) * 1e-3) if e2e else None, "unit": UNIT,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                   "ms_per_step": min(e2e) if e2e else None,
                   "note": "batch creation (H2D staging, FFT tables, graph capture) + one run + "
                           "all results D2H; the batch's release after the results is not timed"},
           "gpu_launches": int(launches), "clocks": clk}
    if dist.rank == 0:
        print(json.dumps(out))


def run_cv(args, dist):
    """Learned control variate on the anisotropic layered system, measured by the variance of
    the estimators over repeated independent direction draws (no reference average needed).

    For each direction budget M and each of R independent draws of M uniform directions,
    one sass_compute_cv call gives the plain Monte Carlo average (the reference's equal-weight
    mean, all_vectors_scatter_device.cpp:355-360) and the control-variate estimate on the same
    directions (FP32 path). Per shell, the relative standard error of an estimate is
    se(q) = max_t sd_r S_r(q,t) / |mean_r S_r(q,0)|; Monte Carlo errors fall as M^-1/2, so an
    estimator reaches 1e-3 on shell q at M*(q) = M (se(q) / 1e-3)^2 directions, and every shell
    at M* = max_q M*(q). Time to 1e-3 = (time per direction at M) x M*, for the FP32 control
    variate, FP32 plain MC and the plain FP64 path (its time per term measured on the GPU).
    The paired difference of the two estimates checks that the control variate is unbiased."""
    import torch

    from sassena_gb300 import abi, cv, synth

    if dist.rank != 0:
        return
    dev = dist.local
    torch.cuda.set_device(dev)
    kw = {}
    if args.nf:
        kw["nf"] = args.nf
    if args.na:
        kw["na"] = args.na
    if args.nq:
        kw["nq"] = args.nq
    w = synth.layered(**kw)
    nclass = len(w.class_names)
    cf = np.ascontiguousarray(w.class_factors)
    budgets = [int(b) for b in args.budgets.split(",")]
    plan = abi.Plan(w.na, w.nf, nclass, "all", "autocorrelate", "fftw", "fp32", device=dev)
    plan.stage(w.coords)
    plan.set_classes(w.atom_class)

    def run_mc(dirs):
        offs = np.arange(w.nq + 1, dtype=np.uintp) * len(dirs)
        sv = (w.shells[:, None, None] * dirs[None]).reshape(-1, 3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = plan.compute(offs, sv, cf)
        return out, (time.perf_counter() - t0) * 1e3

    # control variate: exact training intensities from the library, trained on the GPU
    t0 = time.perf_counter()
    x, t, sc = cv.training_set(plan, w, args.cv_samples, seed=11)
    samp_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    net, loss = cv.fit(x, t, sc, steps=args.cv_steps, batch=4096, lr=2e-3, seed=3, device=dev)
    train_s = time.perf_counter() - t0
    # accuracy of the sphere quadrature the estimator subtracts (32,768 spherical-Fibonacci
    # points, the default of sass_compute_cv) against a 16 times denser set
    g_quad = net.sphere_mean(w.shells, 32768)
    g_dense = net.sphere_mean(w.shells, 16 * 32768)
    quad_dev = float(np.max(np.abs(g_quad / g_dense - 1.0)))
    run_mc(synth.sphere_directions(64, 1))  # warm-up of the plain path
    rows = []
    for m in budgets:
        est_cv, est_mc, ms_cv = [], [], []
        for r in range(args.draws):
            dirs = synth.sphere_directions(m, 1000003 * m + r)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fqt_cv, fqt_mc, _, _, _ = abi.compute_cv(plan, net, w.shells, dirs, cf)
            ms_cv.append((time.perf_counter() - t0) * 1e3)
            est_cv.append(fqt_cv)
            est_mc.append(fqt_mc)
        _, ms_mc = run_mc(synth.sphere_directions(m, 7))
        est_cv, est_mc = np.array(est_cv), np.array(est_mc)  # [R, nq, nf]
        scale = np.abs(est_mc.mean(axis=0)[:, 0])  # |S(q,0)|
        se_cv = est_cv.std(axis=0, ddof=1).max(axis=1) / scale
        se_mc = est_mc.std(axis=0, ddof=1).max(axis=1) / scale
        # paired difference at t = 0: unbiasedness of the control variate
        d0 = (est_cv[:, :, 0] - est_mc[:, :, 0]).real
        d0_se = d0.std(axis=0, ddof=1) / np.sqrt(args.draws)
        z = np.abs(d0.mean(axis=0)) / np.maximum(d0_se, 1e-300)
        # the mean paired difference relative to S(q,0), with its standard error: a bound on
        # any bias of the control variate (its quadrature mean G) at the scale of the target
        bias = np.abs(d0.mean(axis=0)) / scale
        rows.append({"M": m, "draws": args.draws, "terms": w.na * w.nq * m * w.nf,
                     "ms_mc": ms_mc, "ms_cv": float(np.median(ms_cv)),
                     "se_mc_max": float(se_mc.max()), "se_mc_median": float(np.median(se_mc)),
                     "se_cv_max": float(se_cv.max()), "se_cv_median": float(np.median(se_cv)),
                     "variance_ratio_median": float(np.median((se_mc / se_cv) ** 2)),
                     "variance_ratio_per_shell": [float(v) for v in (se_mc / se_cv) ** 2],
                     "unbiased_z_max": float(z.max()), "unbiased_z_over_3": int((z > 3).sum()),
                     "paired_diff_rel_max": float(bias.max()),
                     "paired_diff_rel_se_median": float(np.median(d0_se / scale)),
                     "m_star_mc": float(m * (se_mc.max() / 1e-3) ** 2),
                     "m_star_cv": float(m * (se_cv.max() / 1e-3) ** 2)})
    # plain FP64 path: time per term on two shells x 64 directions
    sub = synth.sphere_directions(64, 7)
    idx = [0, w.nq - 1]
    with abi.Plan(w.na, w.nf, nclass, "all", "autocorrelate", "fftw", "fp64", device=dev) as p64:
        p64.stage(w.coords)
        p64.set_classes(w.atom_class)
        offs = np.arange(3, dtype=np.uintp) * 64
        sv = (w.shells[idx, None, None] * sub[None]).reshape(-1, 3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p64.compute(offs, sv, cf[idx])
        fp64_ms_per_term = (time.perf_counter() - t0) * 1e3 / (w.na * 2 * 64 * w.nf)
    last = rows[-1]  # the largest budget: the best-measured variances
    per_dir_cv, per_dir_mc = last["ms_cv"] / last["M"], last["ms_mc"] / last["M"]
    t_cv = per_dir_cv * last["m_star_cv"]
    t_mc = per_dir_mc * last["m_star_mc"]
    t64 = fp64_ms_per_term * w.na * w.nq * w.nf * last["m_star_mc"]
    out = {"metric": METRIC, "value": last["terms"] / (last["ms_mc"] * 1e-3), "unit": UNIT,
           "n_gpus": 1, "steps": len(budgets) * args.draws, "warmup": 1, "ms_per_step": last["ms_cv"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if args.precision == "fp32" else "f64",
           "data": "synthetic (seeded layered system, density 1 + %.1f cos(2 pi z / %.0f A))"
                   % (w.meta["amplitude"], w.meta["period"]),
           "config": {"workload": "layered_cv", "na": w.na, "nf": w.nf, "nq": w.nq,
                      "shells": [float(w.shells[0]), float(w.shells[-1])], "budgets": budgets,
                      "draws": args.draws,
                      "value_note": "value: FP32 plain path terms/s end to end (host in/out) at M=%d"
                                    % last["M"]},
           "control_variate": {"samples": args.cv_samples, "sample_s": samp_s, "train_s": train_s,
                               "steps": args.cv_steps, "final_loss": loss,
                               "quadrature_rel_dev_vs_16x_denser": quad_dev},
           "budgets": rows,
           "time_to_1e-3": {"from_M": last["M"],
                            "fp32_cv": {"ms": t_cv, "M": last["m_star_cv"]},
                            "fp32_mc": {"ms": t_mc, "M": last["m_star_mc"]},
                            "fp64_mc": {"ms": t64, "M": last["m_star_mc"]},
                            "fp64_mc_over_fp32_cv": t64 / t_cv, "fp32_mc_over_fp32_cv": t_mc / t_cv,
                            "method": "M* = M (max_q se(q) / 1e-3)^2 from the measured standard errors "
                                      "at the largest M; time = time per direction x M*"},
           "fp64_ms_per_term": fp64_ms_per_term}
    print(json.dumps(out))
    plan.close()


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "batched_uneven":
            run_batched(args, dist)
        elif args.workload == "layered_cv":
            run_cv(args, dist)
        elif args.workload in MP_WORKLOADS:
            run_multipole(args, dist)
        elif args.workload == "prepass":
            run_prepass(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
