/*
 * sassena_gb300 — C ABI of the GB300 scattering-amplitude hot path.
 *
 * The reference (Sassena 1.4.2) computes, per q-vector, the orientational average
 * of the autocorrelated (or squared, or plain) scattering amplitude
 *     A(q,t) = sum_j b_j(|q|) exp(i q . r_j(t))
 * inside its scatter devices. This header is the thin C layer under the C++ host
 * devices (sassena_gb300/host/): plain pointers and sizes, int status codes, no
 * exceptions, no CUDA or C++ types in the signatures.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   plan create      ScatterDeviceFactory::create, src/scatter_devices/scatter_device_factory.cpp:23-210
 *                    (device choice by scattering.type :145-201), device ctors
 *                    all_vectors_scatter_device.cpp:32-55, self_vectors_scatter_device.cpp:40-57
 *   stage frames     DataStagerByFrame::stage, src/stager/data_stager.cpp:72-118
 *                    (DataStagerByAtom::stage :214-338 for the incoherent device)
 *   atom classes     ScatterFactors::set_selection / update, src/scatter_devices/scatter_factors.cpp:56-94
 *   compute          AbstractScatterDevice::runner's per-q compute(), abstract_scatter_device.cpp:145-175,
 *                    AllVectorsScatterDevice::compute all_vectors_scatter_device.cpp:238-361,
 *                    SelfVectorsScatterDevice::compute self_vectors_scatter_device.cpp:145-239;
 *                    outputs are the rows HDF5WriterClient::write receives,
 *                    src/services/file_writer_service.cpp:504-531 (fq0 = fqt[0])
 *   amplitudes       AllVectorsScatterDevice::scatter, all_vectors_scatter_device.cpp:388-439
 *   errors           Err::Inst()->write + throw (e.g. all_vectors_scatter_device.cpp:217-227),
 *                    ram_check limits (:57-125) -> status codes + sass_plan_error()
 *
 * Threading: a plan is used by one host thread at a time; distinct plans are
 * independent. All device work of a plan runs on the plan's CUDA stream.
 */
#ifndef SASSENA_GB300_H
#define SASSENA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define SASS_OK 0
#define SASS_ERR_ARG 1          /* invalid argument or shape */
#define SASS_ERR_OOM 2          /* device or host allocation failed */
#define SASS_ERR_UNSUPPORTED 3  /* configuration outside this build (e.g. NF > 524,288 with FFT) */
#define SASS_ERR_CUDA 4         /* CUDA runtime error */
#define SASS_ERR_TIMEOUT 5      /* a bounded device-side wait gave up */
#define SASS_ERR_STATE 6        /* call out of order (e.g. compute before staging) */

/* scattering.type (parameters.cpp:372) */
#define SASS_SCATTERING_ALL 0   /* coherent: AllVectorsScatterDevice */
#define SASS_SCATTERING_SELF 1  /* incoherent: SelfVectorsScatterDevice */

/* scattering.dsp.type (parameters.cpp:375) */
#define SASS_DSP_AUTOCORRELATE 0
#define SASS_DSP_SQUARE 1
#define SASS_DSP_PLAIN 2

/* scattering.dsp.method (parameters.cpp:376): fftw maps to this library's FFT */
#define SASS_METHOD_FFTW 0
#define SASS_METHOD_DIRECT 1

/* Arithmetic of the phase sum. FP64 reproduces the reference's FP64 sums;
 * FP32 is the fast form (FP32 phase, Kahan, FP64 cross-block reductions). */
#define SASS_PRECISION_FP64 0
#define SASS_PRECISION_FP32 1

typedef struct sass_plan sass_plan;

typedef struct sass_plan_desc {
    int scattering;       /* SASS_SCATTERING_* */
    int dsp_type;         /* SASS_DSP_* */
    int dsp_method;       /* SASS_METHOD_* */
    int precision;        /* SASS_PRECISION_* */
    size_t na;            /* atoms of the target selection (stager.target) */
    size_t nf;            /* frames */
    size_t nclass;        /* distinct scattering classes (b depends only on class and |q|) */
    int device;           /* CUDA device ordinal */
    void* stream;         /* cudaStream_t to run on; NULL: the plan creates its own */
    size_t amplitude_budget_bytes; /* cap on the amplitude buffer; 0: 4 GiB */
} sass_plan_desc;

/* Per-call device timings (CUDA events on the plan's stream, milliseconds). */
typedef struct sass_timing {
    double phase_ms;      /* phase-sum kernels (coherent) */
    double corr_ms;       /* correlation / store / incoherent fused kernels */
    double finalize_ms;   /* per-shell FP64 finalisation */
    double h2d_ms;        /* host-to-device copies inside sass_compute */
    double d2h_ms;        /* device-to-host copies inside sass_compute */
    double total_ms;      /* whole sass_compute call on the stream */
    uint64_t kernel_launches; /* kernels this library launched in the call */
    uint64_t phase_launches;  /* of which phase-sum kernels */
    uint64_t h2d_bytes, d2h_bytes;
} sass_timing;

/* Create a plan (device buffers, FFT tables, stream). Replaces the factory +
 * device constructor pair. */
int sass_plan_create(const sass_plan_desc* desc, sass_plan** plan);
void sass_plan_destroy(sass_plan* plan);

/* Last error message of the plan ("" if none); valid until the next call. */
const char* sass_plan_error(const sass_plan* plan);
/* Name of a status code. */
const char* sass_status_name(int status);

/* Stage the trajectory: frame-major float32 [nf][na][3] (the reference's coor_t
 * buffer; replaces DataStagerByFrame::stage, src/stager/data_stager.cpp:72-118).
 * coords_on_device != 0 means `coords` is a device pointer. Host memory is read in
 * place where the device can address it: pinned or registered memory through its device
 * mapping; pageable memory, where the GPU can read it through the host's page tables,
 * page-locked (cudaHostRegister) for the duration of the call and read the same way
 * (read in place unlocked if locking fails); otherwise it is copied first. The call
 * returns after staging: the caller may then free or reuse the buffer. Device memory is
 * reserved before the buffer is read, so SASS_ERR_OOM leaves it unread. */
int sass_stage_frames(sass_plan* plan, const float* coords, int coords_on_device);

/* Request that the host frames of a later sass_stage_frames call be copied ahead: the
 * plan's next sass_compute queues the copy on a copy stream of the plan, behind its own
 * input copies, so that the transfer overlaps its kernels. The next sass_stage_frames of
 * the same pointer then waits for the copy and converts from device memory; the buffer
 * must not change until then. Staging another buffer, or another request, discards it; a
 * request with no compute before the staging is staged as usual. Pageable buffers are
 * page-locked from the request to that staging where the GPU reads pageable memory
 * through the host's page tables. No reference counterpart: DataStagerByFrame::stage
 * (data_stager.cpp:72-118) reads the frames serially before the device runs. */
int sass_prefetch_frames(sass_plan* plan, const float* coords);

/* ---- Staging pre-pass: alignments and motions ------------------------------------
 * Replaces the per-frame work of CoordinateSets::load (src/sample/coordinate_sets.cpp:
 * 244-368): pre-alignments, motions and post-alignments applied in FP64 to the whole
 * system's coordinates, then the reduction to the stager target and the float32
 * staging of DataStagerByFrame (src/stager/data_stager.cpp:102-118). Steps run in the
 * order given (the caller lists pre-alignments, motions, then post-alignments).
 *
 * Every step names atoms by system index. The reference structure of a step is
 * `reference` ([nreference][3], a frame or a file read by the caller) or, when it is
 * NULL, the current frame's atoms reference_selection ("instant"); its centre of mass
 * is sum_i m[reference_selection[i]] R_i / sum_i m[...], summed in list order.
 *   CENTER       (type "center"): translate `selection` by -COM(reference structure).
 *   FITTRANS     translate `selection` by COM(reference structure) - COM(selection).
 *   FITROTTRANS  Fit (center_of_mass.cpp:53-157): the frame's atoms reference_selection
 *                are rotated (Kabsch, SVD of the mass-weighted correlation matrix with
 *                the reflection correction) and moved onto the reference structure;
 *                atom fit_target[k] then takes fitted atom fit_source[k].
 *   FITROT       as FITROTTRANS, then `selection` is translated by its centre of mass
 *                from before the fit (coordinate_sets.cpp:283-287).
 *   MOTION       translation motions (linear, fixed, oscillation; motion_walker.cpp):
 *                x -> ((x - c) + t_f) + c for the atoms of `selection`, c = COM of the
 *                reference structure, t_f = translations[f].
 * Empty lists are allowed (a centre of mass of nothing is 0, as in the reference). */
#define SASS_STEP_CENTER 0
#define SASS_STEP_FITTRANS 1
#define SASS_STEP_FITROTTRANS 2
#define SASS_STEP_FITROT 3
#define SASS_STEP_MOTION 4

typedef struct sass_prepass_step {
    int type;
    int reserved;
    const size_t* selection;            /* atoms translated (and FITTRANS / FITROT centres) */
    size_t nselection;
    const size_t* reference_selection;  /* atoms of the reference structure (masses) */
    size_t nreference;
    const double* reference;            /* [nreference][3] or NULL (the current frame) */
    const size_t* fit_target;           /* fits: atoms written from the fitted copy ... */
    const size_t* fit_source;           /* ... positions in reference_selection they take */
    size_t nfit;
    const double* translations;         /* MOTION: [nf][3] */
} sass_prepass_step;

/* frames: host float32 [nf][nsys][3] of the whole system; masses [nsys]; target [na]
 * system indices of the plan's atoms; staged (optional) receives the float32 frames
 * [nf][na][3] as staged. Replaces sass_stage_frames for configurations with alignments
 * or motions. */
int sass_stage_frames_prepass(sass_plan* plan, const float* frames, size_t nsys, const double* masses,
                              const sass_prepass_step* steps, size_t nsteps, const size_t* target,
                              float* staged);

/* Class index per atom of the selection, int32 [na], each in [0, nclass). */
int sass_set_atom_classes(sass_plan* plan, const int32_t* atom_class, int on_device);

/* Compute nq q-vectors ("shells" here: one q and its orientation sub-vectors).
 *   sub_offsets   [nq+1] host array: sub-vectors of q i are [sub_offsets[i], sub_offsets[i+1])
 *   subvectors    [sub_offsets[nq]][3] FP64 (|q| * orientation, or q itself)
 *   class_factors [nq][nclass] FP64, b_class(|q_i|)
 *   fqt           [nq][nf][2] FP64 out  (orientational average of C(t))
 *   fq, fq2       [nq][2] FP64 out      (afinal, a2final after 1/NM)
 * io_on_device != 0: subvectors, class_factors, fqt, fq, fq2 are device pointers
 * (sub_offsets is always a host array). */
int sass_compute(sass_plan* plan, size_t nq, const size_t* sub_offsets, const double* subvectors,
                 const double* class_factors, double* fqt, double* fq, double* fq2,
                 int io_on_device);

/* Raw coherent amplitudes (no dsp): out [nsub][nf][2] FP64 for the given
 * sub-vectors; sub_shell [nsub] selects the row of class_factors [nshell][nclass]. */
int sass_amplitudes(sass_plan* plan, size_t nsub, const double* subvectors,
                    const int32_t* sub_shell, size_t nshell, const double* class_factors,
                    double* out);

/* Time every instantiated phase-sum tile shape and atom-split size on this
 * workload (the arguments of sass_compute, host arrays) and keep the fastest for the
 * plan's later calls; the choice is cached per process by problem signature. FP32
 * plans whose q-vectors share one direction set also try every shell-recurrence width
 * (and none). The chosen shape is returned through the (optional) out-pointers. */
int sass_autotune(sass_plan* plan, size_t nq, const size_t* sub_offsets, const double* subvectors,
                  const double* class_factors, int repeats, int* q_per_lane, int* warps, int* atoms,
                  int* split_atoms);

/* Timings of the last sass_compute / sass_amplitudes call. */
int sass_last_timing(const sass_plan* plan, sass_timing* out);

/* Tile shape of the phase sum (q per lane, warps = frames per CTA, atoms per
 * stage, atom splits; 0 = automatic). Returns SASS_ERR_UNSUPPORTED for shapes
 * this build does not instantiate. */
int sass_set_phase_tile(sass_plan* plan, int q_per_lane, int warps, int atoms, int atom_splits);

/* FP32 direct kernel: pairs of each lane's q-vectors whose sin/cos are evaluated on the
 * FP32 pipe (Taylor series of the half angle and the double-angle formulas, truncation
 * below 6e-8) instead of the SFU, so that both units carry load; 0 = all on the SFU. Needs
 * the explicit tile shape set by sass_set_phase_tile to instantiate that split
 * (SASS_ERR_UNSUPPORTED otherwise). No counterpart in the reference (libm sin/cos). */
int sass_set_phase_poly(sass_plan* plan, int poly_pairs);

/* Frame centre used by the FP32 form (frame-0 bounding-box midpoint). */
int sass_frame_center(const sass_plan* plan, double* center3);

/* Shell recurrence of the FP32 form. When every q-vector's sub-vectors are multiples of
 * one direction set (the reference's "file" and "sphere" orientation types,
 * abstract_vectors_scatter_device.cpp:112-130) and consecutive |q| lie on a line (linear
 * scans), runs of at least 3 such shells are evaluated by a kernel that carries
 * exp(i q_k u.r) from shell to shell with a three-term recurrence: two reduced sin/cos
 * pairs per atom for up to `shells_per_lane` shells. 0 = automatic (default), -1 = off,
 * else one of 4, 8, 12, 16, 20, 24, 32. FP64 plans ignore it. */
int sass_set_shell_recurrence(sass_plan* plan, int shells_per_lane);

/* How the last sass_compute (or batch run) scheduled the phase sum. */
typedef struct sass_schedule {
    double terms;                  /* atom x sub-vector x frame terms */
    uint64_t direct_tiles;         /* tiles of the direct phase-sum kernel */
    uint64_t rec_tiles;            /* tiles of the shell-recurrence kernel */
    uint64_t rec_shells;           /* q-vectors evaluated by the recurrence */
    int rec_shells_per_lane;       /* 0: recurrence not used */
    int q_per_lane, warps, atoms;  /* direct kernel tile shape */
    int atom_splits;               /* largest atom-split count */
    int poly_pairs;                /* direct kernel: q-vector pairs per lane on the FP32 pipe */
} sass_schedule;
int sass_plan_schedule(const sass_plan* plan, sass_schedule* out);

/* ---- Multipole orientational averages ----
 * The reference's multipole devices (orientation type "multipole",
 * scatter_device_factory.cpp:167-190): MPSphereScatterDevice and MPCylinderScatterDevice
 * (multipole_scatter_device.cpp:278-497, 750-986). For each q and each moment (major l,
 * minor m) the amplitude over frames is summed over atoms, correlated (dsp) and stored
 * as by the vectors devices; the sums over moments are scaled by 1/(4 pi) (sphere) or
 * 1/(2 pi) (cylinder).
 *   sphere:   A_lm(t) = sum_j 4 pi i^l b_j j_l(|q| r_j) conj(Y_l^m(theta_j, phi_j)), |m| <= l
 *   cylinder: A_lm(t) = sqrt(2 pi) sum_j b_j exp(i |z_j q_z|) c_lm J_n(q_r r_j) T_m(n (phi_j - phi_q)),
 *             n = 2l for m = 0, 1 (T = cos, sin) and 2l - 1 for m = 2, 3, in the cylinder frame
 *             of `axis` (CartesianVectorBase, coor3d.cpp:278-295).
 * moments [nmoments][2] (major, minor) as ScatteringAverageOrientationMultipoleMoments
 * lists them (parameters.cpp:1037-1122; the same validity checks, major <= 40 here).
 * Coherent FP64 plans only (SASS_ERR_UNSUPPORTED otherwise). qvectors [nq][3],
 * class_factors [nq][nclass], outputs as sass_compute; all host arrays. */
enum { SASS_MULTIPOLE_SPHERE = 0, SASS_MULTIPOLE_CYLINDER = 1 };
int sass_multipole_compute(sass_plan* plan, int type, size_t nq, const double* qvectors,
                           const double* class_factors, size_t nmoments, const int32_t* moments,
                           const double* axis, double* fqt, double* fq, double* fq2);

/* ---- Batches: many independent systems in one graph-captured launch sequence ----
 * Each system has its own trajectory, atom classes, q-vectors and sub-vector sets of
 * any size. The batch stages everything once; sass_batch_run replays one CUDA graph
 * containing the factor expansion, ONE persistent phase-sum launch over the tiles of all
 * systems (work queue), the batched correlation and the finalisation. No counterpart in
 * the reference, which runs one system per process invocation (sassena.cpp:132-417). */
typedef struct sass_batch sass_batch;

typedef struct sass_system {
    size_t na, nf, nclass;
    const float* coords;          /* host [nf][na][3] float32, frame-major */
    const int32_t* atom_class;    /* host [na] */
    size_t nq;                    /* q-vectors of this system */
    const size_t* sub_offsets;    /* host [nq+1] */
    const double* subvectors;     /* host [sub_offsets[nq]][3] */
    const double* class_factors;  /* host [nq][nclass] */
} sass_system;

/* desc supplies scattering, dsp, method, precision, device and stream (its na, nf,
 * nclass are ignored; each system carries its own). */
int sass_batch_create(const sass_plan_desc* desc, size_t nsystems, const sass_system* systems,
                      sass_batch** batch);
/* Autotune tile shape and atom-split size over the whole batch (coherent). */
int sass_batch_autotune(sass_batch* batch, int repeats, int* q_per_lane, int* warps, int* atoms,
                        int* split_atoms, double* best_ms);
/* Set the tile shape and atom-split size (atoms per tile, a multiple of 128; 0 =
 * automatic), e.g. from sass_batch_autotune on a representative smaller batch. */
int sass_batch_set_tile(sass_batch* batch, int q_per_lane, int warps, int atoms, int split_atoms);
/* Enqueue one replay of the batch's graph (asynchronous on the batch stream). */
int sass_batch_run(sass_batch* batch);
/* Wait for the last run and check the device error word. */
int sass_batch_sync(sass_batch* batch);
/* Copy one system's results to host arrays (fqt [nq][nf][2], fq/fq2 [nq][2]; NULL skips). */
int sass_batch_results(sass_batch* batch, size_t system, double* fqt, double* fq, double* fq2);
int sass_batch_timing(const sass_batch* batch, sass_timing* out);
/* Total atom.q.frame terms, phase-sum tiles and the tile shape of the batch. */
int sass_batch_info(const sass_batch* batch, double* terms, uint64_t* phase_tiles, int* q_per_lane,
                    int* warps, int* atoms, int* split_atoms);
/* Shell recurrence for the batch (as sass_set_shell_recurrence) and its schedule. */
int sass_batch_set_shell_recurrence(sass_batch* batch, int shells_per_lane);
/* Polynomial sin/cos pairs of the batch's tile shape (as sass_set_phase_poly). */
int sass_batch_set_phase_poly(sass_batch* batch, int poly_pairs);
int sass_batch_schedule(const sass_batch* batch, sass_schedule* out);
const char* sass_batch_error(const sass_batch* batch);
void sass_batch_destroy(sass_batch* batch);

/* ---- Learned control variate for the orientational average ----
 * A 4 -> 128 -> 128 -> 1 tanh network g(u, |q|) with BF16 weights and FP32
 * accumulation, trained on the GPU by this library's own kernels on exact intensities
 * (inputs x = (ux, uy, uz, (|q| - q_mid)/q_half), target the normalised log intensity,
 * g = exp(y * y_std + y_mean)). No counterpart in the reference, whose orientational
 * average is the plain mean over random orientations (all_vectors_scatter_device.cpp:355-360). */
typedef struct sass_mlp sass_mlp;
int sass_mlp_create(int device, uint64_t seed, sass_mlp** net);
void sass_mlp_destroy(sass_mlp* net);
const char* sass_mlp_error(const sass_mlp* net);
int sass_mlp_param_count(void);
int sass_mlp_set_scaling(sass_mlp* net, double q_mid, double q_half, double y_mean, double y_std);
/* FP32 master weights and their BF16 copy (either pointer may be NULL). Layout:
 * W1 [128][4], b1 [128], W2 [128][128], b2 [128], W3 [128], b3. */
int sass_mlp_get_params(const sass_mlp* net, float* master, uint16_t* bf16);
int sass_mlp_set_params(sass_mlp* net, const float* master);
/* Gradient of mean (y - t)^2 over the n samples x [n][4], t [n] (no update). */
int sass_mlp_gradient(sass_mlp* net, const float* x, const float* t, size_t n, float* grad, double* loss);
/* Adam steps on consecutive mini-batches of the (caller-shuffled) samples. */
int sass_mlp_train(sass_mlp* net, const float* x, const float* t, size_t n, int steps, int batch, double lr,
                   double* last_loss);
int sass_mlp_predict(sass_mlp* net, const float* x, size_t n, float* y);
/* Mean of g over the sphere at each |q| (spherical-Fibonacci quadrature, FP64 sums). */
int sass_mlp_sphere_mean(sass_mlp* net, const double* qlen, size_t nshell, size_t npoints, double* gbar);
/* Control-variate estimate of S(q,t) and fq for a coherent plan (dsp autocorrelate or
 * square) from m directions shared by all shells, with the plain Monte Carlo estimate on
 * the same directions beside it. fqt_* [nq][nf][2], fq_* [nq][2], diag [nq][3] (optional:
 * quadrature mean of g, mean of g over the directions, variance of g). */
int sass_compute_cv(sass_plan* plan, sass_mlp* net, size_t nq, const double* qlen, size_t m,
                    const double* dirs, const double* class_factors, size_t nquad, double* fqt_cv,
                    double* fqt_mc, double* fq_cv, double* fq_mc, double* diag);

/* Pinned host memory for faster staging (cudaHostAlloc / cudaFreeHost). */
void* sass_host_alloc(size_t bytes);
void sass_host_free(void* p);

/* Measure the SFU (sin/cos results per second) and FP32 FMA (per second)
 * throughput of `device` with pipe microbenchmarks; the phase sum's roofline. */
int sass_probe_pipes(int device, double* sfu_ops_per_s, double* fp32_fma_per_s);
/* FP64 FMA rate of the device (independent fma chains over every SM), FMA/s: the
 * ceiling of the FP64 forms and of the multipole devices. */
int sass_probe_fp64(int device, double* fp64_fma_per_s);

/* Allocation-free coherent autocorrelation + orientational average (FP64), for
 * callers that must not allocate GPU memory while they run: programs that reserve
 * the whole device up front, code running inside a memory-pool callback, services
 * that cannot risk an out-of-memory failure mid-run. No counterpart in the
 * reference (its scatter devices allocate per call, all_vectors_scatter_device.cpp:262).
 *   amplitudes  device [nsub][nf][2] FP64, A_v(t) per sub-vector (sass_amplitudes layout)
 *   sub_offsets device uint64 [nq+1], sub-vectors of q i are [sub_offsets[i], sub_offsets[i+1])
 *   fqt, fq, fq2 device outputs as in sass_compute (dsp = autocorrelate, method fftw/direct)
 * Working memory is one fixed 8.2 MiB device array inside the library; nothing is
 * allocated. Limits: nq <= 128, nf <= 4096 (else SASS_ERR_UNSUPPORTED); sub_offsets
 * must increase and stay below 2^31 (they are read on the device: a q whose range
 * breaks this is treated as empty and its rows come back NaN). Calls share the
 * array: calls that overlap on the GPU race, so issue them in order on one stream.
 * A device reset loses the array's contents and is not supported between calls.
 * Asynchronous on `stream` (a cudaStream_t, NULL = default). */
int sass_correlate_noalloc(int device, void* stream, const double* amplitudes, size_t nf,
                           size_t nq, const uint64_t* sub_offsets, int dsp_method,
                           double* fqt, double* fq, double* fq2);

/* Library version string. */
const char* sass_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SASSENA_GB300_H */
