// Host-side launch interface of the sassena_gb300 kernels (internal, not the C ABI).
//
// Every launch works on lists of descriptors so that one launch can cover many
// systems (trajectories) with different atom counts, frame counts, shells and
// direction sets. A single scatter-device computation is a list with one system.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace sassgpu {

// SM count of the current device, queried once per device. Grids are sized from it, never
// from a fixed count; 1 if the query fails, so grid-stride loops stay valid (only slower).
inline int current_sms() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    static int cache[64] = {0};
    if (dev >= 0 && dev < 64 && cache[dev] > 0) return cache[dev];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    if (dev >= 0 && dev < 64) cache[dev] = n;
    return n;
}

// Blocks of `threads` for a grid-stride loop over n items: enough for every item, at most
// per_sm CTAs per SM of the current device, at least one.
inline unsigned grid_blocks(size_t n, int threads, int per_sm) {
    size_t b = (n + (size_t)threads - 1) / (size_t)threads;
    const size_t cap = (size_t)current_sms() * (size_t)per_sm;
    if (b > cap) b = cap;
    return b < 1 ? 1u : (unsigned)b;
}

enum Precision { PREC_FP64 = 0, PREC_FP32 = 1 };
// Transform arithmetic of the long-series path beyond the two forms: float-float (a value
// as an unevaluated sum of two floats, about 44 significant bits) on the FP32 pipe.
constexpr int PREC_FF = 2;

// Device-side error codes written to the plan's error word (first writer wins).
enum DeviceError : unsigned int {
    DEV_OK = 0,
    DEV_MBAR_TIMEOUT = 1,  // an mbarrier wait exceeded its iteration limit
    DEV_BAD_SHAPE = 2,     // a kernel saw a shape outside what its host check allowed
};

// Atom padding granule: every device coordinate row holds a multiple of this many
// atoms, so every staged tile is whole and 16-byte aligned.
constexpr int kAtomGranule = 128;
// Largest padded FFT length of the correlation kernels (NF <= 4096).
constexpr int kMaxLg = 13;

// ---------------------------------------------------------------------------------------
// Phase sum
// ---------------------------------------------------------------------------------------
// Tile shape: q-vectors per lane, warps (= frames) per CTA, atoms per pipeline stage, and
// (FP32 form) pairs of a lane's q-vectors whose sin/cos are evaluated on the FP32 pipe.
struct PhaseShape {
    int q_per_lane;
    int warps;
    int atoms;
    int poly_pairs;
};

struct PhaseSystem {
    const float4* xyz;     // [nf][na_pad] staged coordinates
    const void* bfac;      // [nshell][na_pad] factors: float (FP32) or double (FP64)
    const double* qv;      // [nv][3] sub-vectors of this system
    double2* out;          // FP64 form: amplitudes [nv][nf], or split partials [nsplit][nv][nf]
    float2* out_f32;       // FP32 amplitudes [nv][nf] (one atom split), or FP32 split partials [nsplit][nv][nf]
    size_t split_stride;   // nv * nf
    int na_pad, nf;
};

struct PhaseTileDesc {
    int system, shell;     // shell index into the system's factor rows
    int v0, nv;            // sub-vectors [v0, v0+nv) of the system, nv <= 32 * q_per_lane
    int f0;                // first frame (one per warp)
    int j_begin, j_end;    // atoms (multiples of the stage size)
    int split;             // atom-split slice written by this tile
};

struct PhaseLaunch {
    int precision;
    PhaseShape shape;
    const PhaseSystem* systems;
    const PhaseTileDesc* tiles;
    int ntiles;
    unsigned int* counter;  // work-queue counter, zero before the launch
    unsigned int* err;
    int max_ctas;           // 0: SMs x resident CTAs per SM
};

bool phase_shape_supported(int precision, PhaseShape t);
std::vector<PhaseShape> phase_shapes(int precision);
cudaError_t launch_phase_sum(const PhaseLaunch& a, cudaStream_t st);
// out[i] = sum_s part[s][i] in split order (FP64), stored as double2 or float2.
cudaError_t launch_split_reduce(const double2* part, int nsplit, size_t n, double2* out,
                                cudaStream_t st);
cudaError_t launch_split_reduce_f32(const float2* part, int nsplit, size_t n, float2* out,
                                    cudaStream_t st);

// ---------------------------------------------------------------------------------------
// Shell-recurrence phase sum (FP32 form): runs of shells lam_k = lam0 + k dlam along
// shared base vectors, evaluated with a three-term recurrence over k.
// ---------------------------------------------------------------------------------------
constexpr int kRecMaxClass = 32;  // scattering classes the recurrence kernel handles

struct RecGroup {
    int system;            // owning system
    int s0, ks;            // shells [s0, s0+ks) of the system, ks <= K
    int pad;
    double lam0, dlam;     // shell s0+k has sub-vectors (lam0 + k dlam) * dirs[d]
};

struct RecSystem {
    const float4* xyzw;       // class-sorted coordinates [nf][na_rec]; padding atoms at the origin
    const int* block_class;   // [na_rec / 32] class (low 16 bits) | padding atoms << 16 of every 32-atom block
    const double* cf;         // [nq][nclass] class factors
    const double* dirs;       // [nd][3] base vectors (FP64)
    double2* out;             // unused by the FP32-only recurrence (kept for the descriptor layout)
    float2* out_f32;          // FP32 amplitudes [nv][nf] (one split), or FP32 split partials [nsplit][nv][nf]
    size_t split_stride;      // nv * nf
    int na_rec, nf, nd, nclass;
    int g_begin;              // first group of this system in the launch's group list
    int pad;
};

struct RecTileDesc {
    int system;
    int p0, np;            // (group, direction) pairs [p0, p0+np) of the system, np <= 32
    int f0;                // first frame (one per warp)
    int j_begin, j_end;    // atoms of the class-sorted rows (multiples of 128; may be empty)
    int split;
    int pad;
};

struct RecLaunch {
    int K;                     // shells per lane (a value of rec_shell_counts())
    const RecSystem* systems;
    const RecGroup* groups;
    const RecTileDesc* tiles;
    int ntiles;
    float* bfac;               // [ngroups][kRecMaxClass][K] filled by launch_rec_factors
    unsigned int* counter;     // work-queue counter, zero before the launch
    unsigned int* err;
    int max_ctas;
};

std::vector<int> rec_shell_counts();
bool rec_shells_supported(int K);
cudaError_t launch_rec_factors(const RecLaunch& a, int ngroups, cudaStream_t st);
cudaError_t launch_phase_rec(const RecLaunch& a, cudaStream_t st);
// dst[f][j] = src[f][map[j]] with w = 1, or a zero row entry with w = 0 where map[j] < 0
cudaError_t launch_permute_stage(const float4* src, int na_pad_src, const int* map, int na_dst, int nf,
                                 float4* dst, cudaStream_t st);

// ---------------------------------------------------------------------------------------
// Correlation, store and orientational average
// ---------------------------------------------------------------------------------------
enum DspType { DSP_AUTOCORRELATE = 0, DSP_SQUARE = 1, DSP_PLAIN = 2 };

// Per-system data of the correlation kernels.
struct CorrSystem {
    const void* A;          // coherent amplitudes [nv][nf]: float2 (FP32) or double2 (FP64)
    const float4* xyz;      // incoherent: staged coordinates [nf][na_pad]
    const void* bfac;       // incoherent: factors [nshell][na_pad]
    const double* qv;       // sub-vectors [nv][3]
    const int* shell_v;     // [nshell+1] sub-vector offsets of each shell
    const void* kbr;        // [L] bit-reversed store kernel: float2 (FP32) or double2 (FP64)
    const float4* qrev;     // FP32 form: sub-vectors in revolutions (q / 2 pi) [nv]
    double cx, cy, cz;      // frame centre (FP32 form) for the plain-dsp phase restore
    int nf, lg, na_pad;
};

// FP32 form: out[v] = (float)(q[v] / 2 pi) once per call, so that the series kernels read the
// sub-vectors they need per (atom, direction) pair without FP64 conversions.
cudaError_t launch_q_revolutions(const double* qv, size_t nv, float4* out, cudaStream_t st);

// Work unit: series [v_begin, v_end) (coherent) or atoms [v_begin, v_end) with all the
// shell's directions (incoherent) of one shell of one system, into one partial slot.
struct CorrChunk {
    int system, shell, v_begin, v_end;
    size_t part_off;        // offset (in doubles) of this slot's partial spectrum / series
    int slot;               // index into apart / a2part
    int pad;
};

struct CorrLaunch {
    int precision, dsp;
    const CorrSystem* systems;
    const CorrChunk* chunks;
    int nchunks;
    int lg_max;             // largest padded length of the batch (shared memory sizing)
    int lg_min;             // smallest padded length (0: not known)
    int nf_max;
    const void* tw;         // [L_max/2] exp(-2 pi i k / L_max), float2 or double2
    int restore_phase;      // FP32 form with dsp=plain: multiply by exp(i q.c)
    double* ppart;          // partial spectra / series (see CorrChunk::part_off)
    double2* apart;         // [nslot]
    double* a2part;         // [nslot]
    unsigned int* err;
};

cudaError_t launch_corr_accumulate(const CorrLaunch& a, cudaStream_t st);  // coherent
cudaError_t launch_self_accumulate(const CorrLaunch& a, cudaStream_t st);  // incoherent

// Per-shell finalisation entry.
struct FinalEntry {
    int slot_begin, slot_end;  // partial slots of this shell (consecutive)
    size_t part_off;           // offset of slot_begin's partial; slots are `part_len` apart
    int part_len;              // L (autocorrelate) or 2*nf (square/plain) doubles per slot
    int f32pair;               // partials are FP32 (Kahan sum, compensation) pairs, not doubles
    int nf, lg;
    double inv_nm;
    double2* fqt;              // [nf]
    double2* fq;
    double2* fq2;
};

struct FinalLaunch {
    int dsp, conj_out;
    const FinalEntry* entries;
    int nentries;
    int lg_max;
    const double* ppart;
    const double2* apart;
    const double* a2part;
    const double2* tw;         // [L_max/2] FP64
};
cudaError_t launch_finalize(const FinalLaunch& a, cudaStream_t st);

// Shared memory of the FFT accumulate kernels for padded length 2^lg.
size_t fft_smem_bytes(int precision, int lg, int nf, bool self);
// Whether the autocorrelation kernels of a launch write their power partials as FP32
// (sum, compensation) pairs (FinalEntry::f32pair): the FP32 form's CTA-per-series kernels.
bool corr_writes_f32_pairs(int precision, int dsp, int lg_max);

// ---------------------------------------------------------------------------------------
// Long series (autocorrelation with padded length 2^14 .. 2^20): four-step FFT through HBM,
// L = R x C with C = 2^kLongRowLg and R = L / C. Spectra are kept in (k1, bit-reversed k2)
// order: index k1 * C + bitrev(k2) holds frequency k1 + R k2.
// ---------------------------------------------------------------------------------------
constexpr int kLongRowLg = 12;
constexpr int kLongLgMax = 20;

struct LongArgs {
    int precision, lg, nf;     // precision of the transforms (Y, twiddles, K)
    int amp_f32;               // the series are float2 (else double2)
    const void* A;             // series [nseries][nf]: the batch's first series
    void* Y;                   // [nseries][L] T2 scratch (column-pass output)
    int nseries;
    const void* tw;            // W_L^j for j < L/2 (T2 of the precision)
    const CorrChunk* chunks;   // row pass: chunk series v reads Y[v - v0]
    int nchunks, v0;
    const void* kbr;           // store kernel K in the long order (T2)
    double* ppart;             // power partial slots (chunk.part_off, L doubles per slot)
    double2* mpart;            // [nv][R] row parts of the series means
    void* xout;                // transform mode: conj(X) in the long order (T2)
};
// Float-float copy (16 bytes per complex value) of an FP64 table: the twiddles and the store
// kernel of the long path's float-float transforms.
cudaError_t launch_to_ff2(const double2* src, size_t n, void* dst, cudaStream_t st);
// Column pass over the batch's series; row pass over its chunks (power, means).
cudaError_t launch_long_columns(const LongArgs& a, cudaStream_t st);
cudaError_t launch_long_rows(const LongArgs& a, cudaStream_t st);
// One series' transform (nseries = 1): xout = conj(FFT_L(x)).
cudaError_t launch_long_transform(const LongArgs& a, cudaStream_t st);
// Incoherent long series: G[p - p0][t] = b_j exp(i q_m . r_j(t)) for pairs p = j * nm + m of
// one shell, p in [p0, p0 + nseries).
struct LongSelfArgs {
    int precision, nf, na_pad, nm, p0, nseries;
    const float4* xyz;         // [nf][na_pad]
    const void* bfac;          // the shell's factor row [na_pad] (T)
    const double* qv;          // the shell's q-vectors [nm][3]
    const float4* qrev;        // FP32 form: the same in revolutions [nm]
    void* G;                   // [nseries][nf] T2
};
cudaError_t launch_long_self_series(const LongSelfArgs& a, cudaStream_t st);
// afinal / a2final partials of every long chunk from the row parts of its series means.
cudaError_t launch_long_means(const CorrChunk* chunks, int nchunks, const double2* mpart, int R, double2* apart,
                              double* a2part, cudaStream_t st);

struct LongFinal {
    const FinalEntry* entries;
    int nentries, lg, conj_out;
    const double* ppart;
    const double2* apart;
    const double* a2part;
    const double2* tw;         // W_L^j, j < L/2, FP64
    double2* Z;                // [nentries][L] scratch
};
cudaError_t launch_long_finalize(const LongFinal& a, cudaStream_t st);
// K of a long system: K(k) = sum_{tau<nf} exp(+2 pi i k tau / L) / (nf L (nf - tau)) in the long
// order, FP64 and FP32 copies; scratch holds nf + L double2.
cudaError_t launch_long_store_kernel(const double2* tw64, int lg, int nf, double2* scratch, double2* k64,
                                     float2* k32, cudaStream_t st);

// FFT tables on the device: tw[k] = exp(-2 pi i k / L) (k < L/2) in FP64 and FP32, and
// the store kernel K at bit-reversed positions for (nf, lg).
cudaError_t launch_twiddles(double2* tw64, float2* tw32, int lg, cudaStream_t st);
cudaError_t launch_store_kernel(const double2* tw64, int lg_tw, double2* k64, float2* k32, int nf,
                                int lg, cudaStream_t st);

// Staging: raw frame-major float [nf][na][3] -> float4 [nf][na_pad] (minus centre); with
// xyz_rec, also the class-sorted copy xyz_rec[f][rec_inv[j]] = (x, y, z, 1). `raw` may be
// host memory the device reads in place.
cudaError_t launch_stage(const float* raw, int nf, int na, int na_pad, double cx, double cy,
                         double cz, int center, float4* xyz, const int* rec_inv, int na_rec,
                         float4* xyz_rec, cudaStream_t st);
// b[s][j] = class_factors[s][cls[j]] (0 for padding atoms), float or double output.
cudaError_t launch_expand_factors(const double* class_factors, int nclass, int nshell,
                                  const int* cls, int na_pad, int precision, void* b,
                                  cudaStream_t st);

}  // namespace sassgpu
