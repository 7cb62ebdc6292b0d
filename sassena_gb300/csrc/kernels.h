// Host-side launch interface of the sassena_gb300 kernels (internal, not the C-ABI).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace sassgpu {

enum Precision { PREC_FP64 = 0, PREC_FP32 = 1 };

// Device-side error codes written to the plan's error word (first writer wins).
enum DeviceError : unsigned int {
    DEV_OK = 0,
    DEV_MBAR_TIMEOUT = 1,  // an mbarrier wait exceeded its iteration limit
    DEV_BAD_SHAPE = 2,     // a kernel saw a shape outside what its host check allowed
};

// Atom padding granule: every device coordinate row holds a multiple of this many
// atoms, so every staged tile is whole and 16-byte aligned.
constexpr int kAtomGranule = 128;

// One CTA-row of the phase sum: `nv` consecutive sub-vectors starting at `v0`,
// all belonging to shell `shell` (so they share the per-atom factors b_j).
struct VecGroup {
    int shell, v0, nv, pad;
};

// Tile shape of the phase-sum kernel: q-vectors per lane, warps (= frames) per
// CTA, atoms per pipeline stage. Only the instantiated shapes are accepted.
struct PhaseTile {
    int q_per_lane;
    int warps;
    int atoms;
};

struct PhaseSumArgs {
    int precision;
    const float4* xyz;        // [nf][na_pad]
    int na_pad, nf;
    const void* bfac;         // [nshell][na_pad] float (FP32) or double (FP64)
    const double* qv;         // [nv_total][3]
    const VecGroup* groups;   // [ngroups]
    int ngroups;
    int nsplit;               // atom splits (grid z)
    int atoms_per_split;      // multiple of the tile's atom count
    double2* out;             // FP64: [nv_total][nf]; FP32 with nsplit > 1: [nsplit][nv_total][nf]
    float2* out_f32;          // FP32 with nsplit == 1: [nv_total][nf]
    size_t split_stride;      // elements between splits of `out`
    unsigned int* err;
    PhaseTile tile;
};

bool phase_tile_supported(int precision, PhaseTile t);
cudaError_t launch_phase_sum(const PhaseSumArgs& a, cudaStream_t st);
// out[v][f] = sum_s part[s][v][f] in split order (FP64), stored as double2 or float2.
cudaError_t launch_split_reduce(const double2* part, int nsplit, size_t n, double2* out,
                                cudaStream_t st);
cudaError_t launch_split_reduce_f32(const double2* part, int nsplit, size_t n, float2* out,
                                    cudaStream_t st);

// Work unit of the correlation / store kernels: series [v_begin, v_end) of one
// shell, reduced into partial slot `slot`.
struct SeriesChunk {
    int shell, v_begin, v_end, slot;
};

// Work unit of the incoherent kernel: atoms [j_begin, j_end) of one shell.
struct AtomChunk {
    int shell, j_begin, j_end, slot;
};

struct CorrArgs {
    int precision;
    int nf, lg;                 // FFT length L = 1 << lg >= 2*nf
    const void* A;              // [nv][nf] amplitudes: float2 (FP32) or double2 (FP64)
    const void* tw;             // [L/2] exp(-2 pi i k / L), float2 (FP32) or double2 (FP64)
    const void* kbr;            // [L] bit-reversed store kernel, same type as tw
    const SeriesChunk* chunks;  // coherent chunks
    const AtomChunk* achunks;   // incoherent chunks
    int nchunks;
    // incoherent inputs
    const float4* xyz;
    int na_pad;
    const double* qv;
    const void* bfac;
    const int* shell_v;         // [nshell+1] sub-vector offsets of each shell
    // plain-dsp phase restore (frame-centred FP32 coordinates): exp(i q.c)
    double cx, cy, cz;
    int restore_phase;
    // partials
    double* ppart;              // [nslot][L] (autocorrelate) or double2 [nslot][nf] (square/plain)
    double2* apart;             // [nslot]
    double* a2part;             // [nslot]
    unsigned int* err;
};

enum DspType { DSP_AUTOCORRELATE = 0, DSP_SQUARE = 1, DSP_PLAIN = 2 };

// Coherent: per series FFT power spectrum / store reductions into partial slots.
cudaError_t launch_corr_accumulate(const CorrArgs& a, int dsp, cudaStream_t st);
// Incoherent: fused series generation + correlation into partial slots.
cudaError_t launch_self_accumulate(const CorrArgs& a, int dsp, cudaStream_t st);

struct FinalizeArgs {
    int nf, lg, dsp, conj_out;
    const double* ppart;        // as produced by the accumulate kernels
    const double2* apart;
    const double* a2part;
    const int* slot_begin;      // [nshell+1] partial slots of each shell
    const double* inv_nm;       // [nshell] 1/NM per shell
    const double2* tw;          // [L/2]
    double2* fqt;               // [nshell][nf]
    double2* fq;                // [nshell]
    double2* fq2;               // [nshell]
    int nshell;
};
cudaError_t launch_finalize(const FinalizeArgs& a, cudaStream_t st);
// Shared memory of the FFT accumulate kernels for padded length 2^lg.
size_t fft_smem_bytes(int precision, int lg, int nf, bool self);

// Staging: raw frame-major float [nf][na][3] -> float4 [nf][na_pad] (minus centre).
cudaError_t launch_stage(const float* raw, int nf, int na, int na_pad, double cx, double cy,
                         double cz, int center, float4* xyz, cudaStream_t st);
// b[s][j] = class_factors[s][cls[j]] (0 for padding atoms), float or double output.
cudaError_t launch_expand_factors(const double* class_factors, int nclass, int nshell,
                                  const int* cls, int na_pad, int precision, void* b,
                                  cudaStream_t st);

}  // namespace sassgpu
