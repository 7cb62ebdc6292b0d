// Scheduling and launch engine shared by the single-plan path (sass_compute), the
// batched path (sass_batch_*) and the autotuner: turns a list of systems with their
// q-vectors into descriptor lists, working buffers and a launch sequence that contains
// no host synchronisation (so it can be captured into a CUDA graph).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "kernels.h"

namespace sassgpu {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n);
    void release();
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
    ~DevBuf() { release(); }
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
};

struct HostPinned {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n);
    void release();
    ~HostPinned() { release(); }
    HostPinned() = default;
    HostPinned(const HostPinned&) = delete;
    HostPinned& operator=(const HostPinned&) = delete;
};

// One staged trajectory on the device.
struct SystemState {
    size_t na = 0, nf = 0, na_pad = 0, nclass = 0;
    int lg = 0;  // padded FFT length 2^lg >= 2 nf
    double center[3] = {0, 0, 0};
    DevBuf raw, xyz, cls, tw64, tw32, k64, k32;
    DevBuf twff, kff;  // long series: float-float twiddles [L/2] and store kernel [L] (16 B each)
    bool staged = false, classes_set = false;
    uint64_t class_gen = 0;  // counts class assignments (part of a prepared engine's key)
    // frames to copy ahead into `raw` (prefetch_system, issue_prefetch): the host buffer, the
    // event that completes the copy once issued (null: not issued yet), and the buffer this
    // library page-locked for it (null: none)
    const float* prefetch_src = nullptr;
    cudaEvent_t prefetch_done = nullptr;
    void* prefetch_locked = nullptr;
    // class-sorted copy for the shell-recurrence kernel (built on first use)
    std::vector<int32_t> h_cls;   // [na] classes (host copy)
    DevBuf xyz_rec, block_class;  // [nf][na_rec] float4 with w; [na_rec / 32] int
    DevBuf rec_map, rec_inv;      // [na_rec] atom of each slot (-1: padding); [na] slot of each atom
    size_t na_rec = 0;
    bool rec_map_ok = false;      // rec_map, rec_inv, block_class and na_rec follow the classes
    bool rec_ready = false;       // xyz_rec exists with this map's padding slots zeroed: staging fills it
    bool rec_valid = false;       // xyz_rec holds the staged frames
    // multipole devices: coordinates in the spherical or cylindrical representation
    DevBuf mp_xyz;  // [nf][na_pad] float4
    int mp_type = -1;
    bool mp_valid = false;
    double mp_axis[3] = {0, 0, 0};
};

struct EngineConfig {
    int scattering = 0, dsp = 0, method = 0, precision = 0;
    PhaseShape shape{0, 0, 0};  // q_per_lane 0: automatic
    int split_atoms = 0;        // atoms per phase-sum tile (0: automatic)
    int rec_k = 0;              // shells per lane of the recurrence kernel: 0 automatic, -1 off
    int device = 0;
};

// One system's q-vectors in a launch. All pointers are device pointers except `offs`.
struct WorkItem {
    SystemState* sys = nullptr;
    std::vector<size_t> offs;  // [nq+1] sub-vector offsets, offs[0] == 0
    const double* d_qv = nullptr;
    // optional product structure: qv[offs[s] + d] = lam[s] * qv[offs[base] + d] for every
    // shell s (see detect_product); empty: general sub-vectors
    std::vector<double> lam;
    int lam_base = -1;
    const double* d_cf = nullptr;  // [nq][nclass]
    double2* d_fqt = nullptr;      // [nq][nf]
    double2* d_fq = nullptr;       // [nq]
    double2* d_fq2 = nullptr;      // [nq]
    // optional (coherent): sqrt of a positive weight per sub-vector; the engine then also
    // writes the weighted averages (1/NM) sum_v w_v C_v(t) into the *_w outputs
    const double* d_wsqrt = nullptr;  // [nv]
    double2* d_fqt_w = nullptr;
    double2* d_fq_w = nullptr;
    double2* d_fq2_w = nullptr;
    // optional (coherent, FP64): amplitudes computed elsewhere ([nv][nf] double2, e.g. the
    // multipole devices); the engine runs no phase sum for the item, only the correlation
    // and the average, scaled by `norm` instead of 1/NM
    const double2* d_amp_given = nullptr;
    double norm = 0;
};

struct EngineStats {
    size_t phase_tiles = 0, corr_chunks = 0, final_entries = 0, launches = 0, phase_launches = 0;
    size_t rec_tiles = 0, rec_shells = 0, rec_groups = 0;
    int rec_k = 0, max_split = 1;
    PhaseShape shape{0, 0, 0};
    int split_atoms = 0;
    double terms = 0;
};

// Allocate the FFT tables of a system (device kernels); needs the stream only for order.
int build_system_tables(SystemState& s, cudaStream_t st, std::string& err);
// Stage frame-major float32 [nf][na][3] (host or device) into `s` (centred for FP32).
int stage_system(SystemState& s, const float* coords, bool on_device, int precision, cudaStream_t st,
                 std::string& err);
int set_system_classes(SystemState& s, const int32_t* cls, bool on_device, cudaStream_t st, std::string& err);
// Request the copy of host frames `coords` into `s.raw` for the next stage_system of the same
// buffer (page-locking pageable memory the device can map). issue_prefetch queues the copy
// on stream `side`, with completion event `done`: the plan calls it once its next compute
// has queued its own input copies, so that the copy engine takes those first and the frame
// copy overlaps the kernels. stage_system of that buffer then waits for `done` and converts
// from `raw`; a request never issued is staged as usual.
int prefetch_system(SystemState& s, const float* coords, std::string& err);
int issue_prefetch(SystemState& s, cudaStream_t side, cudaEvent_t done, std::string& err);
// Wait for an issued prefetch copy (if any) on the host and release what the request holds.
void drop_prefetch(SystemState& s);

// Whether shells [0, nq) of host sub-vectors qv (offsets offs) are multiples of one base
// set: equal counts per shell and qv[offs[s] + d] = lam[s] * qv[offs[base] + d] within
// 1e-12 of the shell's largest sub-vector. Fills lam and base on success.
bool detect_product(const double* qv, const std::vector<size_t>& offs, std::vector<double>& lam, int& base);
// Maximal runs [a, e) of at least min_len shells whose lam lies on a line within
// 2.5e-7 of the run's largest |lam| (float-rounded linear scans qualify).
std::vector<std::pair<int, int>> arithmetic_runs(const std::vector<double>& lam, int min_len);

class Engine {
public:
    // Build descriptors and working buffers for `items`; uploads the descriptors
    // (synchronously) so that enqueue() is free of host work.
    int prepare(const EngineConfig& cfg, const std::vector<WorkItem>& items, std::string& err);
    // Enqueue the whole computation on `st`. With `events` non-null, records
    // [phase start, phase end, corr end, finalize end] (not while capturing).
    int enqueue(cudaStream_t st, std::string& err, cudaEvent_t* events = nullptr);
    const EngineStats& stats() const { return stats_; }
    unsigned int* err_word() const { return err_.as<unsigned int>(); }
    // prepare() calls after the first with the same configuration and items (same inputs,
    // outputs and system generations) keep the descriptors and skip the host work
    // the amplitudes of item i after enqueue() (coherent): float2 (FP32) or double2 [nv][nf]
    const void* amplitudes(int i) const { return amp_.as<unsigned char>() + amp_off_[i]; }
    void release();

private:
    int prepare_full(const EngineConfig& cfg, const std::vector<WorkItem>& items, std::string& err);
    std::vector<uint64_t> key_;  // what the current descriptors were built for (empty: none)
    EngineConfig cfg_;
    EngineStats stats_;
    int lg_max_ = 2, lg_min_ = 2, nf_max_ = 1, nitems_ = 0;
    std::vector<int> nsplit_;
    std::vector<size_t> item_nv_, item_nf_;
    std::vector<std::pair<double2*, double2*>> split_part_;  // (partials, FP64 out) per item
    std::vector<float2*> split_out32_;   // FP32 form: amplitudes the split partials reduce into
    std::vector<float2*> split_part32_;  // FP32 form: the FP32 split partials
    std::vector<const double*> item_cf_;
    std::vector<SystemState*> item_sys_;
    std::vector<size_t> item_nq_;
    int nphase_systems_ = 0, ntiles_ = 0, nchunks_ = 0, nentries_ = 0;
    int nrec_tiles_ = 0, nrec_groups_ = 0, rec_k_ = 0;
    RecSystem* d_rsys_ = nullptr;
    RecGroup* d_rgroups_ = nullptr;
    RecTileDesc* d_rtiles_ = nullptr;
    DevBuf blob_, bfac_, amp_, part_, ppart_, apart_, a2part_, counter_, err_, tw64_, tw32_, rec_bfac_;
    HostPinned hblob_;
    std::vector<size_t> bfac_off_, amp_off_, part_off_;
    PhaseSystem* d_psys_ = nullptr;
    PhaseTileDesc* d_tiles_ = nullptr;
    CorrSystem* d_csys_ = nullptr;
    CorrChunk* d_chunks_ = nullptr;
    FinalEntry* d_entries_ = nullptr;
    FinalEntry* d_entries_w_ = nullptr;  // weighted outputs (same slots)
    std::vector<const double*> item_wsqrt_;
    bool weighted_ = false;
    int tw_lg_ = 0;
    // long series (autocorrelation, padded length above 2^kMaxLg): four-step transform
    struct LongBatch {
        int item, v0, v1, chunk_begin, chunk_end;  // series [v0, v1) in Y; chunks of the batch
        int shell, p0;                             // incoherent: the shell and its first pair
    };
    struct LongItem {
        int item, lg;
        int chunk_begin, chunk_end, entry_begin, entry_end, batch_begin, batch_end;
        size_t mpart_off;  // double2 offset of the item's [nv][R] mean parts
    };
    std::vector<LongBatch> long_batches_;
    std::vector<LongItem> long_items_;
    std::vector<const void*> item_amp_;
    std::vector<std::vector<size_t>> item_offs_;
    std::vector<const double*> item_qv_;
    CorrChunk* d_long_chunks_ = nullptr;
    FinalEntry* d_long_entries_ = nullptr;
    DevBuf long_Y_, long_mpart_, long_Z_, long_G_, qrev_;
    std::vector<size_t> qrev_off_;
};

// HBM scratch for the column-pass output of one batch of long series.
constexpr size_t kLongScratchBytes = (size_t)2 << 30;

int sm_count(int device);

}  // namespace sassgpu
