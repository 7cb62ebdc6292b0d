// Allocation-free entry point: coherent autocorrelation + orientational average
// from caller-provided amplitudes, with all working memory in one fixed,
// file-scope device array.
//
// Who this is for: code that must not allocate GPU memory while it runs. Examples
// are a host program that reserves all device memory up front and forbids further
// cudaMalloc (a fixed memory budget shared with other solvers), code that runs
// inside a memory-pool allocator's callback, and services that must not risk an
// out-of-memory failure in the middle of a run. sass_compute allocates its working
// buffers on demand; sass_correlate_noalloc instead uses the static array below,
// which exists from the moment the library is loaded on a device.
//
// Limits: at most kMaxQ q-vectors per call and NF <= 4096 (padded FFT length 8192).
// The array holds kScratchBytes (8,601,856 bytes, 8.2 MiB) on every GPU that loads the library,
// until the process exits.
//
// Sharing: every call uses the same array and the array keeps the previous call's
// contents. The partial sums are fully rewritten by each call before they are read.
// The FFT twiddles and the store-kernel table depend only on NF; the array records,
// in a tag word written by the device, which NF its tables were built for. Every
// call enqueues the table kernels, and they return at once when the tag already
// names this call's NF, so the decision is taken on the GPU in stream order and no
// host-side cache can go stale. Two calls that overlap on the GPU (different
// streams, or different host threads) race on the array and corrupt each other's
// results. Serialise calls, e.g. by issuing them on one stream.
//
// First call per device: the device address of the array is looked up with
// cudaGetSymbolAddress (with that device current) on the first call that uses the
// device. Make that first call before capturing work into a CUDA graph. A device
// reset (cudaDeviceReset) while the library is loaded is not supported: the
// address looked up before the reset is kept.
//
// Sub-vector offsets are 64-bit in the interface but the correlation descriptors
// index sub-vectors with 32-bit integers: the total number of sub-vectors must stay
// below 2^31. A q whose offsets are not increasing, or lie beyond that limit, gets
// NaN outputs instead of reading outside the amplitudes.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sassena_gb300.h"
#include "common.cuh"
#include "kernels.h"

using namespace sassgpu;

namespace {

constexpr int kNoAllocMaxLg = 13;          // padded length 8192 => NF <= 4096
constexpr int kMaxL = 1 << kNoAllocMaxLg;
constexpr int kMaxQ = 128;                 // q-vectors per call
constexpr int kMaxSlots = 128;             // partial slots (chunks) per call
constexpr int kMaxDevices = 64;

// Byte layout of the scratch array (all offsets multiples of 256).
constexpr size_t kOffPart = 0;                                             // double [slots][L]
constexpr size_t kOffApart = kOffPart + (size_t)kMaxSlots * kMaxL * 8;     // double2 [slots]
constexpr size_t kOffA2 = kOffApart + kMaxSlots * 16;                      // double [slots]
constexpr size_t kOffTag = kOffA2 + kMaxSlots * 8;                         // int: NF of the tables
constexpr size_t kOffTw = kOffA2 + kMaxSlots * 8 + 1024;                   // double2 [L/2]
constexpr size_t kOffK = kOffTw + (size_t)(kMaxL / 2) * 16;                // double2 [L]
constexpr size_t kOffChunks = kOffK + (size_t)kMaxL * 16;                  // CorrChunk [slots]
constexpr size_t kOffEntries = kOffChunks + kMaxSlots * 32;                // FinalEntry [Q]
constexpr size_t kOffSystem = kOffEntries + kMaxQ * 64;                    // CorrSystem
constexpr size_t kScratchBytes = kOffSystem + 256;
static_assert(sizeof(CorrChunk) <= 32 && sizeof(FinalEntry) <= 64 && sizeof(CorrSystem) <= 256,
              "descriptor sizes of the fixed layout");
static_assert(kScratchBytes == 8601856, "documented scratch size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceState {
    bool ready = false;
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch
};
std::mutex g_lock;
DeviceState g_dev[kMaxDevices];

// tw[k] = exp(-2 pi i k / L), k < L/2 (FP64 sincospi). Skipped when the tag says the
// tables already belong to this NF (the tag is written by noalloc_schedule, which runs
// after both table kernels on the stream).
__global__ void noalloc_twiddles(double2* tw, int L, const int* tag, int nf) {
    if (*tag == nf) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L / 2; k += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(-2.0 * (double)k / (double)L, &s, &c);
        tw[k] = make_double2(c, s);
    }
}

// K at bit-reversed position i: K(w) = sum_{tau<NF} exp(+2 pi i w tau / L) / (NF L (NF-tau)),
// the weights that turn a power spectrum into the tau-mean of the normalised correlation.
__global__ void noalloc_store_kernel_table(const double2* __restrict__ tw, double2* kbr, int nf,
                                           int lg, const int* tag) {
    if (*tag == nf) return;
    const int L = 1 << lg;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < L; w += gridDim.x * blockDim.x) {
        double re = 0.0, im = 0.0;
        long long m = 0;  // (w * tau) mod L
        for (int t = 0; t < nf; ++t) {
            const double wt = 1.0 / ((double)nf * (double)L * (double)(nf - t));
            // exp(+2 pi i m / L) = conj(tw[m]) for m < L/2, -conj(tw[m - L/2]) otherwise
            double2 z = m < L / 2 ? tw[m] : tw[m - L / 2];
            double sg = m < L / 2 ? 1.0 : -1.0;
            re += wt * sg * z.x;
            im -= wt * sg * z.y;
            m += w;
            if (m >= L) m -= L;
        }
        int i = __brev((unsigned)w) >> (32 - lg);
        kbr[i] = make_double2(re, im);
    }
}

// Offsets of q s, or an empty range when they are not increasing or exceed the
// 32-bit sub-vector index of the correlation descriptors.
__device__ __forceinline__ bool noalloc_range(const unsigned long long* offs, int s, long long& b,
                                              long long& e) {
    const unsigned long long ub = offs[s], ue = offs[s + 1];
    if (ue < ub || ue > 0x7fffffffull) {
        b = e = 0;
        return false;
    }
    b = (long long)ub;
    e = (long long)ue;
    return true;
}

// Descriptors of one call, written on the device from the device-side offsets: g chunks
// per q (some possibly empty), one finalisation entry per q, the system record. Last,
// the tag records that the tables now hold this call's NF.
__global__ void noalloc_schedule(const unsigned long long* __restrict__ offs, int nq, int g, int nf, int lg,
                                 const double2* A, const double2* kbr, double2* fqt, double2* fq, double2* fq2,
                                 CorrChunk* chunks, FinalEntry* entries, CorrSystem* sys, int* tag) {
    const size_t L = (size_t)1 << lg;
    for (int c = threadIdx.x; c < nq * g; c += blockDim.x) {
        const int s = c / g, k = c - s * g;
        long long b, e;
        noalloc_range(offs, s, b, e);
        const long long nm = e - b;
        const long long len = nm > 0 ? (nm + g - 1) / g : 0;
        long long vb = b + k * len, ve = vb + len;
        if (vb > e) vb = e;
        if (ve > e) ve = e;
        CorrChunk ch;
        ch.system = 0;
        ch.shell = s;
        ch.v_begin = (int)vb;
        ch.v_end = (int)ve;
        ch.part_off = (size_t)c * L;
        ch.slot = c;
        ch.pad = 0;
        chunks[c] = ch;
    }
    for (int s = threadIdx.x; s < nq; s += blockDim.x) {
        long long b, en;
        const bool valid = noalloc_range(offs, s, b, en);
        const long long nm = en - b;
        FinalEntry e;
        e.slot_begin = s * g;
        e.slot_end = (s + 1) * g;
        e.part_off = (size_t)s * g * L;
        e.part_len = L;
        e.f32pair = 0;  // FP64 partials
        e.nf = nf;
        e.lg = lg;
        e.inv_nm = valid && nm > 0 ? 1.0 / (double)nm : __longlong_as_double(0x7ff8000000000000LL);
        e.fqt = fqt + (size_t)s * nf;
        e.fq = fq + s;
        e.fq2 = fq2 + s;
        entries[s] = e;
    }
    if (threadIdx.x == 0) {
        CorrSystem y;
        y.A = A;
        y.xyz = nullptr;
        y.bfac = nullptr;
        y.qv = nullptr;
        y.shell_v = nullptr;
        y.kbr = kbr;
        y.qrev = nullptr;  // FP64 only
        y.cx = y.cy = y.cz = 0.0;
        y.nf = nf;
        y.lg = lg;
        y.na_pad = 0;
        *sys = y;
        *tag = nf;
    }
}

}  // namespace

extern "C" int sass_correlate_noalloc(int device, void* stream, const double* amplitudes, size_t nf,
                                      size_t nq, const uint64_t* sub_offsets, int dsp_method,
                                      double* fqt, double* fq, double* fq2) {
    if (!amplitudes || !sub_offsets || !fqt || !fq || !fq2) return SASS_ERR_ARG;
    if (nf == 0 || nq == 0) return SASS_ERR_ARG;
    if (dsp_method != SASS_METHOD_FFTW && dsp_method != SASS_METHOD_DIRECT) return SASS_ERR_ARG;
    if (device < 0 || device >= kMaxDevices) return SASS_ERR_ARG;
    int lg = 2;
    while (((size_t)1 << lg) < 2 * nf) ++lg;
    if (lg > kNoAllocMaxLg || nq > (size_t)kMaxQ) return SASS_ERR_UNSUPPORTED;  // beyond the fixed array
    cudaStream_t st = (cudaStream_t)stream;

    std::lock_guard<std::mutex> guard(g_lock);
    if (cudaSetDevice(device) != cudaSuccess) return SASS_ERR_CUDA;
    DeviceState& ds = g_dev[device];
    if (!ds.ready) {
        void* addr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
        if (e != cudaSuccess || addr == nullptr) {
            cudaGetLastError();
            return SASS_ERR_CUDA;
        }
        ds.base = static_cast<unsigned char*>(addr);
        ds.ready = true;
    }
    unsigned char* b = ds.base;
    double2* tw = reinterpret_cast<double2*>(b + kOffTw);
    double2* kbr = reinterpret_cast<double2*>(b + kOffK);
    int* tag = reinterpret_cast<int*>(b + kOffTag);
    {
        const int L = 1 << lg;
        noalloc_twiddles<<<(L / 2 + 255) / 256, 256, 0, st>>>(tw, L, tag, (int)nf);
        noalloc_store_kernel_table<<<(L + 127) / 128, 128, 0, st>>>(tw, kbr, (int)nf, lg, tag);
        if (cudaGetLastError() != cudaSuccess) return SASS_ERR_CUDA;
    }
    const int g = kMaxSlots / (int)nq;  // chunks per q (>= 1)
    CorrChunk* chunks = reinterpret_cast<CorrChunk*>(b + kOffChunks);
    FinalEntry* entries = reinterpret_cast<FinalEntry*>(b + kOffEntries);
    CorrSystem* sys = reinterpret_cast<CorrSystem*>(b + kOffSystem);
    noalloc_schedule<<<1, 256, 0, st>>>(reinterpret_cast<const unsigned long long*>(sub_offsets), (int)nq, g,
                                        (int)nf, lg, reinterpret_cast<const double2*>(amplitudes), kbr,
                                        reinterpret_cast<double2*>(fqt), reinterpret_cast<double2*>(fq),
                                        reinterpret_cast<double2*>(fq2), chunks, entries, sys, tag);
    if (cudaGetLastError() != cudaSuccess) return SASS_ERR_CUDA;

    CorrLaunch ca{};
    ca.precision = PREC_FP64;
    ca.dsp = DSP_AUTOCORRELATE;
    ca.systems = sys;
    ca.chunks = chunks;
    ca.nchunks = (int)nq * g;
    ca.lg_max = lg;
    ca.lg_min = lg;
    ca.nf_max = (int)nf;
    ca.tw = tw;
    ca.ppart = reinterpret_cast<double*>(b + kOffPart);
    ca.apart = reinterpret_cast<double2*>(b + kOffApart);
    ca.a2part = reinterpret_cast<double*>(b + kOffA2);
    if (launch_corr_accumulate(ca, st) != cudaSuccess) return SASS_ERR_CUDA;

    FinalLaunch fa{};
    fa.dsp = DSP_AUTOCORRELATE;
    fa.conj_out = dsp_method == SASS_METHOD_DIRECT;
    fa.entries = entries;
    fa.nentries = (int)nq;
    fa.lg_max = lg;
    fa.ppart = ca.ppart;
    fa.apart = ca.apart;
    fa.a2part = ca.a2part;
    fa.tw = tw;
    if (launch_finalize(fa, st) != cudaSuccess) return SASS_ERR_CUDA;
    return SASS_OK;
}
