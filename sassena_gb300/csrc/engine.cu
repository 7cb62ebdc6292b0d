#include "engine.h"
#include "mlp.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sassgpu {

cudaError_t DevBuf::ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    return e;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

cudaError_t HostPinned::ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    release();
    cudaError_t e = cudaHostAlloc(&p, n ? n : 16, cudaHostAllocDefault);
    if (e == cudaSuccess) bytes = n ? n : 16;
    else p = nullptr;
    return e;
}

void HostPinned::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
}

int sm_count(int device) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) n = 1;
    return n;
}

namespace {

// Status codes (mirror include/sassena_gb300.h).
constexpr int kOk = 0, kErrArg = 1, kErrOom = 2, kErrUnsupported = 3, kErrCuda = 4;

int fail_cuda(cudaError_t e, const char* what, std::string& err) {
    cudaGetLastError();
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? kErrOom : kErrCuda;
}

#define ECK(expr)                                               \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return fail_cuda(e_, #expr, err); \
    } while (0)

template <class T>
size_t push(std::vector<unsigned char>& blob, const std::vector<T>& v) {
    size_t off = (blob.size() + 255) & ~(size_t)255;
    blob.resize(off + v.size() * sizeof(T));
    if (!v.empty()) memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
    return off;
}

PhaseShape default_shape(int precision, size_t min_nm) {
    if (precision == PREC_FP64) return PhaseShape{min_nm >= 64 ? 2 : 1, 4, 64};
    int q = 1;
    for (int cand : {8, 4, 2}) {  // the largest Q that wastes little of a shell's lanes
        size_t per = 32 * (size_t)cand;
        size_t groups = (min_nm + per - 1) / per;
        double waste = 1.0 - (double)min_nm / (double)(groups * per);
        if (waste <= 0.15) {
            q = cand;
            break;
        }
    }
    return PhaseShape{q, 8, 128};
}

}  // namespace

int build_system_tables(SystemState& s, cudaStream_t st, std::string& err) {
    const size_t L = (size_t)1 << s.lg;
    ECK(s.tw64.ensure(L / 2 * sizeof(double2)));
    ECK(s.tw32.ensure(L / 2 * sizeof(float2)));
    ECK(s.k64.ensure(L * sizeof(double2)));
    ECK(s.k32.ensure(L * sizeof(float2)));
    ECK(launch_twiddles(s.tw64.as<double2>(), s.tw32.as<float2>(), s.lg, st));
    if (s.lg > kMaxLg) {  // long layout, built by the four-step transform of the window
        DevBuf scratch;
        ECK(scratch.ensure((s.nf + L) * sizeof(double2)));
        ECK(launch_long_store_kernel(s.tw64.as<double2>(), s.lg, (int)s.nf, scratch.as<double2>(),
                                     s.k64.as<double2>(), s.k32.as<float2>(), st));
        // float-float copies for the FP32 form's long transforms
        ECK(s.twff.ensure(L / 2 * 16));
        ECK(s.kff.ensure(L * 16));
        ECK(launch_to_ff2(s.tw64.as<double2>(), L / 2, s.twff.p, st));
        ECK(launch_to_ff2(s.k64.as<double2>(), L, s.kff.p, st));
        ECK(cudaStreamSynchronize(st));
        return kOk;
    }
    ECK(launch_store_kernel(s.tw64.as<double2>(), s.lg, s.k64.as<double2>(), s.k32.as<float2>(), (int)s.nf, s.lg,
                            st));
    ECK(cudaStreamSynchronize(st));
    return kOk;
}

// The address under which the device reads host memory `h` in place, or nullptr: the
// device alias of pinned or registered memory, managed memory as is, and any other host
// pointer where the device reads pageable memory through the host's page tables (Grace
// with address translation over NVLink-C2C; `pageable` is then set). Reading in place
// fuses the transfer with the conversion; the link bounds both equally (about 209 GB/s
// measured on a GB300, copy engine and SM loads alike).
static const float* device_view(const float* h, int device, bool& pageable) {
    pageable = false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return reinterpret_cast<const float*>(a.devicePointer);
    if (a.type == cudaMemoryTypeManaged) return h;
    if (a.type == cudaMemoryTypeDevice) return nullptr;
    int access = 0;
    if (cudaDeviceGetAttribute(&access, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    pageable = access != 0;
    return pageable ? h : nullptr;
}

// Unlocks a caller's buffer that this library page-locked, once the work that reads it is
// done (the stream has drained and, for a prefetch copy, its completion event has fired),
// when it goes out of scope.
struct ScopedHostRegistration {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    ~ScopedHostRegistration() {
        if (!p) return;
        (void)cudaStreamSynchronize(st);
        if (done) (void)cudaEventSynchronize(done);
        if (cudaHostUnregister(p) != cudaSuccess) (void)cudaGetLastError();
    }
};

int stage_system(SystemState& s, const float* coords, bool on_device, int precision, cudaStream_t st,
                 std::string& err) {
    if (!coords) {
        err = "coords is NULL";
        return kErrArg;
    }
    const size_t n = s.nf * s.na * 3;
    // device memory first: a plan that does not fit reads nothing of the caller's buffer
    ECK(s.xyz.ensure(s.nf * s.na_pad * sizeof(float4)));
    const float* src = coords;
    std::vector<float> f0(s.na * 3);
    // A prefetch request: an issued copy may still be writing `raw`, so the stream waits for
    // it, and a copy of this very buffer is the source. A buffer locked for the request is
    // unlocked once the stream has drained (the guards run at return, after the final
    // synchronize). A request never issued is dropped and the frames are staged as usual.
    const bool from_prefetch = s.prefetch_done && !on_device && s.prefetch_src == coords;
    ScopedHostRegistration prefetch_pin;
    if (s.prefetch_src) {
        prefetch_pin.p = s.prefetch_locked;
        prefetch_pin.st = st;
        prefetch_pin.done = s.prefetch_done;
        const cudaEvent_t done = s.prefetch_done;
        s.prefetch_src = nullptr;
        s.prefetch_done = nullptr;
        s.prefetch_locked = nullptr;
        if (done) ECK(cudaStreamWaitEvent(st, done, 0));
    }
    ScopedHostRegistration pin;
    if (from_prefetch) {
        src = s.raw.as<float>();
        memcpy(f0.data(), coords, f0.size() * sizeof(float));
    } else if (!on_device) {
        int device = 0;
        ECK(cudaGetDevice(&device));
        bool pageable = false;
        src = device_view(coords, device, pageable);
        // Pageable memory the device could read through the host's page tables is
        // page-locked for this call and read through its device mapping instead: on a
        // GB300 (Grace host), in-place reads of a buffer the GPU had read before slowed
        // down with every reuse (11.2 GB of coordinates, 64 systems: 1.30, 1.42, 1.63,
        // 1.78 s over four batches), while locking, reading and unlocking took 0.13 to
        // 0.16 s each time. Where locking fails (a range partly locked elsewhere, say),
        // the device reads the pages in place as before.
        if (pageable) {
            if (cudaHostRegister(const_cast<float*>(coords), n * sizeof(float), cudaHostRegisterDefault) ==
                cudaSuccess) {
                pin.p = const_cast<float*>(coords);
                pin.st = st;
                void* dp = nullptr;
                if (cudaHostGetDevicePointer(&dp, pin.p, 0) == cudaSuccess && dp) src = static_cast<const float*>(dp);
                else (void)cudaGetLastError();
            } else {
                (void)cudaGetLastError();
            }
        }
        if (!src) {
            ECK(s.raw.ensure(n * sizeof(float)));
            ECK(cudaMemcpyAsync(s.raw.p, coords, n * sizeof(float), cudaMemcpyHostToDevice, st));
            src = s.raw.as<float>();
        }
        memcpy(f0.data(), coords, f0.size() * sizeof(float));
    } else {
        ECK(cudaMemcpyAsync(f0.data(), coords, f0.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
        ECK(cudaStreamSynchronize(st));
    }
    // FP32 form: fixed centre = midpoint of frame 0's bounding box (FP64)
    double c[3] = {0, 0, 0};
    if (precision == PREC_FP32) {
        for (int k = 0; k < 3; ++k) {
            double lo = f0[k], hi = f0[k];
            for (size_t j = 1; j < s.na; ++j) {
                lo = std::min(lo, (double)f0[3 * j + k]);
                hi = std::max(hi, (double)f0[3 * j + k]);
            }
            c[k] = 0.5 * (lo + hi);
        }
        if (!std::isfinite(c[0]) || !std::isfinite(c[1]) || !std::isfinite(c[2])) {
            err = "non-finite coordinates in frame 0";
            return kErrArg;
        }
    }
    memcpy(s.center, c, sizeof(c));
    // the class-sorted copy, once it exists for the current classes, is filled in the same pass
    const bool rec = s.rec_ready && s.rec_map_ok;
    ECK(launch_stage(src, (int)s.nf, (int)s.na, (int)s.na_pad, c[0], c[1], c[2], precision == PREC_FP32,
                     s.xyz.as<float4>(), rec ? s.rec_inv.as<int>() : nullptr, (int)s.na_rec,
                     rec ? s.xyz_rec.as<float4>() : nullptr, st));
    ECK(cudaStreamSynchronize(st));
    s.staged = true;
    s.rec_valid = rec;
    s.mp_valid = false;
    return kOk;
}

int prefetch_system(SystemState& s, const float* coords, std::string& err) {
    if (!coords) {
        err = "coords is NULL";
        return kErrArg;
    }
    drop_prefetch(s);  // one copy ahead at a time
    const size_t bytes = s.nf * s.na * 3 * sizeof(float);
    ECK(s.raw.ensure(bytes));
    int device = 0;
    ECK(cudaGetDevice(&device));
    bool pageable = false;
    (void)device_view(coords, device, pageable);
    // pageable memory the device can map is locked until the staging that uses the copy, so
    // that the copy engine reads it asynchronously (as the staging itself would lock it)
    if (pageable) {
        if (cudaHostRegister(const_cast<float*>(coords), bytes, cudaHostRegisterDefault) == cudaSuccess)
            s.prefetch_locked = const_cast<float*>(coords);
        else
            (void)cudaGetLastError();
    }
    s.prefetch_src = coords;
    return kOk;
}

int issue_prefetch(SystemState& s, cudaStream_t side, cudaEvent_t done, std::string& err) {
    if (!s.prefetch_src || s.prefetch_done) return kOk;  // nothing requested, or already issued
    // `raw` is free: every staging that reads it synchronises before it returns
    const size_t bytes = s.nf * s.na * 3 * sizeof(float);
    cudaError_t e = cudaMemcpyAsync(s.raw.p, s.prefetch_src, bytes, cudaMemcpyDefault, side);
    if (e == cudaSuccess) e = cudaEventRecord(done, side);
    if (e != cudaSuccess) {
        (void)cudaStreamSynchronize(side);
        if (s.prefetch_locked && cudaHostUnregister(s.prefetch_locked) != cudaSuccess) (void)cudaGetLastError();
        s.prefetch_src = nullptr;
        s.prefetch_locked = nullptr;
        return fail_cuda(e, "prefetch copy", err);
    }
    s.prefetch_done = done;
    return kOk;
}

void drop_prefetch(SystemState& s) {
    if (s.prefetch_done && cudaEventSynchronize(s.prefetch_done) != cudaSuccess) (void)cudaGetLastError();
    if (s.prefetch_locked && cudaHostUnregister(s.prefetch_locked) != cudaSuccess) (void)cudaGetLastError();
    s.prefetch_src = nullptr;
    s.prefetch_done = nullptr;
    s.prefetch_locked = nullptr;
}

int set_system_classes(SystemState& s, const int32_t* cls, bool on_device, cudaStream_t st, std::string& err) {
    if (!cls) {
        err = "atom_class is NULL";
        return kErrArg;
    }
    std::vector<int32_t> h(s.na_pad, -1);
    if (on_device) ECK(cudaMemcpy(h.data(), cls, s.na * sizeof(int32_t), cudaMemcpyDeviceToHost));
    else memcpy(h.data(), cls, s.na * sizeof(int32_t));
    for (size_t j = 0; j < s.na; ++j)
        if (h[j] < 0 || (size_t)h[j] >= s.nclass) {
            err = "atom " + std::to_string(j) + " has class " + std::to_string(h[j]) + " outside [0," +
                  std::to_string(s.nclass) + ")";
            return kErrArg;
        }
    ECK(s.cls.ensure(s.na_pad * sizeof(int32_t)));
    ECK(cudaMemcpyAsync(s.cls.p, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    ECK(cudaStreamSynchronize(st));
    s.h_cls.assign(h.begin(), h.begin() + s.na);
    s.classes_set = true;
    ++s.class_gen;
    s.rec_map_ok = s.rec_ready = s.rec_valid = false;
    s.mp_valid = false;  // the cylinder representation carries the classes
    return kOk;
}

bool detect_product(const double* qv, const std::vector<size_t>& offs, std::vector<double>& lam, int& base) {
    lam.clear();
    base = -1;
    const size_t nq = offs.size() - 1;
    if (nq == 0 || !qv) return false;
    const size_t nd = offs[1] - offs[0];
    for (size_t s = 0; s < nq; ++s)
        if (offs[s + 1] - offs[s] != nd) return false;
    // base: the shell with the largest sub-vector (least relative rounding)
    double best = 0;
    for (size_t s = 0; s < nq; ++s)
        for (size_t d = 0; d < nd; ++d) {
            const double* v = qv + 3 * (offs[s] + d);
            const double n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            if (n2 > best) {
                best = n2;
                base = (int)s;
            }
        }
    if (base < 0 || !(best > 0) || !std::isfinite(best)) return false;
    const double* u = qv + 3 * offs[base];
    double uu = 0;
    for (size_t d = 0; d < nd; ++d) uu += u[3 * d] * u[3 * d] + u[3 * d + 1] * u[3 * d + 1] + u[3 * d + 2] * u[3 * d + 2];
    lam.assign(nq, 0.0);
    for (size_t s = 0; s < nq; ++s) {
        const double* v = qv + 3 * offs[s];
        double uv = 0, vmax = 0;
        for (size_t d = 0; d < 3 * nd; ++d) uv += u[d] * v[d];
        const double l = (int)s == base ? 1.0 : uv / uu;
        for (size_t d = 0; d < nd; ++d) {
            const double* w = v + 3 * d;
            vmax = std::max(vmax, std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]));
        }
        const double tol = 1e-12 * std::max(vmax, std::fabs(l) * std::sqrt(best));
        for (size_t d = 0; d < 3 * nd; ++d)
            if (!(std::fabs(v[d] - l * u[d]) <= tol)) {
                lam.clear();
                base = -1;
                return false;
            }
        lam[s] = l;
    }
    return true;
}

std::vector<std::pair<int, int>> arithmetic_runs(const std::vector<double>& lam, int min_len) {
    std::vector<std::pair<int, int>> out;
    const int n = (int)lam.size();
    auto on_line = [&](int a, int e) {  // shells [a, e] on the line through a and e
        const double step = (lam[e] - lam[a]) / (double)(e - a);
        double scale = 0;
        for (int k = a; k <= e; ++k) scale = std::max(scale, std::fabs(lam[k]));
        for (int k = a + 1; k < e; ++k)
            if (!(std::fabs(lam[k] - (lam[a] + (double)(k - a) * step)) <= 2.5e-7 * scale)) return false;
        return std::isfinite(step);
    };
    int a = 0;
    while (a < n) {
        int e = a + 1;
        while (e < n && on_line(a, e)) ++e;
        if (e - a >= min_len) out.emplace_back(a, e);
        a = (e - a >= min_len) ? e : a + 1;
    }
    return out;
}

namespace {

// Per-lane cost of a group of K shells, in units of one recurrence step (2 FMA + 2 FADD):
// K steps plus the per-atom dot product, two reduced sin/cos pairs and the seed rotation
// (about 22 FP32 operations).
double rec_group_cost(int K) { return K + 5.5; }

int choose_rec_k(const std::vector<std::vector<std::pair<int, int>>>& runs) {
    int best = 0;
    double best_cost = 1e300;
    for (int K : rec_shell_counts()) {
        double c = 0;
        for (const auto& r : runs)
            for (const auto& ae : r) c += std::ceil((double)(ae.second - ae.first) / K) * rec_group_cost(K);
        if (c < best_cost) {
            best_cost = c;
            best = K;
        }
    }
    return best;
}

// Class-sorted layout for the recurrence kernel: class segments padded to 32 atoms, w = 1
// / 0 in float4.w, rows padded to the 128-atom stage. The slot map follows the classes;
// the coordinates follow each staging (filled by the staging kernel once the copy exists).
int build_rec_map(SystemState& s, std::string& err) {
    if (s.h_cls.size() != s.na) {
        err = "atom classes missing";
        return kErrArg;
    }
    std::vector<std::vector<int>> members(s.nclass);
    for (size_t j = 0; j < s.na; ++j) members[s.h_cls[j]].push_back((int)j);
    std::vector<int> map, bcls;
    int last = 0;
    for (size_t c = 0; c < s.nclass; ++c) {
        if (members[c].empty()) continue;
        for (int j : members[c]) map.push_back(j);
        while (map.size() % 32) map.push_back(-1);
        bcls.resize(map.size() / 32, (int)c);
        last = (int)c;
    }
    while (map.size() % 128 || map.empty()) map.push_back(-1);
    bcls.resize(map.size() / 32, last);
    // block information: class in the low 16 bits, padding atoms of the block above
    for (size_t b = 0; b < bcls.size(); ++b) {
        int npad = 0;
        for (int j = 0; j < 32; ++j) npad += map[32 * b + j] < 0;
        bcls[b] |= npad << 16;
    }
    std::vector<int> inv(s.na);
    for (size_t i = 0; i < map.size(); ++i)
        if (map[i] >= 0) inv[map[i]] = (int)i;
    if (s.na_rec != map.size()) s.rec_ready = false;
    s.na_rec = map.size();
    ECK(s.rec_map.ensure(map.size() * sizeof(int)));
    ECK(cudaMemcpy(s.rec_map.p, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice));
    ECK(s.rec_inv.ensure(inv.size() * sizeof(int)));
    ECK(cudaMemcpy(s.rec_inv.p, inv.data(), inv.size() * sizeof(int), cudaMemcpyHostToDevice));
    ECK(s.block_class.ensure(bcls.size() * sizeof(int)));
    ECK(cudaMemcpy(s.block_class.p, bcls.data(), bcls.size() * sizeof(int), cudaMemcpyHostToDevice));
    s.rec_map_ok = true;
    return kOk;
}

int ensure_rec_layout(SystemState& s, std::string& err) {
    if (s.rec_valid && s.rec_map_ok) return kOk;
    if (!s.rec_map_ok) {
        int rc = build_rec_map(s, err);
        if (rc) return rc;
    }
    ECK(s.xyz_rec.ensure(s.nf * s.na_rec * sizeof(float4)));
    ECK(launch_permute_stage(s.xyz.as<float4>(), (int)s.na_pad, s.rec_map.as<int>(), (int)s.na_rec, (int)s.nf,
                             s.xyz_rec.as<float4>(), 0));
    ECK(cudaDeviceSynchronize());
    s.rec_valid = s.rec_ready = true;
    return kOk;
}

}  // namespace

void Engine::release() {
    key_.clear();
    DevBuf* bufs[] = {&blob_,    &bfac_, &amp_, &part_,  &ppart_, &apart_,
                      &a2part_, &counter_, &err_, &tw64_, &tw32_, &rec_bfac_};
    for (DevBuf* b : bufs) b->release();
    hblob_.release();
}

// Everything the descriptors depend on: the configuration and, per item, the system (its
// class assignment's generation, its staged buffers, the staging's centre and whether the
// class-sorted copy holds the staged frames), the sub-vector offsets, the product structure
// and every device pointer. The contents behind the device pointers (coordinates,
// sub-vectors, factors, weights) are read by the kernels at enqueue, not here, so a new
// staging of the same system with the same centre keeps the descriptors.
static std::vector<uint64_t> prepare_key(const EngineConfig& c, const std::vector<WorkItem>& items) {
    std::vector<uint64_t> k;
    auto u = [&](uint64_t v) { k.push_back(v); };
    auto p = [&](const void* v) { k.push_back((uint64_t)(uintptr_t)v); };
    auto d = [&](double v) {
        uint64_t b;
        memcpy(&b, &v, sizeof(b));
        k.push_back(b);
    };
    u((uint64_t)c.scattering);
    u((uint64_t)c.dsp);
    u((uint64_t)c.method);
    u((uint64_t)c.precision);
    u((uint64_t)(uint32_t)c.shape.q_per_lane);
    u((uint64_t)(uint32_t)c.shape.warps);
    u((uint64_t)(uint32_t)c.shape.atoms);
    u((uint64_t)(uint32_t)c.shape.poly_pairs);
    u((uint64_t)(uint32_t)c.split_atoms);
    u((uint64_t)(uint32_t)c.rec_k);
    u((uint64_t)(uint32_t)c.device);
    u(items.size());
    for (const WorkItem& it : items) {
        p(it.sys);
        if (it.sys) {
            const SystemState& s = *it.sys;
            u(s.class_gen);
            u((uint64_t)s.staged | (uint64_t)s.classes_set << 1 | (uint64_t)s.rec_valid << 2 |
              (uint64_t)s.rec_map_ok << 3 | (uint64_t)s.rec_ready << 4);
            for (int c3 = 0; c3 < 3; ++c3) d(s.center[c3]);
            p(s.xyz.p);
            p(s.xyz_rec.p);
            p(s.block_class.p);
            p(s.cls.p);
            u(s.na_rec);
        }
        u(it.offs.size());
        for (size_t o : it.offs) u(o);
        u(it.lam.size());
        for (double l : it.lam) d(l);
        u((uint64_t)(int64_t)it.lam_base);
        for (const void* q : {(const void*)it.d_qv, (const void*)it.d_cf, (const void*)it.d_fqt,
                              (const void*)it.d_fq, (const void*)it.d_fq2, (const void*)it.d_wsqrt,
                              (const void*)it.d_fqt_w, (const void*)it.d_fq_w, (const void*)it.d_fq2_w,
                              (const void*)it.d_amp_given})
            p(q);
        d(it.norm);
    }
    return k;
}

int Engine::prepare(const EngineConfig& cfg, const std::vector<WorkItem>& items, std::string& err) {
    if (!key_.empty() && prepare_key(cfg, items) == key_) return kOk;
    key_.clear();
    const int rc = prepare_full(cfg, items, err);
    // taken after the preparation, which may build the class-sorted copy of a system
    if (rc == kOk) key_ = prepare_key(cfg, items);
    return rc;
}

int Engine::prepare_full(const EngineConfig& cfg, const std::vector<WorkItem>& items, std::string& err) {
    cfg_ = cfg;
    stats_ = EngineStats();
    const bool f32 = cfg.precision == PREC_FP32;
    const bool coherent = cfg.scattering == 0;
    const bool autoc = cfg.dsp == DSP_AUTOCORRELATE;
    const size_t bsz = f32 ? 4 : 8;
    nitems_ = (int)items.size();
    if (items.empty()) {
        err = "no work";
        return kErrArg;
    }
    const int sms = sm_count(cfg.device);

    // ---- shape and sizes ----------------------------------------------------------------
    size_t min_nm = (size_t)-1, total_shells = 0;
    lg_max_ = 2;
    lg_min_ = kMaxLg;
    nf_max_ = 1;
    // systems whose padded length exceeds the shared-memory transforms take the long path
    std::vector<char> long_item(items.size(), 0);
    for (size_t i = 0; i < items.size(); ++i) {
        const WorkItem& it = items[i];
        for (size_t s = 0; s + 1 < it.offs.size(); ++s) min_nm = std::min(min_nm, it.offs[s + 1] - it.offs[s]);
        total_shells += it.offs.size() - 1;
        if (autoc && it.sys->lg > kMaxLg) {
            if (it.sys->lg > kLongLgMax) {
                err = "autocorrelation supports NF <= 524288";
                return kErrUnsupported;
            }
            if (it.d_wsqrt) {
                err = "weighted averages need NF <= 4096";
                return kErrUnsupported;
            }
            long_item[i] = 1;
            continue;
        }
        lg_max_ = std::max(lg_max_, it.sys->lg);
        lg_min_ = std::min(lg_min_, it.sys->lg);
        nf_max_ = std::max(nf_max_, (int)it.sys->nf);
    }
    PhaseShape shape = cfg.shape.q_per_lane ? cfg.shape : default_shape(cfg.precision, min_nm);
    if (coherent && !phase_shape_supported(cfg.precision, shape)) {
        err = "phase tile shape not instantiated";
        return kErrUnsupported;
    }
    stats_.shape = shape;

    // ---- shell-recurrence groups (FP32 form; shells along one direction set) ---------------------
    std::vector<std::vector<char>> rec_on(items.size());
    std::vector<RecGroup> rgroups;
    std::vector<int> item_g0(items.size(), 0), item_ng(items.size(), 0), item_nd(items.size(), 0);
    rec_k_ = 0;
    if (f32 && coherent && cfg.rec_k >= 0) {
        std::vector<std::vector<std::pair<int, int>>> runs(items.size());
        bool any = false;
        for (size_t i = 0; i < items.size(); ++i) {
            const WorkItem& it = items[i];
            if (it.lam.size() + 1 != it.offs.size() || it.lam_base < 0 || it.sys->nclass > (size_t)kRecMaxClass)
                continue;
            runs[i] = arithmetic_runs(it.lam, 3);
            any = any || !runs[i].empty();
        }
        if (any) {
            rec_k_ = cfg.rec_k > 0 ? cfg.rec_k : choose_rec_k(runs);
            if (!rec_shells_supported(rec_k_)) {
                err = "recurrence shell count " + std::to_string(rec_k_) + " not instantiated";
                return kErrUnsupported;
            }
        }
        for (size_t i = 0; rec_k_ && i < items.size(); ++i) {
            if (runs[i].empty()) continue;
            const WorkItem& it = items[i];
            int rc = ensure_rec_layout(*it.sys, err);
            if (rc) return rc;
            rec_on[i].assign(it.offs.size() - 1, 0);
            item_g0[i] = (int)rgroups.size();
            item_nd[i] = (int)(it.offs[1] - it.offs[0]);
            for (const auto& ae : runs[i]) {
                const int n = ae.second - ae.first, ng = (n + rec_k_ - 1) / rec_k_;
                int s0 = ae.first;
                for (int g = 0; g < ng; ++g) {  // near-equal groups of at most K shells
                    const int ks = n / ng + (g < n % ng ? 1 : 0);
                    RecGroup rg{};
                    rg.system = (int)i;
                    rg.s0 = s0;
                    rg.ks = ks;
                    rg.lam0 = it.lam[s0];
                    rg.dlam = ks > 1 ? (it.lam[s0 + ks - 1] - it.lam[s0]) / (double)(ks - 1) : 0.0;
                    rgroups.push_back(rg);
                    for (int k = 0; k < ks; ++k) rec_on[i][s0 + k] = 1;
                    s0 += ks;
                    stats_.rec_shells += ks;
                }
            }
            item_ng[i] = (int)rgroups.size() - item_g0[i];
        }
    }
    auto is_rec = [&](size_t i, size_t sh) { return !rec_on[i].empty() && rec_on[i][sh]; };
    stats_.rec_k = rec_k_;
    stats_.rec_groups = rgroups.size();

    // atom splits: enough tiles for the persistent grid to balance
    nsplit_.assign(items.size(), 1);
    size_t base_tiles = 0;
    for (size_t i = 0; i < items.size(); ++i) {
        const WorkItem& it = items[i];
        size_t groups = 0;
        for (size_t s = 0; s + 1 < it.offs.size(); ++s)
            if (!is_rec(i, s))
                groups += (it.offs[s + 1] - it.offs[s] + 32 * shape.q_per_lane - 1) / (32 * shape.q_per_lane);
        base_tiles += groups * ((it.sys->nf + shape.warps - 1) / shape.warps);
        if (item_ng[i]) base_tiles += ((size_t)item_ng[i] * item_nd[i] + 31) / 32 * ((it.sys->nf + 7) / 8);
    }
    const size_t target = (size_t)sms * 8;
    for (size_t i = 0; i < items.size(); ++i) {
        int max_split = (int)(items[i].sys->na_pad / shape.atoms);
        if (item_ng[i]) max_split = std::min(max_split, (int)(items[i].sys->na_rec / 128));
        int ns = 1;
        if (cfg.split_atoms > 0) {
            ns = (int)((items[i].sys->na_pad + cfg.split_atoms - 1) / cfg.split_atoms);
        } else if (base_tiles < target) {
            ns = (int)((target + base_tiles - 1) / std::max<size_t>(base_tiles, 1));
        } else if (items.size() == 1) {
            // Enough tiles, but the last round of the persistent grid can leave SMs idle:
            // an SM runs about tiles * s / SMs tiles of ceil(stages / s) atom stages each.
            // Take the split count that minimises ceil(tiles * s / SMs) * ceil(stages / s),
            // charging each extra split 0.4 % of the unsplit time for its partials and
            // their reduction. (coherent S(q,t) workload on GB300, 2,048 tiles of 79 stages:
            // s = 2 gives 26.95 tiles per SM and a 2.4 % shorter step than s = 1.)
            const long long nst = item_ng[i] ? (long long)(items[i].sys->na_rec / 128)
                                              : (long long)(items[i].sys->na_pad / shape.atoms);
            const double t1 = (double)base_tiles;
            auto cost = [&](int sp) {
                const double per_sm = std::ceil(t1 * sp / (double)sms - 1e-9);
                return per_sm * (double)((nst + sp - 1) / sp);
            };
            const double c1 = cost(1);
            double best = c1;
            for (int sp = 2; sp <= std::min(8, max_split); ++sp) {
                const double c = cost(sp) + 0.004 * c1 * (sp - 1);
                if (c < best) {
                    best = c;
                    ns = sp;
                }
            }
        }
        // each split writes partials of the item's whole amplitude array (FP32 pairs in the
        // FP32 form, FP64 pairs in the FP64 form): at most 4 GiB of them (items that large have
        // tiles enough without splits, and allocating and freeing tens of GB, as small split
        // sizes on large systems would, slows every later allocation of the process)
        const size_t per_split = (size_t)items[i].offs.back() * items[i].sys->nf * (f32 ? 8 : 16);
        const int budget = (int)std::max<size_t>(1, ((size_t)1 << 32) / std::max<size_t>(per_split, 1));
        nsplit_[i] = items[i].d_amp_given ? 1 : std::max(1, std::min(std::min(ns, max_split), budget));
        stats_.max_split = std::max(stats_.max_split, nsplit_[i]);
    }
    stats_.split_atoms = cfg.split_atoms;

    // ---- working buffers ---------------------------------------------------------------
    bfac_off_.assign(items.size(), 0);
    amp_off_.assign(items.size(), 0);
    part_off_.assign(items.size(), 0);
    size_t bfac_bytes = 0, amp_bytes = 0, part_bytes = 0;
    for (size_t i = 0; i < items.size(); ++i) {
        const WorkItem& it = items[i];
        const size_t nq = it.offs.size() - 1, nv = it.offs.back(), nf = it.sys->nf;
        bfac_off_[i] = bfac_bytes;
        bfac_bytes += ((nq * it.sys->na_pad * bsz + 255) & ~(size_t)255);
        if (coherent && !it.d_amp_given) {
            amp_off_[i] = amp_bytes;
            amp_bytes += ((nv * nf * (f32 ? 8 : 16) + 255) & ~(size_t)255);
            if (nsplit_[i] > 1) {
                part_off_[i] = part_bytes;
                part_bytes += (size_t)nsplit_[i] * nv * nf * (f32 ? 8 : 16);
            }
        }
        stats_.terms += (double)nv * (double)it.sys->na * (double)nf;
    }
    ECK(bfac_.ensure(bfac_bytes));
    if (coherent) ECK(amp_.ensure(amp_bytes));
    if (part_bytes) ECK(part_.ensure(part_bytes));

    // FP32 form: sub-vectors in revolutions, one table per call (filled in enqueue)
    qrev_off_.assign(items.size(), 0);
    size_t qrev_total = 0;
    for (size_t i = 0; i < items.size(); ++i) {
        qrev_off_[i] = qrev_total;
        qrev_total += items[i].offs.back();
    }
    if (f32) ECK(qrev_.ensure(std::max<size_t>(1, qrev_total) * sizeof(float4)));

    // ---- phase-sum descriptors -------------------------------------------------------------
    std::vector<PhaseSystem> psys(items.size());
    std::vector<PhaseTileDesc> tiles;
    std::vector<CorrSystem> csys(items.size());
    std::vector<std::vector<int>> shell_v(items.size());
    item_nv_.assign(items.size(), 0);
    item_nf_.assign(items.size(), 0);
    split_part_.assign(items.size(), {nullptr, nullptr});
    split_out32_.assign(items.size(), nullptr);
    split_part32_.assign(items.size(), nullptr);
    item_cf_.assign(items.size(), nullptr);
    item_sys_.assign(items.size(), nullptr);
    item_nq_.assign(items.size(), 0);
    item_amp_.assign(items.size(), nullptr);
    item_offs_.assign(items.size(), {});
    item_qv_.assign(items.size(), nullptr);
    for (size_t i = 0; i < items.size(); ++i) {
        item_offs_[i] = items[i].offs;
        item_qv_[i] = items[i].d_qv;
    }
    for (size_t i = 0; i < items.size(); ++i) {
        const WorkItem& it = items[i];
        SystemState& s = *it.sys;
        const size_t nq = it.offs.size() - 1, nv = it.offs.back();
        item_nv_[i] = nv;
        item_nf_[i] = s.nf;
        item_cf_[i] = it.d_cf;
        item_sys_[i] = it.sys;
        item_nq_[i] = nq;
        for (size_t k = 0; k <= nq; ++k) shell_v[i].push_back((int)it.offs[k]);
        void* bfac = bfac_.as<unsigned char>() + bfac_off_[i];
        PhaseSystem& p = psys[i];
        p.xyz = s.xyz.as<float4>();
        p.bfac = bfac;
        p.qv = it.d_qv;
        p.na_pad = (int)s.na_pad;
        p.nf = (int)s.nf;
        p.split_stride = nv * s.nf;
        void* amp = coherent ? (void*)(amp_.as<unsigned char>() + amp_off_[i]) : nullptr;
        if (it.d_amp_given) amp = const_cast<double2*>(it.d_amp_given);
        item_amp_[i] = amp;
        if (coherent && !it.d_amp_given) {
            if (nsplit_[i] > 1) {
                unsigned char* part = part_.as<unsigned char>() + part_off_[i];
                if (f32) {  // FP32 partials (8 bytes per frame), summed in float-float by the reduction
                    p.out = nullptr;
                    p.out_f32 = reinterpret_cast<float2*>(part);
                    split_part32_[i] = reinterpret_cast<float2*>(part);
                    split_out32_[i] = reinterpret_cast<float2*>(amp);
                } else {
                    p.out = reinterpret_cast<double2*>(part);
                    p.out_f32 = nullptr;
                    split_part_[i] = {reinterpret_cast<double2*>(part), reinterpret_cast<double2*>(amp)};
                }
            } else {
                p.out = f32 ? nullptr : reinterpret_cast<double2*>(amp);
                p.out_f32 = f32 ? reinterpret_cast<float2*>(amp) : nullptr;
            }
            const int per = 32 * shape.q_per_lane;
            // balanced split of the stages: no slice is empty since nsplit <= stages
            const long long nst = (long long)(s.na_pad / shape.atoms), ns = nsplit_[i];
            // frame tiles outermost: the tiles that read the same frames run together, so
            // the coordinates stream from HBM about once and the other reads hit L2
            for (size_t f0 = 0; f0 < s.nf; f0 += shape.warps)
                for (size_t sh = 0; sh < nq; ++sh) {
                    if (is_rec(i, sh)) continue;
                    for (size_t v = it.offs[sh]; v < it.offs[sh + 1]; v += per)
                        for (int sp = 0; sp < nsplit_[i]; ++sp) {
                            PhaseTileDesc t;
                            t.system = (int)i;
                            t.shell = (int)sh;
                            t.v0 = (int)v;
                            t.nv = (int)std::min<size_t>(per, it.offs[sh + 1] - v);
                            t.f0 = (int)f0;
                            t.j_begin = (int)(sp * nst / ns) * shape.atoms;
                            t.j_end = (int)((sp + 1) * nst / ns) * shape.atoms;
                            t.split = sp;
                            tiles.push_back(t);
                        }
            }
        }
        CorrSystem& c = csys[i];
        c.A = amp;
        c.xyz = s.xyz.as<float4>();
        c.bfac = bfac;
        c.qv = it.d_qv;
        c.shell_v = nullptr;  // patched after upload
        c.kbr = f32 ? (const void*)s.k32.p : (const void*)s.k64.p;
        c.qrev = f32 ? qrev_.as<float4>() + qrev_off_[i] : nullptr;
        c.cx = s.center[0];
        c.cy = s.center[1];
        c.cz = s.center[2];
        c.nf = (int)s.nf;
        c.lg = s.lg;
        c.na_pad = (int)s.na_pad;
    }
    // longest tiles first (cost ~ atoms x active frames) for the persistent queue
    std::stable_sort(tiles.begin(), tiles.end(), [&](const PhaseTileDesc& a, const PhaseTileDesc& b) {
        auto cost = [&](const PhaseTileDesc& t) {
            long long fr = std::min<long long>(shape.warps, (long long)psys[t.system].nf - t.f0);
            return (long long)(t.j_end - t.j_begin) * fr;
        };
        return cost(a) > cost(b);
    });
    ntiles_ = (int)tiles.size();
    nphase_systems_ = (int)items.size();

    // recurrence tiles: 32 (group, direction) pairs x 8 frames x atom slice
    std::vector<RecSystem> rsys(items.size());
    std::vector<RecTileDesc> rtiles;
    for (size_t i = 0; i < items.size(); ++i) {
        if (!item_ng[i]) continue;
        const WorkItem& it = items[i];
        SystemState& s = *it.sys;
        RecSystem& r = rsys[i];
        r.xyzw = s.xyz_rec.as<float4>();
        r.block_class = s.block_class.as<int>();
        r.cf = it.d_cf;
        r.dirs = it.d_qv + 3 * it.offs[it.lam_base];
        r.out = psys[i].out;
        r.out_f32 = psys[i].out_f32;
        r.split_stride = psys[i].split_stride;
        r.na_rec = (int)s.na_rec;
        r.nf = (int)s.nf;
        r.nd = item_nd[i];
        r.nclass = (int)s.nclass;
        r.g_begin = item_g0[i];
        const int pairs = item_ng[i] * item_nd[i];
        const long long nst = (long long)(s.na_rec / 128), ns = nsplit_[i];
        for (size_t f0 = 0; f0 < s.nf; f0 += 8)  // frame tiles outermost (L2 reuse)
            for (int p0 = 0; p0 < pairs; p0 += 32)
                for (int sp = 0; sp < nsplit_[i]; ++sp) {
                    RecTileDesc t{};
                    t.system = (int)i;
                    t.p0 = p0;
                    t.np = std::min(32, pairs - p0);
                    t.f0 = (int)f0;
                    t.j_begin = (int)(sp * nst / ns) * 128;
                    t.j_end = (int)((sp + 1) * nst / ns) * 128;
                    t.split = sp;
                    rtiles.push_back(t);
                }
    }
    std::stable_sort(rtiles.begin(), rtiles.end(), [&](const RecTileDesc& a, const RecTileDesc& b) {
        auto cost = [&](const RecTileDesc& t) {
            long long fr = std::min<long long>(8, (long long)rsys[t.system].nf - t.f0);
            return (long long)(t.j_end - t.j_begin) * fr;
        };
        return cost(a) > cost(b);
    });
    nrec_tiles_ = (int)rtiles.size();
    nrec_groups_ = (int)rgroups.size();
    if (nrec_groups_) ECK(rec_bfac_.ensure((size_t)nrec_groups_ * kRecMaxClass * rec_k_ * sizeof(float)));

    // ---- correlation chunks and finalisation entries ------------------------------------------
    std::vector<CorrChunk> chunks;
    std::vector<FinalEntry> entries, entries_w;
    weighted_ = false;
    item_wsqrt_.assign(items.size(), nullptr);
    for (size_t i = 0; i < items.size(); ++i)
        if (items[i].d_wsqrt) {
            if (!coherent) {
                err = "weighted averages need the coherent path";
                return kErrArg;
            }
            weighted_ = true;
            item_wsqrt_[i] = items[i].d_wsqrt;
        }
    const size_t per_shell = std::max<size_t>(1, ((size_t)sms * 8 + total_shells - 1) / total_shells);
    size_t poff = 0;
    int slot = 0;
    for (size_t i = 0; i < items.size(); ++i) {
        if (long_item[i]) continue;
        const WorkItem& it = items[i];
        SystemState& s = *it.sys;
        const size_t L = (size_t)1 << s.lg;
        const size_t plen = autoc ? L : 2 * s.nf;
        for (size_t sh = 0; sh + 1 < it.offs.size(); ++sh) {
            FinalEntry e{};
            e.slot_begin = slot;
            e.part_off = poff;
            e.part_len = (int)plen;
            e.nf = (int)s.nf;
            e.lg = s.lg;
            e.inv_nm = it.norm > 0 ? it.norm : 1.0 / (double)(it.offs[sh + 1] - it.offs[sh]);
            e.fqt = it.d_fqt + sh * s.nf;
            e.fq = it.d_fq + sh;
            e.fq2 = it.d_fq2 + sh;
            e.f32pair = corr_writes_f32_pairs(cfg.precision, cfg.dsp, lg_max_) ? 1 : 0;
            const size_t units = coherent ? it.offs[sh + 1] - it.offs[sh] : s.na;
            const size_t g = std::min(per_shell, units);
            const size_t len = (units + g - 1) / g;
            for (size_t u = 0; u < units; u += len) {
                CorrChunk c{};
                c.system = (int)i;
                c.shell = (int)sh;
                c.v_begin = (int)((coherent ? it.offs[sh] : 0) + u);
                c.v_end = (int)((coherent ? it.offs[sh] : 0) + std::min(units, u + len));
                c.part_off = poff;
                c.slot = slot++;
                poff += plen;
                chunks.push_back(c);
            }
            e.slot_end = slot;
            entries.push_back(e);
            if (it.d_wsqrt) {
                FinalEntry ew = e;
                ew.fqt = it.d_fqt_w + sh * s.nf;
                ew.fq = it.d_fq_w + sh;
                ew.fq2 = it.d_fq2_w + sh;
                entries_w.push_back(ew);
            }
        }
    }
    // long series: chunks of one shell's series (about 2 CTAs per SM over all rows), batches
    // of consecutive chunks whose series fit the column-pass scratch, one entry per shell
    std::vector<CorrChunk> lchunks;
    std::vector<FinalEntry> lentries;
    long_batches_.clear();
    long_items_.clear();
    size_t mpart_total = 0, ybytes = 0, zbytes = 0, gbytes = 0;
    for (size_t i = 0; i < items.size(); ++i) {
        if (!long_item[i]) continue;
        const WorkItem& it = items[i];
        SystemState& s = *it.sys;
        const size_t L = (size_t)1 << s.lg, R = L >> kLongRowLg, nq = it.offs.size() - 1;
        const size_t esz = sizeof(double2);  // FP64 or float-float transforms: 16 bytes a value (see enqueue)
        const size_t gsz = f32 ? sizeof(float2) : sizeof(double2);
        // incoherent: the (atom, direction) series are generated per batch next to Y
        const size_t S = std::max<size_t>(1, kLongScratchBytes / (L * esz + (coherent ? 0 : s.nf * gsz)));
        LongItem li{};
        li.item = (int)i;
        li.lg = s.lg;
        li.mpart_off = mpart_total;
        li.chunk_begin = (int)lchunks.size();
        li.entry_begin = (int)lentries.size();
        li.batch_begin = (int)long_batches_.size();
        const size_t per = std::max<size_t>(1, (2 * (size_t)sms + R * nq - 1) / (R * nq));
        std::vector<CorrChunk> ic;
        size_t vbase = 0;  // incoherent: first series of the shell (pairs of earlier shells)
        for (size_t sh = 0; sh < nq; ++sh) {
            FinalEntry e{};
            e.slot_begin = slot;
            e.part_off = poff;
            e.part_len = (int)L;
            e.nf = (int)s.nf;
            e.lg = s.lg;
            e.inv_nm = it.norm > 0 ? it.norm : 1.0 / (double)(it.offs[sh + 1] - it.offs[sh]);
            e.fqt = it.d_fqt + sh * s.nf;
            e.fq = it.d_fq + sh;
            e.fq2 = it.d_fq2 + sh;
            const size_t nm = it.offs[sh + 1] - it.offs[sh];
            const size_t units = coherent ? nm : s.na * nm;
            const size_t first = coherent ? it.offs[sh] : vbase;
            vbase += units;
            // chunks short enough that one batch of S series also fills the GPU: the row
            // pass launches R CTAs per chunk of the batch (at 16,384 frames, chunks of 250
            // series left 128 CTAs per launch on 152 SMs)
            const size_t fill = std::max<size_t>(1, S * R / (2 * (size_t)sms));
            const size_t len = std::min(std::min(S, fill), (units + std::min(per, units) - 1) / std::min(per, units));
            for (size_t u = 0; u < units; u += len) {
                CorrChunk c{};
                c.system = (int)i;
                c.shell = (int)sh;
                c.v_begin = (int)(first + u);
                c.v_end = (int)(first + std::min(units, u + len));
                c.part_off = poff;
                c.slot = slot++;
                poff += L;
                ic.push_back(c);
            }
            e.slot_end = slot;
            lentries.push_back(e);
        }
        if (vbase > (size_t)INT32_MAX) {
            err = "too many (atom, direction) series for one call; split the q-vectors";
            return kErrArg;
        }
        mpart_total += (coherent ? it.offs.back() : vbase) * R;
        // batches of consecutive chunks within S series (incoherent: within one shell)
        std::vector<size_t> shell_first(nq + 1, 0);
        for (size_t sh = 0; sh < nq; ++sh) shell_first[sh + 1] = shell_first[sh] + s.na * (it.offs[sh + 1] - it.offs[sh]);
        for (size_t cb = 0; cb < ic.size();) {
            size_t ce = cb + 1;
            while (ce < ic.size() && (size_t)(ic[ce].v_end - ic[cb].v_begin) <= S && ce - cb < 65535 &&
                   (coherent || ic[ce].shell == ic[cb].shell))
                ++ce;
            LongBatch b{(int)i, ic[cb].v_begin, ic[ce - 1].v_end, li.chunk_begin + (int)cb, li.chunk_begin + (int)ce,
                        ic[cb].shell, coherent ? 0 : ic[cb].v_begin - (int)shell_first[ic[cb].shell]};
            long_batches_.push_back(b);
            ybytes = std::max(ybytes, (size_t)(b.v1 - b.v0) * L * esz);
            if (!coherent) gbytes = std::max(gbytes, (size_t)(b.v1 - b.v0) * s.nf * gsz);
            cb = ce;
        }
        lchunks.insert(lchunks.end(), ic.begin(), ic.end());
        li.chunk_end = (int)lchunks.size();
        li.entry_end = (int)lentries.size();
        li.batch_end = (int)long_batches_.size();
        zbytes = std::max(zbytes, (size_t)(li.entry_end - li.entry_begin) * L * sizeof(double2));
        long_items_.push_back(li);
    }
    if (!long_items_.empty()) {
        ECK(long_Y_.ensure(ybytes));
        ECK(long_mpart_.ensure(mpart_total * sizeof(double2)));
        ECK(long_Z_.ensure(zbytes));
        if (gbytes) ECK(long_G_.ensure(gbytes));
    }
    nchunks_ = (int)chunks.size();
    nentries_ = (int)entries.size();
    ECK(ppart_.ensure(poff * sizeof(double)));
    ECK(apart_.ensure(slot * sizeof(double2)));
    ECK(a2part_.ensure(slot * sizeof(double)));
    ECK(counter_.ensure(2 * sizeof(unsigned)));
    ECK(err_.ensure(sizeof(unsigned)));

    // shared twiddle table at the largest length
    if (tw_lg_ != lg_max_ || !tw64_.p) {
        const size_t Lm = (size_t)1 << lg_max_;
        ECK(tw64_.ensure(Lm / 2 * sizeof(double2)));
        ECK(tw32_.ensure(Lm / 2 * sizeof(float2)));
        ECK(launch_twiddles(tw64_.as<double2>(), tw32_.as<float2>(), lg_max_, 0));
        tw_lg_ = lg_max_;
    }

    // ---- upload all descriptors in one copy ------------------------------------------------------
    std::vector<unsigned char> blob;
    std::vector<size_t> shell_off(items.size());
    for (size_t i = 0; i < items.size(); ++i) shell_off[i] = push(blob, shell_v[i]);
    size_t o_psys = push(blob, psys), o_tiles = push(blob, tiles);
    size_t o_rsys = push(blob, rsys), o_rgroups = push(blob, rgroups), o_rtiles = push(blob, rtiles);
    // CorrSystem.shell_v points into the blob: patch with the final device address
    ECK(blob_.ensure(blob.size() + 8192 + csys.size() * sizeof(CorrSystem) +
                     (chunks.size() + lchunks.size()) * sizeof(CorrChunk) +
                     (entries.size() + entries_w.size() + lentries.size()) * sizeof(FinalEntry) + 4096));
    for (size_t i = 0; i < items.size(); ++i)
        csys[i].shell_v = reinterpret_cast<const int*>(blob_.as<unsigned char>() + shell_off[i]);
    size_t o_csys = push(blob, csys), o_chunks = push(blob, chunks), o_entries = push(blob, entries);
    size_t o_entries_w = push(blob, entries_w);
    size_t o_lchunks = push(blob, lchunks), o_lentries = push(blob, lentries);
    if (blob.size() > blob_.bytes) {
        err = "descriptor blob sizing";
        return kErrArg;
    }
    ECK(hblob_.ensure(blob.size()));
    memcpy(hblob_.p, blob.data(), blob.size());
    ECK(cudaMemcpy(blob_.p, hblob_.p, blob.size(), cudaMemcpyHostToDevice));
    unsigned char* base = blob_.as<unsigned char>();
    d_psys_ = reinterpret_cast<PhaseSystem*>(base + o_psys);
    d_tiles_ = reinterpret_cast<PhaseTileDesc*>(base + o_tiles);
    d_rsys_ = reinterpret_cast<RecSystem*>(base + o_rsys);
    d_rgroups_ = reinterpret_cast<RecGroup*>(base + o_rgroups);
    d_rtiles_ = reinterpret_cast<RecTileDesc*>(base + o_rtiles);
    d_csys_ = reinterpret_cast<CorrSystem*>(base + o_csys);
    d_chunks_ = reinterpret_cast<CorrChunk*>(base + o_chunks);
    d_entries_ = reinterpret_cast<FinalEntry*>(base + o_entries);
    d_entries_w_ = reinterpret_cast<FinalEntry*>(base + o_entries_w);
    d_long_chunks_ = reinterpret_cast<CorrChunk*>(base + o_lchunks);
    d_long_entries_ = reinterpret_cast<FinalEntry*>(base + o_lentries);
    ECK(cudaDeviceSynchronize());
    stats_.phase_tiles = tiles.size();
    stats_.rec_tiles = rtiles.size();
    stats_.corr_chunks = chunks.size() + lchunks.size();
    stats_.final_entries = entries.size() + lentries.size();
    return kOk;
}

int Engine::enqueue(cudaStream_t st, std::string& err, cudaEvent_t* ev) {
    const bool f32 = cfg_.precision == PREC_FP32;
    const bool coherent = cfg_.scattering == 0;
    size_t launches = 0, phase_launches = 0;
    ECK(cudaMemsetAsync(err_.p, 0, sizeof(unsigned), st));
    ECK(cudaMemsetAsync(counter_.p, 0, 2 * sizeof(unsigned), st));
    for (int i = 0; i < nitems_; ++i) {
        SystemState& s = *item_sys_[i];
        ECK(launch_expand_factors(item_cf_[i], (int)s.nclass, (int)item_nq_[i], s.cls.as<int>(), (int)s.na_pad,
                                  cfg_.precision, bfac_.as<unsigned char>() + bfac_off_[i], st));
        ++launches;
    }
    if (ev) ECK(cudaEventRecord(ev[0], st));
    if (coherent && nrec_tiles_) {
        RecLaunch rl{};
        rl.K = rec_k_;
        rl.systems = d_rsys_;
        rl.groups = d_rgroups_;
        rl.tiles = d_rtiles_;
        rl.ntiles = nrec_tiles_;
        rl.bfac = rec_bfac_.as<float>();
        rl.counter = counter_.as<unsigned>() + 1;
        rl.err = err_.as<unsigned>();
        ECK(launch_rec_factors(rl, nrec_groups_, st));
        ECK(launch_phase_rec(rl, st));
        launches += 2;
        ++phase_launches;
    }
    if (coherent) {
        PhaseLaunch pl{};
        pl.precision = cfg_.precision;
        pl.shape = stats_.shape;
        pl.systems = d_psys_;
        pl.tiles = d_tiles_;
        pl.ntiles = ntiles_;
        pl.counter = counter_.as<unsigned>();
        pl.err = err_.as<unsigned>();
        if (ntiles_) {
            ECK(launch_phase_sum(pl, st));
            ++launches;
            ++phase_launches;
        }
        for (int i = 0; i < nitems_; ++i) {
            if (nsplit_[i] <= 1) continue;
            const size_t n = item_nv_[i] * item_nf_[i];
            if (f32) ECK(launch_split_reduce_f32(split_part32_[i], nsplit_[i], n, split_out32_[i], st));
            else ECK(launch_split_reduce(split_part_[i].first, nsplit_[i], n, split_part_[i].second, st));
            ++launches;
        }
    }
    if (ev) ECK(cudaEventRecord(ev[1], st));
    if (f32)
        for (int i = 0; i < nitems_; ++i)
            if (item_qv_[i]) {
                ECK(launch_q_revolutions(item_qv_[i], item_offs_[i].back(), qrev_.as<float4>() + qrev_off_[i], st));
                ++launches;
            }
    CorrLaunch cl{};
    cl.precision = cfg_.precision;
    cl.dsp = cfg_.dsp;
    cl.systems = d_csys_;
    cl.chunks = d_chunks_;
    cl.nchunks = nchunks_;
    cl.lg_max = lg_max_;
    cl.lg_min = lg_min_;
    cl.nf_max = nf_max_;
    cl.tw = f32 ? (const void*)tw32_.p : (const void*)tw64_.p;
    cl.restore_phase = f32;
    cl.ppart = ppart_.as<double>();
    cl.apart = apart_.as<double2>();
    cl.a2part = a2part_.as<double>();
    cl.err = err_.as<unsigned>();
    ECK(coherent ? launch_corr_accumulate(cl, st) : launch_self_accumulate(cl, st));
    ++launches;
    for (const LongItem& li : long_items_) {
        SystemState& s = *item_sys_[li.item];
        const size_t esz = f32 ? sizeof(float2) : sizeof(double2);
        for (int b = li.batch_begin; b < li.batch_end; ++b) {
            const LongBatch& lb = long_batches_[b];
            // The transforms need more than FP32: the 1/(NF - tau) normalisation amplifies
            // transform rounding at large lags in proportion to NF. The FP64 form runs them in
            // FP64, the FP32 form in float-float on the FP32 pipe (about 44 bits).
            LongArgs la{};
            la.precision = f32 ? PREC_FF : PREC_FP64;
            la.amp_f32 = f32;
            la.lg = s.lg;
            la.nf = (int)s.nf;
            if (coherent) {
                la.A = static_cast<const unsigned char*>(item_amp_[li.item]) + (size_t)lb.v0 * s.nf * esz;
            } else {  // generate the batch's (atom, direction) series
                LongSelfArgs g{};
                g.precision = cfg_.precision;
                g.nf = (int)s.nf;
                g.na_pad = (int)s.na_pad;
                g.nm = (int)(item_offs_[li.item][lb.shell + 1] - item_offs_[li.item][lb.shell]);
                g.p0 = lb.p0;
                g.nseries = lb.v1 - lb.v0;
                g.xyz = s.xyz.as<float4>();
                g.bfac = bfac_.as<unsigned char>() + bfac_off_[li.item] + (size_t)lb.shell * s.na_pad * (f32 ? 4 : 8);
                g.qv = item_qv_[li.item] + 3 * item_offs_[li.item][lb.shell];
                g.qrev = f32 ? qrev_.as<float4>() + qrev_off_[li.item] + item_offs_[li.item][lb.shell] : nullptr;
                g.G = long_G_.p;
                ECK(launch_long_self_series(g, st));
                ++launches;
                la.A = long_G_.p;
            }
            la.Y = long_Y_.p;
            la.nseries = lb.v1 - lb.v0;
            la.tw = f32 ? s.twff.p : s.tw64.p;
            la.chunks = d_long_chunks_ + lb.chunk_begin;
            la.nchunks = lb.chunk_end - lb.chunk_begin;
            la.v0 = lb.v0;
            la.kbr = f32 ? s.kff.p : s.k64.p;
            la.ppart = ppart_.as<double>();
            la.mpart = long_mpart_.as<double2>() + li.mpart_off;
            ECK(launch_long_columns(la, st));
            ECK(launch_long_rows(la, st));
            launches += 2;
        }
        ECK(launch_long_means(d_long_chunks_ + li.chunk_begin, li.chunk_end - li.chunk_begin,
                              long_mpart_.as<double2>() + li.mpart_off, 1 << (s.lg - kLongRowLg), apart_.as<double2>(),
                              a2part_.as<double>(), st));
        ++launches;
    }
    if (ev) ECK(cudaEventRecord(ev[2], st));
    FinalLaunch fl{};
    fl.dsp = cfg_.dsp;
    fl.conj_out = cfg_.dsp == DSP_AUTOCORRELATE && cfg_.method == 1;
    fl.entries = d_entries_;
    fl.nentries = nentries_;
    fl.lg_max = lg_max_;
    fl.ppart = ppart_.as<double>();
    fl.apart = apart_.as<double2>();
    fl.a2part = a2part_.as<double>();
    fl.tw = tw64_.as<double2>();
    ECK(launch_finalize(fl, st));
    ++launches;
    for (const LongItem& li : long_items_) {
        SystemState& s = *item_sys_[li.item];
        LongFinal lf{};
        lf.entries = d_long_entries_ + li.entry_begin;
        lf.nentries = li.entry_end - li.entry_begin;
        lf.lg = s.lg;
        lf.conj_out = fl.conj_out;
        lf.ppart = ppart_.as<double>();
        lf.apart = apart_.as<double2>();
        lf.a2part = a2part_.as<double>();
        lf.tw = s.tw64.as<double2>();
        lf.Z = long_Z_.as<double2>();
        ECK(launch_long_finalize(lf, st));
        launches += 2;
    }
    if (weighted_) {
        // the autocorrelation is quadratic in A: scaling A_v by sqrt(w_v) turns the same
        // correlation pass into (1/NM) sum_v w_v C_v(t)
        for (int i = 0; i < nitems_; ++i) {
            if (!item_wsqrt_[i]) continue;
            ECK(launch_scale_series(const_cast<void*>(amplitudes(i)), f32, item_wsqrt_[i], item_nv_[i],
                                    (int)item_nf_[i], st));
            ++launches;
        }
        ECK(launch_corr_accumulate(cl, st));
        FinalLaunch fw = fl;
        fw.entries = d_entries_w_;
        int nw = 0;
        for (int i = 0; i < nitems_; ++i)
            if (item_wsqrt_[i]) nw += (int)item_nq_[i];
        fw.nentries = nw;
        ECK(launch_finalize(fw, st));
        launches += 2;
    }
    if (ev) ECK(cudaEventRecord(ev[3], st));
    stats_.launches = launches;
    stats_.phase_launches = phase_launches;
    return kOk;
}

}  // namespace sassgpu
