// Internal definition of the plan object, shared by the C ABI translation units.
#pragma once

#include <string>

#include "../../include/sassena_gb300.h"
#include "engine.h"

namespace sassgpu {
constexpr int kEvents = 12;
}

struct sass_plan {
    sass_plan_desc d{};
    sassgpu::SystemState sys;
    sassgpu::Engine eng;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    // sass_prefetch_frames: the copy stream and the copy's completion event (created lazily)
    cudaStream_t side = nullptr;
    cudaEvent_t pf_done = nullptr;
    std::string msg;
    sass_timing timing{};
    cudaEvent_t ev[sassgpu::kEvents] = {};
    sassgpu::PhaseShape shape{0, 0, 0};
    int split_atoms = 0;
    int rec_k = 0;  // shell recurrence: 0 automatic, -1 off, else shells per lane
    sassgpu::DevBuf qv, cf, fqt, fq, fq2, amp_tmp;
    // multipole devices: packed per-call inputs, basis batch, amplitudes, results
    sassgpu::DevBuf mp_in, mp_Jb, mp_Yc, mp_amp, mp_out, mp_ycf, mp_slot;
    // staging pre-pass: packed lists, FP64 system frames, float upload, fit copy, vectors
    sassgpu::DevBuf pp_lists, pp_W, pp_F, pp_C, pp_vec;
};
