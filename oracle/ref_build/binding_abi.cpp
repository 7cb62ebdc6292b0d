// Recording stand-in of this project's C ABI for the binding check (test infrastructure).
//
// GpuVectorsScatterDevice (sassena_gb300/integration) is compiled here against the
// reference's own headers and driven by the reference's own run(). The GPU is not
// reachable in this build, so the C ABI calls it makes are recorded instead of run: the
// plan description, the staged frames, the atom classes and every sass_compute call
// (sub-vector offsets, sub-vectors, class factors). The rows it returns are zero. The
// recorded calls are replayed through the real library on the GPU by
// tests/test_gpu_binding.py and checked against the reference device's rows.
// The library is linked with -Bsymbolic, so the binding calls these definitions even in a
// process that has also loaded the real library.
#include <cstring>
#include <string>
#include <vector>

#include "sassena_gb300.h"

struct sass_plan {
    sass_plan_desc desc;
};

namespace {
struct Record {
    sass_plan_desc desc;
    std::vector<float> frames;
    std::vector<int32_t> classes;
    std::vector<size_t> offs;
    std::vector<double> subvectors, class_factors;
    int computes = 0;
} g_rec;
}  // namespace

extern "C" {

int sass_plan_create(const sass_plan_desc* desc, sass_plan** plan) {
    g_rec = Record();
    g_rec.desc = *desc;
    *plan = new sass_plan;
    (*plan)->desc = *desc;
    return SASS_OK;
}

void sass_plan_destroy(sass_plan* plan) { delete plan; }

const char* sass_plan_error(const sass_plan*) { return ""; }

int sass_stage_frames(sass_plan* plan, const float* coords, int) {
    g_rec.frames.assign(coords, coords + plan->desc.nf * plan->desc.na * 3);
    return SASS_OK;
}

int sass_set_atom_classes(sass_plan* plan, const int32_t* atom_class, int) {
    g_rec.classes.assign(atom_class, atom_class + plan->desc.na);
    return SASS_OK;
}

int sass_compute(sass_plan* plan, size_t nq, const size_t* sub_offsets, const double* subvectors,
                 const double* class_factors, double* fqt, double* fq, double* fq2, int) {
    ++g_rec.computes;
    g_rec.offs.assign(sub_offsets, sub_offsets + nq + 1);
    g_rec.subvectors.assign(subvectors, subvectors + 3 * sub_offsets[nq]);
    g_rec.class_factors.assign(class_factors, class_factors + nq * plan->desc.nclass);
    std::memset(fqt, 0, nq * plan->desc.nf * 2 * sizeof(double));
    std::memset(fq, 0, nq * 2 * sizeof(double));
    std::memset(fq2, 0, nq * 2 * sizeof(double));
    return SASS_OK;
}

/* What the binding passed in its last run. ints[8]: scattering, dsp_type, dsp_method,
 * precision, na, nf, nclass, number of sass_compute calls; sizes[4]: offsets, sub-vector
 * values, class-factor values, staged floats. */
void bind_last_sizes(long* ints, size_t* sizes) {
    ints[0] = g_rec.desc.scattering;
    ints[1] = g_rec.desc.dsp_type;
    ints[2] = g_rec.desc.dsp_method;
    ints[3] = g_rec.desc.precision;
    ints[4] = (long)g_rec.desc.na;
    ints[5] = (long)g_rec.desc.nf;
    ints[6] = (long)g_rec.desc.nclass;
    ints[7] = g_rec.computes;
    sizes[0] = g_rec.offs.size();
    sizes[1] = g_rec.subvectors.size();
    sizes[2] = g_rec.class_factors.size();
    sizes[3] = g_rec.frames.size();
}

void bind_last_calls(size_t* offs, double* subvectors, double* class_factors, int32_t* classes, float* frames) {
    std::memcpy(offs, g_rec.offs.data(), g_rec.offs.size() * sizeof(size_t));
    std::memcpy(subvectors, g_rec.subvectors.data(), g_rec.subvectors.size() * sizeof(double));
    std::memcpy(class_factors, g_rec.class_factors.data(), g_rec.class_factors.size() * sizeof(double));
    std::memcpy(classes, g_rec.classes.data(), g_rec.classes.size() * sizeof(int32_t));
    std::memcpy(frames, g_rec.frames.data(), g_rec.frames.size() * sizeof(float));
}

}  // extern "C"
