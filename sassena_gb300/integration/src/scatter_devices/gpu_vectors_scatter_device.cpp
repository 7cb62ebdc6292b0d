// GpuVectorsScatterDevice: the reference-side scatter device that runs the vectors
// orientational average on the GB300 through this project's C ABI. See the header for
// what it keeps from the reference and what it changes.
#include <complex>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>

#include "control.hpp"
#include "exceptions/exceptions.hpp"
#include "log.hpp"
#include "sample.hpp"
#include "scatter_devices/gpu_vectors_scatter_device.hpp"
#include "stager/data_stager.hpp"

GpuVectorsScatterDevice::GpuVectorsScatterDevice(boost::mpi::communicator allcomm,
                                                 boost::mpi::communicator partitioncomm, Sample& sample,
                                                 std::vector<CartesianCoor3D> vectors, size_t NAF,
                                                 boost::asio::ip::tcp::endpoint fileservice_endpoint,
                                                 boost::asio::ip::tcp::endpoint monitorservice_endpoint,
                                                 int precision)
    : AbstractVectorsScatterDevice(allcomm, partitioncomm, sample, vectors, NAF, fileservice_endpoint,
                                   monitorservice_endpoint),
      plan_(NULL),
      precision_(precision),
      computed_(false) {
    p_coordinates = NULL;
    const std::string& type = Params::Inst()->scattering.type;
    const std::string& dsp = Params::Inst()->scattering.dsp.type;
    const std::string& method = Params::Inst()->scattering.dsp.method;
    sass_plan_desc d;
    std::memset(&d, 0, sizeof(d));
    // the keys AllVectorsScatterDevice::dsp and SelfVectorsScatterDevice::dsp accept
    d.scattering = type == "self" ? SASS_SCATTERING_SELF : SASS_SCATTERING_ALL;
    if (dsp == "autocorrelate") d.dsp_type = SASS_DSP_AUTOCORRELATE;
    else if (dsp == "square") d.dsp_type = SASS_DSP_SQUARE;
    else if (dsp == "plain") d.dsp_type = SASS_DSP_PLAIN;
    else fail(("DSP type not understood: " + dsp).c_str());
    if (method == "fftw") d.dsp_method = SASS_METHOD_FFTW;
    else if (method == "direct") d.dsp_method = SASS_METHOD_DIRECT;
    else fail(("Correlation method not understood: " + method).c_str());
    d.precision = precision_;
    assign_classes();
    d.na = NA;
    d.nf = NF;
    d.nclass = class_atom_.size();
    d.device = 0;
    d.stream = NULL;
    d.amplitude_budget_bytes = 0;
    if (sass_plan_create(&d, &plan_) != SASS_OK) fail("sass_plan_create");
}

GpuVectorsScatterDevice::~GpuVectorsScatterDevice() {
    if (plan_ != NULL) sass_plan_destroy(plan_);
    if (p_coordinates != NULL) {
        free(p_coordinates);
        p_coordinates = NULL;
    }
}

void GpuVectorsScatterDevice::fail(const char* what) {
    std::string msg = std::string("GPU scatter device: ") + what;
    if (plan_ != NULL && sass_plan_error(plan_)[0] != '\0') msg += std::string(": ") + sass_plan_error(plan_);
    Err::Inst()->write(msg);
    throw sassena::terminate_request();
}

// Atoms of the target selection that share the database ID and the background kappa get the
// same factor from ScatterFactors::update for every q (scatter_factors.cpp:56-78); kappas
// default to 1 and are set per selection as ScatterFactors::update_kappas does (:29-44).
void GpuVectorsScatterDevice::assign_classes() {
    IAtomselection* target = sample_.atoms.selections[Params::Inst()->stager.target];
    std::vector<double> kappa(sample_.atoms.size(), 1.0);
    std::vector<ScatteringBackgroundKappaParameters>& kp = Params::Inst()->scattering.background.kappas;
    for (size_t i = 0; i < kp.size(); ++i) {
        IAtomselection* sel = sample_.atoms.selections[kp[i].selection];
        for (size_t j = 0; j < sel->size(); ++j) kappa[(*sel)[j]] = kp[i].value;
    }
    std::map<std::pair<size_t, double>, int32_t> index;
    class_of_atom_.resize(target->size());
    class_atom_.clear();
    for (size_t i = 0; i < target->size(); ++i) {
        const size_t atom = (*target)[i];
        const std::pair<size_t, double> key(sample_.atoms[atom], kappa[atom]);
        std::map<std::pair<size_t, double>, int32_t>::iterator it = index.find(key);
        if (it == index.end()) {
            it = index.insert(std::make_pair(key, (int32_t)class_atom_.size())).first;
            class_atom_.push_back(i);
        }
        class_of_atom_[i] = it->second;
    }
}

// Frames as DataStagerByFrame stages them (float32 [NF][NA][3]; the incoherent device
// takes the same layout here, where the reference stages it by atom) into the plan.
void GpuVectorsScatterDevice::stage_data() {
    Timer& timer = timer_[boost::this_thread::get_id()];
    DataStagerByFrame data_stager(sample_, allcomm_, partitioncomm_, timer);
    p_coordinates = data_stager.stage();
    if (sass_stage_frames(plan_, p_coordinates, 0) != SASS_OK) fail("sass_stage_frames");
    if (sass_set_atom_classes(plan_, &class_of_atom_[0], 0) != SASS_OK) fail("sass_set_atom_classes");
}

// Every q-vector of the device in one call: the sub-vectors of init_subvectors and the
// class factors of ScatterFactors::update, per q in the order of vectors_.
void GpuVectorsScatterDevice::compute_all() {
    const size_t nq = vectors_.size(), nclass = class_atom_.size();
    std::vector<size_t> offs(1, 0);
    std::vector<double> sv, cf(nq * nclass);
    for (size_t i = 0; i < nq; ++i) {
        CartesianCoor3D q = vectors_[i];
        init_subvectors(q);
        for (size_t m = 0; m < subvector_index_.size(); ++m) {
            sv.push_back(subvector_index_[m].x);
            sv.push_back(subvector_index_[m].y);
            sv.push_back(subvector_index_[m].z);
        }
        offs.push_back(offs.back() + subvector_index_.size());
        scatterfactors.update(q);
        std::vector<double>& f = scatterfactors.get_all();
        for (size_t c = 0; c < nclass; ++c) cf[i * nclass + c] = f[class_atom_[c]];
    }
    fqt_.assign(nq * NF * 2, 0.0);
    fq_.assign(nq * 2, 0.0);
    fq2_.assign(nq * 2, 0.0);
    if (nq > 0 && sass_compute(plan_, nq, &offs[0], &sv[0], &cf[0], &fqt_[0], &fq_[0], &fq2_[0], 0) != SASS_OK)
        fail("sass_compute");
    computed_ = true;
}

// The row of the current q-vector, left as AllVectorsScatterDevice::compute leaves it:
// atfinal_ [NF], afinal_ and a2final_, averaged over the orientations.
void GpuVectorsScatterDevice::compute() {
    if (!computed_) compute_all();
    const size_t i = current_vector_;
    CartesianCoor3D q = vectors_[i];
    init_subvectors(q);  // NM and subvector_index_ of this q, as the reference leaves them
    std::memcpy(atfinal_, &fqt_[i * NF * 2], NF * sizeof(fftw_complex));
    afinal_ = std::complex<double>(fq_[2 * i], fq_[2 * i + 1]);
    a2final_ = std::complex<double>(fq2_[2 * i], fq2_[2 * i + 1]);
}

// The GPU needs no worker threads: each joins the start-up barrier of
// AbstractScatterDevice::start_workers (abstract_scatter_device.cpp:178-211) and ends.
void GpuVectorsScatterDevice::worker() { workerbarrier->wait(); }
