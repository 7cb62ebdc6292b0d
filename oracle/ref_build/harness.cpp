// Harness around the reference's own compiled scatter devices (test infrastructure).
//
// The reference cannot be built whole here (MPI, Boost, FFTW3, HDF5 and libxml2 are
// absent), but its hot path compiles unmodified from its own sources against the small
// stand-ins in shim/: smath.cpp, coor3d.cpp, assignment.cpp, scatter_factors.cpp and the
// abstract, vectors, all and self scatter devices, plus the database getters and
// create_from_scans cut from database.cpp and parameters.cpp by line range (the
// Makefile checks the cut lines). This file plays the parts of the reference that
// are not compiled: it fills Params, Database and the Sample the way the reference's
// configuration and sample loading would for the case, constructs a device as
// ScatterDeviceFactory::create does for one rank (scatter_device_factory.cpp:145-201),
// calls run() (abstract_scatter_device.cpp:105-143) and collects the rows the device
// writes through HDF5WriterClient::write.
//
// Nothing in the product links this library; tests/golden/make_reference_golden.py
// turns its outputs into committed fixtures.
#include <cmath>
#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "control.hpp"
#include "log.hpp"
#include "sample.hpp"
#include "scatter_devices/all_vectors_scatter_device.hpp"
#include "scatter_devices/gpu_vectors_scatter_device.hpp"
#include "scatter_devices/self_vectors_scatter_device.hpp"
#include "services.hpp"

// --- definitions from reference sources that are not compiled (log.cpp needs
// boost::format); messages are kept for the caller instead of printed.
size_t Info::counter = 0;
size_t Warn::counter = 0;
size_t Err::counter = 0;
static std::string g_errors;
void Info::write(std::string) {}
void Warn::write(std::string) {}
void Err::write(std::string s) { g_errors += s + "\n"; }

SignalRowSink& signal_row_sink() {
    static SignalRowSink sink;
    return sink;
}

namespace {

// The device destructors are protected; these expose run() and delete.
class RunAll : public AllVectorsScatterDevice {
public:
    using AllVectorsScatterDevice::AllVectorsScatterDevice;
    ~RunAll() {}
};
class RunSelf : public SelfVectorsScatterDevice {
public:
    using SelfVectorsScatterDevice::SelfVectorsScatterDevice;
    ~RunSelf() {}
};

size_t g_id_base = 0;  // fresh database IDs per run: sfactors caches values per (q, ID)

}  // namespace

// One run of a vectors device (the reference's, or the binding's GpuVectorsScatterDevice)
// on the case the arguments describe; see ref_run_vectors.
static long run_device(bool binding, int self, const char* dsp_type, const char* dsp_method, size_t nthreads,
                const float* coords, size_t nf, size_t na, const int* atom_type, size_t ntype, const int* sf_type,
                const double* sf_const, const double* vol, const int* ex_type, const double* ex_const,
                double background, size_t nq, const double* qvectors, size_t nm, const double* orient,
                double* q_out, double* fqt, double* fq, double* fq2) {
    g_errors.clear();
    Params* P = Params::Inst();
    P->scattering.type = self ? "self" : "all";
    P->scattering.dsp.type = dsp_type;
    P->scattering.dsp.method = dsp_method;
    P->scattering.background.factor = background;
    P->scattering.background.kappas.clear();
    P->scattering.average.orientation.type = "vectors";
    ScatteringAverageOrientationVectorsParameters& ov = P->scattering.average.orientation.vectors;
    ov.clear();
    ov.type = "file";
    for (size_t i = 0; i < nm; ++i) {
        CartesianCoor3D q(orient[3 * i], orient[3 * i + 1], orient[3 * i + 2]);
        double ql = q.length();
        if (ql != 0) q = (1.0 / ql) * q;  // as create() normalises file orientations
        ov.push_back(q);
    }
    P->stager.target = "system";
    P->limits.computation.threads = nthreads;
    P->limits.computation.memory.scale = 1;
    P->limits.computation.memory.result_buffer = (size_t)1 << 40;
    P->limits.computation.memory.alignpad_buffer = (size_t)1 << 40;
    P->limits.computation.memory.exchange_buffer = (size_t)1 << 40;
    P->limits.computation.memory.signal_buffer = (size_t)1 << 40;
    P->limits.services.monitor.sampling = 1;
    P->debug.print.orientations = false;

    Database* D = Database::Inst();
    const size_t base = g_id_base;
    g_id_base += ntype;
    for (size_t t = 0; t < ntype; ++t) {
        D->sfactors.reg(base + t, std::vector<double>(sf_const + 9 * t, sf_const + 9 * t + 9), sf_type[t]);
        D->volumes.reg(base + t, std::vector<double>(1, vol[t]), 0);
        D->exclusionfactors.reg(base + t, std::vector<double>(1, ex_const[t]), ex_type[t]);
    }

    Sample sample;
    IAtomselection system;
    for (size_t j = 0; j < na; ++j) {
        sample.atoms.ids.push_back(base + (size_t)atom_type[j]);
        system.indexes.push_back(j);
    }
    sample.atoms.selections["system"] = &system;
    sample.coordinate_sets.nframes = nf;
    sample.target_frames = coords;

    std::vector<CartesianCoor3D> qs;
    for (size_t i = 0; i < nq; ++i) qs.push_back(CartesianCoor3D(qvectors[3 * i], qvectors[3 * i + 1], qvectors[3 * i + 2]));

    long rows = 0;
    signal_row_sink() = [&](const CartesianCoor3D& q, const fftw_complex* data, size_t NF, std::complex<double> a,
                            std::complex<double> a2) {
        if ((size_t)rows >= nq || NF != nf) throw std::runtime_error("unexpected row");
        q_out[3 * rows] = q.x;
        q_out[3 * rows + 1] = q.y;
        q_out[3 * rows + 2] = q.z;
        std::memcpy(fqt + (size_t)rows * nf * 2, data, nf * sizeof(fftw_complex));
        fq[2 * rows] = a.real();
        fq[2 * rows + 1] = a.imag();
        fq2[2 * rows] = a2.real();
        fq2[2 * rows + 1] = a2.imag();
        ++rows;
    };

    boost::mpi::communicator comm;
    boost::asio::ip::tcp::endpoint ep;
    try {
        if (binding) {
            GpuVectorsScatterDevice dev(comm, comm, sample, qs, self ? na : nf, ep, ep);
            dev.run();
        } else if (self) {
            RunSelf dev(comm, comm, sample, qs, na, ep, ep);  // NAF = NA (scatter_device_factory.cpp:60-65)
            dev.run();
        } else {
            RunAll dev(comm, comm, sample, qs, nf, ep, ep);  // NAF = NF
            dev.run();
        }
    } catch (std::exception& e) {
        g_errors += e.what();
        signal_row_sink() = nullptr;
        return -1;
    }
    signal_row_sink() = nullptr;
    return rows;
}

extern "C" {

/* One run of the reference's coherent (self = 0) or incoherent (self = 1) vectors device.
 *   dsp_type "autocorrelate" | "square" | "plain"; dsp_method "fftw" | "direct"
 *   coords      float32 [nf][na][3], the target selection's staged frames
 *   atom_type   [na] index into the per-type database tables below
 *   sf_type     [ntype] sfactor function type (0 constant, 2 four Gaussians + c)
 *   sf_const    [ntype][9] its constants (database.cpp:469-528)
 *   vol         [ntype] volume (volume function type 0, a constant)
 *   ex_type     [ntype] exclusion function type (0 constant, 1 linear, 2 Gaussian)
 *   ex_const    [ntype] its constant
 *   background  scattering.background.factor (kappa 1 for every atom)
 *   qvectors    [nq][3] scattering vectors, in the order the device writes them
 *   orient      [nm][3] orientations of vectors.type = file, normalised here as
 *               ScatteringAverageOrientationVectorsParameters::create does; nm = 0
 *               means no orientational averaging (the q-vectors themselves)
 * Outputs per written row r: q_out[r][3], fqt[r][nf][2], fq[r][2], fq2[r][2].
 * Returns the number of rows, or -1 with a message in ref_last_error(). */
long ref_run_vectors(int self, const char* dsp_type, const char* dsp_method, size_t nthreads,
                     const float* coords, size_t nf, size_t na, const int* atom_type, size_t ntype,
                     const int* sf_type, const double* sf_const, const double* vol, const int* ex_type,
                     const double* ex_const, double background, size_t nq, const double* qvectors,
                     size_t nm, const double* orient, double* q_out, double* fqt, double* fq, double* fq2) {
    return run_device(false, self, dsp_type, dsp_method, nthreads, coords, nf, na, atom_type, ntype, sf_type,
                      sf_const, vol, ex_type, ex_const, background, nq, qvectors, nm, orient, q_out, fqt, fq, fq2);
}

/* The same run with this project's GpuVectorsScatterDevice (the binding a maintainer adds,
 * sassena_gb300/integration) in place of the reference's device, driven by the reference's
 * run(). The C ABI it calls is the recording stand-in of binding_abi.cpp: the rows it writes
 * are zero, and bind_last_* return what it passed to the library. */
long bind_run_vectors(int self, const char* dsp_type, const char* dsp_method, size_t nthreads,
                      const float* coords, size_t nf, size_t na, const int* atom_type, size_t ntype,
                      const int* sf_type, const double* sf_const, const double* vol, const int* ex_type,
                      const double* ex_const, double background, size_t nq, const double* qvectors,
                      size_t nm, const double* orient, double* q_out, double* fqt, double* fq, double* fq2) {
    return run_device(true, self, dsp_type, dsp_method, nthreads, coords, nf, na, atom_type, ntype, sf_type,
                      sf_const, vol, ex_type, ex_const, background, nq, qvectors, nm, orient, q_out, fqt, fq, fq2);
}



/* The reference's q-vector scans (ScatteringVectorsParameters::create_from_scans) for up to
 * three scans; base[s][3], from/to/exponent[s], points[s]. Writes at most cap vectors to
 * out[][3] and returns how many the scans made, or -1 on error. */
long ref_scans(size_t nscan, const double* from, const double* to, const size_t* points, const double* exponent,
               const double* base, size_t cap, double* out) {
    g_errors.clear();
    ScatteringVectorsParameters v;
    for (size_t s = 0; s < nscan; ++s) {
        ScatteringVectorsScanParameters sc;
        sc.from = from[s];
        sc.to = to[s];
        sc.points = points[s];
        sc.exponent = exponent[s];
        sc.basevector = CartesianCoor3D(base[3 * s], base[3 * s + 1], base[3 * s + 2]);
        v.scans.push_back(sc);
    }
    try {
        v.create_from_scans();
    } catch (...) {
        return -1;
    }
    for (size_t i = 0; i < v.size() && i < cap; ++i) {
        out[3 * i] = v[i].x;
        out[3 * i + 1] = v[i].y;
        out[3 * i + 2] = v[i].z;
    }
    return (long)v.size();
}

/* Database getters (database.cpp:391-528) for one registered entry. */
double ref_sfactor(int type, const double* constants, size_t n, double q) {
    const size_t id = g_id_base++;
    Database::Inst()->sfactors.reg(id, std::vector<double>(constants, constants + n), type);
    return Database::Inst()->sfactors.get(id, q);
}
double ref_volume(int type, const double* constants, size_t n) {
    const size_t id = g_id_base++;
    Database::Inst()->volumes.reg(id, std::vector<double>(constants, constants + n), type);
    return Database::Inst()->volumes.get(id);
}
double ref_exclusion(int type, const double* constants, size_t n, double effvolume, double q) {
    const size_t id = g_id_base++;
    Database::Inst()->exclusionfactors.reg(id, std::vector<double>(constants, constants + n), type);
    return Database::Inst()->exclusionfactors.get(id, effvolume, q);
}

const char* ref_last_error(void) { return g_errors.c_str(); }

}  // extern "C"
