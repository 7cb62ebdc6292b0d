// C entry points of the host layer (no GPU): signal-file writing/reading and
// configuration parsing, for callers that drive the devices themselves and for tests.
#include <cstring>
#include <stdexcept>
#include <string>

#include "config.hpp"
#include "signal_file.hpp"

using namespace sassgpu;

namespace {
thread_local std::string g_err;
}

extern "C" {

const char* sass_host_error(void) { return g_err.c_str(); }

// Write a signal file. flags: bit0 fqt, bit1 fq0, bit2 fq, bit3 fq2 (datasets written).
// fqt [nq][nf][2], fq0/fq/fq2 [nq][2]; NULL for datasets not written. chunksize: rows
// per chunk (limits.signal.chunksize; 0 = the default 10000).
int sass_host_signal_write(const char* path, size_t nq, size_t nf, const double* qvectors,
                           const double* fqt, const double* fq0, const double* fq, const double* fq2,
                           int flags, const char* rawconfig, const char* database, size_t chunksize) {
    try {
        SignalData d;
        d.nf = nf;
        if (chunksize) d.chunksize = chunksize;
        for (size_t i = 0; i < nq; ++i) d.qvectors.push_back(Vec3{qvectors[3 * i], qvectors[3 * i + 1], qvectors[3 * i + 2]});
        d.has_fqt = flags & 1;
        d.has_fq0 = flags & 2;
        d.has_fq = flags & 4;
        d.has_fq2 = flags & 8;
        if (d.has_fqt) d.fqt.assign(fqt, fqt + nq * nf * 2);
        if (d.has_fq0) d.fq0.assign(fq0, fq0 + nq * 2);
        if (d.has_fq) d.fq.assign(fq, fq + nq * 2);
        if (d.has_fq2) d.fq2.assign(fq2, fq2 + nq * 2);
        d.rawconfig = rawconfig ? rawconfig : "";
        d.config = d.rawconfig;
        d.database = database ? database : "";
        write_signal_file(path, d);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// Read a signal file. First call with NULL arrays to get *nq, *nf and *flags; then
// again with arrays of that size.
int sass_host_signal_read(const char* path, size_t* nq, size_t* nf, int* flags, double* qvectors,
                          double* fqt, double* fq0, double* fq, double* fq2) {
    try {
        SignalData d = read_signal_file(path);
        *nq = d.nq();
        *nf = d.nf;
        *flags = (d.has_fqt ? 1 : 0) | (d.has_fq0 ? 2 : 0) | (d.has_fq ? 4 : 0) | (d.has_fq2 ? 8 : 0);
        if (qvectors)
            for (size_t i = 0; i < d.nq(); ++i)
                for (int k = 0; k < 3; ++k) qvectors[3 * i + k] = d.qvectors[i][k];
        if (fqt && d.has_fqt) memcpy(fqt, d.fqt.data(), d.fqt.size() * 8);
        if (fq0 && d.has_fq0) memcpy(fq0, d.fq0.data(), d.fq0.size() * 8);
        if (fq && d.has_fq) memcpy(fq, d.fq.data(), d.fq.size() * 8);
        if (fq2 && d.has_fq2) memcpy(fq2, d.fq2.data(), d.fq2.size() * 8);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// q-vectors generated by the configuration's scattering.vectors section
// (single / scans / file), written to out (3 doubles each, up to cap vectors).
int sass_host_config_qvectors(const char* config, double* out, size_t cap, size_t* n) {
    try {
        Params p;
        p.read_xml(config);
        *n = p.qvectors.size();
        for (size_t i = 0; i < p.qvectors.size() && i < cap; ++i)
            for (int k = 0; k < 3; ++k) out[3 * i + k] = p.qvectors[i][k];
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

}  // extern "C"
