// signal.h5 writer and reader (no libhdf5).
//
// The reference writes, through its HDF5 writer service (src/services/
// file_writer_service.cpp:44-171, :314-484, :504-531):
//   /qvectors f64 [NQ,3]   /fqt f64 [NQ,NF,2]   /fq0 /fq /fq2 f64 [NQ,2]
//   /meta/rawconfig int8 [n]   /meta/config string   /meta/database string
// each of fqt, fq0, fq, fq2 only if its scattering.signal.* flag is set, rows in
// completion order. This module writes the same names, shapes, element types and
// row order in the HDF5 file format's classic encoding (superblock version 0,
// symbol-table groups, version-1 object headers). Like the reference's writer, the
// root datasets are chunked with an unlimited first dimension (rows of
// limits.signal.chunksize, a version-1 B-tree chunk index); the /meta datasets are
// contiguous. Appending rewrites the file with the new rows after the old ones. The
// reader understands contiguous and chunked datasets, so a run can resume from a file
// written by either program.
#pragma once

#include <string>
#include <vector>

#include "config.hpp"

namespace sassgpu {

struct SignalData {
    size_t nf = 0;
    size_t chunksize = 10000;  // limits.signal.chunksize (rows per chunk)
    std::vector<Vec3> qvectors;
    bool has_fqt = true, has_fq0 = true, has_fq = true, has_fq2 = true;
    std::vector<double> fqt;  // [NQ][NF][2]
    std::vector<double> fq0, fq, fq2;  // [NQ][2]
    std::string rawconfig, config, database;

    size_t nq() const { return qvectors.size(); }
};

// Write `d` to `path` (replacing the file). Throws std::runtime_error on I/O failure.
void write_signal_file(const std::string& path, const SignalData& d);
// Read datasets of an existing signal file (qvectors always; the others if present).
// Throws on files that are not HDF5 or use encodings outside the ones described above.
SignalData read_signal_file(const std::string& path);
bool is_hdf5_file(const std::string& path);

}  // namespace sassgpu
