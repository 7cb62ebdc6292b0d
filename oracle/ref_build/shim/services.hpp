// Stand-in for the reference's writer and monitor services with one process: the
// writer client hands every row (q, fqt, fq, fq2; fq0 = fqt[0]) to a sink the harness
// installs, in the order the device writes them; the monitor ignores progress.
#pragma once
#include <complex>
#include <cstddef>
#include <functional>

#include <boost/asio.hpp>
#include <fftw3.h>

#include "math/coor3d.hpp"

typedef std::function<void(const CartesianCoor3D&, const fftw_complex*, size_t, std::complex<double>,
                           std::complex<double>)>
    SignalRowSink;
SignalRowSink& signal_row_sink();

class HDF5WriterClient {
public:
    HDF5WriterClient(boost::asio::ip::tcp::endpoint) {}
    void write(CartesianCoor3D qvector, const fftw_complex* data, size_t NF, const std::complex<double> data2,
               const std::complex<double> data3) {
        signal_row_sink()(qvector, data, NF, data2, data3);
    }
    void flush() {}
};

class MonitorClient {
public:
    MonitorClient(boost::asio::ip::tcp::endpoint) {}
    void reset_server() {}
    void set_samplingfactor(size_t) {}
    void set_samplingfactor_server(size_t) {}
    void update(size_t, double) {}
};
