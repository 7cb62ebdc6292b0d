// GpuVectorsScatterDevice: the scatter device a Sassena maintainer adds to the reference
// tree (src/scatter_devices/, next to AllVectorsScatterDevice) to run the vectors
// orientational average of the coherent ("all") and incoherent ("self") devices on the
// GB300 through this project's C ABI (include/sassena_gb300.h).
//
// It is an AbstractVectorsScatterDevice (include/scatter_devices/
// abstract_vectors_scatter_device.hpp), so the reference's own run() drives it
// (src/scatter_devices/abstract_scatter_device.cpp:105-143): ram_check, stage_data, then
// for every q compute(), write() and next(). The device keeps the reference's inputs and
// outputs:
//   - q-vectors: the `vectors` the factory hands it, in that order;
//   - sub-vectors: init_subvectors (abstract_vectors_scatter_device.cpp:112-175), unchanged;
//   - scattering lengths: ScatterFactors::update (scatter_factors.cpp:56-78), unchanged;
//   - frames: DataStagerByFrame (data_stager.cpp:72-118), float32 [NF][NA][3];
//   - rows: atfinal_, afinal_, a2final_ as AllVectorsScatterDevice::compute leaves them
//     (all_vectors_scatter_device.cpp:238-361), written by the reference's write().
// What changes is where the work runs: the first compute() sends every q-vector of the
// device to the GPU in one sass_compute call, and each compute() then hands its row to
// write(). Atoms share a scattering class when they share the database ID and the kappa
// of the background correction, which is all ScatterFactors::update looks at, so the
// per-class factors of a q are the factors ScatterFactors computes for one atom of each
// class.
//
// Factory hook (scatter_device_factory.cpp:145-201), for orientation.type = vectors:
//     return new GpuVectorsScatterDevice(allcomm, partitioncomm, sample, vectors, NAF,
//                                        fileservice_endpoint, monitorservice_endpoint);
// Link with -lsassena_gb300.
#ifndef SCATTER_DEVICES__GPU_VECTORS_SCATTER_DEVICE_HPP_
#define SCATTER_DEVICES__GPU_VECTORS_SCATTER_DEVICE_HPP_

#include <cstdint>
#include <vector>

#include "sassena_gb300.h"
#include "scatter_devices/abstract_vectors_scatter_device.hpp"

class GpuVectorsScatterDevice : public AbstractVectorsScatterDevice {
protected:
    sass_plan* plan_;
    int precision_;
    std::vector<int32_t> class_of_atom_;  // scattering class of every target atom
    std::vector<size_t> class_atom_;      // one target atom of every class
    std::vector<double> fqt_, fq_, fq2_;  // rows of every q-vector, [nq][NF][2], [nq][2]
    bool computed_;

    void stage_data();
    void compute();
    void worker();
    void fail(const char* what);
    void assign_classes();
    void compute_all();

public:
    // precision: SASS_PRECISION_FP64 (the reference's arithmetic) or SASS_PRECISION_FP32
    GpuVectorsScatterDevice(boost::mpi::communicator allcomm, boost::mpi::communicator partitioncomm,
                            Sample& sample, std::vector<CartesianCoor3D> vectors, size_t NAF,
                            boost::asio::ip::tcp::endpoint fileservice_endpoint,
                            boost::asio::ip::tcp::endpoint monitorservice_endpoint,
                            int precision = SASS_PRECISION_FP64);
    ~GpuVectorsScatterDevice();
};

#endif
