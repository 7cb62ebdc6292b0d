// Two functions of the reference's parameters.cpp compiled as they stand:
// SampleParameters::~SampleParameters (lines 924-928; Params' destructor needs it) and
// ScatteringVectorsParameters::create_from_scans (lines 1125-1189). The Makefile cuts the
// lines into the .inc files and checks the cut.
#include <cmath>
#include <string>
#include <vector>

#include "control.hpp"
#include "log.hpp"

using namespace std;

#include "sample_parameters_dtor.inc"
#include "create_from_scans.inc"
