// Stand-in: the sample parts ScatterFactors reads are in sample.hpp.
#pragma once
#include "sample.hpp"
