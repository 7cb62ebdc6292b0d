// The reference's database getters (reg, quick-lookup and get of volumes, exclusion
// factors and scattering factors), compiled from database.cpp lines 375-528 as they
// stand; the Makefile cuts the lines into database_getters.inc and checks the cut.
#include <cmath>
#include <string>
#include <vector>

#include <boost/lexical_cast.hpp>
#include <boost/math/special_functions/factorial.hpp>

#include "control.hpp"
#include "log.hpp"

using namespace std;

#include "database_getters.inc"
