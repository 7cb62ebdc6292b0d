// Stand-in for boost/math/special_functions/factorial.hpp: the database's Slater-type
// scattering factor (type 1) calls factorial<double>; no workload uses that type.
#pragma once
#include <cmath>
namespace boost { namespace math {
template <class T>
T factorial(unsigned i) { return std::tgamma((T)i + 1); }
} }
