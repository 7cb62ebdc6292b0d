// Stand-in for boost/numeric/ublas/matrix.hpp: the coherent device's scatter() opens
// boost::numeric::ublas::detail with a using-directive and uses nothing from it.
#pragma once
namespace boost { namespace numeric { namespace ublas { namespace detail {} } } }
