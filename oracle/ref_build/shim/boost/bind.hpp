// Stand-in for boost/bind.hpp (start_workers binds the virtual worker() to this).
#pragma once
#include <functional>
#include <utility>
namespace boost {
template <class... A>
auto bind(A&&... a) -> decltype(std::bind(std::forward<A>(a)...)) { return std::bind(std::forward<A>(a)...); }
}
