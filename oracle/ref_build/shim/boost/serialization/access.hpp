// Stand-in for boost/serialization/access.hpp: the reference's classes befriend
// boost::serialization::access and name base_object inside serialize() templates that
// the compiled functions never instantiate.
#pragma once
namespace boost {
namespace serialization {
class access {};
template <class Base, class Derived>
Base& base_object(Derived& d) { return d; }
}  // namespace serialization
}  // namespace boost
