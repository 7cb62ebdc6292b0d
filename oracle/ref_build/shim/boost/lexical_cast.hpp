// Stand-in for boost/lexical_cast.hpp: conversion through a string stream (the
// reference uses it for log messages only).
#pragma once
#include <sstream>
#include <string>
namespace boost {
template <class T, class S>
T lexical_cast(const S& s) {
    std::stringstream io;
    io << s;
    T t;
    io >> t;
    return t;
}
template <>
inline std::string lexical_cast<std::string, std::string>(const std::string& s) { return s; }
}  // namespace boost
