// Minimal stand-in for boost::program_options::variables_map, enough for the
// reference's CPU solvers to compile without Boost.  Test infrastructure only.
#pragma once
#include <any>
#include <map>
#include <string>
namespace boost {
namespace program_options {
struct variable_value {
    std::any value;
    variable_value() = default;
    template <class T> variable_value(const T &v) : value(v) {}
    template <class T> const T &as() const { return std::any_cast<const T &>(value); }
};
struct variables_map : std::map<std::string, variable_value> {};
}  // namespace program_options
}  // namespace boost
