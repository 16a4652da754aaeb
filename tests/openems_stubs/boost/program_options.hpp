// Compile-time stand-in for <boost/program_options.hpp>: the declarations
// openEMS's tools/global.h names (its option registry), so that glue code
// including the engine headers can be compiled without Boost.  Nothing here
// is called.
#pragma once
#include <string>
#include <vector>

namespace boost {
namespace program_options {
class options_description {
public:
    options_description() {}
    explicit options_description(const std::string&) {}
};
class variable_value {
public:
    template <class T>
    const T& as() const { static T t; return t; }
    bool empty() const { return true; }
};
class variables_map {
public:
    size_t count(const std::string&) const { return 0; }
    const variable_value& operator[](const std::string&) const { static variable_value v; return v; }
};
}  // namespace program_options
}  // namespace boost
