// Test infrastructure for the oracle build only (never shipped, never on the product path).
//
// Minimal stand-in for boost::program_options, just large enough for the reference's
// include/io/configuration.h to compile. That header's Config class is parsed but never
// instantiated by the oracle harness, so every member here is an inert no-op.
#pragma once

#include <cstdint>
#include <cassert>
#include <iostream>
#include <list>
#include <string>

namespace boost {
namespace program_options {

template <typename T>
struct typed_value {
    typed_value* default_value(const T&) { return this; }
    typed_value* required() { return this; }
};

template <typename T>
typed_value<T>* value(T*) {
    static typed_value<T> v;
    return &v;
}

struct options_description;

struct options_description_easy_init {
    options_description_easy_init& operator()(const char*, const char*) { return *this; }
    template <typename V>
    options_description_easy_init& operator()(const char*, V*, const char*) { return *this; }
};

struct options_description {
    options_description() = default;
    explicit options_description(const std::string&) {}
    options_description_easy_init add_options() { return {}; }
    options_description& add(const options_description&) { return *this; }
};

inline std::ostream& operator<<(std::ostream& os, const options_description&) { return os; }

struct positional_options_description {
    positional_options_description& add(const char*, int) { return *this; }
};

struct variable_value {
    template <typename T>
    T as() const { return T{}; }
};

struct variables_map {
    std::size_t count(const std::string&) const { return 0; }
    variable_value operator[](const std::string&) const { return {}; }
};

struct parsed_options {};

struct command_line_parser {
    command_line_parser(int, char**) {}
    command_line_parser& options(const options_description&) { return *this; }
    command_line_parser& allow_unregistered() { return *this; }
    command_line_parser& positional(const positional_options_description&) { return *this; }
    parsed_options run() { return {}; }
};

template <typename Char>
parsed_options parse_config_file(const Char*, const options_description&) { return {}; }

inline void store(const parsed_options&, variables_map&) {}
inline void notify(variables_map&) {}

}  // namespace program_options
}  // namespace boost
