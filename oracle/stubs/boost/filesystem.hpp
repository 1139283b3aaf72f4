// Test infrastructure for the oracle build only (never shipped, never on the product path).
//
// Minimal stand-in for boost::filesystem so that the reference's include/io/configuration.h
// compiles. The Config constructor that uses it is never called by the oracle harness.
#pragma once

#include <string>

namespace boost {
namespace filesystem {

struct path {
    path() = default;
    explicit path(const std::string&) {}
};

inline bool exists(const path&) { return false; }
inline bool create_directory(const path&) { return false; }
inline bool remove(const path&) { return false; }

struct directory_entry {
    path path() const { return {}; }
};

struct directory_iterator {
    directory_iterator() = default;
    explicit directory_iterator(const path&) {}
    directory_iterator& operator++() { return *this; }
    const directory_entry* operator->() const { return &entry; }
    bool operator!=(const directory_iterator&) const { return false; }
    directory_entry entry;
};

}  // namespace filesystem
}  // namespace boost
