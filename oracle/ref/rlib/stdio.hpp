// Print-only stand-in for recolic's un-vendored `rlib/stdio.hpp`, used when
// the reference headers are compiled as the layout oracle. The reference only
// calls rlib::printfln / rlib::println / rlib::printable_iter for diagnostics
// (gpma.cuh:86-87,923,931; gpma_bfs.cuh:87,91) and imports rlib::literals
// (utils.cuh:12); none of them affects the data structure, so they are no-ops.
#pragma once
#include <string>
namespace rlib {
namespace literals {}
template <typename... A> inline void printfln(A &&...) {}
template <typename... A> inline void println(A &&...) {}
template <typename T> inline int printable_iter(const T &) { return 0; }
} // namespace rlib
