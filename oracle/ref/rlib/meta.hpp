// Empty stand-in for recolic's un-vendored `rlib/meta.hpp` (included by
// multidev.cuh:7, which uses nothing from it on the oracle path).
#pragma once
#include "stdio.hpp"
