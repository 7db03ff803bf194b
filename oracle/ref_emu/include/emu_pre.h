// Force-included ahead of every reference translation unit compiled for the
// CPU emulation (TEST INFRASTRUCTURE ONLY).
#pragma once

#include <cmath>

// libstdc++ has no std::sqrtf; the reference calls it in device code
// (range_alignment.cu:103).
namespace std {
inline float sqrtf(float x) { return ::sqrtf(x); }
}  // namespace std

#include "emu_launch.h"
