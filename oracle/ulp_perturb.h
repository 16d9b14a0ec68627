// ULP perturbation of the transcendental calls of the OpenPBR BSDF — TEST
// INFRASTRUCTURE.
//
// Force-included (g++ -include) into a second build of the oracle by
// tests/test_openpbr_conditioning.py: every unqualified powf/expf/logf/sinf/
// cosf/acosf call returns the libm result moved up by one ulp for half of the
// inputs (chosen by a hash of the argument bits). Comparing that build with
// the plain oracle measures how far one-ulp differences between two math
// libraries (CUDA's and the host's) carry along a path.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

inline float orc_ulp_nudge(float result, float key) {
    uint32_t bits;
    std::memcpy(&bits, &key, sizeof bits);
    return ((bits * 2654435761u) >> 31) != 0u ? std::nextafter(result, 1e30f) : result;
}

#define powf(a, b) orc_ulp_nudge(std::pow(static_cast<float>(a), static_cast<float>(b)), static_cast<float>(a) + static_cast<float>(b))
#define expf(a) orc_ulp_nudge(std::exp(static_cast<float>(a)), static_cast<float>(a))
#define logf(a) orc_ulp_nudge(std::log(static_cast<float>(a)), static_cast<float>(a))
#define sinf(a) orc_ulp_nudge(std::sin(static_cast<float>(a)), static_cast<float>(a))
#define cosf(a) orc_ulp_nudge(std::cos(static_cast<float>(a)), static_cast<float>(a))
#define acosf(a) orc_ulp_nudge(std::acos(static_cast<float>(a)), static_cast<float>(a))
