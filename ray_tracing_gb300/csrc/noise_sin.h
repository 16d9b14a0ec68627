// The sine of the hash-noise texture, identical on the host and the device.
//
// The reference's noise texture (programs.cu:184-209: hash_noise and
// turbulence, evaluated by evaluate_texture at :268-302) hashes a point with
// fract(sin(dot(p, k)) * 43758.5453). The factor 43758 turns a one-ulp
// difference of sin into a change of about 3e-3 in the hash, so two correct
// single-precision sines (CUDA's sinf and the host libm's sinf) that differ in
// the last bit give visibly different noise. This file evaluates that sine with
// one sequence of IEEE single-precision operations (+, -, *, fused multiply-add,
// floor and round-to-nearest-integer, each correctly rounded on both
// processors), so the CUDA kernels and the CPU oracle produce the same bits.
//
// Method: Cody-Waite argument reduction (W. J. Cody and W. Waite, "Software
// Manual for the Elementary Functions", 1980) by the nearest multiple k of
// pi/2, with pi/2 split into three single-precision parts applied by fused
// multiply-adds (the first product is exact for |x| < 2^24, so the reduced
// argument carries an absolute error of about 2^-25), then the Taylor series of
// sin and cos about 0 on |r| <= pi/4 (+ the reduction's slack), truncated after
// r^9 and r^10 (truncation error below 2e-9), chosen by the quadrant k mod 4.
// Accuracy (measured against the double-precision libm sine rounded to float):
// within 1 ulp for |x| < 2^17 and 3 ulp (absolute error below 2e-7) for
// |x| < 2^22; larger or non-finite arguments still give one deterministic
// result on both sides.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define RTGB_NOISE_HD __host__ __device__ __forceinline__
#else
#define RTGB_NOISE_HD inline
#endif

namespace rtgb_noise {

RTGB_NOISE_HD float fma_rn(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

RTGB_NOISE_HD float round_even(float v) {
#if defined(__CUDA_ARCH__)
    return rintf(v);
#else
    return std::nearbyint(v);  // the default rounding mode: to nearest, ties to even
#endif
}

RTGB_NOISE_HD float floor_f(float v) {
#if defined(__CUDA_ARCH__)
    return floorf(v);
#else
    return std::floor(v);
#endif
}

// sin(x) for the noise texture (see the file comment).
RTGB_NOISE_HD float noise_sinf(float x) {
    // pi/2 = kP1 + kP2 + kP3 (the leading 72 bits, each part a float)
    constexpr float kTwoOverPi = 0.6366197466850281f;
    constexpr float kP1 = 1.5707963705062866f;
    constexpr float kP2 = -4.371138828673793e-08f;
    constexpr float kP3 = -1.7151245100058819e-15f;
    const float k = round_even(x * kTwoOverPi);
    float r = fma_rn(-k, kP1, x);
    r = fma_rn(-k, kP2, r);
    r = fma_rn(-k, kP3, r);
    // quadrant k mod 4, exact for integer-valued k below 2^24
    const float kq = k - 4.0f * floor_f(k * 0.25f);
    const int q = kq >= 0.0f && kq < 4.0f ? static_cast<int>(kq) : 0;
    const float r2 = r * r;
    // Taylor coefficients 1/n! with alternating signs
    float s = fma_rn(r2, 2.7557318844628753e-06f, -0.00019841270113829523f);  // 1/9!, -1/7!
    s = fma_rn(r2, s, 0.008333333767950535f);                                 // 1/5!
    s = fma_rn(r2, s, -0.1666666716337204f);                                  // -1/3!
    const float sin_r = fma_rn(r * r2, s, r);
    float c = fma_rn(r2, -2.755731998149713e-07f, 2.4801587642286904e-05f);   // -1/10!, 1/8!
    c = fma_rn(r2, c, -0.0013888889225199819f);                               // -1/6!
    c = fma_rn(r2, c, 0.0416666679084301f);                                   // 1/4!
    c = fma_rn(r2, c, -0.5f);                                                 // -1/2!
    const float cos_r = fma_rn(r2, c, 1.0f);
    const float v = (q & 1) ? cos_r : sin_r;
    return (q & 2) ? -v : v;
}

}  // namespace rtgb_noise
