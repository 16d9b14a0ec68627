// Small dense-matrix helpers of the SceneIR v2 layer (row-major 4x4 affine
// and 3x3 matrices as std::array<double>), in place of the Eigen calls the
// reference's scene code makes.
#pragma once

#include <array>
#include <cmath>

#include "rtgb_scene_ir_v2.hpp"

namespace rtgb::scene::math {

using Mat3 = std::array<double, 9>;

inline double at(const Mat4& m, int r, int c) { return m[static_cast<size_t>(4 * r + c)]; }

inline Mat4 mul(const Mat4& a, const Mat4& b) {
    Mat4 out {};
    for (int r = 0; r < 4; ++r) {
        for (int c = 0; c < 4; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += at(a, r, k) * at(b, k, c);
            out[static_cast<size_t>(4 * r + c)] = s;
        }
    }
    return out;
}

inline Mat3 linear(const Mat4& m) {
    return {at(m, 0, 0), at(m, 0, 1), at(m, 0, 2), at(m, 1, 0), at(m, 1, 1), at(m, 1, 2), at(m, 2, 0), at(m, 2, 1),
        at(m, 2, 2)};
}

inline Vec3 translation(const Mat4& m) { return {at(m, 0, 3), at(m, 1, 3), at(m, 2, 3)}; }

inline double det(const Mat3& a) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
}

// inverse by the adjugate; the caller checks the determinant
inline Mat3 inverse(const Mat3& a) {
    const double d = det(a);
    Mat3 out {a[4] * a[8] - a[5] * a[7], a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
        a[5] * a[6] - a[3] * a[8], a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
        a[3] * a[7] - a[4] * a[6], a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
    const double inv = 1.0 / d;  // cofactors scaled by 1/det, as Eigen's 3x3 inverse does
    for (double& v : out) v *= inv;
    return out;
}

inline Vec3 mul3(const Mat3& a, const Vec3& v) {
    return {a[0] * v[0] + a[1] * v[1] + a[2] * v[2], a[3] * v[0] + a[4] * v[1] + a[5] * v[2],
        a[6] * v[0] + a[7] * v[1] + a[8] * v[2]};
}

inline Vec3 mul3_transposed(const Mat3& a, const Vec3& v) {
    return {a[0] * v[0] + a[3] * v[1] + a[6] * v[2], a[1] * v[0] + a[4] * v[1] + a[7] * v[2],
        a[2] * v[0] + a[5] * v[1] + a[8] * v[2]};
}

inline Vec3 column(const Mat3& a, int c) { return {a[static_cast<size_t>(c)], a[static_cast<size_t>(3 + c)], a[static_cast<size_t>(6 + c)]}; }

inline Vec3 point(const Mat4& m, const Vec3& p) {
    const Vec3 l = mul3(linear(m), p);
    return {l[0] + at(m, 0, 3), l[1] + at(m, 1, 3), l[2] + at(m, 2, 3)};
}

inline Vec3 cross(const Vec3& a, const Vec3& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}

inline double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline double norm(const Vec3& a) { return std::sqrt(dot(a, a)); }

template <class A>
bool all_finite(const A& a) {
    for (const auto& v : a) {
        if (!std::isfinite(static_cast<double>(v))) return false;
    }
    return true;
}

template <class A>
bool any_negative(const A& a) {
    for (const auto& v : a) {
        if (v < 0) return true;
    }
    return false;
}

}  // namespace rtgb::scene::math
