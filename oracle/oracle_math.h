// Oracle math kernel — TEST INFRASTRUCTURE ONLY.
//
// Scalar CPU restatement of the reference's device vector math
// (src/realtime/gpu/device_math.h:20-88), its RNG (src/realtime/gpu/programs.cu:104-137)
// and the shared light / reservoir helpers (src/common/light_sampling.h:64-124,
// src/common/restir_di.h:58-199). Only tests/, __graft_entry__.smoke() and
// bench.py's cpu_baseline / reference legs use it, as the oracle.
//
// Build with -ffp-contract=off so every a*b+c rounds twice, as the CUDA
// product does under --fmad=false.
#pragma once

#include <cmath>
#include <cstdint>

namespace orc {

struct V3 {
    float x, y, z;
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(const V3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 mul(const V3& v, float s) { return {v.x * s, v.y * s, v.z * s}; }
// device_math.h:36-39: division is a multiply by the reciprocal.
inline V3 divs(const V3& v, float s) {
    const float inv = 1.0f / s;
    return {v.x * inv, v.y * inv, v.z * inv};
}
inline float dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float len_sq(const V3& v) { return dot(v, v); }
inline float len(const V3& v) { return std::sqrt(len_sq(v)); }
// device_math.h:59-65: a vector no longer than 1e-8 normalizes to zero.
inline V3 normalize(const V3& v) {
    const float l = len(v);
    if (l <= 1e-8f) return {0.0f, 0.0f, 0.0f};
    return divs(v, l);
}
inline V3 reflect(const V3& i, const V3& n) { return sub(i, mul(n, 2.0f * dot(i, n))); }
inline V3 refract(const V3& i, const V3& n, float eta) {
    const float cos_theta = std::fmin(dot(mul(i, -1.0f), n), 1.0f);
    const V3 perp = mul(add(i, mul(n, cos_theta)), eta);
    const float k = 1.0f - len_sq(perp);
    const V3 par = mul(n, -std::sqrt(std::fmax(k, 0.0f)));
    return add(perp, par);
}
inline float max_comp(const V3& v) { return std::fmax(v.x, std::fmax(v.y, v.z)); }
inline V3 clamp3(const V3& v, float lo, float hi) {
    return {std::fmin(std::fmax(v.x, lo), hi), std::fmin(std::fmax(v.y, lo), hi),
        std::fmin(std::fmax(v.z, lo), hi)};
}
inline bool near_zero(const V3& v) {
    return std::fabs(v.x) < 1e-7f && std::fabs(v.y) < 1e-7f && std::fabs(v.z) < 1e-7f;
}
inline V3 from3(const float* p) { return {p[0], p[1], p[2]}; }

// ---- RNG: programs.cu:104-137 --------------------------------------------
inline uint32_t hash_u32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
inline uint32_t rng_for(int pixel_index, int sample, uint32_t stream) {
    const uint32_t seed = static_cast<uint32_t>(pixel_index) * 1973u
                          ^ static_cast<uint32_t>(sample + 1) * 9277u
                          ^ static_cast<uint32_t>(stream + 1) * 26699u ^ 0x9e3779b9u;
    return hash_u32(seed);
}
inline float rnd(uint32_t& s) {
    s = s * 1664525u + 1013904223u;
    return static_cast<float>(s & 0x00ffffffu) * (1.0f / 16777216.0f);
}
// Multi-draw calls evaluate their draws left to right (x, then y, then z).
inline V3 random_in_unit_sphere(uint32_t& rng) {
    for (;;) {
        const float a = rnd(rng) * 2.0f - 1.0f;
        const float b = rnd(rng) * 2.0f - 1.0f;
        const float c = rnd(rng) * 2.0f - 1.0f;
        const V3 p{a, b, c};
        if (len_sq(p) < 1.0f) return p;
    }
}
inline V3 random_unit_vector(uint32_t& rng) { return normalize(random_in_unit_sphere(rng)); }

// ---- light_sampling.h:64-124 ----------------------------------------------
constexpr float kPi = 3.14159265358979323846f;
inline float uniform_sphere_pdf() { return 0.07957747154594767f; }
inline float uniform_cone_pdf(float cos_theta_max) {
    const float solid_angle = 6.28318530717958648f * (1.0f - cos_theta_max);
    return solid_angle > 1e-12f ? 1.0f / solid_angle : 0.0f;
}
inline float area_to_solid_angle_pdf(float area, float d2, float abs_cos) {
    if (area <= 1e-12f || d2 <= 0.0f || abs_cos <= 1e-8f) return 0.0f;
    return d2 / (area * abs_cos);
}
inline float power_heuristic(float a, float b) {
    if (a <= 0.0f) return 0.0f;
    const float a2 = a * a;
    const float b2 = b * b;
    return a2 / (a2 + b2);
}
// Linear CDF scan of light_sampling.h:90-116 (first i with u < cdf[i]).
template <typename CdfAt>
inline int sample_cdf(int count, float u, CdfAt cdf_at) {
    if (count <= 0) return -1;
    const float s = u < 0.0f ? 0.0f : (u < 1.0f ? u : 0.99999994f);
    for (int i = 0; i < count; ++i) {
        if (s < cdf_at(i)) return i;
    }
    return count - 1;
}
inline void sample_uniform_triangle(float u0, float u1, float& w0, float& w1, float& w2) {
    const float su = std::sqrt(u0 < 0.0f ? 0.0f : (u0 < 1.0f ? u0 : 1.0f));
    w0 = 1.0f - su;
    w1 = su * (1.0f - u1);
    w2 = su * u1;
}

// ---- restir_di.h:21-199 ---------------------------------------------------
struct Candidate {
    int light_index = -1;
    float u0 = 0.0f;
    float u1 = 0.0f;
};
struct Surface {
    float position[3] = {0, 0, 0};
    float normal[3] = {0, 0, 0};
    int material_type = -1;
    int primitive_type = -1;
    int primitive_index = -1;
};
// 84-byte layout of RestirReservoir.
struct Reservoir {
    Candidate selected;
    Surface surface;
    float weight_sum = 0.0f;
    float selected_target = 0.0f;
    float estimator_weight = 0.0f;
    int candidate_count = 0;
    int temporal_candidate_count = 0;
    int spatial_candidate_count = 0;
    int bias_correction_source_count = 0;
    int age = 0;
    int valid = 0;
};
static_assert(sizeof(Reservoir) == 84, "reservoir layout");

struct MergeResult {
    int multiplicity = 0;
    int selected = 0;
};

inline float clamp_unit(float v) { return v < 0.0f ? 0.0f : (v < 1.0f ? v : 0.99999994f); }
inline bool finite_positive(float v) { return v > 0.0f && std::isfinite(v); }

inline bool reservoir_update(Reservoir& r, const Candidate& c, float target, float weight,
    int multiplicity, float u) {
    if (c.light_index < 0 || multiplicity <= 0) return false;
    r.candidate_count += multiplicity;
    if (!finite_positive(target) || !finite_positive(weight)) return false;
    const float next = r.weight_sum + weight;
    if (!finite_positive(next)) return false;
    const bool selected = clamp_unit(u) * next < weight;
    if (selected) {
        r.selected = c;
        r.selected_target = target;
        r.valid = 1;
    }
    r.weight_sum = next;
    return selected;
}

inline void reservoir_finalize(Reservoir& r) {
    r.estimator_weight = 0.0f;
    if (r.valid == 0 || r.candidate_count <= 0 || !finite_positive(r.selected_target)
        || !finite_positive(r.weight_sum)) {
        r.valid = 0;
        return;
    }
    r.estimator_weight = r.weight_sum / (static_cast<float>(r.candidate_count) * r.selected_target);
    if (!finite_positive(r.estimator_weight)) {
        r.valid = 0;
        r.estimator_weight = 0.0f;
    }
}

inline void reservoir_finalize_basic(Reservoir& r, float selected_source_target,
    float source_target_sum, int source_count) {
    r.estimator_weight = 0.0f;
    r.bias_correction_source_count = source_count > 0 ? source_count : 0;
    if (r.valid == 0 || source_count <= 0 || !finite_positive(r.selected_target)
        || !finite_positive(r.weight_sum) || !finite_positive(selected_source_target)
        || !finite_positive(source_target_sum)) {
        r.valid = 0;
        return;
    }
    r.estimator_weight =
        r.weight_sum * selected_source_target / (r.selected_target * source_target_sum);
    if (!finite_positive(r.estimator_weight)) {
        r.valid = 0;
        r.estimator_weight = 0.0f;
    }
}

inline bool surface_valid(const Surface& cur, const Reservoir& prev, float max_dist,
    float min_dot, int max_age) {
    if (prev.valid == 0 || prev.selected.light_index < 0 || prev.age < 0 || prev.age >= max_age
        || cur.material_type != prev.surface.material_type
        || cur.primitive_type != prev.surface.primitive_type
        || cur.primitive_index != prev.surface.primitive_index) {
        return false;
    }
    const float limit = max_dist > 0.0f ? max_dist : 0.0f;
    const float dx = cur.position[0] - prev.surface.position[0];
    const float dy = cur.position[1] - prev.surface.position[1];
    const float dz = cur.position[2] - prev.surface.position[2];
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float nd = cur.normal[0] * prev.surface.normal[0] + cur.normal[1] * prev.surface.normal[1]
                     + cur.normal[2] * prev.surface.normal[2];
    return d2 <= limit * limit && nd >= min_dot;
}

inline MergeResult reservoir_merge(Reservoir& cur, const Reservoir& prev, float target_at_current,
    int max_candidates, float u, bool temporal) {
    if (prev.valid == 0 || prev.candidate_count <= 0 || !finite_positive(prev.estimator_weight)) {
        return {};
    }
    int m = prev.candidate_count;
    if (max_candidates > 0 && m > max_candidates) m = max_candidates;
    const float w = finite_positive(target_at_current)
                        ? target_at_current * prev.estimator_weight * static_cast<float>(m)
                        : 0.0f;
    const bool sel = reservoir_update(cur, prev.selected, target_at_current, w, m, u);
    if (temporal) {
        cur.temporal_candidate_count += m;
        cur.age = prev.age + 1;
    } else {
        cur.spatial_candidate_count += m;
    }
    return MergeResult{m, sel ? 1 : 0};
}

}  // namespace orc
