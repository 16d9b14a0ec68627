// Device building blocks of the wavefront path tracer (sm_103a).
//
// Per-path arithmetic follows the reference's device functions operation for
// operation (src/realtime/gpu/programs.cu, src/realtime/gpu/device_math.h,
// src/common/light_sampling.h, src/common/restir_di.h) so that, compiled with
// --fmad=false, one path reproduces the reference's radiance. The data layout
// around it (SoA path streams, leaf-ordered primitive records, BVH2 nodes with
// child boxes inline) is this project's own.
#pragma once

#include <climits>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "rtgb.h"

#define RTGB_HD __host__ __device__ __forceinline__
#define RTGB_D __device__ __forceinline__

namespace rtgb {

constexpr float kRayEpsilon = 1e-3f;
constexpr float kRayFar = 1e30f;
constexpr float kPi = 3.14159265358979323846f;
constexpr double kCameraEpsilon = 1e-12;
constexpr int kTraversalStack = 64;

// ---- float3 arithmetic (device_math.h:20-88) --------------------------------
RTGB_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
RTGB_HD float3 add(const float3& a, const float3& b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
RTGB_HD float3 sub(const float3& a, const float3& b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
RTGB_HD float3 mul(const float3& a, const float3& b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
RTGB_HD float3 mul(const float3& v, float s) { return f3(v.x * s, v.y * s, v.z * s); }
RTGB_HD float3 divs(const float3& v, float s) {
    const float inv = 1.0f / s;
    return f3(v.x * inv, v.y * inv, v.z * inv);
}
RTGB_HD float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RTGB_HD float3 cross(const float3& a, const float3& b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
RTGB_HD float len_sq(const float3& v) { return dot(v, v); }
RTGB_HD float len(const float3& v) { return sqrtf(len_sq(v)); }
RTGB_HD float3 normalize(const float3& v) {
    const float l = len(v);
    if (l <= 1e-8f) return f3(0.0f, 0.0f, 0.0f);
    return divs(v, l);
}
RTGB_HD float3 reflect(const float3& i, const float3& n) { return sub(i, mul(n, 2.0f * dot(i, n))); }
RTGB_HD float3 refract(const float3& i, const float3& n, float eta) {
    const float ct = fminf(dot(mul(i, -1.0f), n), 1.0f);
    const float3 perp = mul(add(i, mul(n, ct)), eta);
    const float k = 1.0f - len_sq(perp);
    return add(perp, mul(n, -sqrtf(fmaxf(k, 0.0f))));
}
RTGB_HD float max_comp(const float3& v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
RTGB_HD float3 clamp3(const float3& v, float lo, float hi) {
    return f3(fminf(fmaxf(v.x, lo), hi), fminf(fmaxf(v.y, lo), hi), fminf(fmaxf(v.z, lo), hi));
}
RTGB_HD bool near_zero(const float3& v) {
    return fabsf(v.x) < 1e-7f && fabsf(v.y) < 1e-7f && fabsf(v.z) < 1e-7f;
}
RTGB_HD float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
RTGB_HD float3 xyz(const float4& v) { return f3(v.x, v.y, v.z); }
RTGB_HD float4 f4(const float3& v, float w) { return make_float4(v.x, v.y, v.z, w); }

// ---- per-path RNG (programs.cu:104-137) ---------------------------------------
RTGB_HD uint32_t hash_u32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
RTGB_HD uint32_t rng_for(int pixel, int sample, uint32_t stream) {
    return hash_u32(static_cast<uint32_t>(pixel) * 1973u ^ static_cast<uint32_t>(sample + 1) * 9277u
                    ^ static_cast<uint32_t>(stream + 1) * 26699u ^ 0x9e3779b9u);
}
RTGB_HD float rnd(uint32_t& s) {
    s = s * 1664525u + 1013904223u;
    return static_cast<float>(s & 0x00ffffffu) * (1.0f / 16777216.0f);
}
// Bounds of the device loops that have no fixed trip count. The defaults never
// bind on real inputs; a smaller limit (rtgb_create_info's debug fields) makes
// a loop give up early so the error path can be exercised. A loop that reaches
// its bound counts itself in *gave_up and returns a defined value.
constexpr int kDefaultTraversalLimit = 1 << 24;
constexpr int kDefaultRejectionLimit = 1000000;

struct LoopBounds {
    int traversal;   // wide-BVH node visits per ray
    int rejection;   // draws of random_in_unit_sphere
    int* gave_up;    // per-frame count of loops that reached their bound (device word)
};

// Draws are consumed left to right (x, y, z).
RTGB_D float3 random_in_unit_sphere(uint32_t& rng, const LoopBounds& lb) {
    // The reference loops until acceptance; 1e6 rejections have probability
    // (1 - pi/6)^1e6, so the default bound never binds but keeps the loop finite.
    for (int guard = 0; guard < lb.rejection; ++guard) {
        const float a = rnd(rng) * 2.0f - 1.0f;
        const float b = rnd(rng) * 2.0f - 1.0f;
        const float c = rnd(rng) * 2.0f - 1.0f;
        const float3 p = f3(a, b, c);
        if (len_sq(p) < 1.0f) return p;
    }
    if (lb.gave_up) atomicAdd(lb.gave_up, 1);
    return f3(0.0f, 0.0f, 0.0f);
}
RTGB_D float3 random_unit_vector(uint32_t& rng, const LoopBounds& lb) {
    return normalize(random_in_unit_sphere(rng, lb));
}

// ---- light pdfs (light_sampling.h:64-124) --------------------------------------
RTGB_HD float uniform_sphere_pdf() { return 0.07957747154594767f; }
RTGB_HD float uniform_cone_pdf(float ctm) {
    const float sa = 6.28318530717958648f * (1.0f - ctm);
    return sa > 1e-12f ? 1.0f / sa : 0.0f;
}
RTGB_HD float area_pdf(float area, float d2, float ac) {
    if (area <= 1e-12f || d2 <= 0.0f || ac <= 1e-8f) return 0.0f;
    return d2 / (area * ac);
}
RTGB_HD float power_heuristic(float a, float b) {
    if (a <= 0.0f) return 0.0f;
    const float a2 = a * a;
    const float b2 = b * b;
    return a2 / (a2 + b2);
}
// First i with u < cdf[i] (else count-1): an upper-bound binary search over the
// non-decreasing CDF returns the same index as the reference's linear scan
// (light_sampling.h:90-116) in O(log n).
RTGB_D int sample_cdf(const float* cdf, int count, float u) {
    if (count <= 0) return -1;
    const float s = u < 0.0f ? 0.0f : (u < 1.0f ? u : 0.99999994f);
    int lo = 0, hi = count;  // first index in [lo, hi) with s < cdf[i]
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s < cdf[mid]) hi = mid;  // cdf may live in shared or global memory
        else lo = mid + 1;
    }
    return lo < count ? lo : count - 1;
}
constexpr int kGuide = 1024;          // CDF guide-table buckets

// First i with u < cdf[i] (else count-1), the same index as sample_cdf, found
// from a guide table: guide[j] = first i with j/kGuide < cdf[i] bounds the
// answer for u in [j/kGuide, (j+1)/kGuide) between guide[j] and guide[j+1]
// (guide[kGuide] = count), so the bisection covers one bucket.
RTGB_D int sample_cdf_guided(const float* cdf, const int* guide, int count, float u) {
    if (count <= 0) return -1;
    const float s = u < 0.0f ? 0.0f : (u < 1.0f ? u : 0.99999994f);
    const int j = static_cast<int>(s * static_cast<float>(kGuide));
    int lo = guide[j], hi = guide[j + 1];
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s < cdf[mid]) hi = mid;
        else lo = mid + 1;
    }
    return lo < count ? lo : count - 1;
}

RTGB_HD void sample_uniform_triangle(float u0, float u1, float& w0, float& w1, float& w2) {
    const float su = sqrtf(u0 < 0.0f ? 0.0f : (u0 < 1.0f ? u0 : 1.0f));
    w0 = 1.0f - su;
    w1 = su * (1.0f - u1);
    w2 = su * u1;
}

// ---- reservoirs (restir_di.h:21-199), the reference's 84-byte layout ----------
struct Candidate {
    int light_index;
    float u0;
    float u1;
};
struct Surface {
    float position[3];
    float normal[3];
    int material_type;
    int primitive_type;
    int primitive_index;
};
struct Reservoir {
    Candidate selected;
    Surface surface;
    float weight_sum;
    float selected_target;
    float estimator_weight;
    int candidate_count;
    int temporal_candidate_count;
    int spatial_candidate_count;
    int bias_correction_source_count;
    int age;
    int valid;
};
static_assert(sizeof(Reservoir) == 84, "RestirReservoir layout");

RTGB_HD Reservoir empty_reservoir() {
    Reservoir r;
    r.selected = Candidate{-1, 0.0f, 0.0f};
    for (int i = 0; i < 3; ++i) {
        r.surface.position[i] = 0.0f;
        r.surface.normal[i] = 0.0f;
    }
    r.surface.material_type = -1;
    r.surface.primitive_type = -1;
    r.surface.primitive_index = -1;
    r.weight_sum = 0.0f;
    r.selected_target = 0.0f;
    r.estimator_weight = 0.0f;
    r.candidate_count = 0;
    r.temporal_candidate_count = 0;
    r.spatial_candidate_count = 0;
    r.bias_correction_source_count = 0;
    r.age = 0;
    r.valid = 0;
    return r;
}

// The per-launch cudaMemsetAsync of the reservoir buffer (optix_renderer.cpp:
// 253-254): every field zero, which is what pixels without ReSTIR keep.
RTGB_HD Reservoir zero_reservoir() {
    Reservoir r = empty_reservoir();
    r.selected.light_index = 0;
    r.surface.material_type = 0;
    r.surface.primitive_type = 0;
    r.surface.primitive_index = 0;
    return r;
}

RTGB_HD float clamp_unit(float v) { return v < 0.0f ? 0.0f : (v < 1.0f ? v : 0.99999994f); }
RTGB_HD bool finite_positive(float v) { return v > 0.0f && isfinite(v); }

RTGB_HD bool reservoir_update(Reservoir& r, const Candidate& c, float target, float weight, int m, float u) {
    if (c.light_index < 0 || m <= 0) return false;
    r.candidate_count += m;
    if (!finite_positive(target) || !finite_positive(weight)) return false;
    const float next = r.weight_sum + weight;
    if (!finite_positive(next)) return false;
    const bool sel = clamp_unit(u) * next < weight;
    if (sel) {
        r.selected = c;
        r.selected_target = target;
        r.valid = 1;
    }
    r.weight_sum = next;
    return sel;
}

RTGB_HD void reservoir_finalize(Reservoir& r) {
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

RTGB_HD void reservoir_finalize_basic(Reservoir& r, float sel_t, float sum, int n) {
    r.estimator_weight = 0.0f;
    r.bias_correction_source_count = n > 0 ? n : 0;
    if (r.valid == 0 || n <= 0 || !finite_positive(r.selected_target) || !finite_positive(r.weight_sum)
        || !finite_positive(sel_t) || !finite_positive(sum)) {
        r.valid = 0;
        return;
    }
    r.estimator_weight = r.weight_sum * sel_t / (r.selected_target * sum);
    if (!finite_positive(r.estimator_weight)) {
        r.valid = 0;
        r.estimator_weight = 0.0f;
    }
}

RTGB_HD bool surface_valid(const Surface& cur, const Reservoir& prev, float max_dist, float min_dot, int max_age) {
    if (prev.valid == 0 || prev.selected.light_index < 0 || prev.age < 0 || prev.age >= max_age
        || cur.material_type != prev.surface.material_type || cur.primitive_type != prev.surface.primitive_type
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

struct MergeResult {
    int multiplicity;
    int selected;
};

RTGB_HD MergeResult reservoir_merge(Reservoir& cur, const Reservoir& prev, float target, int max_c, float u,
    bool temporal) {
    if (prev.valid == 0 || prev.candidate_count <= 0 || !finite_positive(prev.estimator_weight)) {
        return MergeResult{0, 0};
    }
    int m = prev.candidate_count;
    if (max_c > 0 && m > max_c) m = max_c;
    const float w = finite_positive(target) ? target * prev.estimator_weight * static_cast<float>(m) : 0.0f;
    const bool sel = reservoir_update(cur, prev.selected, target, w, m, u);
    if (temporal) {
        cur.temporal_candidate_count += m;
        cur.age = prev.age + 1;
    } else {
        cur.spatial_candidate_count += m;
    }
    return MergeResult{m, sel ? 1 : 0};
}

// ---- reservoirs in HBM ----------------------------------------------------------
//
// A frame reservoir is stored as 96 bytes on a 32-byte boundary, three DRAM
// sectors ordered by which pass reads them, instead of the 84-byte record the
// algebra above works on:
//   sector 0 (q[0], q[1]) surface: position xyz, normal xyz, primitive index,
//            material type and primitive type (8 bits each, sign-extended)
//   sector 1 (q[2], q[3]) sample: selected light, u0, u1, valid; age,
//            candidate count, estimator weight, (spare)
//   sector 2 (q[4], q[5]) sums: weight sum, selected target, temporal,
//            spatial and bias-correction source counts, (spare)
// A temporal or spatial reuse reads sectors 0 and 1 (surface_valid and
// reservoir_merge read nothing else), a bias-correction ray sector 0, the
// finalisation sectors 1 and 2. All-zero bits decode to zero_reservoir().
struct alignas(32) ReservoirRec {
    float4 q[6];
};
static_assert(sizeof(ReservoirRec) == 96, "ReservoirRec layout");

// Bit casts usable on the host (the record is converted there for downloads).
RTGB_HD float bits_f(int v) {
    float f;
    memcpy(&f, &v, sizeof f);
    return f;
}
RTGB_HD int bits_i(float v) {
    int i;
    memcpy(&i, &v, sizeof i);
    return i;
}

RTGB_HD int pack_types(int material_type, int primitive_type) {
    return (material_type & 0xff) | ((primitive_type & 0xff) << 8);
}
RTGB_HD int unpack_type(int packed, int shift) {
    return static_cast<int>(static_cast<signed char>((packed >> shift) & 0xff));
}

RTGB_HD void pack_surface(const Surface& s, float4& a, float4& b) {
    a = make_float4(s.position[0], s.position[1], s.position[2], s.normal[0]);
    b = make_float4(s.normal[1], s.normal[2], bits_f(s.primitive_index),
        bits_f(pack_types(s.material_type, s.primitive_type)));
}
RTGB_HD Surface unpack_surface(const float4& a, const float4& b) {
    Surface s;
    s.position[0] = a.x;
    s.position[1] = a.y;
    s.position[2] = a.z;
    s.normal[0] = a.w;
    s.normal[1] = b.x;
    s.normal[2] = b.y;
    s.primitive_index = bits_i(b.z);
    const int t = bits_i(b.w);
    s.material_type = unpack_type(t, 0);
    s.primitive_type = unpack_type(t, 8);
    return s;
}

RTGB_HD void pack_sample(const Reservoir& r, float4& a, float4& b) {
    a = make_float4(bits_f(r.selected.light_index), r.selected.u0, r.selected.u1, bits_f(r.valid));
    b = make_float4(bits_f(r.age), bits_f(r.candidate_count), r.estimator_weight, 0.0f);
}
RTGB_HD void unpack_sample(const float4& a, const float4& b, Reservoir& r) {
    r.selected.light_index = bits_i(a.x);
    r.selected.u0 = a.y;
    r.selected.u1 = a.z;
    r.valid = bits_i(a.w);
    r.age = bits_i(b.x);
    r.candidate_count = bits_i(b.y);
    r.estimator_weight = b.z;
}

RTGB_HD void pack_sums(const Reservoir& r, float4& a, float4& b) {
    a = make_float4(r.weight_sum, r.selected_target, bits_f(r.temporal_candidate_count),
        bits_f(r.spatial_candidate_count));
    b = make_float4(bits_f(r.bias_correction_source_count), 0.0f, 0.0f, 0.0f);
}
RTGB_HD void unpack_sums(const float4& a, const float4& b, Reservoir& r) {
    r.weight_sum = a.x;
    r.selected_target = a.y;
    r.temporal_candidate_count = bits_i(a.z);
    r.spatial_candidate_count = bits_i(a.w);
    r.bias_correction_source_count = bits_i(b.x);
}

RTGB_HD void store_reservoir(ReservoirRec* p, const Reservoir& r) {
    float4 q[6];
    pack_surface(r.surface, q[0], q[1]);
    pack_sample(r, q[2], q[3]);
    pack_sums(r, q[4], q[5]);
#pragma unroll
    for (int k = 0; k < 6; ++k) p->q[k] = q[k];
}

RTGB_HD Reservoir load_reservoir(const ReservoirRec* p) {
    Reservoir r;
    r.surface = unpack_surface(p->q[0], p->q[1]);
    unpack_sample(p->q[2], p->q[3], r);
    unpack_sums(p->q[4], p->q[5], r);
    return r;
}

// The fields a temporal or spatial reuse reads (sectors 0 and 1); the sums
// are left zero (surface_valid and reservoir_merge do not read them).
RTGB_HD Reservoir load_reuse(const ReservoirRec* p) {
    Reservoir r = zero_reservoir();
    r.surface = unpack_surface(p->q[0], p->q[1]);
    unpack_sample(p->q[2], p->q[3], r);
    return r;
}

// ---- device scene ------------------------------------------------------------

// Emissive-geometry light (PackedLight, light_sampling.h:22-27).
struct PackedLight {
    int type;  // 0 sphere, 1 quad, 2 triangle, 3 environment
    int primitive_index;
    float selection_pdf;
    float cdf;
};

// One leaf-ordered primitive record, 64 bytes (four float4):
//   sphere:   [0] center.xyz radius
//   quad:     [0] origin.xyz n.x  [1] edge_u.xyz n.y  [2] edge_v.xyz n.z  [3] w.xyz
//   triangle: [0] p0.xyz          [1] e1.xyz          [2] e2.xyz
// [3].w always holds the primitive code (type << 28 | index) as int bits.
// n = unit quad normal and w = n / |n|^2 are computed on the host with the
// reference's float operations (programs.cu:1451-1476), e1/e2 = p1-p0, p2-p0.
struct PrimRecord {
    float4 q[4];
};

// BVH2 node with both children's boxes inline, 64 bytes:
//   a = (c0.lo.xyz, c0 child) b = (c0.hi.xyz, c1 child) c = (c1.lo.xyz, -) d = (c1.hi.xyz, -)
// A child >= 0 is an internal node; a child < 0 is the leaf of sorted slot ~child.
struct BvhNode {
    float4 a, b, c, d;
};

constexpr int kAnalyticHot = 5;

// Wide (4-ary) BVH node, 128 bytes = 8 float4, collapsed from the binary LBVH
// (every BVH4 node is a binary node at even depth, its children the binary
// node's children or grandchildren) and numbered breadth-first, so the top
// levels are a prefix of the array that kernels can stage in shared memory:
//   q[0..2] = lo.x, lo.y, lo.z of children 0..3, q[3..5] = hi.x, hi.y, hi.z,
//   q[6] = child indices as int bits (>= 0 a BVH4 node, < 0 the leaf of sorted
//   slot ~c, kEmptyChild unused), q[7] unused.
constexpr int kNode4 = 8;                 // float4 per BVH4 node
constexpr int kEmptyChild = INT_MIN;
constexpr int kStagedNodes4 = 64;         // BVH4 nodes the trace kernels keep in shared memory (8 KB)

struct DeviceScene {
    const PrimRecord* prims;      // leaf order
    const BvhNode* nodes;         // binary LBVH (build, refit, parity downloads)
    int prim_count;
    int node_count;
    const float4* nodes4;         // wide BVH traversed by every ray (kNode4 float4 per node)
    int node4_count;
    const rtgb_sphere* spheres;
    const rtgb_quad* quads;
    const rtgb_triangle* triangles;
    const rtgb_medium* media;
    const rtgb_material* materials;
    const rtgb_texture* textures;
    const float* texels;           // RGB triplets
    int sphere_count, quad_count, triangle_count, medium_count, material_count, texture_count, texel_count;
    const PackedLight* lights;
    const float* light_cdf;
    const int* light_guide;       // kGuide + 1 bucket starts over light_cdf (sample_cdf_guided)
    int light_count;
    int environment_light;        // index into lights or -1
    const int* sphere_light;       // primitive -> light index or -1
    const int* quad_light;
    const int* triangle_light;
    const rtgb_analytic_light* analytic;
    // per light, kAnalyticHot float4 built once at prepare with the fields the
    // light sampler reads (one aligned 16-byte load each instead of scalar
    // loads of the 108-byte rtgb_analytic_light): (position, selection_pdf),
    // (basis_x, width or radius), (basis_y, height or length),
    // (radiance, world_area), (analytic_light_normal, type as int bits)
    const float4* analytic_hot;
    const float* analytic_cdf;
    const int* analytic_guide;    // kGuide + 1 bucket starts over analytic_cdf
    int analytic_count;
    const BvhNode* analytic_nodes;  // BVH over finite, non-point analytic lights
    const int* analytic_leaf;       // sorted slot -> analytic light index
    int analytic_bvh_count;
    int analytic_node_count;
    const int* infinite_analytic;   // distant/dome light indices, reference order
    int infinite_analytic_count;
    const rtgb_openpbr_material* openpbr;  // compiled OpenPBR materials (rtgb_material::openpbr_index)
    int openpbr_count;
    float background[3];
    LoopBounds bounds;              // traversal / rejection bounds and the gave-up word
};

// ---- cameras: programs.cu:304-537 ------------------------------------------------

struct CameraDev {
    int width, height, model, lut_monotone;
    long long pixel_offset;   // first pixel of this camera in frame-wide arrays
    long long path_offset;    // pixel_offset * spp
    float origin_f[3], bx_f[3], by_f[3], bz_f[3];  // static_cast<float> of the double pose
    double origin[3], bx[3], by[3], bz[3];
    double pin[9];                                  // fx fy cx cy k1 k2 k3 p1 p2
    double eq_fx, eq_fy, eq_cx, eq_cy, eq_tan[2], lut_step;
    const double* lut;                              // 1024 doubles (device)
    const float4* dirs;                             // per-pixel camera-space direction
};

struct D2 {
    double x, y;
};

RTGB_HD D2 distort_pinhole(const double* p, const D2& xy) {
    const double x = xy.x, y = xy.y;
    const double x2 = x * x, y2 = y * y, xyt = x * y;
    const double r2 = x2 + y2, r4 = r2 * r2, r6 = r4 * r2;
    const double radial = 1.0 + p[4] * r2 + p[5] * r4 + p[6] * r6;
    return D2{x * radial + p[8] * (r2 + 2.0 * x2) + 2.0 * p[7] * xyt,
        y * radial + p[7] * (r2 + 2.0 * y2) + 2.0 * p[8] * xyt};
}

RTGB_HD bool solve2(double a00, double a01, double a10, double a11, const D2& rhs, D2& d) {
    const double det = a00 * a11 - a01 * a10;
    if (fabs(det) < kCameraEpsilon) return false;
    const double inv = 1.0 / det;
    d.x = (a11 * rhs.x - a01 * rhs.y) * inv;
    d.y = (-a10 * rhs.x + a00 * rhs.y) * inv;
    return true;
}

RTGB_HD float3 unproject_pinhole(const double* p, double px, double py) {
    const D2 xd{(px - p[2]) / p[0], (py - p[3]) / p[1]};
    D2 xy = xd;
    for (int it = 0; it < 24; ++it) {
        const D2 dist = distort_pinhole(p, xy);
        const D2 err{xd.x - dist.x, xd.y - dist.y};
        if (err.x * err.x + err.y * err.y < 1e-20) break;
        const double x = xy.x, y = xy.y;
        const double r2 = x * x + y * y, r4 = r2 * r2, r6 = r4 * r2;
        const double radial = 1.0 + p[4] * r2 + p[5] * r4 + p[6] * r6;
        const double drdx = 2.0 * x * (p[4] + 2.0 * p[5] * r2 + 3.0 * p[6] * r4);
        const double drdy = 2.0 * y * (p[4] + 2.0 * p[5] * r2 + 3.0 * p[6] * r4);
        D2 d{0.0, 0.0};
        if (!solve2(radial + x * drdx + 6.0 * p[8] * x + 2.0 * p[7] * y, x * drdy + 2.0 * p[7] * x + 2.0 * p[8] * y,
                y * drdx + 2.0 * p[7] * x + 2.0 * p[8] * y, radial + y * drdy + 6.0 * p[7] * y + 2.0 * p[8] * x, err,
                d)) {
            break;
        }
        xy.x += d.x;
        xy.y += d.y;
    }
    return normalize(f3(static_cast<float>(xy.x), static_cast<float>(xy.y), 1.0f));
}

RTGB_HD float2 project_pinhole(const double* p, const float3& dir) {
    if (fabsf(dir.z) < 1e-7f) return make_float2(-1.0f, -1.0f);
    const double inv_z = 1.0 / static_cast<double>(dir.z);
    const D2 xu{static_cast<double>(dir.x) * inv_z, static_cast<double>(dir.y) * inv_z};
    const D2 xd = distort_pinhole(p, xu);
    return make_float2(static_cast<float>(xd.x * p[0] + p[2]), static_cast<float>(xd.y * p[1] + p[3]));
}

RTGB_HD D2 equi_tangential(const D2& xy, const double* t) {
    const double xr = xy.x, yr = xy.y;
    const double xr2 = xr * xr, yr2 = yr * yr, xryr = xr * yr;
    return D2{xr + 2.0 * t[0] * xryr + t[1] * (xr2 + yr2 + 2.0 * xr2), yr + t[0] * (xr2 + yr2 + 2.0 * yr2) + 2.0 * t[1] * xryr};
}

RTGB_HD D2 remove_equi_tangential(const D2& xy, const double* t) {
    const D2 dist = equi_tangential(xy, t);
    D2 d{0.0, 0.0};
    if (!solve2(1.0 + 2.0 * t[0] * xy.y + 6.0 * t[1] * xy.x, 2.0 * t[0] * xy.x + 2.0 * t[1] * xy.y,
            2.0 * t[0] * xy.x + 2.0 * t[1] * xy.y, 1.0 + 6.0 * t[0] * xy.y + 2.0 * t[1] * xy.x,
            D2{xy.x - dist.x, xy.y - dist.y}, d)) {
        return xy;
    }
    return D2{xy.x + d.x, xy.y + d.y};
}

// Unprojection of one pixel centre for a camera (FP64, computed once per
// intrinsics change into the camera's direction table).
RTGB_HD float3 unproject_equi(const double fx, const double fy, const double cx, const double cy, const double* tan2,
    const double* lut, double lut_step, double px, double py) {
    const D2 xy{(px - cx) / fx, (py - cy) / fy};
    if (xy.x * xy.x + xy.y * xy.y < kCameraEpsilon * kCameraEpsilon) return f3(0.0f, 0.0f, 1.0f);
    const D2 xr = remove_equi_tangential(xy, tan2);
    const double rd = sqrt(xr.x * xr.x + xr.y * xr.y);
    if (rd < kCameraEpsilon) return f3(0.0f, 0.0f, 1.0f);
    double theta = 0.0;
    bool ok = true;
    if (rd <= 0.0 || lut_step <= 0.0) {
        theta = 0.0;
    } else {
        const double pos = rd / lut_step;
        if (pos > 1023.0) {
            ok = false;
        } else if (pos >= 1023.0) {
            theta = lut[1023];
        } else {
            const int i = static_cast<int>(pos);
            const double a = pos - static_cast<double>(i);
            theta = (1.0 - a) * lut[i] + a * lut[i + 1];
        }
    }
    if (!ok) return normalize(f3(static_cast<float>(xy.x), static_cast<float>(xy.y), 1.0f));
    const double scale = tan(theta) / rd;
    return normalize(f3(static_cast<float>(xr.x * scale), static_cast<float>(xr.y * scale), 1.0f));
}

// invert_lut_theta (programs.cu:435-450): first i with lut[i] <= theta <= lut[i+1].
// On a non-decreasing LUT that is lower_bound(theta) - 1, found by bisection.
RTGB_D double invert_lut_theta(const CameraDev& c, double theta) {
    if (theta <= 0.0 || c.lut_step <= 0.0) return 0.0;
    if (theta >= c.lut[1023]) return 1023.0 * c.lut_step;
    if (c.lut_monotone) {
        int lo = 0, hi = 1024;  // first j with lut[j] >= theta
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (c.lut[mid] < theta) lo = mid + 1;
            else hi = mid;
        }
        const int i = lo - 1;
        if (i >= 0 && i < 1023) {
            const double den = c.lut[i + 1] - c.lut[i];
            const double a = den > 0.0 ? (theta - c.lut[i]) / den : 0.0;
            return (static_cast<double>(i) + a) * c.lut_step;
        }
    }
    for (int i = 0; i < 1023; ++i) {
        if (c.lut[i] <= theta && theta <= c.lut[i + 1]) {
            const double den = c.lut[i + 1] - c.lut[i];
            const double a = den > 0.0 ? (theta - c.lut[i]) / den : 0.0;
            return (static_cast<double>(i) + a) * c.lut_step;
        }
    }
    return 1023.0 * c.lut_step;
}

RTGB_D float2 project_camera(const CameraDev& c, const float3& dir) {
    if (c.model != RTGB_CAMERA_EQUI62_LUT1D) return project_pinhole(c.pin, dir);
    const double dx = dir.x, dy = dir.y, dz = dir.z;
    const double r = sqrt(dx * dx + dy * dy);
    if (r < kCameraEpsilon) return make_float2(static_cast<float>(c.eq_cx), static_cast<float>(c.eq_cy));
    const double theta = atan2(r, dz);
    const double rd = invert_lut_theta(c, theta);
    const D2 xr{dx / r * rd, dy / r * rd};
    const D2 xd = equi_tangential(xr, c.eq_tan);
    return make_float2(static_cast<float>(xd.x * c.eq_fx + c.eq_cx), static_cast<float>(xd.y * c.eq_fy + c.eq_cy));
}

RTGB_D float3 cam_to_world(const CameraDev& c, const float3& d) {
    return normalize(add(add(mul(ld3(c.bx_f), d.x), mul(ld3(c.by_f), d.y)), mul(ld3(c.bz_f), d.z)));
}

// ---- primitive tests (programs.cu:1421-1547) on leaf records -------------------

RTGB_D int prim_code(const PrimRecord& p) { return __float_as_int(p.q[3].w); }

// Sphere: returns the accepted root or -1 (no hit) for (tmin, tmax).
RTGB_D bool sphere_t(const float3& center, float radius, const float3& o, const float3& d, float tmin, float tmax,
    float& t) {
    const float3 oc = sub(o, center);
    const float a = len_sq(d);
    const float hb = dot(oc, d);
    const float c = len_sq(oc) - radius * radius;
    const float disc = hb * hb - a * c;
    if (disc <= 0.0f) return false;
    const float sd = sqrtf(disc);
    float root = (-hb - sd) / a;
    if (root <= tmin || root >= tmax) {
        root = (-hb + sd) / a;
        if (root <= tmin || root >= tmax) return false;
    }
    t = root;
    return true;
}

RTGB_D bool quad_t(const float3& origin, const float3& normal, const float3& w, const float3& eu, const float3& ev,
    const float3& o, const float3& d, float tmin, float tmax, float& t, float& u, float& v) {
    const float denom = dot(normal, d);
    if (fabsf(denom) < 1e-6f) return false;
    const float tt = dot(sub(origin, o), normal) / denom;
    if (tt <= tmin || tt >= tmax) return false;
    const float3 p = add(o, mul(d, tt));
    const float3 rel = sub(p, origin);
    const float uu = dot(w, cross(rel, ev));
    const float vv = dot(w, cross(eu, rel));
    if (uu < 0.0f || uu > 1.0f || vv < 0.0f || vv > 1.0f) return false;
    t = tt;
    u = uu;
    v = vv;
    return true;
}

RTGB_D bool triangle_t(const float3& p0, const float3& e1, const float3& e2, const float3& o, const float3& d,
    float tmin, float tmax, float& t, float& u, float& v) {
    const float3 pvec = cross(d, e2);
    const float det = dot(e1, pvec);
    if (fabsf(det) <= 1e-8f) return false;
    const float inv = 1.0f / det;
    const float3 tvec = sub(o, p0);
    const float uu = dot(tvec, pvec) * inv;
    if (uu < 0.0f || uu > 1.0f) return false;
    const float3 qvec = cross(tvec, e1);
    const float vv = dot(d, qvec) * inv;
    if (vv < 0.0f || (uu + vv) > 1.0f) return false;
    const float tt = dot(e2, qvec) * inv;
    if (tt <= tmin || tt >= tmax) return false;
    t = tt;
    u = uu;
    v = vv;
    return true;
}

// Tests one leaf record; on a hit inside (tmin, tmax) returns t.
RTGB_D bool prim_hit(const PrimRecord& p, const float3& o, const float3& d, float tmin, float tmax, float& t) {
    const int type = static_cast<unsigned>(prim_code(p)) >> 28;
    float u, v;
    if (type == 2) return triangle_t(xyz(p.q[0]), xyz(p.q[1]), xyz(p.q[2]), o, d, tmin, tmax, t, u, v);
    if (type == 0) return sphere_t(xyz(p.q[0]), p.q[0].w, o, d, tmin, tmax, t);
    return quad_t(xyz(p.q[0]), f3(p.q[0].w, p.q[1].w, p.q[2].w), xyz(p.q[3]), xyz(p.q[1]), xyz(p.q[2]), o, d, tmin,
        tmax, t, u, v);
}

RTGB_D PrimRecord load_prim(const PrimRecord* __restrict__ prims, int slot) {
    PrimRecord r;
    const float4* src = reinterpret_cast<const float4*>(prims + slot);
    r.q[0] = __ldg(src + 0);
    r.q[1] = __ldg(src + 1);
    r.q[2] = __ldg(src + 2);
    r.q[3] = __ldg(src + 3);
    return r;
}

// Slab test of one child box; boxes were widened at build time, so the fused
// form below never rejects a box the exact test accepts.
RTGB_D bool box_hit(const float3& lo, const float3& hi, const float3& inv, const float3& oinv, float tmin, float tmax,
    float& tnear) {
    const float tx0 = __fmaf_rn(lo.x, inv.x, -oinv.x), tx1 = __fmaf_rn(hi.x, inv.x, -oinv.x);
    const float ty0 = __fmaf_rn(lo.y, inv.y, -oinv.y), ty1 = __fmaf_rn(hi.y, inv.y, -oinv.y);
    const float tz0 = __fmaf_rn(lo.z, inv.z, -oinv.z), tz1 = __fmaf_rn(hi.z, inv.z, -oinv.z);
    const float n = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    const float f = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tnear = n;
    return n <= f;
}

struct RayInv {
    float3 inv, oinv;
};

RTGB_D RayInv ray_inv(const float3& o, const float3& d) {
    // Zero direction components get a huge finite reciprocal so slabs stay ordered.
    auto rcp = [](float x) { return fabsf(x) > 1e-20f ? 1.0f / x : copysignf(1e20f, x); };
    RayInv r;
    r.inv = f3(rcp(d.x), rcp(d.y), rcp(d.z));
    r.oinv = f3(o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z);
    return r;
}

RTGB_D float lane4(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }

// The node's eight float4, from the shared-memory copy of the first `staged`
// nodes when it is there, else through the read-only cache.
RTGB_D void load_node4(const DeviceScene& s, const float4* staged, int staged_count, int node, float4 (&q)[kNode4]) {
    if (node < staged_count) {
        const float4* src = staged + static_cast<long long>(kNode4) * node;
#pragma unroll
        for (int k = 0; k < kNode4 - 1; ++k) q[k] = src[k];
    } else {
        const float4* src = s.nodes4 + static_cast<long long>(kNode4) * node;
#pragma unroll
        for (int k = 0; k < kNode4 - 1; ++k) q[k] = __ldg(src + k);
    }
}

// Inserts (t, c) into the ascending list (t0, c0) .. (t3, c3) (INF-padded);
// equal t keeps the earlier child first.
RTGB_D void insert4(float t, int c, float& t0, int& c0, float& t1, int& c1, float& t2, int& c2, float& t3, int& c3) {
    if (!(t < t3)) return;
    t3 = t;
    c3 = c;
    if (t3 < t2) {
        const float tt = t2; t2 = t3; t3 = tt;
        const int cc = c2; c2 = c3; c3 = cc;
    }
    if (t2 < t1) {
        const float tt = t1; t1 = t2; t2 = tt;
        const int cc = c1; c1 = c2; c2 = cc;
    }
    if (t1 < t0) {
        const float tt = t0; t0 = t1; t1 = tt;
        const int cc = c0; c0 = c1; c1 = cc;
    }
}

// Closest hit over the scene's wide BVH: strict t < closest like the
// reference, so equal-t primitives keep the first one traversed. Leaves are
// tested as soon as their box is hit; internal children are visited nearest
// first. Returns the code or -1. `overflow` counts subtrees dropped by a full
// stack (never silently). `staged` / `staged_count`: a shared-memory copy of
// the first nodes (or null / 0).
RTGB_D int traverse_closest(const DeviceScene& s, const float3& o, const float3& d, float tmin, float& closest,
    int& overflow, const float4* staged = nullptr, int staged_count = 0) {
    int best = -1;
    if (s.prim_count <= 0) return -1;
    if (s.prim_count == 1) {
        const PrimRecord p = load_prim(s.prims, 0);
        float t;
        if (prim_hit(p, o, d, tmin, closest, t)) {
            closest = t;
            best = prim_code(p);
        }
        return best;
    }
    const RayInv ri = ray_inv(o, d);
    int stack[kTraversalStack];
    int sp = 0;
    int node = 0;
    const float kInf = __int_as_float(0x7f800000);
    const int limit = s.bounds.traversal;
    int guard = 0;
    for (; guard < limit; ++guard) {
        float4 q[kNode4];
        load_node4(s, staged, staged_count, node, q);
        float t0 = kInf, t1 = kInf, t2 = kInf, t3 = kInf;
        int c0 = -1, c1 = -1, c2 = -1, c3 = -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = __float_as_int(lane4(q[6], k));
            if (c == kEmptyChild) continue;
            float tn;
            if (!box_hit(f3(lane4(q[0], k), lane4(q[1], k), lane4(q[2], k)), f3(lane4(q[3], k), lane4(q[4], k), lane4(q[5], k)),
                    ri.inv, ri.oinv, tmin, closest, tn)) {
                continue;
            }
            if (c < 0) {
                const PrimRecord p = load_prim(s.prims, ~c);
                float t;
                if (prim_hit(p, o, d, tmin, closest, t)) {
                    closest = t;
                    best = prim_code(p);
                }
            } else {
                insert4(tn, c, t0, c0, t1, c1, t2, c2, t3, c3);
            }
        }
        if (t0 < kInf) {
            // farthest first onto the stack, continue with the nearest
            if (t3 < kInf) {
                if (sp < kTraversalStack) stack[sp++] = c3;
                else ++overflow;
            }
            if (t2 < kInf) {
                if (sp < kTraversalStack) stack[sp++] = c2;
                else ++overflow;
            }
            if (t1 < kInf) {
                if (sp < kTraversalStack) stack[sp++] = c1;
                else ++overflow;
            }
            node = c0;
            continue;
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    if (guard >= limit && s.bounds.gave_up) atomicAdd(s.bounds.gave_up, 1);
    return best;
}

// Any hit in (tmin, tmax): the reference's occlusion test is a closest-hit
// query whose `hit` flag alone is used (programs.cu:1759-1762), so the first
// hit found gives the same answer.
RTGB_D bool traverse_any(const DeviceScene& s, const float3& o, const float3& d, float tmin, float tmax, int& overflow,
    const float4* staged = nullptr, int staged_count = 0) {
    if (s.prim_count <= 0) return false;
    if (s.prim_count == 1) {
        float t;
        return prim_hit(load_prim(s.prims, 0), o, d, tmin, tmax, t);
    }
    const RayInv ri = ray_inv(o, d);
    int stack[kTraversalStack];
    int sp = 0;
    int node = 0;
    const int limit = s.bounds.traversal;
    int guard = 0;
    for (; guard < limit; ++guard) {
        float4 q[kNode4];
        load_node4(s, staged, staged_count, node, q);
        int next = -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = __float_as_int(lane4(q[6], k));
            if (c == kEmptyChild) continue;
            float tn;
            if (!box_hit(f3(lane4(q[0], k), lane4(q[1], k), lane4(q[2], k)), f3(lane4(q[3], k), lane4(q[4], k), lane4(q[5], k)),
                    ri.inv, ri.oinv, tmin, tmax, tn)) {
                continue;
            }
            if (c < 0) {
                float t;
                if (prim_hit(load_prim(s.prims, ~c), o, d, tmin, tmax, t)) return true;
            } else if (next < 0) {
                next = c;
            } else if (sp < kTraversalStack) {
                stack[sp++] = c;
            } else {
                ++overflow;
            }
        }
        if (next >= 0) {
            node = next;
            continue;
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    if (guard >= limit && s.bounds.gave_up) atomicAdd(s.bounds.gave_up, 1);
    return false;
}

}  // namespace rtgb
