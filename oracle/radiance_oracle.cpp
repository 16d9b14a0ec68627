// Radiance oracle — TEST INFRASTRUCTURE ONLY.
//
// A scalar, per-pixel CPU restatement of the reference's realtime radiance
// path, src/realtime/gpu/programs.cu (radiance_kernel :1828-1953,
// resolve_reprojection_kernel :1955-2067 and every helper they call), driven
// the way src/realtime/gpu/optix_renderer.cpp:230-277 drives it (frame buffers
// zeroed per launch, history captured and copied after the resolve pass).
// It is the oracle of the CUDA path: only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference legs load it.
//
// Intersection runs either brute force (programs.cu:1664-1710, the
// reference's non-accelerated order: spheres, quads, triangles) or over the
// reference's own host BVH (median split, leaf <= 4,
// src/realtime/gpu/gpu_scene_acceleration.cpp:145-179, traversed as in
// programs.cu:1619-1652). Both give the same closest hit up to equal-t ties.
//
// OpenPBR materials run through ray_tracing_gb300/csrc/openpbr.h, the same
// host/device header the CUDA path uses (as the reference shares
// src/common/openpbr_core.h); that header is pinned word for word to the
// reference's by tests/test_openpbr_kats.py.
//
// Compiled with -ffp-contract=off; multi-draw RNG calls evaluate left to right.
#include "../include/rtgb.h"
#include "oracle_math.h"
#include "noise_sin.h"
#include "openpbr.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

namespace orc {
namespace {

constexpr float kRayEpsilon = 1e-3f;
constexpr float kRayFar = 1e30f;
constexpr double kCameraEpsilon = 1e-12;

namespace pbr = rtgb::pbr;

struct Ray {
    V3 origin;
    V3 direction;
};

struct Hit {
    bool hit = false;
    float t = 0.0f;
    V3 position{0, 0, 0};
    float tex_u = 0.0f;
    float tex_v = 0.0f;
    V3 geometric_normal{0, 0, 1};
    V3 shading_normal{0, 0, 1};
    V3 base_color{0, 0, 0};
    V3 emission{0, 0, 0};
    float fuzz = 0.0f;
    float ior = 1.0f;
    int openpbr_index = -1;
    int material_type = 0;
    int primitive_type = -1;
    int primitive_index = -1;
    bool front_face = true;
    int record_code = -1;  // parity record: which primitive/medium produced the hit
};

struct AnalyticHit {
    bool hit = false;
    float t = 0.0f;
    V3 position{0, 0, 0};
    V3 normal{0, 0, 1};
    int light_index = -1;
};

struct PathState {
    V3 throughput{1, 1, 1};
    V3 radiance{0, 0, 0};
    V3 prev_position{0, 0, 0};
    V3 prev_normal{0, 0, 1};
    float prev_bsdf_pdf = 0.0f;
    int prev_material_type = -1;
    int prev_primitive_type = -1;
    int prev_primitive_index = -1;
    bool prev_valid = false;
    bool prev_delta = true;
    Ray ray{};
    bool alive = true;
    pbr::Medium subsurface{};       // OpenPBR random-walk medium the path is inside
    int subsurface_material = -1;   // its OpenPBR material index
    int decisions = 0;              // this bounce's discrete outcomes, for the parity record
};

// Parity record of one bounce: (k << 28) | (decisions << 22) | index, where the
// decisions are bit 0 emissive NEE visible, bit 1 analytic (or ReSTIR) NEE
// visible, bits 2-5 the scatter event (OpenPBR sample event 1-9, 10 a
// random-walk scattering inside the medium, 0 otherwise).
constexpr int kDecisionShift = 22;
constexpr int kDecisionNeeEmissive = 1;
constexpr int kDecisionNeeAnalytic = 2;
constexpr int kDecisionWalk = 10;

struct LightSample {
    V3 position{0, 0, 0};
    V3 normal{0, 0, 1};
    V3 direction{0, 0, 1};
    V3 emission{0, 0, 0};
    float distance = 0.0f;
    float pdf = 0.0f;
    int material_index = -1;
    int light_index = -1;
    bool infinite = false;
    bool delta = false;
    bool valid = false;
};

// PackedLight (light_sampling.h:15-27).
struct PackedLight {
    int type = 0;  // 0 sphere, 1 quad, 2 triangle, 3 environment
    int primitive_index = -1;
    float selection_pdf = 0.0f;
    float cdf = 0.0f;
};

struct Camera {
    int width = 0;
    int height = 0;
    int model = 0;
    double origin[3]{};
    double basis_x[3]{};
    double basis_y[3]{};
    double basis_z[3]{};
    rtgb_pinhole32 pinhole{};
    rtgb_equi62_lut1d equi{};
};

struct BvhNode {
    float bmin[3];
    float bmax[3];
    int left = -1;
    int right = -1;
    int first = 0;
    int count = 0;
};

struct PrimRef {
    int type;
    int index;
    float bmin[3];
    float bmax[3];
};

struct Scene {
    std::vector<rtgb_texture> textures;
    std::vector<float> texels;
    std::vector<rtgb_material> materials;
    std::vector<rtgb_sphere> spheres;
    std::vector<rtgb_quad> quads;
    std::vector<rtgb_triangle> triangles;
    std::vector<rtgb_medium> media;
    std::vector<rtgb_analytic_light> analytic;
    std::vector<rtgb_openpbr_material> openpbr;
    std::vector<PackedLight> lights;
    V3 background{0, 0, 0};
    bool use_bvh = false;
    std::vector<BvhNode> nodes;
    std::vector<PrimRef> refs;
};

// ---- scene preparation: packed_scene_preparation.cpp:191-302 --------------

float luminance(const V3& v) {
    return std::max(0.0f, 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z);
}

V3 average_texture(const Scene& s, int index, int depth) {
    if (index < 0 || index >= static_cast<int>(s.textures.size()) || depth >= 8) return {0, 0, 0};
    const rtgb_texture& t = s.textures[static_cast<size_t>(index)];
    if (t.type == 0) return {std::max(t.color[0], 0.0f), std::max(t.color[1], 0.0f), std::max(t.color[2], 0.0f)};
    if (t.type == 1) {
        const V3 e = average_texture(s, t.even_texture, depth + 1);
        const V3 o = average_texture(s, t.odd_texture, depth + 1);
        return mul(add(e, o), 0.5f);
    }
    if (t.type == 2 && t.image_width > 0 && t.image_height > 0) {
        const int count = t.image_width * t.image_height;
        if (t.image_offset < 0 || t.image_offset + count > static_cast<int>(s.texels.size() / 3)) return {0, 0, 0};
        V3 sum{0, 0, 0};
        for (int i = 0; i < count; ++i) sum = add(sum, from3(&s.texels[3 * static_cast<size_t>(t.image_offset + i)]));
        // sum / count per component, as the reference divides (not a multiply by the reciprocal)
        const float n = static_cast<float>(count);
        return {std::max(sum.x / n, 0.0f), std::max(sum.y / n, 0.0f), std::max(sum.z / n, 0.0f)};
    }
    if (t.type == 3) return {0.5f, 0.5f, 0.5f};
    return {0, 0, 0};
}

pbr::V3 pv(const V3& v) { return pbr::V3{v.x, v.y, v.z}; }
V3 fv(const pbr::V3& v) { return V3{v.x, v.y, v.z}; }

// The OpenPBR parameter block is the first 204 bytes of rtgb_openpbr_material.
pbr::Mat openpbr_parameters(const rtgb_openpbr_material& c) {
    pbr::Mat m;
    std::memcpy(&m, &c, sizeof m);
    return m;
}

// material_emission_luminance, packed_scene_preparation.cpp:227-251
float emission_luminance(const Scene& s, int material_index) {
    if (material_index < 0 || material_index >= static_cast<int>(s.materials.size())) return 0.0f;
    const rtgb_material& m = s.materials[static_cast<size_t>(material_index)];
    if (m.type == 3) return luminance(average_texture(s, m.emission_texture, 0));
    if (m.type != 5 || m.openpbr_index < 0 || m.openpbr_index >= static_cast<int>(s.openpbr.size())) return 0.0f;
    const rtgb_openpbr_material& c = s.openpbr[static_cast<size_t>(m.openpbr_index)];
    pbr::Mat params = openpbr_parameters(c);
    if (c.color_texture[3] >= 0) {
        pbr::apply_color(params, 3, pv(average_texture(s, c.color_texture[3], 0)), c.color_space[3]);
    }
    return pbr::luminance(pbr::emission(params));
}

void build_light_distribution(Scene& s) {
    auto append = [&](int type, int index, float weight) {
        if (!std::isfinite(weight) || weight <= 1e-12f) return;
        s.lights.push_back(PackedLight{type, index, weight, 0.0f});
    };
    for (size_t i = 0; i < s.spheres.size(); ++i) {
        const rtgb_sphere& sp = s.spheres[i];
        const float area = 4.0f * kPi * sp.radius * sp.radius;
        append(0, static_cast<int>(i), area * emission_luminance(s, sp.material_index));
    }
    for (size_t i = 0; i < s.quads.size(); ++i) {
        const rtgb_quad& q = s.quads[i];
        const float area = len(cross(from3(q.edge_u), from3(q.edge_v)));
        append(1, static_cast<int>(i), area * emission_luminance(s, q.material_index));
    }
    for (size_t i = 0; i < s.triangles.size(); ++i) {
        const rtgb_triangle& t = s.triangles[i];
        const float area = 0.5f * len(cross(sub(from3(t.p1), from3(t.p0)), sub(from3(t.p2), from3(t.p0))));
        append(2, static_cast<int>(i), area * emission_luminance(s, t.material_index));
    }
    append(3, -1, 4.0f * kPi * luminance(s.background));
    float total = 0.0f;
    for (const PackedLight& l : s.lights) total += l.selection_pdf;
    float cdf = 0.0f;
    for (PackedLight& l : s.lights) {
        l.selection_pdf /= total;
        cdf += l.selection_pdf;
        l.cdf = cdf;
    }
    if (!s.lights.empty()) s.lights.back().cdf = 1.0f;
}

// ---- reference host BVH: gpu_scene_acceleration.cpp:18-179 ---------------

void ext(float* mn, float* mx, const V3& p) {
    mn[0] = std::min(mn[0], p.x); mn[1] = std::min(mn[1], p.y); mn[2] = std::min(mn[2], p.z);
    mx[0] = std::max(mx[0], p.x); mx[1] = std::max(mx[1], p.y); mx[2] = std::max(mx[2], p.z);
}

void pad_bounds(float* mn, float* mx) {
    for (int a = 0; a < 3; ++a) {
        if (mx[a] - mn[a] < 1e-5f) {
            mn[a] -= 1e-5f;
            mx[a] += 1e-5f;
        }
    }
}

int build_node(Scene& s, int begin, int end) {
    const int node_index = static_cast<int>(s.nodes.size());
    s.nodes.emplace_back();
    const float inf = std::numeric_limits<float>::infinity();
    float nb_min[3] = {inf, inf, inf}, nb_max[3] = {-inf, -inf, -inf};
    float cb_min[3] = {inf, inf, inf}, cb_max[3] = {-inf, -inf, -inf};
    auto centroid = [](const PrimRef& r) {
        return V3{(r.bmin[0] + r.bmax[0]) * 0.5f, (r.bmin[1] + r.bmax[1]) * 0.5f, (r.bmin[2] + r.bmax[2]) * 0.5f};
    };
    for (int i = begin; i < end; ++i) {
        const PrimRef& r = s.refs[static_cast<size_t>(i)];
        ext(nb_min, nb_max, V3{r.bmin[0], r.bmin[1], r.bmin[2]});
        ext(nb_min, nb_max, V3{r.bmax[0], r.bmax[1], r.bmax[2]});
        ext(cb_min, cb_max, centroid(r));
    }
    const int count = end - begin;
    BvhNode& node = s.nodes[static_cast<size_t>(node_index)];
    std::memcpy(node.bmin, nb_min, sizeof nb_min);
    std::memcpy(node.bmax, nb_max, sizeof nb_max);
    if (count <= 4) {
        node.first = begin;
        node.count = count;
        return node_index;
    }
    const float ex = cb_max[0] - cb_min[0], ey = cb_max[1] - cb_min[1], ez = cb_max[2] - cb_min[2];
    int axis = 0;
    if (ey > ex && ey >= ez) axis = 1;
    else axis = ez > ex ? 2 : 0;
    const int middle = begin + count / 2;
    std::nth_element(s.refs.begin() + begin, s.refs.begin() + middle, s.refs.begin() + end,
        [&](const PrimRef& a, const PrimRef& b) {
            const V3 ca = centroid(a), cb = centroid(b);
            const float va = axis == 0 ? ca.x : (axis == 1 ? ca.y : ca.z);
            const float vb = axis == 0 ? cb.x : (axis == 1 ? cb.y : cb.z);
            return va < vb;
        });
    const int left = build_node(s, begin, middle);
    const int right = build_node(s, middle, end);
    s.nodes[static_cast<size_t>(node_index)].left = left;
    s.nodes[static_cast<size_t>(node_index)].right = right;
    return node_index;
}

void build_reference_bvh(Scene& s) {
    const float inf = std::numeric_limits<float>::infinity();
    for (size_t i = 0; i < s.spheres.size(); ++i) {
        const rtgb_sphere& sp = s.spheres[i];
        const float r = std::fabs(sp.radius);
        PrimRef ref{0, static_cast<int>(i), {sp.center[0] - r, sp.center[1] - r, sp.center[2] - r},
            {sp.center[0] + r, sp.center[1] + r, sp.center[2] + r}};
        s.refs.push_back(ref);
    }
    for (size_t i = 0; i < s.quads.size(); ++i) {
        const rtgb_quad& q = s.quads[i];
        PrimRef ref{1, static_cast<int>(i), {inf, inf, inf}, {-inf, -inf, -inf}};
        const V3 o = from3(q.origin), u = from3(q.edge_u), v = from3(q.edge_v);
        ext(ref.bmin, ref.bmax, o);
        ext(ref.bmin, ref.bmax, add(o, u));
        ext(ref.bmin, ref.bmax, add(o, v));
        ext(ref.bmin, ref.bmax, add(add(o, u), v));
        pad_bounds(ref.bmin, ref.bmax);
        s.refs.push_back(ref);
    }
    for (size_t i = 0; i < s.triangles.size(); ++i) {
        const rtgb_triangle& t = s.triangles[i];
        PrimRef ref{2, static_cast<int>(i), {inf, inf, inf}, {-inf, -inf, -inf}};
        ext(ref.bmin, ref.bmax, from3(t.p0));
        ext(ref.bmin, ref.bmax, from3(t.p1));
        ext(ref.bmin, ref.bmax, from3(t.p2));
        pad_bounds(ref.bmin, ref.bmax);
        s.refs.push_back(ref);
    }
    if (!s.refs.empty()) build_node(s, 0, static_cast<int>(s.refs.size()));
}

// ---- textures: programs.cu:184-302 -----------------------------------------

float fractf(float v) { return v - std::floor(v); }
float clamp01(float v) { return std::fmin(std::fmax(v, 0.0f), 1.0f); }

void sphere_uv(const V3& p, float& u, float& v) {
    const float theta = std::acos(std::fmin(std::fmax(-p.y, -1.0f), 1.0f));
    const float phi = std::atan2(-p.z, p.x) + kPi;
    u = phi / (2.0f * kPi);
    v = theta / kPi;
}

// programs.cu:184-209. The sine is rtgb_noise::noise_sinf, the one the
// kernels use: the hash multiplies sin by 43758, so two correct sines that
// differ in the last bit (CUDA's and glibc's) give different noise.
float hash_noise(const V3& p) {
    const float n = rtgb_noise::noise_sinf(dot(p, V3{12.9898f, 78.233f, 37.719f})) * 43758.5453f;
    return fractf(n) * 2.0f - 1.0f;
}

float turbulence(V3 p) {
    float acc = 0.0f, w = 1.0f;
    for (int i = 0; i < 7; ++i) {
        acc += w * hash_noise(p);
        p = mul(p, 2.0f);
        w *= 0.5f;
    }
    return std::fabs(acc);
}

float address_coord(float c, int mode, bool& valid) {
    if (mode == 0 && (c < 0.0f || c > 1.0f)) {
        valid = false;
        return 0.0f;
    }
    if (mode == 2) return c - std::floor(c);
    if (mode == 3) {
        const float period = c - 2.0f * std::floor(0.5f * c);
        return period <= 1.0f ? period : 2.0f - period;
    }
    return clamp01(c);
}

V3 image_texel(const Scene& s, const rtgb_texture& t, int x, int y) {
    x = x < 0 ? 0 : (x >= t.image_width ? t.image_width - 1 : x);
    y = y < 0 ? 0 : (y >= t.image_height ? t.image_height - 1 : y);
    const int idx = t.image_offset + y * t.image_width + x;
    return idx >= 0 && idx < static_cast<int>(s.texels.size() / 3) ? from3(&s.texels[3 * static_cast<size_t>(idx)])
                                                                   : V3{0, 1, 1};
}

V3 sample_image(const Scene& s, const rtgb_texture& t, float u, float v) {
    if (s.texels.empty() || t.image_width <= 0 || t.image_height <= 0) return {0, 1, 1};
    bool valid = true;
    const float au = address_coord(u, t.u_address_mode, valid);
    const float av = 1.0f - address_coord(v, t.v_address_mode, valid);
    if (!valid) return {0, 0, 0};
    if (t.filter_type == 0) {
        int x = static_cast<int>(au * static_cast<float>(t.image_width));
        int y = static_cast<int>(av * static_cast<float>(t.image_height));
        x = x >= t.image_width ? t.image_width - 1 : x;
        y = y >= t.image_height ? t.image_height - 1 : y;
        return image_texel(s, t, x, y);
    }
    const float x = au * static_cast<float>(t.image_width - 1);
    const float y = av * static_cast<float>(t.image_height - 1);
    const int x0 = static_cast<int>(std::floor(x));
    const int y0 = static_cast<int>(std::floor(y));
    const float tx = x - static_cast<float>(x0);
    const float ty = y - static_cast<float>(y0);
    const V3 top = add(mul(image_texel(s, t, x0, y0), 1.0f - tx), mul(image_texel(s, t, x0 + 1, y0), tx));
    const V3 bot = add(mul(image_texel(s, t, x0, y0 + 1), 1.0f - tx), mul(image_texel(s, t, x0 + 1, y0 + 1), tx));
    return add(mul(top, 1.0f - ty), mul(bot, ty));
}

V3 eval_texture(const Scene& s, int index, float u, float v, const V3& p) {
    for (int depth = 0; depth < 8; ++depth) {
        if (index < 0 || index >= static_cast<int>(s.textures.size())) return {1, 0, 1};
        const rtgb_texture& t = s.textures[static_cast<size_t>(index)];
        if (t.type == 0) return from3(t.color);
        if (t.type == 1) {
            if (std::fabs(t.scale) < 1e-8f) {
                index = t.even_texture;
                continue;
            }
            const int x = static_cast<int>(std::floor(p.x / t.scale));
            const int y = static_cast<int>(std::floor(p.y / t.scale));
            const int z = static_cast<int>(std::floor(p.z / t.scale));
            index = ((x + y + z) % 2) == 0 ? t.even_texture : t.odd_texture;
            continue;
        }
        if (t.type == 2) return sample_image(s, t, u, v);
        if (t.type == 3) {
            const float turb = turbulence(p);
            const float value = 0.5f * (1.0f + rtgb_noise::noise_sinf(t.scale * p.z + 10.0f * turb));
            return {value, value, value};
        }
        return {1, 0, 1};
    }
    return {1, 0, 1};
}

// ---- cameras: programs.cu:304-537 ------------------------------------------

struct D2 {
    double x, y;
};

D2 distort_pinhole(const rtgb_pinhole32& p, const D2& xy) {
    const double x = xy.x, y = xy.y;
    const double x2 = x * x, y2 = y * y, xyt = x * y;
    const double r2 = x2 + y2, r4 = r2 * r2, r6 = r4 * r2;
    const double radial = 1.0 + p.k1 * r2 + p.k2 * r4 + p.k3 * r6;
    return {x * radial + p.p2 * (r2 + 2.0 * x2) + 2.0 * p.p1 * xyt,
        y * radial + p.p1 * (r2 + 2.0 * y2) + 2.0 * p.p2 * xyt};
}

bool solve2(double a00, double a01, double a10, double a11, const D2& rhs, D2& d) {
    const double det = a00 * a11 - a01 * a10;
    if (std::fabs(det) < kCameraEpsilon) return false;
    const double inv = 1.0 / det;
    d.x = (a11 * rhs.x - a01 * rhs.y) * inv;
    d.y = (-a10 * rhs.x + a00 * rhs.y) * inv;
    return true;
}

V3 unproject_pinhole(const rtgb_pinhole32& p, double px, double py) {
    const D2 xd{(px - p.cx) / p.fx, (py - p.cy) / p.fy};
    D2 xy = xd;
    for (int it = 0; it < 24; ++it) {
        const D2 dist = distort_pinhole(p, xy);
        const D2 err{xd.x - dist.x, xd.y - dist.y};
        if (err.x * err.x + err.y * err.y < 1e-20) break;
        const double x = xy.x, y = xy.y;
        const double r2 = x * x + y * y, r4 = r2 * r2, r6 = r4 * r2;
        const double radial = 1.0 + p.k1 * r2 + p.k2 * r4 + p.k3 * r6;
        const double drdx = 2.0 * x * (p.k1 + 2.0 * p.k2 * r2 + 3.0 * p.k3 * r4);
        const double drdy = 2.0 * y * (p.k1 + 2.0 * p.k2 * r2 + 3.0 * p.k3 * r4);
        D2 d{0, 0};
        if (!solve2(radial + x * drdx + 6.0 * p.p2 * x + 2.0 * p.p1 * y,
                x * drdy + 2.0 * p.p1 * x + 2.0 * p.p2 * y,
                y * drdx + 2.0 * p.p1 * x + 2.0 * p.p2 * y,
                radial + y * drdy + 6.0 * p.p1 * y + 2.0 * p.p2 * x, err, d)) {
            break;
        }
        xy.x += d.x;
        xy.y += d.y;
    }
    return normalize(V3{static_cast<float>(xy.x), static_cast<float>(xy.y), 1.0f});
}

V3 project_pinhole(const rtgb_pinhole32& p, const V3& dir) {
    if (std::fabs(dir.z) < 1e-7f) return {-1.0f, -1.0f, 0.0f};
    const double inv_z = 1.0 / static_cast<double>(dir.z);
    const D2 xu{static_cast<double>(dir.x) * inv_z, static_cast<double>(dir.y) * inv_z};
    const D2 xd = distort_pinhole(p, xu);
    return {static_cast<float>(xd.x * p.fx + p.cx), static_cast<float>(xd.y * p.fy + p.cy), 1.0f};
}

D2 equi_tangential(const D2& xy, const double* t) {
    const double xr = xy.x, yr = xy.y;
    const double xr2 = xr * xr, yr2 = yr * yr, xryr = xr * yr;
    const double p1 = t[0], p2 = t[1];
    return {xr + 2.0 * p1 * xryr + p2 * (xr2 + yr2 + 2.0 * xr2), yr + p1 * (xr2 + yr2 + 2.0 * yr2) + 2.0 * p2 * xryr};
}

D2 remove_equi_tangential(const D2& xy, const double* t) {
    const D2 dist = equi_tangential(xy, t);
    D2 d{0, 0};
    if (!solve2(1.0 + 2.0 * t[0] * xy.y + 6.0 * t[1] * xy.x, 2.0 * t[0] * xy.x + 2.0 * t[1] * xy.y,
            2.0 * t[0] * xy.x + 2.0 * t[1] * xy.y, 1.0 + 6.0 * t[0] * xy.y + 2.0 * t[1] * xy.x,
            D2{xy.x - dist.x, xy.y - dist.y}, d)) {
        return xy;
    }
    return {xy.x + d.x, xy.y + d.y};
}

bool lut_theta(const rtgb_equi62_lut1d& p, double rd, double& theta) {
    if (rd <= 0.0 || p.lut_step <= 0.0) {
        theta = 0.0;
        return true;
    }
    const double pos = rd / p.lut_step;
    if (pos > 1023.0) return false;
    if (pos >= 1023.0) {
        theta = p.lut[1023];
        return true;
    }
    const int i = static_cast<int>(pos);
    const double a = pos - static_cast<double>(i);
    theta = (1.0 - a) * p.lut[i] + a * p.lut[i + 1];
    return true;
}

double invert_lut_theta(const rtgb_equi62_lut1d& p, double theta) {
    if (theta <= 0.0 || p.lut_step <= 0.0) return 0.0;
    if (theta >= p.lut[1023]) return 1023.0 * p.lut_step;
    for (int i = 0; i < 1023; ++i) {
        if (p.lut[i] <= theta && theta <= p.lut[i + 1]) {
            const double den = p.lut[i + 1] - p.lut[i];
            const double a = den > 0.0 ? (theta - p.lut[i]) / den : 0.0;
            return (static_cast<double>(i) + a) * p.lut_step;
        }
    }
    return 1023.0 * p.lut_step;
}

V3 project_equi(const rtgb_equi62_lut1d& p, const V3& dir) {
    const double dx = dir.x, dy = dir.y, dz = dir.z;
    const double r = std::sqrt(dx * dx + dy * dy);
    if (r < kCameraEpsilon) return {static_cast<float>(p.cx), static_cast<float>(p.cy), 1.0f};
    const double theta = std::atan2(r, dz);
    const double rd = invert_lut_theta(p, theta);
    const D2 xr{dx / r * rd, dy / r * rd};
    const D2 xd = equi_tangential(xr, p.tangential);
    return {static_cast<float>(xd.x * p.fx + p.cx), static_cast<float>(xd.y * p.fy + p.cy), 1.0f};
}

V3 unproject_equi(const rtgb_equi62_lut1d& p, double px, double py) {
    const D2 xy{(px - p.cx) / p.fx, (py - p.cy) / p.fy};
    if (xy.x * xy.x + xy.y * xy.y < kCameraEpsilon * kCameraEpsilon) return {0, 0, 1};
    const D2 xr = remove_equi_tangential(xy, p.tangential);
    const double rd = std::sqrt(xr.x * xr.x + xr.y * xr.y);
    if (rd < kCameraEpsilon) return {0, 0, 1};
    double theta = 0.0;
    if (!lut_theta(p, rd, theta)) return normalize(V3{static_cast<float>(xy.x), static_cast<float>(xy.y), 1.0f});
    const double scale = std::tan(theta) / rd;
    return normalize(V3{static_cast<float>(xr.x * scale), static_cast<float>(xr.y * scale), 1.0f});
}

V3 unproject(const Camera& c, double px, double py) {
    return c.model == 1 ? unproject_equi(c.equi, px, py) : unproject_pinhole(c.pinhole, px, py);
}

V3 project(const Camera& c, const V3& d) {
    return c.model == 1 ? project_equi(c.equi, d) : project_pinhole(c.pinhole, d);
}

V3 basis_f(const double* b) { return {static_cast<float>(b[0]), static_cast<float>(b[1]), static_cast<float>(b[2])}; }

V3 to_world(const Camera& c, const V3& d) {
    return normalize(add(add(mul(basis_f(c.basis_x), d.x), mul(basis_f(c.basis_y), d.y)), mul(basis_f(c.basis_z), d.z)));
}

V3 cam_origin(const Camera& c) { return basis_f(c.origin); }

Camera make_camera(const rtgb_camera& pc) {
    Camera c{};
    c.width = pc.width;
    c.height = pc.height;
    c.model = pc.model;
    for (int r = 0; r < 3; ++r) {
        c.origin[r] = pc.translation[r];
        c.basis_x[r] = pc.rotation[r * 3 + 0];
        c.basis_y[r] = pc.rotation[r * 3 + 1];
        c.basis_z[r] = pc.rotation[r * 3 + 2];
    }
    c.pinhole = pc.pinhole;
    c.equi = pc.equi;
    return c;
}

// ---- light helpers: programs.cu:539-891 -------------------------------------

V3 cone_direction(const V3& axis, float cos_theta_max, float u0, float u1) {
    const float ct = 1.0f - u0 * (1.0f - cos_theta_max);
    const float st = std::sqrt(std::fmax(0.0f, 1.0f - ct * ct));
    const float phi = 2.0f * kPi * u1;
    const V3 helper = std::fabs(axis.x) > 0.9f ? V3{0, 1, 0} : V3{1, 0, 0};
    const V3 tangent = normalize(cross(helper, axis));
    const V3 bitangent = cross(axis, tangent);
    return normalize(add(mul(axis, ct), add(mul(tangent, st * std::cos(phi)), mul(bitangent, st * std::sin(phi)))));
}

V3 sphere_direction(float u0, float u1) {
    const float z = 1.0f - 2.0f * u0;
    const float r = std::sqrt(std::fmax(0.0f, 1.0f - z * z));
    const float phi = 2.0f * kPi * u1;
    return {r * std::cos(phi), r * std::sin(phi), z};
}

class Tracer {
public:
    explicit Tracer(const Scene& s) : s_(s) {}

    const PackedLight* find_light(int type, int prim) const {
        for (const PackedLight& l : s_.lights) {
            if (l.type == type && l.primitive_index == prim) return &l;
        }
        return nullptr;
    }

    float effective_selection_pdf(const PackedLight& light, int ex_type, int ex_index) const {
        const PackedLight* ex = ex_type < 0 ? nullptr : find_light(ex_type, ex_index);
        if (ex == &light) return 0.0f;
        const float eligible = ex == nullptr ? 1.0f : 1.0f - ex->selection_pdf;
        return eligible > 1e-8f ? light.selection_pdf / eligible : 0.0f;
    }

    float conditional_pdf_for_hit(const PackedLight& light, const V3& origin, const V3& dir, const Hit* hit) const {
        if (light.type == 3) return uniform_sphere_pdf();
        if (hit == nullptr || !hit->hit || hit->primitive_type != light.type
            || hit->primitive_index != light.primitive_index || !hit->front_face) {
            return 0.0f;
        }
        if (light.type == 0) {
            const rtgb_sphere& sp = s_.spheres[static_cast<size_t>(light.primitive_index)];
            const float d2 = len_sq(sub(from3(sp.center), origin));
            const float r2 = sp.radius * sp.radius;
            if (d2 <= r2) return 0.0f;
            const float ctm = std::sqrt(std::fmax(0.0f, 1.0f - r2 / d2));
            return uniform_cone_pdf(ctm);
        }
        const float d2 = len_sq(sub(hit->position, origin));
        const float ac = std::fmax(dot(hit->geometric_normal, mul(dir, -1.0f)), 0.0f);
        if (light.type == 1) {
            const rtgb_quad& q = s_.quads[static_cast<size_t>(light.primitive_index)];
            const float area = len(cross(from3(q.edge_u), from3(q.edge_v)));
            return area_to_solid_angle_pdf(area, d2, ac);
        }
        const rtgb_triangle& t = s_.triangles[static_cast<size_t>(light.primitive_index)];
        const float area = 0.5f * len(cross(sub(from3(t.p1), from3(t.p0)), sub(from3(t.p2), from3(t.p0))));
        return area_to_solid_angle_pdf(area, d2, ac);
    }

    float emission_mis_weight(const PathState& st, const Hit* hit, bool env) const {
        if (!st.prev_valid || st.prev_delta) return 1.0f;
        if (!env && (hit == nullptr || hit->primitive_type < 0)) return 1.0f;
        const PackedLight* light = env ? find_light(3, -1) : find_light(hit->primitive_type, hit->primitive_index);
        if (light == nullptr) return 1.0f;
        const V3 dir = normalize(st.ray.direction);
        const float cond = env ? (st.prev_material_type == 4 ? uniform_sphere_pdf()
                                                             : std::fmax(dot(st.prev_normal, dir), 0.0f) / kPi)
                               : conditional_pdf_for_hit(*light, st.prev_position, dir, hit);
        const float sel = effective_selection_pdf(*light, st.prev_primitive_type, st.prev_primitive_index);
        return power_heuristic(st.prev_bsdf_pdf, sel * cond);
    }

    static bool finite_analytic(int type) { return type == 0 || type == 1 || type == 2 || type == 3; }

    static V3 analytic_normal(const rtgb_analytic_light& l) {
        return normalize(mul(cross(from3(l.basis_x), from3(l.basis_y)), -1.0f));
    }

    static bool plane_coords(const rtgb_analytic_light& l, const V3& p, float& lx, float& ly) {
        const V3 bx = from3(l.basis_x), by = from3(l.basis_y);
        const V3 local = sub(p, from3(l.position));
        const float xx = dot(bx, bx), xy = dot(bx, by), yy = dot(by, by);
        const float det = xx * yy - xy * xy;
        if (det <= 1e-16f) return false;
        const float px = dot(local, bx), py = dot(local, by);
        lx = (px * yy - py * xy) / det;
        ly = (py * xx - px * xy) / det;
        return true;
    }

    static bool hit_analytic(const rtgb_analytic_light& l, const Ray& ray, float tmin, float tmax, AnalyticHit& h) {
        const V3 center = from3(l.position);
        if (l.type == 0) {
            const float radius = l.radius * len(from3(l.basis_x));
            const V3 oc = sub(ray.origin, center);
            const float a = len_sq(ray.direction);
            const float hb = dot(oc, ray.direction);
            const float c = len_sq(oc) - radius * radius;
            const float disc = hb * hb - a * c;
            if (a <= 1e-16f || disc < 0.0f) return false;
            const float rt = std::sqrt(disc);
            float root = (-hb - rt) / a;
            if (root <= tmin || root >= tmax) root = (-hb + rt) / a;
            if (root <= tmin || root >= tmax) return false;
            const V3 pos = add(ray.origin, mul(ray.direction, root));
            const V3 n = normalize(sub(pos, center));
            if (dot(ray.direction, n) >= 0.0f) return false;
            h.hit = true;
            h.t = root;
            h.position = pos;
            h.normal = n;
            return true;
        }
        if (l.type == 1 || l.type == 2) {
            const V3 n = analytic_normal(l);
            const float den = dot(ray.direction, n);
            if (den >= -1e-8f) return false;
            const float t = dot(sub(center, ray.origin), n) / den;
            if (t <= tmin || t >= tmax) return false;
            const V3 pos = add(ray.origin, mul(ray.direction, t));
            float lx = 0.0f, ly = 0.0f;
            if (!plane_coords(l, pos, lx, ly)) return false;
            const bool inside = l.type == 1 ? lx * lx + ly * ly <= l.radius * l.radius
                                            : std::fabs(lx) <= 0.5f * l.width && std::fabs(ly) <= 0.5f * l.height;
            if (!inside) return false;
            h.hit = true;
            h.t = t;
            h.position = pos;
            h.normal = n;
            return true;
        }
        if (l.type != 3) return false;
        const V3 bx = from3(l.basis_x), by = from3(l.basis_y), bz = from3(l.basis_z);
        const float scale = len(bx);
        if (scale <= 1e-8f) return false;
        const V3 ax = divs(bx, scale), ay = divs(by, scale), az = normalize(bz);
        const V3 lo = sub(ray.origin, center);
        const float ox = dot(lo, ax), oy = dot(lo, ay), oz = dot(lo, az);
        const float dx = dot(ray.direction, ax), dy = dot(ray.direction, ay), dz = dot(ray.direction, az);
        const float radius = l.radius * scale;
        const float a = dx * dx + dy * dy;
        const float hb = ox * dx + oy * dy;
        const float c = ox * ox + oy * oy - radius * radius;
        const float disc = hb * hb - a * c;
        if (a <= 1e-16f || disc < 0.0f) return false;
        const float rt = std::sqrt(disc);
        float root = (-hb - rt) / a;
        float z = oz + root * dz;
        const float half_len = 0.5f * l.length * len(bz);
        if (root <= tmin || root >= tmax || std::fabs(z) > half_len) {
            root = (-hb + rt) / a;
            z = oz + root * dz;
        }
        if (root <= tmin || root >= tmax || std::fabs(z) > half_len) return false;
        const float x = ox + root * dx, y = oy + root * dy;
        const V3 n = normalize(add(mul(ax, x), mul(ay, y)));
        if (dot(ray.direction, n) >= 0.0f) return false;
        h.hit = true;
        h.t = root;
        h.position = add(ray.origin, mul(ray.direction, root));
        h.normal = n;
        return true;
    }

    AnalyticHit intersect_analytic(const Ray& ray, float tmin, float tmax) const {
        AnalyticHit best{};
        float closest = tmax;
        for (size_t i = 0; i < s_.analytic.size(); ++i) {
            const rtgb_analytic_light& l = s_.analytic[i];
            if (!finite_analytic(l.type) || l.treat_as_point != 0) continue;
            AnalyticHit c{};
            if (!hit_analytic(l, ray, tmin, closest, c)) continue;
            c.light_index = static_cast<int>(i);
            closest = c.t;
            best = c;
        }
        return best;
    }

    static float analytic_pdf_for_hit(const rtgb_analytic_light& l, const V3& origin, const V3& dir, const AnalyticHit& h) {
        if (l.delta != 0 || l.treat_as_point != 0 || l.treat_as_line != 0) return 0.0f;
        if (l.type == 0) {
            const V3 center = from3(l.position);
            const float radius = l.radius * len(from3(l.basis_x));
            const float d2 = len_sq(sub(center, origin));
            const float r2 = radius * radius;
            if (d2 <= r2) return 0.0f;
            return uniform_cone_pdf(std::sqrt(std::fmax(0.0f, 1.0f - r2 / d2)));
        }
        const float d2 = len_sq(sub(h.position, origin));
        const float ac = std::fmax(dot(h.normal, mul(dir, -1.0f)), 0.0f);
        return area_to_solid_angle_pdf(l.world_area, d2, ac);
    }

    float analytic_emission_mis(const PathState& st, const AnalyticHit& h) const {
        if (!st.prev_valid || st.prev_delta || h.light_index < 0) return 1.0f;
        const rtgb_analytic_light& l = s_.analytic[static_cast<size_t>(h.light_index)];
        const V3 dir = normalize(st.ray.direction);
        const float lp = l.selection_pdf * analytic_pdf_for_hit(l, st.prev_position, dir, h);
        return power_heuristic(st.prev_bsdf_pdf, lp);
    }

    V3 analytic_infinite_radiance(const PathState& st) const {
        V3 rad{0, 0, 0};
        const V3 dir = normalize(st.ray.direction);
        for (const rtgb_analytic_light& l : s_.analytic) {
            bool in_dir = false;
            if (l.type == 5) {
                in_dir = true;
            } else if (l.type == 4) {
                const V3 axis = normalize(from3(l.basis_z));
                const float thr = l.delta != 0 ? 0.999999f : l.cos_theta_max;
                in_dir = dot(axis, dir) >= thr;
            }
            if (!in_dir) continue;
            float w = 1.0f;
            if (st.prev_valid && !st.prev_delta) {
                const float cond = l.delta != 0 ? 0.0f : (l.type == 5 ? uniform_sphere_pdf() : uniform_cone_pdf(l.cos_theta_max));
                if (cond <= 0.0f) continue;
                w = power_heuristic(st.prev_bsdf_pdf, l.selection_pdf * cond);
            }
            rad = add(rad, mul(from3(l.radiance), w));
        }
        return rad;
    }

    // ---- surfaces: programs.cu:903-1009, 1421-1547 ------------------------

    static void set_face(const Ray& ray, const V3& outward, Hit& h) {
        h.front_face = dot(ray.direction, outward) < 0.0f;
        h.geometric_normal = outward;
        h.shading_normal = h.front_face ? outward : mul(outward, -1.0f);
    }

    void populate_material(int mi, Hit& h) const {
        if (mi < 0 || mi >= static_cast<int>(s_.materials.size())) {
            h.base_color = {0, 0, 0};
            h.emission = {0, 0, 0};
            h.material_type = 0;
            h.ior = 1.0f;
            h.fuzz = 0.0f;
            h.openpbr_index = -1;
            return;
        }
        const rtgb_material& m = s_.materials[static_cast<size_t>(mi)];
        h.openpbr_index = m.openpbr_index;
        h.material_type = m.type;
        h.fuzz = m.fuzz;
        h.ior = m.ior;
        h.base_color = eval_texture(s_, m.albedo_texture, h.tex_u, h.tex_v, h.position);
        h.emission = eval_texture(s_, m.emission_texture, h.tex_u, h.tex_v, h.position);
        if (h.material_type == 2) {
            h.base_color = {0.92f, 0.95f, 1.0f};
            h.emission = {0, 0, 0};
        }
        if (h.material_type == 3 && !h.front_face) h.emission = {0, 0, 0};
        if (h.material_type != 3) h.emission = {0, 0, 0};
        if (h.material_type == 5) {
            const rtgb_openpbr_material* c = openpbr_material(m.openpbr_index);
            if (c == nullptr) {
                h.material_type = -1;
                h.base_color = {0, 0, 0};
                h.emission = {0, 0, 0};
                return;
            }
            pbr::Mat params = openpbr_parameters(*c);
            apply_color_binding(params, *c, 0, h.tex_u, h.tex_v, h.position);
            apply_color_binding(params, *c, 3, h.tex_u, h.tex_v, h.position);
            h.base_color = fv(params.base_color);
            h.emission = fv(pbr::emission(params));
        }
    }

    // resolve_openpbr_material, programs.cu:909-921
    const rtgb_openpbr_material* openpbr_material(int index) const {
        if (index < 0 || index >= static_cast<int>(s_.openpbr.size())) return nullptr;
        return &s_.openpbr[static_cast<size_t>(index)];
    }

    // evaluate_openpbr_color_binding, programs.cu:923-932 (input: 0 base, 1 specular,
    // 2 transmission, 3 emission color)
    void apply_color_binding(pbr::Mat& params, const rtgb_openpbr_material& c, int input, float u, float v,
        const V3& p) const {
        if (c.color_texture[input] < 0) return;
        pbr::apply_color(params, input, pv(eval_texture(s_, c.color_texture[input], u, v, p)), c.color_space[input]);
    }

    // evaluate_openpbr_scattering_material, programs.cu:944-960
    pbr::Mat scattering_parameters(const Hit& h) const {
        const rtgb_openpbr_material& c = *openpbr_material(h.openpbr_index);
        pbr::Mat params = openpbr_parameters(c);
        if (c.color_texture[0] >= 0) params.base_color = pv(h.base_color);
        apply_color_binding(params, c, 1, h.tex_u, h.tex_v, h.position);
        apply_color_binding(params, c, 2, h.tex_u, h.tex_v, h.position);
        for (int k = 0; k < 2; ++k) {
            if (c.scalar_texture[k] >= 0) {
                pbr::apply_scalar(params, k, eval_texture(s_, c.scalar_texture[k], h.tex_u, h.tex_v, h.position).x);
            }
        }
        return params;
    }

    static pbr::Context transport_context(const PathState& st) {
        pbr::Context ctx = pbr::default_context();
        ctx.throughput = pv(st.throughput);
        return ctx;
    }

    static bool try_sphere(const rtgb_sphere& sp, const Ray& ray, float tmin, float tmax, Hit& h) {
        const V3 center = from3(sp.center);
        const V3 oc = sub(ray.origin, center);
        const float radius = sp.radius;
        const float a = len_sq(ray.direction);
        const float hb = dot(oc, ray.direction);
        const float c = len_sq(oc) - radius * radius;
        const float disc = hb * hb - a * c;
        if (disc <= 0.0f) return false;
        const float sd = std::sqrt(disc);
        float root = (-hb - sd) / a;
        if (root <= tmin || root >= tmax) {
            root = (-hb + sd) / a;
            if (root <= tmin || root >= tmax) return false;
        }
        h.hit = true;
        h.t = root;
        h.position = add(ray.origin, mul(ray.direction, root));
        const V3 outward = divs(sub(h.position, center), radius);
        sphere_uv(outward, h.tex_u, h.tex_v);
        set_face(ray, outward, h);
        return true;
    }

    static bool try_quad(const rtgb_quad& q, const Ray& ray, float tmin, float tmax, Hit& h) {
        const V3 origin = from3(q.origin), eu = from3(q.edge_u), ev = from3(q.edge_v);
        const V3 n = cross(eu, ev);
        const float nls = len_sq(n);
        if (nls <= 1e-12f) return false;
        const V3 normal = divs(n, std::sqrt(nls));
        const float denom = dot(normal, ray.direction);
        if (std::fabs(denom) < 1e-6f) return false;
        const float t = dot(sub(origin, ray.origin), normal) / denom;
        if (t <= tmin || t >= tmax) return false;
        const V3 p = add(ray.origin, mul(ray.direction, t));
        const V3 rel = sub(p, origin);
        const V3 w = divs(n, nls);
        const float u = dot(w, cross(rel, ev));
        const float v = dot(w, cross(eu, rel));
        if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f) return false;
        h.hit = true;
        h.t = t;
        h.position = p;
        h.tex_u = u;
        h.tex_v = v;
        set_face(ray, normal, h);
        return true;
    }

    static bool try_triangle(const rtgb_triangle& tr, const Ray& ray, float tmin, float tmax, Hit& h) {
        const V3 p0 = from3(tr.p0), p1 = from3(tr.p1), p2 = from3(tr.p2);
        const V3 e1 = sub(p1, p0), e2 = sub(p2, p0);
        const V3 pvec = cross(ray.direction, e2);
        const float det = dot(e1, pvec);
        if (std::fabs(det) <= 1e-8f) return false;
        const float inv = 1.0f / det;
        const V3 tvec = sub(ray.origin, p0);
        const float u = dot(tvec, pvec) * inv;
        if (u < 0.0f || u > 1.0f) return false;
        const V3 qvec = cross(tvec, e1);
        const float v = dot(ray.direction, qvec) * inv;
        if (v < 0.0f || (u + v) > 1.0f) return false;
        const float t = dot(e2, qvec) * inv;
        if (t <= tmin || t >= tmax) return false;
        const V3 normal = normalize(cross(e1, e2));
        const float w = 1.0f - u - v;
        h.hit = true;
        h.t = t;
        h.position = add(ray.origin, mul(ray.direction, t));
        if (tr.has_texcoords != 0) {
            h.tex_u = tr.uv0[0] * w + tr.uv1[0] * u + tr.uv2[0] * v;
            h.tex_v = tr.uv0[1] * w + tr.uv1[1] * u + tr.uv2[1] * v;
        } else {
            h.tex_u = u;
            h.tex_v = v;
        }
        set_face(ray, normal, h);
        if (tr.has_vertex_normals != 0) {
            V3 sh = add(mul(from3(tr.n0), w), add(mul(from3(tr.n1), u), mul(from3(tr.n2), v)));
            if (!near_zero(sh)) {
                sh = normalize(sh);
                if (dot(sh, normal) < 0.0f) sh = mul(sh, -1.0f);
                h.shading_normal = h.front_face ? sh : mul(sh, -1.0f);
            }
        }
        return true;
    }

    void try_prim(int type, int index, const Ray& ray, float tmin, float& closest, Hit& hit, bool& found) const {
        Hit c{};
        bool ok = false;
        int mi = -1;
        if (type == 0) {
            const rtgb_sphere& sp = s_.spheres[static_cast<size_t>(index)];
            ok = try_sphere(sp, ray, tmin, closest, c);
            mi = sp.material_index;
        } else if (type == 1) {
            const rtgb_quad& q = s_.quads[static_cast<size_t>(index)];
            ok = try_quad(q, ray, tmin, closest, c);
            mi = q.material_index;
        } else {
            const rtgb_triangle& t = s_.triangles[static_cast<size_t>(index)];
            ok = try_triangle(t, ray, tmin, closest, c);
            mi = t.material_index;
        }
        if (!ok) return;
        c.primitive_type = type;
        c.primitive_index = index;
        c.record_code = (type << 28) | index;
        populate_material(mi, c);
        closest = c.t;
        hit = c;
        found = true;
    }

    static bool hit_bounds(const BvhNode& n, const Ray& ray, float tmin, float tmax) {
        const float o[3] = {ray.origin.x, ray.origin.y, ray.origin.z};
        const float d[3] = {ray.direction.x, ray.direction.y, ray.direction.z};
        for (int a = 0; a < 3; ++a) {
            if (std::fabs(d[a]) <= 1e-12f) {
                if (o[a] < n.bmin[a] || o[a] > n.bmax[a]) return false;
                continue;
            }
            const float inv = 1.0f / d[a];
            float nt = (n.bmin[a] - o[a]) * inv;
            float ft = (n.bmax[a] - o[a]) * inv;
            if (nt > ft) std::swap(nt, ft);
            tmin = std::fmax(tmin, nt);
            tmax = std::fmin(tmax, ft);
            if (tmax < tmin) return false;
        }
        return true;
    }

    bool medium_boundary(const rtgb_medium& m, const Ray& ray, float tmin, float tmax, float& entry, float& exit) const {
        const V3 shifted = sub(ray.origin, from3(m.translation));
        const V3 r0 = from3(m.rotation_row0), r1 = from3(m.rotation_row1), r2 = from3(m.rotation_row2);
        const V3 lo{dot(r0, shifted), dot(r1, shifted), dot(r2, shifted)};
        const V3 ld{dot(r0, ray.direction), dot(r1, ray.direction), dot(r2, ray.direction)};
        if (m.boundary_type == 0) {
            const V3 center = from3(m.local_center_or_min);
            const V3 oc = sub(lo, center);
            const float a = len_sq(ld);
            const float hb = dot(oc, ld);
            const float c = len_sq(oc) - m.radius * m.radius;
            const float disc = hb * hb - a * c;
            if (disc <= 0.0f) return false;
            const float sd = std::sqrt(disc);
            float t0 = (-hb - sd) / a, t1 = (-hb + sd) / a;
            if (t0 > t1) std::swap(t0, t1);
            entry = std::fmax(t0, tmin);
            exit = std::fmin(t1, tmax);
            return entry < exit;
        }
        if (m.boundary_type == 1) {
            float t0 = tmin, t1 = tmax;
            const float o[3] = {lo.x, lo.y, lo.z}, d[3] = {ld.x, ld.y, ld.z};
            for (int a = 0; a < 3; ++a) {
                if (std::fabs(d[a]) < 1e-8f) {
                    if (o[a] < m.local_center_or_min[a] || o[a] > m.local_max[a]) return false;
                    continue;
                }
                float a0 = (m.local_center_or_min[a] - o[a]) / d[a];
                float a1 = (m.local_max[a] - o[a]) / d[a];
                if (a0 > a1) std::swap(a0, a1);
                t0 = std::fmax(t0, a0);
                t1 = std::fmin(t1, a1);
                if (t0 >= t1) return false;
            }
            entry = t0;
            exit = t1;
            return true;
        }
        return false;
    }

    // intersect_scene, programs.cu:1654-1757
    Hit intersect(const Ray& ray, float tmin, float tmax, uint32_t* rng) const {
        Hit hit{};
        float closest = tmax;
        bool found = false;
        if (s_.use_bvh && !s_.nodes.empty()) {
            int stack[64];
            int sp = 1;
            stack[0] = 0;
            while (sp > 0) {
                const int ni = stack[--sp];
                if (ni < 0 || ni >= static_cast<int>(s_.nodes.size())) continue;
                const BvhNode& n = s_.nodes[static_cast<size_t>(ni)];
                if (!hit_bounds(n, ray, tmin, closest)) continue;
                if (n.count > 0) {
                    for (int i = 0; i < n.count; ++i) {
                        const PrimRef& r = s_.refs[static_cast<size_t>(n.first + i)];
                        try_prim(r.type, r.index, ray, tmin, closest, hit, found);
                    }
                    continue;
                }
                if (sp + 2 > 64) continue;
                stack[sp++] = n.right;
                stack[sp++] = n.left;
            }
        } else {
            for (size_t i = 0; i < s_.spheres.size(); ++i) try_prim(0, static_cast<int>(i), ray, tmin, closest, hit, found);
            for (size_t i = 0; i < s_.quads.size(); ++i) try_prim(1, static_cast<int>(i), ray, tmin, closest, hit, found);
            for (size_t i = 0; i < s_.triangles.size(); ++i) try_prim(2, static_cast<int>(i), ray, tmin, closest, hit, found);
        }
        if (rng != nullptr) {
            const float ray_len = len(ray.direction);
            if (ray_len > 1e-8f) {
                for (size_t i = 0; i < s_.media.size(); ++i) {
                    const rtgb_medium& m = s_.media[i];
                    if (m.density <= 0.0f) continue;
                    float entry = 0.0f, exit = 0.0f;
                    if (!medium_boundary(m, ray, tmin, closest, entry, exit)) continue;
                    entry = std::fmax(entry, tmin);
                    exit = std::fmin(exit, closest);
                    if (entry >= exit) continue;
                    const float inside = (exit - entry) * ray_len;
                    const float u = std::fmax(rnd(*rng), 1e-6f);
                    const float hd = -std::log(u) / m.density;
                    if (hd >= inside) continue;
                    Hit c{};
                    c.hit = true;
                    c.t = entry + hd / ray_len;
                    c.position = add(ray.origin, mul(ray.direction, c.t));
                    c.front_face = true;
                    c.geometric_normal = mul(normalize(ray.direction), -1.0f);
                    c.shading_normal = c.geometric_normal;
                    c.tex_u = 0.0f;
                    c.tex_v = 0.0f;
                    c.record_code = (4 << 28) | static_cast<int>(i);
                    populate_material(m.material_index, c);
                    closest = c.t;
                    hit = c;
                    found = true;
                }
            }
        }
        hit.hit = found;
        return hit;
    }

    bool occluded(const Ray& ray, float max_t) const { return intersect(ray, kRayEpsilon, max_t, nullptr).hit; }

    // ---- shading: programs.cu:1011-1354 ----------------------------------

    // evaluate_material_emission, programs.cu:1011-1024
    V3 material_emission(const rtgb_material& m, float u, float v, const V3& p) const {
        if (m.type == 5) {
            const rtgb_openpbr_material* c = openpbr_material(m.openpbr_index);
            if (c == nullptr) return {0, 0, 0};
            pbr::Mat params = openpbr_parameters(*c);
            apply_color_binding(params, *c, 3, u, v, p);
            return fv(pbr::emission(params));
        }
        return eval_texture(s_, m.emission_texture, u, v, p);
    }

    // direct_material_response, programs.cu:1026-1055
    V3 direct_response(const Hit& h, const PathState& st, const V3& ldir, float& bsdf_pdf) const {
        bsdf_pdf = 0.0f;
        if (h.material_type == 5) {
            if (openpbr_material(h.openpbr_index) == nullptr) return {0, 0, 0};
            const pbr::Mat params = scattering_parameters(h);
            const pbr::Frame frame = pbr::make_frame(pv(h.geometric_normal), pbr::V3{0.0f, 0.0f, 0.0f});
            const pbr::Eval e = pbr::evaluate(params, frame, pv(mul(normalize(st.ray.direction), -1.0f)), pv(ldir),
                transport_context(st));
            const float cosine = std::fabs(dot(h.shading_normal, ldir));
            bsdf_pdf = e.pdf;
            return mul(fv(e.value), cosine);
        }
        if (h.material_type == 0) {
            const float c = std::fmax(dot(h.shading_normal, ldir), 0.0f);
            bsdf_pdf = c / kPi;
            return mul(h.base_color, bsdf_pdf);
        }
        if (h.material_type == 4) {
            bsdf_pdf = uniform_sphere_pdf();
            return mul(h.base_color, bsdf_pdf);
        }
        return {0, 0, 0};
    }

    LightSample sample_direct(const Hit& rcv, uint32_t& rng) const {
        LightSample smp{};
        const V3 sp = rcv.position;
        const PackedLight* ex = rcv.primitive_type < 0 ? nullptr : find_light(rcv.primitive_type, rcv.primitive_index);
        const float eligible = ex == nullptr ? 1.0f : 1.0f - ex->selection_pdf;
        if (eligible <= 1e-8f) return smp;
        const int count = static_cast<int>(s_.lights.size());
        int li = -1;
        if (ex == nullptr) {
            li = sample_cdf(count, rnd(rng), [&](int i) { return s_.lights[static_cast<size_t>(i)].cdf; });
        } else {
            const float target = rnd(rng) * eligible;
            float acc = 0.0f;
            for (int i = 0; i < count; ++i) {
                if (&s_.lights[static_cast<size_t>(i)] == ex) continue;
                acc += s_.lights[static_cast<size_t>(i)].selection_pdf;
                if (target < acc) {
                    li = i;
                    break;
                }
            }
            if (li < 0) {
                for (int i = count - 1; i >= 0; --i) {
                    if (&s_.lights[static_cast<size_t>(i)] != ex) {
                        li = i;
                        break;
                    }
                }
            }
        }
        if (li < 0) return smp;
        const PackedLight& light = s_.lights[static_cast<size_t>(li)];
        const float sel = light.selection_pdf / eligible;
        if (sel <= 0.0f) return smp;
        if (light.type == 3) {
            if (rcv.material_type == 4) {
                smp.direction = random_unit_vector(rng);
                smp.pdf = sel * uniform_sphere_pdf();
            } else {
                smp.direction = add(rcv.shading_normal, random_unit_vector(rng));
                if (near_zero(smp.direction)) smp.direction = rcv.shading_normal;
                smp.direction = normalize(smp.direction);
                const float c = std::fmax(dot(rcv.shading_normal, smp.direction), 0.0f);
                smp.pdf = sel * c / kPi;
            }
            smp.emission = s_.background;
            smp.distance = kRayFar;
            smp.infinite = true;
            smp.valid = smp.pdf > 0.0f;
            return smp;
        }
        float tu = 0.0f, tv = 0.0f, cond = 0.0f;
        if (light.type == 0) {
            if (light.primitive_index < 0 || light.primitive_index >= static_cast<int>(s_.spheres.size())) return smp;
            const rtgb_sphere& sph = s_.spheres[static_cast<size_t>(light.primitive_index)];
            const V3 center = from3(sph.center);
            const V3 tc = sub(center, sp);
            const float d2 = len_sq(tc);
            const float r2 = sph.radius * sph.radius;
            if (d2 <= r2 * (1.0f + 1e-6f)) return smp;
            const float ctm = std::sqrt(std::fmax(0.0f, 1.0f - r2 / d2));
            const V3 axis = normalize(tc);
            const float u0 = rnd(rng);
            const float u1 = rnd(rng);
            smp.direction = cone_direction(axis, ctm, u0, u1);
            const V3 oc = sub(sp, center);
            const float hb = dot(oc, smp.direction);
            const float disc = hb * hb - (len_sq(oc) - r2);
            if (disc <= 0.0f) return smp;
            smp.distance = -hb - std::sqrt(disc);
            if (smp.distance <= kRayEpsilon) return smp;
            smp.position = add(sp, mul(smp.direction, smp.distance));
            smp.normal = normalize(sub(smp.position, center));
            sphere_uv(smp.normal, tu, tv);
            smp.material_index = sph.material_index;
            cond = uniform_cone_pdf(ctm);
        } else if (light.type == 1) {
            if (light.primitive_index < 0 || light.primitive_index >= static_cast<int>(s_.quads.size())) return smp;
            const rtgb_quad& q = s_.quads[static_cast<size_t>(light.primitive_index)];
            const V3 o = from3(q.origin), eu = from3(q.edge_u), ev = from3(q.edge_v);
            tu = rnd(rng);
            tv = rnd(rng);
            smp.position = add(o, add(mul(eu, tu), mul(ev, tv)));
            const V3 an = cross(eu, ev);
            const float area = len(an);
            if (area <= 1e-12f) return smp;
            smp.normal = divs(an, area);
            smp.material_index = q.material_index;
            const V3 tl = sub(smp.position, sp);
            const float d2 = len_sq(tl);
            if (d2 <= 1e-12f) return LightSample{};
            smp.distance = std::sqrt(d2);
            smp.direction = divs(tl, smp.distance);
            const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
            cond = area_to_solid_angle_pdf(area, d2, ac);
        } else {
            if (light.primitive_index < 0 || light.primitive_index >= static_cast<int>(s_.triangles.size())) return smp;
            const rtgb_triangle& t = s_.triangles[static_cast<size_t>(light.primitive_index)];
            const V3 p0 = from3(t.p0), p1 = from3(t.p1), p2 = from3(t.p2);
            float w0 = 0.0f, w1 = 0.0f, w2 = 0.0f;
            const float u0 = rnd(rng);
            const float u1 = rnd(rng);
            sample_uniform_triangle(u0, u1, w0, w1, w2);
            smp.position = add(mul(p0, w0), add(mul(p1, w1), mul(p2, w2)));
            if (t.has_texcoords != 0) {
                tu = t.uv0[0] * w0 + t.uv1[0] * w1 + t.uv2[0] * w2;
                tv = t.uv0[1] * w0 + t.uv1[1] * w1 + t.uv2[1] * w2;
            } else {
                tu = w1;
                tv = w2;
            }
            const V3 an = cross(sub(p1, p0), sub(p2, p0));
            const float da = len(an);
            if (da <= 1e-12f) return smp;
            smp.normal = divs(an, da);
            smp.material_index = t.material_index;
            const V3 tl = sub(smp.position, sp);
            const float d2 = len_sq(tl);
            if (d2 <= 1e-12f) return LightSample{};
            smp.distance = std::sqrt(d2);
            smp.direction = divs(tl, smp.distance);
            const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
            cond = area_to_solid_angle_pdf(0.5f * da, d2, ac);
        }
        if (cond <= 0.0f || smp.material_index < 0 || smp.material_index >= static_cast<int>(s_.materials.size())) {
            return LightSample{};
        }
        smp.emission = material_emission(s_.materials[static_cast<size_t>(smp.material_index)], tu, tv, smp.position);
        smp.pdf = sel * cond;
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }

    LightSample analytic_candidate(const Hit& rcv, int li, float u0, float u1) const {
        LightSample smp{};
        if (li < 0 || li >= static_cast<int>(s_.analytic.size())) return smp;
        const rtgb_analytic_light& l = s_.analytic[static_cast<size_t>(li)];
        if (l.selection_pdf <= 0.0f) return smp;
        smp.light_index = li;
        smp.emission = from3(l.radiance);
        if (l.type == 5) {
            smp.direction = sphere_direction(u0, u1);
            smp.distance = kRayFar;
            smp.pdf = l.selection_pdf * uniform_sphere_pdf();
            smp.infinite = true;
            smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
            return smp;
        }
        if (l.type == 4) {
            const V3 axis = normalize(from3(l.basis_z));
            smp.direction = l.delta != 0 ? axis : cone_direction(axis, l.cos_theta_max, u0, u1);
            smp.distance = kRayFar;
            smp.pdf = l.selection_pdf * (l.delta != 0 ? 1.0f : uniform_cone_pdf(l.cos_theta_max));
            smp.infinite = true;
            smp.delta = l.delta != 0;
            smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
            return smp;
        }
        const V3 sp = rcv.position;
        const V3 center = from3(l.position);
        if (l.type == 0) {
            const V3 tc = sub(center, sp);
            const float d2 = len_sq(tc);
            const float radius = l.radius * len(from3(l.basis_x));
            const float r2 = radius * radius;
            if (d2 <= r2 * (1.0f + 1e-6f)) return smp;
            if (l.treat_as_point != 0) {
                smp.distance = std::sqrt(d2);
                smp.direction = divs(tc, smp.distance);
                const float iscale = l.world_area > 1e-12f ? l.world_area : 1.0f;
                smp.emission = mul(smp.emission, iscale / d2);
                smp.pdf = l.selection_pdf;
                smp.delta = true;
                smp.valid = max_comp(smp.emission) > 0.0f;
                return smp;
            }
            const float ctm = std::sqrt(std::fmax(0.0f, 1.0f - r2 / d2));
            smp.direction = cone_direction(normalize(tc), ctm, u0, u1);
            AnalyticHit sh{};
            if (!hit_analytic(l, Ray{sp, smp.direction}, kRayEpsilon, kRayFar, sh)) return LightSample{};
            smp.position = sh.position;
            smp.normal = sh.normal;
            smp.distance = sh.t;
            smp.pdf = l.selection_pdf * uniform_cone_pdf(ctm);
            smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
            return smp;
        }
        if (l.type == 1) {
            const float radial = l.radius * std::sqrt(u0);
            const float phi = 2.0f * kPi * u1;
            smp.position = add(center, add(mul(from3(l.basis_x), radial * std::cos(phi)), mul(from3(l.basis_y), radial * std::sin(phi))));
            smp.normal = analytic_normal(l);
        } else if (l.type == 2) {
            smp.position = add(center, add(mul(from3(l.basis_x), (u0 - 0.5f) * l.width), mul(from3(l.basis_y), (u1 - 0.5f) * l.height)));
            smp.normal = analytic_normal(l);
        } else if (l.type == 3) {
            const float phi = 2.0f * kPi * u0;
            const float rx = l.radius * std::cos(phi);
            const float ry = l.radius * std::sin(phi);
            smp.position = add(center, add(add(mul(from3(l.basis_x), rx), mul(from3(l.basis_y), ry)),
                                           mul(from3(l.basis_z), (u1 - 0.5f) * l.length)));
            smp.normal = normalize(add(mul(from3(l.basis_x), rx), mul(from3(l.basis_y), ry)));
        } else {
            return LightSample{};
        }
        const V3 tl = sub(smp.position, sp);
        const float d2 = len_sq(tl);
        if (d2 <= 1e-12f) return LightSample{};
        smp.distance = std::sqrt(d2);
        smp.direction = divs(tl, smp.distance);
        const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
        smp.pdf = l.selection_pdf * area_to_solid_angle_pdf(l.world_area, d2, ac);
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }

    int sample_analytic_index(float u) const {
        return sample_cdf(static_cast<int>(s_.analytic.size()), u,
            [&](int i) { return s_.analytic[static_cast<size_t>(i)].cdf; });
    }

    const Scene& scene() const { return s_; }

private:
    const Scene& s_;
};

// ---- per-camera renderer state (optix_renderer.cpp, device_frame_buffers.cpp) ----

struct FrameBuffers {
    std::vector<float> beauty, normal, dnormal, albedo;  // 4 floats per pixel
    std::vector<float> depth, flow, trust;
    std::vector<Reservoir> reservoirs;
    void resize(size_t n) {
        beauty.assign(n * 4, 0.0f);
        normal.assign(n * 4, 0.0f);
        dnormal.assign(n * 4, 0.0f);
        albedo.assign(n * 4, 0.0f);
        depth.assign(n, 0.0f);
        flow.assign(n * 2, 0.0f);
        trust.assign(n, 0.0f);
        Reservoir zero{};
        std::memset(&zero, 0, sizeof zero);  // the reference memsets the buffer every launch
        reservoirs.assign(n, zero);
    }
};

struct CameraState {
    int width = 0, height = 0;
    FrameBuffers frame, history;
    int history_w = 0, history_h = 0;
    int history_length = 0;
    Camera previous{};
    int previous_valid = 0;
    // parity records
    std::vector<int32_t> codes;
    std::vector<float> path_radiance;
    int record_bounces = 0;
    int record_spp = 0;
    // diagnostics of the last frame: number of ReSTIR visibility rays etc.
    uint64_t rays = 0;
};

struct Params {
    const Camera* cam;
    const Camera* prev;
    int prev_valid;
    int history_length;
    const FrameBuffers* history;
    FrameBuffers* frame;
    uint32_t stream;
    rtgb_render_profile profile;
    int restir_enabled;
    int width, height;
    CameraState* state;
};

class Renderer {
public:
    Renderer(const rtgb_scene& sc, bool use_bvh, int threads) : tracer_(scene_) {
        scene_.textures.assign(sc.textures, sc.textures + sc.texture_count);
        scene_.texels.assign(sc.image_texels, sc.image_texels + 3 * static_cast<size_t>(sc.image_texel_count));
        scene_.materials.assign(sc.materials, sc.materials + sc.material_count);
        scene_.spheres.assign(sc.spheres, sc.spheres + sc.sphere_count);
        scene_.quads.assign(sc.quads, sc.quads + sc.quad_count);
        scene_.triangles.assign(sc.triangles, sc.triangles + sc.triangle_count);
        scene_.media.assign(sc.media, sc.media + sc.medium_count);
        scene_.analytic.assign(sc.analytic_lights, sc.analytic_lights + sc.analytic_light_count);
        if (sc.openpbr_materials != nullptr && sc.openpbr_material_count > 0) {
            scene_.openpbr.assign(sc.openpbr_materials, sc.openpbr_materials + sc.openpbr_material_count);
        }
        scene_.background = from3(sc.background);
        scene_.use_bvh = use_bvh;
        build_light_distribution(scene_);
        if (use_bvh) build_reference_bvh(scene_);
        threads_ = threads > 0 ? threads : static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    }

    void reset_sequence(uint32_t s) {
        stream_ = s;
        reset_accumulation();
    }
    void reset_accumulation() {
        for (CameraState& c : cams_) {
            c.history_length = 0;
            c.previous_valid = 0;
        }
    }

    void set_record(bool on) { record_ = on; }

    // launch_radiance_pipeline for every active camera; rows [y0, y1) only
    // when y1 > y0 (a bounded sample for timing).
    int render_frame(const rtgb_camera_rig& rig, const rtgb_render_profile& profile, int active, int y0, int y1,
        int stride) {
        if (active < 1 || active > RTGB_MAX_CAMERAS || active > rig.active_count) return RTGB_INVALID_ARGUMENT;
        if (cams_.size() < static_cast<size_t>(active)) cams_.resize(static_cast<size_t>(active));
        const uint32_t stream = stream_++;
        for (int ci = 0; ci < active; ++ci) {
            const rtgb_camera& pc = rig.cameras[ci];
            if (pc.enabled == 0 || pc.width <= 0 || pc.height <= 0) return RTGB_INVALID_ARGUMENT;
            CameraState& cs = cams_[static_cast<size_t>(ci)];
            const Camera cam = make_camera(pc);
            const size_t n = static_cast<size_t>(pc.width) * static_cast<size_t>(pc.height);
            cs.frame.resize(n);
            if (cs.history_w != pc.width || cs.history_h != pc.height) {
                cs.history.resize(n);
                cs.history_w = pc.width;
                cs.history_h = pc.height;
                cs.history_length = 0;
                cs.previous_valid = 0;
            }
            cs.width = pc.width;
            cs.height = pc.height;
            Params p{};
            p.cam = &cam;
            p.prev = &cs.previous;
            p.prev_valid = cs.previous_valid;
            p.history_length = cs.history_length;
            p.history = &cs.history;
            p.frame = &cs.frame;
            p.stream = stream;
            p.profile = profile;
            const int min_lights = profile.restir_min_analytic_lights > 0 ? profile.restir_min_analytic_lights : 1;
            p.restir_enabled = profile.enable_restir_di != 0 && static_cast<int>(scene_.analytic.size()) >= min_lights ? 1 : 0;
            p.width = pc.width;
            p.height = pc.height;
            p.state = &cs;
            const int spp = profile.samples_per_pixel > 0 ? profile.samples_per_pixel : 1;
            const int mb = profile.max_bounces > 0 ? profile.max_bounces : 1;
            if (record_) {
                cs.codes.assign(n * static_cast<size_t>(spp) * static_cast<size_t>(mb), -2);
                cs.path_radiance.assign(n * static_cast<size_t>(spp) * 3, 0.0f);
                cs.record_bounces = mb;
                cs.record_spp = spp;
            }
            const int ry0 = y1 > y0 ? std::max(0, y0) : 0;
            const int ry1 = y1 > y0 ? std::min(pc.height, y1) : pc.height;
            std::atomic<uint64_t> rays{0};
            const int step = stride > 1 ? stride : 1;
            const int nrows = (ry1 - ry0 + step - 1) / step;
            parallel_rows(0, nrows, [&](int r) {
                const int y = ry0 + r * step;
                uint64_t local = 0;
                for (int x = 0; x < pc.width; ++x) local += radiance_pixel(p, x, y);
                rays.fetch_add(local, std::memory_order_relaxed);
            });
            parallel_rows(0, nrows, [&](int r) {
                const int y = ry0 + r * step;
                for (int x = 0; x < pc.width; ++x) resolve_pixel(p, x, y);
            });
            cs.rays = rays.load();
            // capture_launch_history (radiance_launch_setup.cpp:122-136) and copy_frame_to_history
            cs.previous = cam;
            cs.previous_valid = 1;
            cs.history_length = cs.history_length == 0 ? 1 : cs.history_length + 1;
            cs.history.beauty = cs.frame.beauty;
            cs.history.normal = cs.frame.normal;
            cs.history.depth = cs.frame.depth;
            cs.history.reservoirs = cs.frame.reservoirs;
        }
        return RTGB_OK;
    }

    CameraState* camera(int i) { return i >= 0 && i < static_cast<int>(cams_.size()) ? &cams_[static_cast<size_t>(i)] : nullptr; }
    uint32_t stream() const { return stream_; }
    const Tracer& tracer() const { return tracer_; }
    const Scene& scene() const { return scene_; }

private:
    template <typename F>
    void parallel_rows(int y0, int y1, F&& fn) {
        const int rows = y1 - y0;
        if (rows <= 0) return;
        const int nt = std::min(threads_, rows);
        std::atomic<int> next{y0};
        std::vector<std::thread> pool;
        pool.reserve(static_cast<size_t>(nt));
        for (int t = 0; t < nt; ++t) {
            pool.emplace_back([&]() {
                for (;;) {
                    const int y = next.fetch_add(1);
                    if (y >= y1) break;
                    fn(y);
                }
            });
        }
        for (std::thread& th : pool) th.join();
    }

    // ---- ReSTIR: programs.cu:2105-2449 -------------------------------------

    static Surface restir_surface(const Hit& h) {
        Surface s{};
        s.position[0] = h.position.x; s.position[1] = h.position.y; s.position[2] = h.position.z;
        s.normal[0] = h.shading_normal.x; s.normal[1] = h.shading_normal.y; s.normal[2] = h.shading_normal.z;
        s.material_type = h.material_type;
        s.primitive_type = h.primitive_type;
        s.primitive_index = h.primitive_index;
        return s;
    }

    static float restir_lum(const V3& v) { return std::fmax(0.0f, 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z); }

    V3 unshadowed(const Hit& h, const PathState& st, const LightSample& l, bool bsdf_avail, float& target) const {
        target = 0.0f;
        if (!l.valid || l.pdf <= 0.0f) return {0, 0, 0};
        float bp = 0.0f;
        const V3 resp = tracer_.direct_response(h, st, l.direction, bp);
        if (max_comp(resp) <= 0.0f) return {0, 0, 0};
        const float mis = l.delta || !bsdf_avail ? 1.0f : power_heuristic(l.pdf, bp);
        const V3 num = mul(mul(l.emission, resp), mis);
        target = restir_lum(num);
        return num;
    }

    static bool previous_pixel(const Params& p, const Hit& h, int& index) {
        index = -1;
        if (p.history_length <= 0 || p.prev_valid == 0) return false;
        const Camera& c = *p.prev;
        const V3 off = sub(h.position, cam_origin(c));
        const V3 cp{dot(off, basis_f(c.basis_x)), dot(off, basis_f(c.basis_y)), dot(off, basis_f(c.basis_z))};
        const V3 px = project(c, cp);
        if (!std::isfinite(px.x) || !std::isfinite(px.y)) return false;
        const int x = static_cast<int>(std::floor(px.x));
        const int y = static_cast<int>(std::floor(px.y));
        if (x < 0 || x >= p.width || y < 0 || y >= p.height) return false;
        index = y * p.width + x;
        return true;
    }

    float target_at_previous(const Params& p, const Reservoir& src, const Candidate& sel, bool bsdf_avail, uint64_t& rays) const {
        if (p.prev_valid == 0) return 0.0f;
        const V3 spos = from3(src.surface.position);
        const V3 origin = cam_origin(*p.prev);
        const V3 off = sub(spos, origin);
        const float dist = len(off);
        if (!std::isfinite(dist) || dist <= kRayEpsilon) return 0.0f;
        PathState ss{};
        ss.ray.origin = origin;
        ss.ray.direction = mul(off, 1.0f / dist);
        ++rays;
        const Hit sh = tracer_.intersect(ss.ray, kRayEpsilon, dist + 0.05f, nullptr);
        if (!sh.hit || sh.material_type != src.surface.material_type || sh.primitive_type != src.surface.primitive_type
            || sh.primitive_index != src.surface.primitive_index) {
            return 0.0f;
        }
        const float tol = std::fmax(0.01f, 0.02f * dist);
        if (len_sq(sub(sh.position, spos)) > tol * tol || dot(sh.shading_normal, from3(src.surface.normal)) < 0.95f) return 0.0f;
        const LightSample l = tracer_.analytic_candidate(sh, sel.light_index, sel.u0, sel.u1);
        float t = 0.0f;
        unshadowed(sh, ss, l, bsdf_avail, t);
        return t;
    }

    void restir_direct(const Params& p, const Hit& h, int x, int y, uint32_t& rng, bool bsdf_avail, PathState& st, uint64_t& rays) const {
        const Scene& sc = tracer_.scene();
        if (h.material_type == 3 || sc.analytic.empty()) return;
        Reservoir r{};
        const int req = p.profile.restir_initial_candidates > 0 ? p.profile.restir_initial_candidates : 1;
        const int count = req < 32 ? req : 32;
        for (int c = 0; c < count; ++c) {
            const int li = tracer_.sample_analytic_index(rnd(rng));
            Candidate cand{};
            cand.light_index = li;
            cand.u0 = rnd(rng);
            cand.u1 = rnd(rng);
            const LightSample l = tracer_.analytic_candidate(h, cand.light_index, cand.u0, cand.u1);
            float t = 0.0f;
            unshadowed(h, st, l, bsdf_avail, t);
            const float w = l.pdf > 0.0f ? t / l.pdf : 0.0f;
            reservoir_update(r, cand, t, w, 1, rnd(rng));
        }
        const int canonical = r.candidate_count;
        Reservoir sources[9];
        int mult[9] = {0};
        int nsrc = 0;
        int selected_src = -1;
        const FrameBuffers& hist = *p.history;
        if (p.profile.restir_temporal_reuse != 0) {
            int pi = -1;
            if (previous_pixel(p, h, pi)) {
                const Reservoir prev = hist.reservoirs[static_cast<size_t>(pi)];
                const float tol = std::fmax(0.005f, 0.01f * h.t);
                if (surface_valid(restir_surface(h), prev, tol, 0.95f, p.profile.restir_max_history_age)) {
                    const LightSample l = tracer_.analytic_candidate(h, prev.selected.light_index, prev.selected.u0, prev.selected.u1);
                    float t = 0.0f;
                    unshadowed(h, st, l, bsdf_avail, t);
                    const MergeResult m = reservoir_merge(r, prev, t, p.profile.restir_max_temporal_candidates, rnd(rng), true);
                    if (m.multiplicity > 0) {
                        sources[nsrc] = prev;
                        mult[nsrc] = m.multiplicity;
                        if (m.selected != 0) selected_src = nsrc;
                        ++nsrc;
                    }
                }
            }
        }
        const int nbrs = p.profile.restir_spatial_neighbors < 8 ? p.profile.restir_spatial_neighbors : 8;
        if (nbrs > 0) {
            int ri = -1;
            if (previous_pixel(p, h, ri)) {
                static const int kOff[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
                const int rot = (x * 3 + y * 5 + static_cast<int>(p.stream)) & 7;
                for (int k = 0; k < nbrs; ++k) {
                    const int oi = (rot + k) & 7;
                    const int bx = ri % p.width, by = ri / p.width;
                    const int nx = bx + kOff[oi][0], ny = by + kOff[oi][1];
                    if (nx < 0 || nx >= p.width || ny < 0 || ny >= p.height) continue;
                    const Reservoir prev = hist.reservoirs[static_cast<size_t>(ny * p.width + nx)];
                    const float tol = std::fmax(0.01f, 0.02f * h.t);
                    if (!surface_valid(restir_surface(h), prev, tol, 0.95f, p.profile.restir_max_history_age)) continue;
                    const LightSample l = tracer_.analytic_candidate(h, prev.selected.light_index, prev.selected.u0, prev.selected.u1);
                    float t = 0.0f;
                    unshadowed(h, st, l, bsdf_avail, t);
                    const MergeResult m = reservoir_merge(r, prev, t, p.profile.restir_max_spatial_candidates, rnd(rng), false);
                    if (m.multiplicity > 0 && nsrc < 9) {
                        sources[nsrc] = prev;
                        mult[nsrc] = m.multiplicity;
                        if (m.selected != 0) selected_src = nsrc;
                        ++nsrc;
                    }
                }
            }
        }
        r.surface = restir_surface(h);
        if (p.profile.restir_bias_correction == 1 && nsrc > 0 && r.valid != 0) {
            float sel_t = r.selected_target;
            float sum = r.selected_target * static_cast<float>(canonical);
            for (int s = 0; s < nsrc; ++s) {
                const float t = target_at_previous(p, sources[s], r.selected, bsdf_avail, rays);
                sum += t * static_cast<float>(mult[s]);
                if (selected_src == s) sel_t = t;
            }
            reservoir_finalize_basic(r, sel_t, sum, nsrc);
        } else {
            reservoir_finalize(r);
        }
        p.frame->reservoirs[static_cast<size_t>(y * p.width + x)] = r;
        if (r.valid == 0) return;
        const LightSample l = tracer_.analytic_candidate(h, r.selected.light_index, r.selected.u0, r.selected.u1);
        float t = 0.0f;
        const V3 num = unshadowed(h, st, l, bsdf_avail, t);
        if (!l.valid || t <= 0.0f) return;
        const Ray shadow{add(h.position, mul(l.direction, kRayEpsilon * 2.0f)), l.direction};
        const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
        if (max_t <= kRayEpsilon) return;
        ++rays;
        if (tracer_.occluded(shadow, max_t)) return;
        st.decisions |= kDecisionNeeAnalytic;
        st.radiance = add(st.radiance, mul(st.throughput, mul(num, r.estimator_weight)));
    }

    void direct_emissive(const Hit& h, uint32_t& rng, bool bsdf_avail, PathState& st, uint64_t& rays) const {
        if (h.material_type == 3 || tracer_.scene().lights.empty()) return;
        const LightSample l = tracer_.sample_direct(h, rng);
        if (!l.valid) return;
        float bp = 0.0f;
        const V3 resp = tracer_.direct_response(h, st, l.direction, bp);
        if (max_comp(resp) <= 0.0f) return;
        const Ray shadow{add(h.position, mul(l.direction, kRayEpsilon * 2.0f)), l.direction};
        const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
        if (max_t <= kRayEpsilon) return;
        ++rays;
        if (tracer_.occluded(shadow, max_t)) return;
        const float mis = bsdf_avail ? power_heuristic(l.pdf, bp) : 1.0f;
        const V3 direct = mul(mul(l.emission, resp), mis / l.pdf);
        st.decisions |= kDecisionNeeEmissive;
        st.radiance = add(st.radiance, mul(st.throughput, direct));
    }

    void direct_analytic(const Hit& h, uint32_t& rng, bool bsdf_avail, PathState& st, uint64_t& rays) const {
        if (h.material_type == 3 || tracer_.scene().analytic.empty()) return;
        const int li = tracer_.sample_analytic_index(rnd(rng));
        const float u0 = rnd(rng);
        const float u1 = rnd(rng);
        const LightSample l = tracer_.analytic_candidate(h, li, u0, u1);
        if (!l.valid) return;
        float bp = 0.0f;
        const V3 resp = tracer_.direct_response(h, st, l.direction, bp);
        if (max_comp(resp) <= 0.0f) return;
        const Ray shadow{add(h.position, mul(l.direction, kRayEpsilon * 2.0f)), l.direction};
        const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
        if (max_t <= kRayEpsilon) return;
        ++rays;
        if (tracer_.occluded(shadow, max_t)) return;
        const float mis = l.delta || !bsdf_avail ? 1.0f : power_heuristic(l.pdf, bp);
        const V3 direct = mul(mul(l.emission, resp), mis / l.pdf);
        st.decisions |= kDecisionNeeAnalytic;
        st.radiance = add(st.radiance, mul(st.throughput, direct));
    }

    static void record_scatter(PathState& st, const Hit& h, float pdf, bool delta) {
        st.prev_position = h.position;
        st.prev_normal = h.shading_normal;
        st.prev_bsdf_pdf = pdf;
        st.prev_material_type = h.material_type;
        st.prev_primitive_type = h.primitive_type;
        st.prev_primitive_index = h.primitive_index;
        st.prev_valid = true;
        st.prev_delta = delta;
    }

    // sample_bsdf, programs.cu:2463-2565
    void sample_bsdf(const Hit& h, uint32_t& rng, PathState& st) const {
        if (!st.alive) return;
        if (h.material_type == 3) {
            st.alive = false;
            return;
        }
        if (h.material_type == 0) {
            V3 d = add(h.shading_normal, random_unit_vector(rng));
            if (near_zero(d)) d = h.shading_normal;
            st.ray.origin = add(h.position, mul(h.shading_normal, kRayEpsilon));
            st.ray.direction = normalize(d);
            st.throughput = mul(st.throughput, h.base_color);
            const float c = std::fmax(dot(h.shading_normal, st.ray.direction), 0.0f);
            record_scatter(st, h, c / kPi, false);
            return;
        }
        if (h.material_type == 1) {
            const V3 refl = reflect(normalize(st.ray.direction), h.shading_normal);
            const V3 fz = mul(random_in_unit_sphere(rng), std::fmin(std::fmax(h.fuzz, 0.0f), 1.0f));
            const V3 sc = normalize(add(refl, fz));
            if (dot(sc, h.shading_normal) <= 0.0f) {
                st.alive = false;
                return;
            }
            st.ray.origin = add(h.position, mul(h.shading_normal, kRayEpsilon));
            st.ray.direction = sc;
            st.throughput = mul(st.throughput, h.base_color);
            record_scatter(st, h, 0.0f, true);
            return;
        }
        if (h.material_type == 2) {
            const float ratio = h.front_face ? (1.0f / std::fmax(h.ior, 1e-4f)) : std::fmax(h.ior, 1e-4f);
            const V3 ud = normalize(st.ray.direction);
            const float ct = std::fmin(dot(mul(ud, -1.0f), h.shading_normal), 1.0f);
            const float stt = std::sqrt(std::fmax(0.0f, 1.0f - ct * ct));
            const bool cannot = ratio * stt > 1.0f;
            V3 dir;
            bool refl = cannot;
            if (!refl) {
                float r0 = (1.0f - ratio) / (1.0f + ratio);
                r0 *= r0;
                const float fres = r0 + (1.0f - r0) * std::pow(1.0f - ct, 5.0f);
                refl = fres > rnd(rng);
            }
            dir = refl ? reflect(ud, h.shading_normal) : refract(ud, h.shading_normal, ratio);
            st.ray.origin = add(h.position, mul(dir, kRayEpsilon));
            st.ray.direction = normalize(dir);
            st.throughput = mul(st.throughput, h.base_color);
            record_scatter(st, h, 0.0f, true);
            return;
        }
        if (h.material_type == 5) {
            if (tracer_.openpbr_material(h.openpbr_index) == nullptr) {
                st.alive = false;
                return;
            }
            const pbr::Mat params = tracer_.scattering_parameters(h);
            const pbr::Frame frame = pbr::make_frame(pv(h.geometric_normal), pbr::V3{0.0f, 0.0f, 0.0f});
            const float u_lobe = rnd(rng);
            const float u1 = rnd(rng);
            const float u2 = rnd(rng);
            const pbr::Sample smp = pbr::sample(params, frame, pv(mul(normalize(st.ray.direction), -1.0f)), u_lobe, u1,
                u2, Tracer::transport_context(st));
            if (smp.valid == 0) {
                st.alive = false;
                return;
            }
            const V3 d = fv(smp.wi);
            st.ray.origin = add(h.position, mul(d, kRayEpsilon));
            st.ray.direction = normalize(d);
            st.throughput = mul(st.throughput, fv(smp.weight));
            st.decisions |= smp.event << 2;
            record_scatter(st, h, smp.pdf, smp.delta != 0);
            if (smp.event == pbr::kSubsurfaceEntry) {
                st.subsurface = pbr::subsurface_medium(params);
                st.subsurface_material = h.openpbr_index;
            } else if (smp.event == pbr::kSubsurfaceExit) {
                st.subsurface = pbr::Medium{};
                st.subsurface_material = -1;
            }
            return;
        }
        if (h.material_type == 4) {
            const V3 d = random_unit_vector(rng);
            st.ray.origin = add(h.position, mul(d, kRayEpsilon));
            st.ray.direction = d;
            st.throughput = mul(st.throughput, h.base_color);
            record_scatter(st, h, uniform_sphere_pdf(), false);
            return;
        }
        st.alive = false;
    }

    // radiance_kernel, programs.cu:1828-1953, for one pixel. Returns rays traced.
    uint64_t radiance_pixel(const Params& p, int x, int y) const {
        const Scene& sc = tracer_.scene();
        const int pixel = y * p.width + x;
        const int spp = p.profile.samples_per_pixel > 0 ? p.profile.samples_per_pixel : 1;
        const int mb = p.profile.max_bounces > 0 ? p.profile.max_bounces : 1;
        V3 beauty{0, 0, 0}, nsum{0, 0, 0}, asum{0, 0, 0};
        float dsum = 0.0f;
        int aux = 0;
        uint64_t rays = 0;
        const float pxf = static_cast<float>(x) + 0.5f;
        const float pyf = static_cast<float>(y) + 0.5f;
        const V3 dir_cam = unproject(*p.cam, pxf, pyf);
        for (int s = 0; s < spp; ++s) {
            uint32_t rng = rng_for(pixel, s, p.stream);
            PathState st{};
            st.ray.origin = cam_origin(*p.cam);
            st.ray.direction = to_world(*p.cam, dir_cam);
            V3 sn{0, 0, 1}, sa{0, 0, 0};
            float sd = 0.0f;
            bool captured = false;
            int32_t* codes = nullptr;
            if (!p.state->codes.empty()) {
                codes = &p.state->codes[(static_cast<size_t>(pixel) * static_cast<size_t>(spp) + static_cast<size_t>(s)) * static_cast<size_t>(mb)];
            }
            int last_b = -1;
            for (int b = 0; b < mb && st.alive; ++b) {
                if (codes && last_b >= 0) codes[last_b] |= st.decisions << kDecisionShift;
                st.decisions = 0;
                last_b = b;
                ++rays;
                Hit h = tracer_.intersect(st.ray, kRayEpsilon, kRayFar, &rng);
                const AnalyticHit ah = tracer_.intersect_analytic(st.ray, kRayEpsilon, h.hit ? h.t : kRayFar);
                if (codes) codes[b] = ah.hit ? ((5 << 28) | ah.light_index) : (h.hit ? h.record_code : -1);
                if (ah.hit) {
                    const rtgb_analytic_light& l = sc.analytic[static_cast<size_t>(ah.light_index)];
                    const float w = tracer_.analytic_emission_mis(st, ah);
                    st.radiance = add(st.radiance, mul(st.throughput, mul(from3(l.radiance), w)));
                    st.alive = false;
                    break;
                }
                if (!h.hit) {
                    const float w = tracer_.emission_mis_weight(st, nullptr, true);
                    st.radiance = add(st.radiance, mul(st.throughput, mul(sc.background, w)));
                    st.radiance = add(st.radiance, mul(st.throughput, tracer_.analytic_infinite_radiance(st)));
                    st.alive = false;
                    break;
                }
                // OpenPBR random-walk segment inside the entered material (programs.cu:1878-1902)
                if (st.subsurface.active != 0) {
                    if (h.material_type != 5 || h.openpbr_index != st.subsurface_material || h.front_face) {
                        st.alive = false;
                        break;
                    }
                    const float ray_len = std::sqrt(len_sq(st.ray.direction));
                    const pbr::Segment seg = pbr::subsurface_segment(st.subsurface, h.t * ray_len, rnd(rng),
                        Tracer::transport_context(st));
                    st.throughput = mul(st.throughput, fv(seg.weight));
                    if (seg.scattered != 0) {
                        const V3 incident = normalize(st.ray.direction);
                        const float g1 = rnd(rng);
                        const float g2 = rnd(rng);
                        const V3 dir = fv(pbr::sample_hg(pv(incident), st.subsurface.anisotropy, g1, g2));
                        st.ray.origin = add(st.ray.origin, mul(st.ray.direction, seg.distance / std::fmax(ray_len, 1e-8f)));
                        st.ray.direction = dir;
                        st.ray.origin = add(st.ray.origin, mul(st.ray.direction, kRayEpsilon));
                        st.prev_valid = false;
                        st.decisions |= kDecisionWalk << 2;
                        continue;
                    }
                }
                if (!captured && b == 0) {
                    sn = h.shading_normal;
                    sa = h.base_color;
                    sd = h.t;
                    captured = true;
                }
                const float ew = tracer_.emission_mis_weight(st, &h, false);
                st.radiance = add(st.radiance, mul(st.throughput, mul(h.emission, ew)));
                const bool bsdf_avail = b + 1 < mb;
                direct_emissive(h, rng, bsdf_avail, st, rays);
                const bool use_restir = p.restir_enabled != 0 && b == 0;
                if (use_restir) {
                    restir_direct(p, h, x, y, rng, bsdf_avail, st, rays);
                } else {
                    direct_analytic(h, rng, bsdf_avail, st, rays);
                }
                if (!bsdf_avail) {
                    st.alive = false;
                    break;
                }
                sample_bsdf(h, rng, st);
                if (st.alive && b >= p.profile.rr_start_bounce) {
                    const float q = std::fmin(std::fmax(max_comp(st.throughput), 0.05f), 0.95f);
                    if (rnd(rng) > q) {
                        st.alive = false;
                    } else {
                        st.throughput = divs(st.throughput, q);
                    }
                }
            }
            if (codes && last_b >= 0) codes[last_b] |= st.decisions << kDecisionShift;
            beauty = add(beauty, st.radiance);
            if (!p.state->path_radiance.empty()) {
                float* pr = &p.state->path_radiance[(static_cast<size_t>(pixel) * static_cast<size_t>(spp) + static_cast<size_t>(s)) * 3];
                pr[0] = st.radiance.x;
                pr[1] = st.radiance.y;
                pr[2] = st.radiance.z;
            }
            if (captured) {
                nsum = add(nsum, sn);
                asum = add(asum, sa);
                dsum += sd;
                ++aux;
            }
        }
        const float inv_spp = 1.0f / static_cast<float>(spp);
        const V3 bavg = mul(beauty, inv_spp);
        const float inv_aux = aux > 0 ? (1.0f / static_cast<float>(aux)) : 0.0f;
        const V3 navg = aux > 0 ? normalize(mul(nsum, inv_aux)) : V3{0, 0, 1};
        const V3 aavg = aux > 0 ? mul(asum, inv_aux) : V3{0, 0, 0};
        const float davg = aux > 0 ? dsum * inv_aux : 0.0f;
        // store_output, programs.cu:1773-1805
        FrameBuffers& f = *p.frame;
        const size_t i4 = static_cast<size_t>(pixel) * 4;
        f.beauty[i4 + 0] = bavg.x; f.beauty[i4 + 1] = bavg.y; f.beauty[i4 + 2] = bavg.z; f.beauty[i4 + 3] = 1.0f;
        const V3 enc = clamp3(add(mul(navg, 0.5f), V3{0.5f, 0.5f, 0.5f}), 0.0f, 1.0f);
        f.normal[i4 + 0] = enc.x; f.normal[i4 + 1] = enc.y; f.normal[i4 + 2] = enc.z; f.normal[i4 + 3] = 1.0f;
        const V3 cn = normalize(V3{dot(navg, basis_f(p.cam->basis_x)), dot(navg, basis_f(p.cam->basis_y)), dot(navg, basis_f(p.cam->basis_z))});
        f.dnormal[i4 + 0] = cn.x; f.dnormal[i4 + 1] = cn.y; f.dnormal[i4 + 2] = cn.z; f.dnormal[i4 + 3] = 1.0f;
        const V3 ca = clamp3(aavg, 0.0f, 1.0f);
        f.albedo[i4 + 0] = ca.x; f.albedo[i4 + 1] = ca.y; f.albedo[i4 + 2] = ca.z; f.albedo[i4 + 3] = 1.0f;
        f.depth[static_cast<size_t>(pixel)] = davg;
        return rays;
    }

    // resolve_reprojection_kernel, programs.cu:1955-2067
    static void resolve_pixel(const Params& p, int x, int y) {
        const int pi = y * p.width + x;
        FrameBuffers& f = *p.frame;
        f.flow[2 * static_cast<size_t>(pi)] = 0.0f;
        f.flow[2 * static_cast<size_t>(pi) + 1] = 0.0f;
        f.trust[static_cast<size_t>(pi)] = 0.0f;
        if (p.history_length <= 0) return;
        const FrameBuffers& h = *p.history;
        const size_t i4 = static_cast<size_t>(pi) * 4;
        const float cb[4] = {f.beauty[i4], f.beauty[i4 + 1], f.beauty[i4 + 2], f.beauty[i4 + 3]};
        const float cn[4] = {f.normal[i4], f.normal[i4 + 1], f.normal[i4 + 2], f.normal[i4 + 3]};
        const float cd = f.depth[static_cast<size_t>(pi)];
        const float pxf = static_cast<float>(x) + 0.5f;
        const float pyf = static_cast<float>(y) + 0.5f;
        const V3 dc = unproject(*p.cam, pxf, pyf);
        const V3 dw = to_world(*p.cam, dc);
        const V3 wp = add(cam_origin(*p.cam), mul(dw, cd));
        const Camera& prev_src = p.prev_valid != 0 ? *p.prev : *p.cam;
        // prev_origin/prev_basis come from the captured history (the previous camera).
        const V3 off{static_cast<float>(wp.x - p.prev->origin[0]), static_cast<float>(wp.y - p.prev->origin[1]),
            static_cast<float>(wp.z - p.prev->origin[2])};
        const V3 pcs{dot(off, basis_f(p.prev->basis_x)), dot(off, basis_f(p.prev->basis_y)), dot(off, basis_f(p.prev->basis_z))};
        const V3 pp = project(prev_src, pcs);
        const bool finite = std::isfinite(pp.x) && std::isfinite(pp.y);
        if (finite) {
            f.flow[2 * static_cast<size_t>(pi)] = pxf - pp.x;
            f.flow[2 * static_cast<size_t>(pi) + 1] = pyf - pp.y;
        }
        const int px = finite ? static_cast<int>(std::floor(pp.x)) : -1;
        const int py = finite ? static_cast<int>(std::floor(pp.y)) : -1;
        bool valid = false;
        if (finite && px >= 0 && px < p.width && py >= 0 && py < p.height) {
            const size_t pj = static_cast<size_t>(py * p.width + px);
            const V3 hn{h.normal[pj * 4] * 2.0f - 1.0f, h.normal[pj * 4 + 1] * 2.0f - 1.0f, h.normal[pj * 4 + 2] * 2.0f - 1.0f};
            const V3 cur{cn[0] * 2.0f - 1.0f, cn[1] * 2.0f - 1.0f, cn[2] * 2.0f - 1.0f};
            const float nd = dot(cur, hn);
            const float hd = h.depth[pj];
            const float ed = len(pcs);
            const float tol = std::fmax(0.02f, 0.05f * std::fmax(ed, hd));
            if (nd > 0.95f && std::fabs(ed - hd) < tol) valid = true;
        }
        if (!valid) return;
        f.trust[static_cast<size_t>(pi)] = 1.0f;
        const size_t pj = static_cast<size_t>(py * p.width + px);
        const float hb[4] = {h.beauty[pj * 4], h.beauty[pj * 4 + 1], h.beauty[pj * 4 + 2], h.beauty[pj * 4 + 3]};
        const float hn[4] = {h.normal[pj * 4], h.normal[pj * 4 + 1], h.normal[pj * 4 + 2], h.normal[pj * 4 + 3]};
        const float hd = h.depth[pj];
        const int next_len = p.history_length + 1;
        const float blend = 1.0f / static_cast<float>(next_len);
        const float cc[3] = {std::fmin(std::fmax(cb[0], 0.0f), 10.0f), std::fmin(std::fmax(cb[1], 0.0f), 10.0f),
            std::fmin(std::fmax(cb[2], 0.0f), 10.0f)};
        if (p.restir_enabled == 0) {
            for (int c = 0; c < 3; ++c) f.beauty[i4 + static_cast<size_t>(c)] = hb[c] + (cc[c] - hb[c]) * blend;
            f.beauty[i4 + 3] = 1.0f;
        }
        for (int c = 0; c < 4; ++c) f.normal[i4 + static_cast<size_t>(c)] = hn[c] + (cn[c] - hn[c]) * blend;
        f.depth[static_cast<size_t>(pi)] = hd + (cd - hd) * blend;
    }

    Scene scene_;
    Tracer tracer_;
    std::vector<CameraState> cams_;
    uint32_t stream_ = 0;
    int threads_ = 1;
    bool record_ = false;
};

}  // namespace
}  // namespace orc

// ---- C interface for tests and bench -----------------------------------------

extern "C" {

struct orc_renderer {
    orc::Renderer* r;
};

orc_renderer* orc_create(const rtgb_scene* scene, int use_reference_bvh, int threads) {
    if (scene == nullptr) return nullptr;
    return new orc_renderer{new orc::Renderer(*scene, use_reference_bvh != 0, threads)};
}

void orc_destroy(orc_renderer* h) {
    if (h) {
        delete h->r;
        delete h;
    }
}

void orc_reset_sequence(orc_renderer* h, uint32_t s) { h->r->reset_sequence(s); }
void orc_reset_accumulation(orc_renderer* h) { h->r->reset_accumulation(); }
void orc_set_path_records(orc_renderer* h, int on) { h->r->set_record(on != 0); }
uint32_t orc_sample_stream(orc_renderer* h) { return h->r->stream(); }

// The emissive light table of build_light_distribution: up to `capacity`
// 16-byte PackedLight records into `lights` (may be null); returns the count.
int orc_light_table(orc_renderer* h, void* lights, int capacity) {
    const std::vector<orc::PackedLight>& L = h->r->scene().lights;
    const int n = static_cast<int>(L.size());
    if (lights != nullptr && capacity > 0) {
        std::memcpy(lights, L.data(), sizeof(orc::PackedLight) * static_cast<size_t>(std::min(n, capacity)));
    }
    return n;
}

int orc_render_frame(orc_renderer* h, const rtgb_camera_rig* rig, const rtgb_render_profile* profile,
    int active, int row_begin, int row_end, int row_stride) {
    if (!h || !rig || !profile) return RTGB_INVALID_ARGUMENT;
    return h->r->render_frame(*rig, *profile, active, row_begin, row_end, row_stride);
}

// which: 0 beauty, 1 normal, 2 denoiser_normal, 3 albedo, 4 depth, 5 flow, 6 trust, 7 reservoirs
int orc_get_buffer(orc_renderer* h, int cam, int which, void* dst, size_t bytes) {
    orc::CameraState* c = h->r->camera(cam);
    if (!c) return RTGB_INVALID_ARGUMENT;
    const void* src = nullptr;
    size_t n = 0;
    switch (which) {
        case 0: src = c->frame.beauty.data(); n = c->frame.beauty.size() * 4; break;
        case 1: src = c->frame.normal.data(); n = c->frame.normal.size() * 4; break;
        case 2: src = c->frame.dnormal.data(); n = c->frame.dnormal.size() * 4; break;
        case 3: src = c->frame.albedo.data(); n = c->frame.albedo.size() * 4; break;
        case 4: src = c->frame.depth.data(); n = c->frame.depth.size() * 4; break;
        case 5: src = c->frame.flow.data(); n = c->frame.flow.size() * 4; break;
        case 6: src = c->frame.trust.data(); n = c->frame.trust.size() * 4; break;
        case 7: src = c->frame.reservoirs.data(); n = c->frame.reservoirs.size() * sizeof(orc::Reservoir); break;
        default: return RTGB_INVALID_ARGUMENT;
    }
    if (bytes != n) return RTGB_INVALID_ARGUMENT;
    std::memcpy(dst, src, n);
    return RTGB_OK;
}

int orc_get_path_records(orc_renderer* h, int cam, int32_t* codes, int max_bounces, float* radiance, int64_t paths) {
    orc::CameraState* c = h->r->camera(cam);
    if (!c || c->codes.empty() || max_bounces != c->record_bounces) return RTGB_INVALID_ARGUMENT;
    if (static_cast<size_t>(paths) * static_cast<size_t>(max_bounces) != c->codes.size()) return RTGB_INVALID_ARGUMENT;
    std::memcpy(codes, c->codes.data(), c->codes.size() * sizeof(int32_t));
    std::memcpy(radiance, c->path_radiance.data(), c->path_radiance.size() * sizeof(float));
    return RTGB_OK;
}

uint64_t orc_last_rays(orc_renderer* h, int cam) {
    orc::CameraState* c = h->r->camera(cam);
    return c ? c->rays : 0;
}

// direction_debug_kernel, programs.cu:1807-1826
int orc_direction_debug(const rtgb_camera* cam, uint8_t* rgba) {
    const orc::Camera c = orc::make_camera(*cam);
    for (int y = 0; y < c.height; ++y) {
        for (int x = 0; x < c.width; ++x) {
            const float px = static_cast<float>(x) + 0.5f, py = static_cast<float>(y) + 0.5f;
            const orc::V3 d = orc::to_world(c, orc::unproject(c, px, py));
            const size_t i = 4 * (static_cast<size_t>(y) * static_cast<size_t>(c.width) + static_cast<size_t>(x));
            auto enc = [](float v) { return static_cast<uint8_t>(255.0f * orc::clamp01(0.5f * (v + 1.0f))); };
            rgba[i] = enc(d.x);
            rgba[i + 1] = enc(d.y);
            rgba[i + 2] = enc(d.z);
            rgba[i + 3] = 255;
        }
    }
    return RTGB_OK;
}

// Camera-space direction of a pixel (unproject), and projection, for KATs.
float orc_noise_sinf(float x) { return rtgb_noise::noise_sinf(x); }

void orc_unproject(const rtgb_camera* cam, double px, double py, float out[3]) {
    const orc::Camera c = orc::make_camera(*cam);
    const orc::V3 d = orc::unproject(c, px, py);
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

void orc_project(const rtgb_camera* cam, const float dir[3], float out[2]) {
    const orc::Camera c = orc::make_camera(*cam);
    const orc::V3 p = orc::project(c, orc::V3{dir[0], dir[1], dir[2]});
    out[0] = p.x; out[1] = p.y;
}

// Reservoir KAT entry points (restir_di.h:67-199) on the 84-byte layout.
int orc_reservoir_update(void* r, int light, float u0, float u1, float target, float weight, int mult, float u) {
    orc::Candidate c{light, u0, u1};
    return orc::reservoir_update(*static_cast<orc::Reservoir*>(r), c, target, weight, mult, u) ? 1 : 0;
}
void orc_reservoir_finalize(void* r) { orc::reservoir_finalize(*static_cast<orc::Reservoir*>(r)); }
void orc_reservoir_finalize_basic(void* r, float sel, float sum, int n) {
    orc::reservoir_finalize_basic(*static_cast<orc::Reservoir*>(r), sel, sum, n);
}
void orc_reservoir_merge(void* cur, const void* prev, float target, int max_c, float u, int temporal, int out[2]) {
    const orc::MergeResult m = orc::reservoir_merge(*static_cast<orc::Reservoir*>(cur),
        *static_cast<const orc::Reservoir*>(prev), target, max_c, u, temporal != 0);
    out[0] = m.multiplicity;
    out[1] = m.selected;
}
int orc_surface_valid(const void* cur_surface, const void* prev, float max_dist, float min_dot, int max_age) {
    return orc::surface_valid(*static_cast<const orc::Surface*>(cur_surface), *static_cast<const orc::Reservoir*>(prev),
               max_dist, min_dot, max_age) ? 1 : 0;
}

// Light-sampling KATs (light_sampling.h:64-124).
float orc_uniform_cone_pdf(float c) { return orc::uniform_cone_pdf(c); }
float orc_area_pdf(float a, float d2, float c) { return orc::area_to_solid_angle_pdf(a, d2, c); }
float orc_power_heuristic(float a, float b) { return orc::power_heuristic(a, b); }
int orc_sample_cdf(const float* cdf, int n, float u) {
    return orc::sample_cdf(n, u, [&](int i) { return cdf[i]; });
}
uint32_t orc_rng_for(int pixel, int sample, uint32_t stream) { return orc::rng_for(pixel, sample, stream); }
float orc_rnd(uint32_t* s) { return orc::rnd(*s); }

}  // extern "C"
