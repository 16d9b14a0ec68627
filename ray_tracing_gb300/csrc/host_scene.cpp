// Host-side authoring helpers of the C ABI: builtin and procedural scenes,
// camera packing, equi62 LUT construction and render-profile presets.
//
// Scene contents restate the reference's builders
// (src/scene/shared_scene_builders.cpp, utils/render_restir_acceptance.cpp)
// after the realtime adapter (src/scene/realtime_scene_adapter.cpp:371-486):
// textures first, then materials, then one primitive per instance, boxes
// expanded into six quads in the adapter's face order (:76-110).
#include "rtgb.h"

#include <algorithm>
#include <array>
#include <bit>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numbers>
#include <string>
#include <vector>

#include "host_scene.h"

namespace rtgb {
namespace {

using Vec3 = std::array<double, 3>;

Vec3 legacy_to_world(const Vec3& v) { return {v[0], -v[2], v[1]}; }  // frame_convention.h:33-35

void set3(float* dst, const Vec3& v) {
    dst[0] = static_cast<float>(v[0]);
    dst[1] = static_cast<float>(v[1]);
    dst[2] = static_cast<float>(v[2]);
}

// SplitMix64: the seeded stream of every procedural scene here.
struct SplitMix {
    uint64_t state;
    explicit SplitMix(uint64_t seed) : state(seed) {}
    uint64_t next() {
        uint64_t z = (state += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
};

class Builder {
public:
    explicit Builder(rtgb_host_scene& s) : s_(s) {}

    int constant_texture(const Vec3& c) {
        rtgb_texture t {};
        t.type = RTGB_TEXTURE_CONSTANT;
        t.even_texture = -1;
        t.odd_texture = -1;
        t.u_address_mode = 1;
        t.v_address_mode = 1;
        t.filter_type = 1;
        t.scale = 1.0f;
        set3(t.color, c);
        s_.textures.push_back(t);
        return static_cast<int>(s_.textures.size()) - 1;
    }
    int checker_texture(double scale, int even, int odd) {
        rtgb_texture t {};
        t.type = RTGB_TEXTURE_CHECKER;
        t.even_texture = even;
        t.odd_texture = odd;
        t.u_address_mode = 1;
        t.v_address_mode = 1;
        t.filter_type = 1;
        t.scale = static_cast<float>(scale);
        s_.textures.push_back(t);
        return static_cast<int>(s_.textures.size()) - 1;
    }
    int noise_texture(double scale) {
        rtgb_texture t {};
        t.type = RTGB_TEXTURE_NOISE;
        t.even_texture = -1;
        t.odd_texture = -1;
        t.u_address_mode = 1;
        t.v_address_mode = 1;
        t.filter_type = 1;
        t.scale = static_cast<float>(scale);
        s_.textures.push_back(t);
        return static_cast<int>(s_.textures.size()) - 1;
    }
    int material(int type, int albedo_tex, int emission_tex, double ior, double fuzz) {
        rtgb_material m {};
        m.type = type;
        m.albedo_texture = albedo_tex;
        m.emission_texture = emission_tex;
        m.ior = static_cast<float>(ior);
        m.fuzz = static_cast<float>(fuzz);
        m.openpbr_index = -1;
        s_.materials.push_back(m);
        return static_cast<int>(s_.materials.size()) - 1;
    }
    // Image texture over texels appended to the scene's texel array (RGB rows).
    int image_texture(int width, int height, const std::vector<float>& rgb) {
        rtgb_texture t {};
        t.type = RTGB_TEXTURE_IMAGE;
        t.even_texture = -1;
        t.odd_texture = -1;
        t.image_offset = static_cast<int32_t>(s_.texels.size() / 3);
        t.image_width = width;
        t.image_height = height;
        t.u_address_mode = 2;
        t.v_address_mode = 2;
        t.filter_type = 1;
        t.scale = 1.0f;
        s_.texels.insert(s_.texels.end(), rgb.begin(), rgb.end());
        s_.textures.push_back(t);
        return static_cast<int>(s_.textures.size()) - 1;
    }
    // An OpenPBR material (OpenPbrMaterialDesc) and its compiled parameter block.
    int openpbr(const rtgb_openpbr_material& om) {
        s_.openpbr.push_back(om);
        const int m = material(RTGB_MATERIAL_OPENPBR, -1, -1, 1.0, 0.0);
        s_.materials[static_cast<size_t>(m)].openpbr_index = static_cast<int32_t>(s_.openpbr.size()) - 1;
        return m;
    }
    // add_diffuse_color / add_emissive_color (shared_scene_builders.cpp:41-53)
    int diffuse(const Vec3& c) { return material(RTGB_MATERIAL_LAMBERTIAN, constant_texture(c), -1, 1.0, 0.0); }
    int emissive(const Vec3& c) { return material(RTGB_MATERIAL_DIFFUSE_LIGHT, -1, constant_texture(c), 1.0, 0.0); }
    int metal(const Vec3& c, double fuzz) { return material(RTGB_MATERIAL_METAL, constant_texture(c), -1, 1.0, fuzz); }
    int dielectric(double ior) { return material(RTGB_MATERIAL_DIELECTRIC, -1, -1, ior, 0.0); }

    void sphere(int m, const Vec3& c, double r) {
        rtgb_sphere sp {};
        set3(sp.center, c);
        sp.radius = static_cast<float>(r);
        sp.material_index = m;
        s_.spheres.push_back(sp);
    }
    void quad(int m, const Vec3& o, const Vec3& u, const Vec3& v) {
        rtgb_quad q {};
        set3(q.origin, o);
        set3(q.edge_u, u);
        set3(q.edge_v, v);
        q.material_index = m;
        s_.quads.push_back(q);
    }
    void triangle(int m, const Vec3& a, const Vec3& b, const Vec3& c) {
        rtgb_triangle t {};
        set3(t.p0, a);
        set3(t.p1, b);
        set3(t.p2, c);
        t.material_index = m;
        s_.triangles.push_back(t);
    }
    // add_box_instance (shared_scene_builders.cpp:82-92) + add_box_quads
    // (realtime_scene_adapter.cpp:76-110): yaw about +Y, then translate.
    void box(int m, const Vec3& mn, const Vec3& mx, const Vec3& translation, double yaw_deg) {
        const double a = yaw_deg * std::numbers::pi / 180.0;
        const double c = std::cos(a), s = std::sin(a);
        auto rot = [&](const Vec3& p) { return Vec3 {c * p[0] + s * p[2], p[1], -s * p[0] + c * p[2]}; };
        auto point = [&](const Vec3& p) {
            const Vec3 r = rot(p);
            return Vec3 {r[0] + translation[0], r[1] + translation[1], r[2] + translation[2]};
        };
        auto diff = [](const Vec3& p, const Vec3& q) { return Vec3 {p[0] - q[0], p[1] - q[1], p[2] - q[2]}; };
        const Vec3 p000 {mn[0], mn[1], mn[2]}, p001 {mn[0], mn[1], mx[2]}, p010 {mn[0], mx[1], mn[2]},
            p011 {mn[0], mx[1], mx[2]}, p100 {mx[0], mn[1], mn[2]}, p101 {mx[0], mn[1], mx[2]},
            p110 {mx[0], mx[1], mn[2]}, p111 {mx[0], mx[1], mx[2]};
        auto face = [&](const Vec3& o, const Vec3& u, const Vec3& v) { quad(m, point(o), rot(u), rot(v)); };
        face(p001, diff(p101, p001), diff(p011, p001));
        face(p100, diff(p000, p100), diff(p110, p100));
        face(p000, diff(p001, p000), diff(p010, p000));
        face(p101, diff(p100, p101), diff(p111, p101));
        face(p010, diff(p110, p010), diff(p011, p010));
        face(p000, diff(p100, p000), diff(p001, p000));
    }
    rtgb_analytic_light& analytic(int type) {
        rtgb_analytic_light l {};
        l.type = type;
        l.radius = 0.5f;
        l.width = 1.0f;
        l.height = 1.0f;
        l.length = 1.0f;
        l.cos_theta_max = 1.0f;
        s_.analytic.push_back(l);
        return s_.analytic.back();
    }
    void background(const Vec3& b) { set3(s_.background.data(), b); }

private:
    rtgb_host_scene& s_;
};

// finalize_analytic_light_distribution (src/scene/analytic_light_compiler.cpp:15-39),
// computed in double from per-light selection weights.
void finalize_analytic_distribution(rtgb_host_scene& s, const std::vector<double>& weights) {
    double total = 0.0;
    std::vector<double> w(weights.size());
    for (size_t i = 0; i < weights.size(); ++i) {
        w[i] = std::isfinite(weights[i]) ? std::max(0.0, weights[i]) : 0.0;
        total += w[i];
    }
    double cdf = 0.0;
    for (size_t i = 0; i < w.size(); ++i) {
        const double pdf = total > 0.0 ? w[i] / total : 0.0;
        cdf += pdf;
        s.analytic[i].selection_pdf = static_cast<float>(pdf);
        s.analytic[i].cdf = static_cast<float>(cdf);
    }
    if (total > 0.0) {
        size_t last = w.size();
        for (size_t i = w.size(); i-- > 0;) {
            if (s.analytic[i].selection_pdf > 0.0f) {
                last = i;
                break;
            }
        }
        for (size_t i = last; i < w.size(); ++i) s.analytic[i].cdf = 1.0f;
    }
}

void build_cornell(rtgb_host_scene& s) {
    Builder b(s);
    const int red = b.diffuse({0.65, 0.05, 0.05});
    const int white = b.diffuse({0.73, 0.73, 0.73});
    const int green = b.diffuse({0.12, 0.45, 0.15});
    const int light = b.emissive({15.0, 15.0, 15.0});
    b.quad(green, {555, 0, 0}, {0, 555, 0}, {0, 0, 555});
    b.quad(red, {0, 0, 0}, {0, 555, 0}, {0, 0, 555});
    b.quad(light, {343, 554, 332}, {-130, 0, 0}, {0, 0, -105});
    b.quad(white, {0, 0, 0}, {555, 0, 0}, {0, 0, 555});
    b.quad(white, {555, 555, 555}, {-555, 0, 0}, {0, 0, -555});
    b.quad(white, {0, 0, 555}, {555, 0, 0}, {0, 555, 0});
    b.box(white, {0, 0, 0}, {165, 330, 165}, {265, 0, 295}, 15.0);
    b.box(white, {0, 0, 0}, {165, 165, 165}, {130, 0, 65}, -18.0);
}

void build_smoke(rtgb_host_scene& s) {
    Builder b(s);
    const int diffuse = b.diffuse({0.75, 0.25, 0.2});
    const int light = b.emissive({10.0, 10.0, 10.0});
    b.sphere(diffuse, legacy_to_world({0.0, 0.0, -1.0}), 0.5);
    b.quad(light, legacy_to_world({-0.75, 1.25, -1.5}), legacy_to_world({1.5, 0.0, 0.0}),
        legacy_to_world({0.0, 0.0, 1.5}));
}

void build_final_room(rtgb_host_scene& s) {
    Builder b(s);
    const int white = b.diffuse({0.73, 0.73, 0.73});
    const int green = b.diffuse({0.30, 0.70, 0.35});
    const int red = b.diffuse({0.72, 0.25, 0.22});
    const int blue = b.diffuse({0.25, 0.35, 0.75});
    const int light = b.emissive({10.0, 10.0, 10.0});
    auto q = [&](int m, Vec3 o, Vec3 u, Vec3 v) { b.quad(m, legacy_to_world(o), legacy_to_world(u), legacy_to_world(v)); };
    q(white, {-4.0, -1.0, -4.0}, {0.0, 0.0, 8.0}, {8.0, 0.0, 0.0});
    q(white, {-4.0, 3.5, -4.0}, {8.0, 0.0, 0.0}, {0.0, 0.0, 8.0});
    q(green, {-4.0, -1.0, -4.0}, {0.0, 4.5, 0.0}, {0.0, 0.0, 8.0});
    q(red, {4.0, -1.0, -4.0}, {0.0, 0.0, 8.0}, {0.0, 4.5, 0.0});
    q(white, {-4.0, -1.0, -4.0}, {8.0, 0.0, 0.0}, {0.0, 4.5, 0.0});
    q(blue, {-4.0, -1.0, 4.0}, {0.0, 4.5, 0.0}, {8.0, 0.0, 0.0});
    q(light, {-1.0, 3.15, -1.0}, {2.0, 0.0, 0.0}, {0.0, 0.0, 2.0});
    q(white, {-3.2, -0.25, -3.0}, {0.0, 0.0, 1.8}, {1.8, 0.0, 0.0});
    q(white, {1.2, 0.15, 1.0}, {0.0, 0.0, 1.6}, {1.6, 0.0, 0.0});
    const double spheres[8][4] = {{0.0, 0.25, -1.2, 0.55}, {-1.6, 0.35, 1.7, 0.55}, {-3.1, 1.0, 0.8, 0.55},
        {3.0, 1.35, -0.9, 0.65}, {1.1, 1.1, -3.0, 0.60}, {-0.8, 2.55, 2.2, 0.45}, {0.9, 0.55, -0.1, 0.45},
        {-0.35, 0.4, -1.15, 0.35}};
    for (const auto& sp : spheres) b.sphere(white, legacy_to_world({sp[0], sp[1], sp[2]}), sp[3]);
}

void build_bouncing_spheres(rtgb_host_scene& s) {
    Builder b(s);
    const int ground = b.diffuse({0.5, 0.5, 0.5});
    const int diffuse = b.diffuse({0.4, 0.2, 0.1});
    const int metal_tex = b.constant_texture({0.7, 0.6, 0.5});
    const int metal = b.material(RTGB_MATERIAL_METAL, metal_tex, -1, 1.0, 0.0);
    const int glass = b.dielectric(1.5);
    const int blue_tex = b.constant_texture({0.2, 0.3, 0.8});
    const int blue_metal = b.material(RTGB_MATERIAL_METAL, blue_tex, -1, 1.0, 0.25);
    b.sphere(ground, {0.0, -1000.0, 0.0}, 1000.0);
    b.sphere(glass, {0.0, 1.0, 0.0}, 1.0);
    b.sphere(diffuse, {-4.0, 1.0, 0.0}, 1.0);
    b.sphere(metal, {4.0, 1.0, 0.0}, 1.0);
    for (int x = -2; x <= 2; ++x) {
        for (int z = -2; z <= 2; ++z) {
            const int m = ((x + z) % 3 == 0) ? glass : (((x + z) % 2 == 0) ? diffuse : blue_metal);
            b.sphere(m, {x * 1.2, 0.2, z * 1.2}, 0.2);
        }
    }
    b.background({0.70, 0.80, 1.00});
}

// utils/render_restir_acceptance.cpp:41-93. SceneDescription::add_material
// (src/realtime/scene_description.cpp:25-44) turns the receiver's albedo
// colour into a constant texture appended to the texture table.
void build_restir_acceptance(rtgb_host_scene& s) {
    Builder b(s);
    const int receiver = b.diffuse({0.65, 0.58, 0.5});
    b.quad(receiver, legacy_to_world({-2.5, -2.5, -4.0}), legacy_to_world({5.0, 0.0, 0.0}), legacy_to_world({0.0, 5.0, 0.0}));
    for (int i = 0; i < 128; ++i) {
        const double x = 20.0 + static_cast<double>(i % 16);
        const double y = -8.0 + static_cast<double>(i / 16);
        const double z = -2.0 - 0.1 * static_cast<double>(i % 7);
        b.sphere(receiver, legacy_to_world({x, y, z}), 0.2);
    }
    std::vector<double> weights;
    for (int i = 0; i < 64; ++i) {
        const int column = i % 8, row = i / 8;
        const double x = -2.1 + 0.6 * column;
        const double y = -2.1 + 0.6 * row;
        const double z = -1.5 - 0.15 * static_cast<double>((i * 7) % 5);
        const double strength = 0.35 + 0.08 * static_cast<double>((i * 13) % 17);
        rtgb_analytic_light& l = b.analytic(RTGB_ANALYTIC_SPHERE);
        set3(l.position, legacy_to_world({x, y, z}));
        set3(l.basis_x, legacy_to_world({1, 0, 0}));
        set3(l.basis_y, legacy_to_world({0, 1, 0}));
        set3(l.basis_z, legacy_to_world({0, 0, 1}));
        set3(l.radiance, {strength, strength, strength});
        l.radius = 0.02f;
        l.world_area = 1.0f;
        l.treat_as_point = 1;
        l.delta = 1;
        weights.push_back(strength);
    }
    finalize_analytic_distribution(s, weights);
}

// Seeded random-sphere field: ground sphere r=1000, a 22x22 grid of r=0.2
// spheres jittered by U(0,0.9) (80% Lambertian albedo U^2, 15% metal
// albedo U(0.5,1) fuzz U(0,0.5), 5% dielectric 1.5) and `light_count`
// emissive rect lights (area U(0.01,0.1), radiance U(1,20)) facing down,
// expressed as analytic rect lights so ReSTIR DI samples them.
void build_random_spheres(rtgb_host_scene& s, uint32_t seed, int64_t detail) {
    Builder b(s);
    SplitMix rng(0x5eed0000ull ^ seed);
    const int ground = b.diffuse({0.5, 0.5, 0.5});
    b.sphere(ground, {0.0, -1000.0, 0.0}, 1000.0);
    for (int a = -11; a < 11; ++a) {
        for (int c = -11; c < 11; ++c) {
            const double choose = rng.uniform();
            const Vec3 center {a + 0.9 * rng.uniform(), 0.2, c + 0.9 * rng.uniform()};
            int m;
            if (choose < 0.8) {
                const double r = rng.uniform() * rng.uniform();
                const double g = rng.uniform() * rng.uniform();
                const double bl = rng.uniform() * rng.uniform();
                m = b.diffuse({r, g, bl});
            } else if (choose < 0.95) {
                const Vec3 alb {rng.uniform(0.5, 1.0), rng.uniform(0.5, 1.0), rng.uniform(0.5, 1.0)};
                m = b.metal(alb, rng.uniform(0.0, 0.5));
            } else {
                m = b.dielectric(1.5);
            }
            b.sphere(m, center, 0.2);
        }
    }
    const int light_count = detail > 0 ? static_cast<int>(detail) : 1024;
    std::vector<double> weights;
    for (int i = 0; i < light_count; ++i) {
        const double area = rng.uniform(0.01, 0.1);
        const double aspect = rng.uniform(0.5, 2.0);
        const double width = std::sqrt(area * aspect);
        const double height = area / width;
        const double radiance = rng.uniform(1.0, 20.0);
        const Vec3 pos {rng.uniform(-11.0, 11.0), rng.uniform(1.2, 3.0), rng.uniform(-11.0, 11.0)};
        rtgb_analytic_light& l = b.analytic(RTGB_ANALYTIC_RECT);
        set3(l.position, pos);
        // basis_x x basis_y = +Y, so the emitting side (-(bx x by)) faces down.
        set3(l.basis_x, {1.0, 0.0, 0.0});
        set3(l.basis_y, {0.0, 0.0, -1.0});
        set3(l.basis_z, {0.0, -1.0, 0.0});
        set3(l.radiance, {radiance, radiance, radiance});
        l.width = static_cast<float>(width);
        l.height = static_cast<float>(height);
        l.world_area = static_cast<float>(width * height);
        weights.push_back(radiance * width * height);
    }
    finalize_analytic_distribution(s, weights);
    b.background({0.02, 0.025, 0.04});
}

// OpenPbrCoreMaterial defaults (src/common/openpbr_core.h:33-77), all
// textures unbound, color bindings in linear sRGB.
rtgb_openpbr_material openpbr_defaults() {
    rtgb_openpbr_material m {};
    auto c3 = [](float* d, float x, float y, float z) {
        d[0] = x;
        d[1] = y;
        d[2] = z;
    };
    m.base_weight = 1.0f;
    c3(m.base_color, 0.8f, 0.8f, 0.8f);
    m.specular_weight = 1.0f;
    c3(m.specular_color, 1.0f, 1.0f, 1.0f);
    m.specular_roughness = 0.3f;
    m.specular_ior = 1.5f;
    c3(m.transmission_color, 1.0f, 1.0f, 1.0f);
    m.transmission_dispersion_abbe_number = 20.0f;
    c3(m.subsurface_color, 0.8f, 0.8f, 0.8f);
    m.subsurface_radius = 1.0f;
    c3(m.subsurface_radius_scale, 1.0f, 0.5f, 0.25f);
    c3(m.fuzz_color, 1.0f, 1.0f, 1.0f);
    m.fuzz_roughness = 0.5f;
    c3(m.coat_color, 1.0f, 1.0f, 1.0f);
    m.coat_ior = 1.6f;
    m.coat_darkening = 1.0f;
    m.thin_film_thickness = 0.5f;
    m.thin_film_ior = 1.4f;
    c3(m.emission_color, 1.0f, 1.0f, 1.0f);
    m.geometry_opacity = 1.0f;
    for (int k = 0; k < 4; ++k) {
        m.color_texture[k] = -1;
        m.color_space[k] = 1;
    }
    m.scalar_texture[0] = -1;
    m.scalar_texture[1] = -1;
    return m;
}

// OpenPBR material gallery: a row of spheres, one per feature of the OpenPBR
// BSDF (F82 metal, smooth and rough glass, thin-walled glass, dispersion, thin
// film, coat, fuzz, random-walk and thin-walled subsurface, cut-out opacity,
// texture-bound roughness/metalness/specular color), on an OpenPBR floor with
// an sRGB checker base color, lit by an OpenPBR emissive quad and sphere (the
// sphere's emission color texture-bound) and `detail` analytic sphere lights
// (default 24) for ReSTIR DI. Camera slot 0 of the default rig looks at it.
void build_openpbr_gallery(rtgb_host_scene& s, uint32_t seed, int64_t detail) {
    Builder b(s);
    SplitMix rng(0x09e7b7c0ull ^ seed);
    auto base = [](float r, float g, float bl) {
        rtgb_openpbr_material m = openpbr_defaults();
        m.base_color[0] = r;
        m.base_color[1] = g;
        m.base_color[2] = bl;
        return m;
    };
    // floor: OpenPBR dielectric with an sRGB-encoded checker base color
    {
        rtgb_openpbr_material m = base(0.5f, 0.5f, 0.5f);
        m.base_diffuse_roughness = 0.5f;
        m.specular_roughness = 0.45f;
        m.color_texture[0] = b.checker_texture(0.5, b.constant_texture({0.85, 0.82, 0.75}), b.constant_texture({0.25, 0.3, 0.35}));
        m.color_space[0] = 2;
        // 1 cm below the spheres: a solid checker flips sign on the plane y = 0,
        // where the cell of a hit would hang on the last bit of its position
        b.quad(b.openpbr(m), {-8.0, -0.01, -2.0}, {16.0, 0.0, 0.0}, {0.0, 0.0, 14.0});
    }
    b.quad(b.diffuse({0.6, 0.55, 0.5}), {-8.0, 0.0, 9.0}, {16.0, 0.0, 0.0}, {0.0, 5.0, 0.0});
    std::vector<rtgb_openpbr_material> row;
    {
        rtgb_openpbr_material m = base(1.0f, 0.78f, 0.34f);  // gold, F82 tint
        m.base_metalness = 1.0f;
        m.specular_roughness = 0.25f;
        m.specular_color[2] = 0.6f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(1.0f, 1.0f, 1.0f);  // smooth glass
        m.transmission_weight = 1.0f;
        m.specular_roughness = 0.0f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(1.0f, 1.0f, 1.0f);  // rough tinted glass
        m.transmission_weight = 1.0f;
        m.specular_roughness = 0.3f;
        m.transmission_color[0] = 0.6f;
        m.transmission_color[1] = 0.9f;
        m.transmission_color[2] = 0.8f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(1.0f, 1.0f, 1.0f);  // thin-walled glass
        m.transmission_weight = 1.0f;
        m.specular_roughness = 0.1f;
        m.geometry_thin_walled = 1;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(1.0f, 1.0f, 1.0f);  // dispersive glass
        m.transmission_weight = 1.0f;
        m.specular_roughness = 0.0f;
        m.specular_ior = 1.7f;
        m.transmission_dispersion_scale = 1.0f;
        m.transmission_dispersion_abbe_number = 18.0f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(0.05f, 0.05f, 0.08f);  // thin-film soap-bubble dielectric
        m.thin_film_weight = 1.0f;
        m.thin_film_thickness = 0.45f;
        m.thin_film_ior = 1.33f;
        m.specular_roughness = 0.15f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(0.7f, 0.1f, 0.08f);  // clear-coated car paint
        m.base_metalness = 0.6f;
        m.specular_roughness = 0.4f;
        m.coat_weight = 1.0f;
        m.coat_roughness = 0.05f;
        m.coat_color[2] = 0.85f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(0.2f, 0.05f, 0.3f);  // velvet
        m.fuzz_weight = 1.0f;
        m.fuzz_color[0] = 0.9f;
        m.fuzz_color[1] = 0.6f;
        m.fuzz_color[2] = 1.0f;
        m.fuzz_roughness = 0.5f;
        m.base_diffuse_roughness = 1.0f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(0.9f, 0.7f, 0.6f);  // skin-like random walk
        m.subsurface_weight = 1.0f;
        m.subsurface_color[0] = 0.9f;
        m.subsurface_color[1] = 0.6f;
        m.subsurface_color[2] = 0.5f;
        m.subsurface_radius = 0.25f;
        m.subsurface_scatter_anisotropy = 0.3f;
        m.specular_roughness = 0.35f;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(0.3f, 0.8f, 0.3f);  // leaf: thin-walled subsurface
        m.subsurface_weight = 0.8f;
        m.subsurface_color[0] = 0.4f;
        m.subsurface_color[1] = 0.9f;
        m.subsurface_color[2] = 0.3f;
        m.subsurface_scatter_anisotropy = 0.4f;
        m.geometry_thin_walled = 1;
        row.push_back(m);
    }
    {
        rtgb_openpbr_material m = base(0.2f, 0.4f, 0.9f);  // cut-out
        m.geometry_opacity = 0.45f;
        row.push_back(m);
    }
    {
        // roughness and metalness from a small image, specular color from a checker
        rtgb_openpbr_material m = base(0.8f, 0.8f, 0.85f);
        const int w = 8, h = 8;
        std::vector<float> rough(static_cast<size_t>(w * h * 3)), metal(static_cast<size_t>(w * h * 3));
        for (int y = 0; y < h; ++y) {
            for (int x = 0; x < w; ++x) {
                const float r = static_cast<float>(rng.uniform(0.05, 0.9));
                const float mt = ((x / 2 + y / 2) & 1) ? 1.0f : 0.0f;
                for (int k = 0; k < 3; ++k) {
                    rough[static_cast<size_t>((y * w + x) * 3 + k)] = r;
                    metal[static_cast<size_t>((y * w + x) * 3 + k)] = mt;
                }
            }
        }
        m.scalar_texture[1] = b.image_texture(w, h, rough);
        m.scalar_texture[0] = b.image_texture(w, h, metal);
        m.color_texture[1] = b.checker_texture(4.0, b.constant_texture({1.0, 0.8, 0.6}), b.constant_texture({0.6, 0.8, 1.0}));
        row.push_back(m);
    }
    const int n = static_cast<int>(row.size());
    for (int i = 0; i < n; ++i) {
        const int col = i % 6, line = i / 6;
        const double x = -2.75 + 1.1 * col;
        const double z = 4.0 + 1.4 * line;
        b.sphere(b.openpbr(row[static_cast<size_t>(i)]), {x, 0.45, z}, 0.45);
    }
    // emitters: an OpenPBR quad overhead (one-sided geometry, two-sided OpenPBR emission)
    // and a small OpenPBR sphere whose emission color is texture-bound
    {
        rtgb_openpbr_material m = base(0.0f, 0.0f, 0.0f);
        m.emission_luminance = 6.0f;
        m.emission_color[0] = 1.0f;
        m.emission_color[1] = 0.9f;
        m.emission_color[2] = 0.75f;
        b.quad(b.openpbr(m), {-1.5, 3.2, 3.5}, {3.0, 0.0, 0.0}, {0.0, 0.0, 2.5});
    }
    {
        rtgb_openpbr_material m = base(0.1f, 0.1f, 0.1f);
        m.emission_luminance = 4.0f;
        m.color_texture[3] = b.checker_texture(8.0, b.constant_texture({1.0, 0.3, 0.2}), b.constant_texture({0.2, 0.5, 1.0}));
        m.color_space[3] = 1;
        b.sphere(b.openpbr(m), {3.6, 1.4, 6.5}, 0.3);
    }
    const int lights = detail > 0 ? static_cast<int>(detail) : 24;
    std::vector<double> weights;
    for (int i = 0; i < lights; ++i) {
        const double strength = rng.uniform(2.0, 12.0);
        rtgb_analytic_light& l = b.analytic(RTGB_ANALYTIC_SPHERE);
        set3(l.position, {rng.uniform(-4.0, 4.0), rng.uniform(1.5, 3.5), rng.uniform(1.0, 8.0)});
        set3(l.basis_x, {1.0, 0.0, 0.0});
        set3(l.basis_y, {0.0, 1.0, 0.0});
        set3(l.basis_z, {0.0, 0.0, 1.0});
        set3(l.radiance, {strength, strength * rng.uniform(0.6, 1.0), strength * rng.uniform(0.5, 1.0)});
        l.radius = static_cast<float>(rng.uniform(0.05, 0.15));
        l.world_area = static_cast<float>(4.0 * std::numbers::pi * l.radius * l.radius);
        weights.push_back(strength * l.world_area);
    }
    finalize_analytic_distribution(s, weights);
    b.background({0.03, 0.035, 0.05});
}

// Unit icosphere subdivided twice: 162 vertices, 320 faces.
void icosphere2(std::vector<Vec3>& verts, std::vector<std::array<int, 3>>& faces) {
    verts.clear();
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    const double v[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
        {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (const auto& p : v) {
        const double l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        verts.push_back({p[0] / l, p[1] / l, p[2] / l});
    }
    faces = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4}, {11, 10, 2},
        {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8}, {3, 8, 9}, {4, 9, 5}, {2, 4, 11},
        {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    for (int level = 0; level < 2; ++level) {
        std::vector<std::array<int, 3>> next;
        auto mid = [&](int i, int j) {
            Vec3 m {(verts[i][0] + verts[j][0]) * 0.5, (verts[i][1] + verts[j][1]) * 0.5,
                (verts[i][2] + verts[j][2]) * 0.5};
            const double l = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            verts.push_back({m[0] / l, m[1] / l, m[2] / l});
            return static_cast<int>(verts.size()) - 1;
        };
        for (const auto& f : faces) {
            const int a = mid(f[0], f[1]), bb = mid(f[1], f[2]), c = mid(f[2], f[0]);
            next.push_back({f[0], a, c});
            next.push_back({f[1], bb, a});
            next.push_back({f[2], c, bb});
            next.push_back({a, bb, c});
        }
        faces = next;
    }
}

// Seeded procedural triangle scene: a displaced-grid terrain plus icosphere
// instances, constant per-object materials, and `emissive` emissive
// triangles (a fraction of the icosphere faces). The triangle budget is
// `detail` (default 1,000,000).
// The 1 M-triangle terrain with 200 icosphere instances and 256 emissive
// triangles; with `pbr` every non-emissive surface is an OpenPBR material
// with constant parameters (the instances: base colour U(0,1)^3, specular
// roughness U(0.05,1), metalness Bernoulli(0.3), specular IOR 1.5).
void build_triangle_terrain(rtgb_host_scene& s, uint32_t seed, int64_t detail, bool pbr = false) {
    Builder b(s);
    SplitMix rng(0x7e77a1000ull ^ seed);
    const int64_t budget = detail > 0 ? detail : 1000000;
    const int instances = 200;
    // icosphere subdivided twice: 320 faces
    std::vector<Vec3> verts;
    std::vector<std::array<int, 3>> faces;
    icosphere2(verts, faces);
    const int64_t sphere_tris = static_cast<int64_t>(instances) * static_cast<int64_t>(faces.size());
    const int64_t terrain_tris = std::max<int64_t>(2, budget - sphere_tris);
    const int n = std::max(1, static_cast<int>(std::sqrt(static_cast<double>(terrain_tris) / 2.0)));
    const double extent = 40.0;
    const double phase[4] = {rng.uniform(0, 6.283), rng.uniform(0, 6.283), rng.uniform(0, 6.283), rng.uniform(0, 6.283)};
    auto height = [&](double x, double z) {
        return 0.8 * std::sin(0.21 * x + phase[0]) * std::cos(0.17 * z + phase[1])
               + 0.35 * std::sin(0.57 * x + 0.31 * z + phase[2]) + 0.12 * std::cos(1.3 * z - 0.7 * x + phase[3]);
    };
    auto pbr_material = [&](const Vec3& color, double roughness, double metalness) {
        rtgb_openpbr_material om = openpbr_defaults();
        for (int k = 0; k < 3; ++k) om.base_color[k] = static_cast<float>(color[k]);
        om.specular_roughness = static_cast<float>(roughness);
        om.base_metalness = static_cast<float>(metalness);
        om.specular_ior = 1.5f;
        return b.openpbr(om);
    };
    const int terrain = pbr ? pbr_material({0.45, 0.42, 0.38}, 0.6, 0.0) : b.diffuse({0.45, 0.42, 0.38});
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < n; ++i) {
            const double x0 = -extent + 2.0 * extent * i / n, x1 = -extent + 2.0 * extent * (i + 1) / n;
            const double z0 = -extent + 2.0 * extent * j / n, z1 = -extent + 2.0 * extent * (j + 1) / n;
            const Vec3 a {x0, height(x0, z0), z0}, c {x1, height(x1, z0), z0}, d {x0, height(x0, z1), z1},
                e {x1, height(x1, z1), z1};
            b.triangle(terrain, a, d, c);
            b.triangle(terrain, c, d, e);
        }
    }
    const int emissive_target = 256;
    int emitted = 0;
    for (int k = 0; k < instances; ++k) {
        const double r = rng.uniform(0.3, 1.2);
        const double cx = rng.uniform(-extent * 0.8, extent * 0.8), cz = rng.uniform(-extent * 0.8, extent * 0.8);
        const Vec3 center {cx, height(cx, cz) + r * 1.05, cz};
        const Vec3 color {rng.uniform(), rng.uniform(), rng.uniform()};
        const int m = pbr ? pbr_material(color, rng.uniform(0.05, 1.0), rng.uniform() < 0.3 ? 1.0 : 0.0) : b.diffuse(color);
        const bool is_light_host = k % 25 == 0;
        const int light_m = is_light_host ? b.emissive({8.0, 7.0, 6.0}) : -1;
        for (size_t f = 0; f < faces.size(); ++f) {
            auto P = [&](int vi) {
                return Vec3 {center[0] + r * verts[vi][0], center[1] + r * verts[vi][1], center[2] + r * verts[vi][2]};
            };
            const bool emissive = is_light_host && emitted < emissive_target && f % 10 == 0;
            if (emissive) ++emitted;
            b.triangle(emissive ? light_m : m, P(faces[f][0]), P(faces[f][1]), P(faces[f][2]));
        }
    }
    b.background({0.05, 0.06, 0.09});
}

// The 4 M-triangle textured room: a 30 x 8 x 30 room whose floor, ceiling and
// four walls are fine triangle grids (the floor gently undulating), textured
// OpenPBR (a checker base colour on the floor, 3D noise on the walls), 600
// icosphere props with constant OpenPBR materials, and 16 ceiling panels of
// 256 emissive OpenPBR triangles each (4096). `detail` is the triangle budget
// (default 4,000,000).
void build_textured_room(rtgb_host_scene& s, uint32_t seed, int64_t detail) {
    Builder b(s);
    SplitMix rng(0x7e4700ull ^ seed);
    const int64_t budget = detail > 0 ? detail : 4000000;
    const double hx = 15.0, hz = 15.0, top = 8.0;
    auto pbr = [&](const Vec3& color, double roughness, double metalness) {
        rtgb_openpbr_material om = openpbr_defaults();
        for (int k = 0; k < 3; ++k) om.base_color[k] = static_cast<float>(color[k]);
        om.specular_roughness = static_cast<float>(roughness);
        om.base_metalness = static_cast<float>(metalness);
        return om;
    };
    rtgb_openpbr_material floor_m = pbr({0.6, 0.6, 0.6}, 0.5, 0.0);
    floor_m.color_texture[0] = b.checker_texture(1.5, b.constant_texture({0.75, 0.72, 0.66}), b.constant_texture({0.18, 0.2, 0.24}));
    rtgb_openpbr_material wall_m = pbr({0.7, 0.7, 0.7}, 0.8, 0.0);
    wall_m.color_texture[0] = b.noise_texture(1.3);
    const int floor = b.openpbr(floor_m), wall = b.openpbr(wall_m), ceiling = b.openpbr(pbr({0.85, 0.85, 0.82}, 0.9, 0.0));
    rtgb_openpbr_material lamp = pbr({0.0, 0.0, 0.0}, 0.5, 0.0);
    lamp.emission_luminance = 12.0f;
    lamp.emission_color[0] = 1.0f;
    lamp.emission_color[1] = 0.92f;
    lamp.emission_color[2] = 0.8f;
    const int light = b.openpbr(lamp);

    // a grid of cu x cv quads (two triangles each) spanning o + [0,1] u + [0,1] v
    auto grid_cells = [&](int m, const Vec3& o, const Vec3& u, const Vec3& v, int cu, int cv, auto&& lift) {
        auto P = [&](int i, int j) {
            const double a = static_cast<double>(i) / cu, c = static_cast<double>(j) / cv;
            Vec3 q {o[0] + a * u[0] + c * v[0], o[1] + a * u[1] + c * v[1], o[2] + a * u[2] + c * v[2]};
            q[1] += lift(q[0], q[2]);
            return q;
        };
        for (int j = 0; j < cv; ++j) {
            for (int i = 0; i < cu; ++i) {
                const Vec3 p00 = P(i, j), p10 = P(i + 1, j), p01 = P(i, j + 1), p11 = P(i + 1, j + 1);
                b.triangle(m, p00, p01, p10);
                b.triangle(m, p10, p01, p11);
            }
        }
    };
    // a square grid of about `tris` triangles
    auto grid = [&](int m, const Vec3& o, const Vec3& u, const Vec3& v, int64_t tris, auto&& lift) {
        const int cells = std::max(1, static_cast<int>(std::sqrt(static_cast<double>(tris) / 2.0)));
        grid_cells(m, o, u, v, cells, cells, lift);
    };
    const auto flat = [](double, double) { return 0.0; };
    const auto bumps = [](double x, double z) { return 0.03 * std::sin(1.7 * x) * std::cos(1.3 * z); };

    const int props = 600, panels = 16;
    const int64_t prop_tris = static_cast<int64_t>(props) * 320, lamp_tris = static_cast<int64_t>(panels) * 256;
    const int64_t rest = std::max<int64_t>(12, budget - prop_tris - lamp_tris);
    grid(floor, {-hx, 0.0, -hz}, {2 * hx, 0.0, 0.0}, {0.0, 0.0, 2 * hz}, rest * 4 / 10, bumps);
    grid(ceiling, {-hx, top, -hz}, {0.0, 0.0, 2 * hz}, {2 * hx, 0.0, 0.0}, rest * 2 / 10, flat);
    grid(wall, {-hx, 0.0, -hz}, {0.0, top, 0.0}, {2 * hx, 0.0, 0.0}, rest / 10, flat);
    grid(wall, {-hx, 0.0, hz}, {2 * hx, 0.0, 0.0}, {0.0, top, 0.0}, rest / 10, flat);
    grid(wall, {-hx, 0.0, -hz}, {0.0, 0.0, 2 * hz}, {0.0, top, 0.0}, rest / 10, flat);
    grid(wall, {hx, 0.0, -hz}, {0.0, top, 0.0}, {0.0, 0.0, 2 * hz}, rest / 10, flat);
    // ceiling panels: 4 x 4 layout, each 8 x 16 quads just below the ceiling, facing down
    for (int k = 0; k < panels; ++k) {
        const double cx = -11.25 + 7.5 * (k % 4), cz = -11.25 + 7.5 * (k / 4);
        grid_cells(light, {cx - 1.5, top - 0.02, cz - 0.75}, {3.0, 0.0, 0.0}, {0.0, 0.0, 1.5}, 16, 8, flat);
    }
    // icosphere props (the 320-face sphere of the terrain scene)
    std::vector<Vec3> verts;
    std::vector<std::array<int, 3>> faces;
    icosphere2(verts, faces);
    for (int k = 0; k < props; ++k) {
        const double r = rng.uniform(0.2, 0.8);
        const double cx = rng.uniform(-hx + 1.0, hx - 1.0), cz = rng.uniform(-hz + 1.0, hz - 1.0);
        const Vec3 center {cx, bumps(cx, cz) + r * 1.02, cz};
        const int m = b.openpbr(pbr({rng.uniform(), rng.uniform(), rng.uniform()}, rng.uniform(0.05, 1.0),
            rng.uniform() < 0.3 ? 1.0 : 0.0));
        for (const auto& f : faces) {
            auto P = [&](int vi) { return Vec3 {center[0] + r * verts[vi][0], center[1] + r * verts[vi][1], center[2] + r * verts[vi][2]}; };
            b.triangle(m, P(f[0]), P(f[1]), P(f[2]));
        }
    }
    b.background({0.0, 0.0, 0.0});
}

// ---- cameras -----------------------------------------------------------------

// invert_equi_theta_distortion (src/realtime/camera_models.cpp:74-119)
double eval_theta_d(const double* radial, double theta) {
    const double t2 = theta * theta;
    double scale = 1.0, tp = t2;
    for (int i = 0; i < 6; ++i) {
        scale += radial[i] * tp;
        tp *= t2;
    }
    return theta * scale;
}
double eval_theta_d_derivative(const double* radial, double theta) {
    const double t2 = theta * theta;
    double d = 1.0, tp = t2;
    for (int i = 0; i < 6; ++i) {
        d += static_cast<double>(2 * i + 3) * radial[i] * tp;
        tp *= t2;
    }
    return d;
}
double invert_theta_d(const double* radial, double thetad) {
    constexpr double eps = 1e-12;
    double theta = std::cbrt(std::max(thetad, 0.0));
    for (int it = 0; it < 30; ++it) {
        const double err = thetad - eval_theta_d(radial, theta);
        if (std::abs(err) < eps) break;
        const double der = eval_theta_d_derivative(radial, theta);
        if (std::abs(der) < eps) break;
        const double delta = err / der;
        theta += delta;
        if (std::abs(delta) < eps || std::abs(delta) > 3.1416) break;
    }
    return theta;
}

void mat3_mul(const double* a, const double* b, double* out) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[r * 3 + c] = a[r * 3] * b[c] + a[r * 3 + 1] * b[3 + c] + a[r * 3 + 2] * b[6 + c];
}

// camera_to_world_matrix / body_to_world_matrix (frame_convention.h:7-21), row-major.
constexpr double kCameraToRenderer[9] = {1, 0, 0, 0, 0, 1, 0, -1, 0};
constexpr double kBodyToRenderer[9] = {0, -1, 0, 0, 0, -1, 1, 0, 0};

// A camera at `eye` looking at `target` with world `up`: rotation columns are
// the world directions of camera x (right), y (down) and z (forward).
void look_at(rtgb_camera& cam, const Vec3& eye, const Vec3& target, const Vec3& up) {
    auto norm = [](Vec3 v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        return Vec3 {v[0] / l, v[1] / l, v[2] / l};
    };
    auto crs = [](const Vec3& a, const Vec3& b) {
        return Vec3 {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    };
    const Vec3 fwd = norm({target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]});
    const Vec3 right = norm(crs(fwd, up));
    const Vec3 down = crs(fwd, right);
    for (int r = 0; r < 3; ++r) {
        cam.rotation[r * 3 + 0] = right[r];
        cam.rotation[r * 3 + 1] = down[r];
        cam.rotation[r * 3 + 2] = fwd[r];
        cam.translation[r] = eye[r];
    }
}

rtgb_camera pinhole_camera(int w, int h, double hfov_deg) {
    rtgb_camera c {};
    c.enabled = 1;
    c.width = w;
    c.height = h;
    c.model = RTGB_CAMERA_PINHOLE32;
    const double f = 0.5 * w / std::tan(0.5 * hfov_deg * std::numbers::pi / 180.0);
    c.pinhole = rtgb_pinhole32 {f, f, 0.5 * w, 0.5 * h, 0, 0, 0, 0, 0};
    return c;
}

rtgb_camera equi_camera(int w, int h, double hfov_deg) {
    rtgb_camera c {};
    c.enabled = 1;
    c.width = w;
    c.height = h;
    c.model = RTGB_CAMERA_EQUI62_LUT1D;
    // derive_default_camera_intrinsics (camera_models.cpp:164-204): equidistant focal
    const double f = 0.5 * w / (0.5 * hfov_deg * std::numbers::pi / 180.0);
    const double radial[6] = {0, 0, 0, 0, 0, 0};
    const double tangential[2] = {0, 0};
    rtgb_make_equi62_lut1d(w, h, f, f, 0.5 * w, 0.5 * h, radial, tangential, &c.equi);
    return c;
}

Vec3 rotate_about(const Vec3& v, const Vec3& axis, double deg) {
    const double a = deg * std::numbers::pi / 180.0, c = std::cos(a), s = std::sin(a);
    const double d = v[0] * axis[0] + v[1] * axis[1] + v[2] * axis[2];
    const Vec3 x {axis[1] * v[2] - axis[2] * v[1], axis[2] * v[0] - axis[0] * v[2], axis[0] * v[1] - axis[1] * v[0]};
    return {v[0] * c + x[0] * s + axis[0] * d * (1 - c), v[1] * c + x[1] * s + axis[1] * d * (1 - c),
        v[2] * c + x[2] * s + axis[2] * d * (1 - c)};
}

}  // namespace
}  // namespace rtgb

using namespace rtgb;

namespace {

constexpr char kSceneMagic[8] = {'R', 'T', 'G', 'B', 'S', 'C', 'N', '1'};
constexpr uint32_t kSceneVersion = 1;
static_assert(std::endian::native == std::endian::little, "scene files are written in host byte order");

// record sizes, in file order; a reader with other layouts refuses the file
constexpr std::array<uint32_t, 9> kRecordSizes {sizeof(rtgb_texture), sizeof(float), sizeof(rtgb_material),
    sizeof(rtgb_sphere), sizeof(rtgb_quad), sizeof(rtgb_triangle), sizeof(rtgb_medium), sizeof(rtgb_analytic_light),
    sizeof(rtgb_openpbr_material)};

template <class F>
void for_each_array(rtgb_host_scene& s, F&& f) {
    f(s.textures);
    f(s.texels);
    f(s.materials);
    f(s.spheres);
    f(s.quads);
    f(s.triangles);
    f(s.media);
    f(s.analytic);
    f(s.openpbr);
}

template <class T>
void copy_array(std::vector<T>& dst, const T* src, int32_t n) {
    dst.assign(src, src + (src && n > 0 ? n : 0));
}

}  // namespace

extern "C" {

rtgb_status rtgb_host_scene_create(const char* name, uint32_t seed, int64_t detail, rtgb_host_scene** out) {
    if (name == nullptr || out == nullptr) return RTGB_INVALID_ARGUMENT;
    auto* s = new rtgb_host_scene();
    const std::string n(name);
    if (n == "cornell_box") build_cornell(*s);
    else if (n == "smoke") build_smoke(*s);
    else if (n == "final_room") build_final_room(*s);
    else if (n == "bouncing_spheres") build_bouncing_spheres(*s);
    else if (n == "restir_acceptance") build_restir_acceptance(*s);
    else if (n == "random_spheres") build_random_spheres(*s, seed, detail);
    else if (n == "triangle_terrain") build_triangle_terrain(*s, seed, detail);
    else if (n == "triangle_terrain_pbr") build_triangle_terrain(*s, seed, detail, true);
    else if (n == "openpbr_gallery") build_openpbr_gallery(*s, seed, detail);
    else if (n == "textured_room") build_textured_room(*s, seed, detail);
    else {
        delete s;
        return RTGB_INVALID_ARGUMENT;
    }
    *out = s;
    return RTGB_OK;
}

void rtgb_host_scene_destroy(rtgb_host_scene* s) { delete s; }

rtgb_status rtgb_host_scene_view(const rtgb_host_scene* s, rtgb_scene* v) {
    if (s == nullptr || v == nullptr) return RTGB_INVALID_ARGUMENT;
    *v = rtgb_scene {};
    v->textures = s->textures.data();
    v->texture_count = static_cast<int32_t>(s->textures.size());
    v->image_texels = s->texels.data();
    v->image_texel_count = static_cast<int32_t>(s->texels.size() / 3);
    v->materials = s->materials.data();
    v->material_count = static_cast<int32_t>(s->materials.size());
    v->spheres = s->spheres.data();
    v->sphere_count = static_cast<int32_t>(s->spheres.size());
    v->quads = s->quads.data();
    v->quad_count = static_cast<int32_t>(s->quads.size());
    v->triangles = s->triangles.data();
    v->triangle_count = static_cast<int32_t>(s->triangles.size());
    v->media = s->media.data();
    v->medium_count = static_cast<int32_t>(s->media.size());
    v->analytic_lights = s->analytic.data();
    v->analytic_light_count = static_cast<int32_t>(s->analytic.size());
    v->openpbr_materials = s->openpbr.data();
    v->openpbr_material_count = static_cast<int32_t>(s->openpbr.size());
    std::memcpy(v->background, s->background.data(), sizeof v->background);
    return RTGB_OK;
}


rtgb_status rtgb_host_scene_save(const rtgb_host_scene* s, const char* path) {
    if (s == nullptr || path == nullptr) return RTGB_INVALID_ARGUMENT;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return RTGB_INVALID_ARGUMENT;
    bool ok = std::fwrite(kSceneMagic, 1, 8, f) == 8 && std::fwrite(&kSceneVersion, 4, 1, f) == 1 &&
              std::fwrite(kRecordSizes.data(), 4, kRecordSizes.size(), f) == kRecordSizes.size();
    for_each_array(const_cast<rtgb_host_scene&>(*s), [&](auto& v) {
        const uint64_t n = v.size();
        ok = ok && std::fwrite(&n, 8, 1, f) == 1 && (n == 0 || std::fwrite(v.data(), sizeof v[0], n, f) == n);
    });
    ok = ok && std::fwrite(s->background.data(), 4, 3, f) == 3;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? RTGB_OK : RTGB_INVALID_ARGUMENT;
}

rtgb_status rtgb_host_scene_load(const char* path, rtgb_host_scene** out) {
    if (path == nullptr || out == nullptr) return RTGB_INVALID_ARGUMENT;
    *out = nullptr;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return RTGB_INVALID_ARGUMENT;
    auto s = std::make_unique<rtgb_host_scene>();
    char magic[8] = {};
    uint32_t version = 0;
    std::array<uint32_t, 9> sizes {};
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::equal(magic, magic + 8, kSceneMagic) &&
              std::fread(&version, 4, 1, f) == 1 && version == kSceneVersion &&
              std::fread(sizes.data(), 4, sizes.size(), f) == sizes.size() && sizes == kRecordSizes;
    // counts are bounded by what is left in the file before anything is allocated
    long here = ok ? std::ftell(f) : 0;
    std::fseek(f, 0, SEEK_END);
    const long end = std::ftell(f);
    std::fseek(f, here, SEEK_SET);
    for_each_array(*s, [&](auto& v) {
        uint64_t n = 0;
        ok = ok && std::fread(&n, 8, 1, f) == 1;
        here += 8;
        ok = ok && n <= static_cast<uint64_t>(end - here) / sizeof v[0] && n <= static_cast<uint64_t>(INT32_MAX);
        if (!ok) return;
        v.resize(static_cast<size_t>(n));
        ok = n == 0 || std::fread(v.data(), sizeof v[0], n, f) == n;
        here += static_cast<long>(n * sizeof v[0]);
    });
    ok = ok && std::fread(s->background.data(), 4, 3, f) == 3;
    std::fclose(f);
    if (!ok) return RTGB_INVALID_ARGUMENT;
    *out = s.release();
    return RTGB_OK;
}

rtgb_status rtgb_host_scene_from_view(const rtgb_scene* v, rtgb_host_scene** out) {
    if (v == nullptr || out == nullptr) return RTGB_INVALID_ARGUMENT;
    auto s = std::make_unique<rtgb_host_scene>();
    copy_array(s->textures, v->textures, v->texture_count);
    copy_array(s->texels, v->image_texels, v->image_texel_count > 0 ? 3 * v->image_texel_count : 0);
    copy_array(s->materials, v->materials, v->material_count);
    copy_array(s->spheres, v->spheres, v->sphere_count);
    copy_array(s->quads, v->quads, v->quad_count);
    copy_array(s->triangles, v->triangles, v->triangle_count);
    copy_array(s->media, v->media, v->medium_count);
    copy_array(s->analytic, v->analytic_lights, v->analytic_light_count);
    copy_array(s->openpbr, v->openpbr_materials, v->openpbr_material_count);
    std::memcpy(s->background.data(), v->background, sizeof v->background);
    *out = s.release();
    return RTGB_OK;
}

rtgb_status rtgb_make_equi62_lut1d(int32_t width, int32_t height, double fx, double fy, double cx, double cy,
    const double radial[6], const double tangential[2], rtgb_equi62_lut1d* out) {
    if (out == nullptr || radial == nullptr || tangential == nullptr || fx == 0.0 || fy == 0.0) return RTGB_INVALID_ARGUMENT;
    *out = rtgb_equi62_lut1d {};
    out->width = width;
    out->height = height;
    out->fx = fx;
    out->fy = fy;
    out->cx = cx;
    out->cy = cy;
    for (int i = 0; i < 6; ++i) out->radial[i] = radial[i];
    out->tangential[0] = tangential[0];
    out->tangential[1] = tangential[1];
    const double x = (static_cast<double>(width) + 10.0 - cx) / fx;
    const double y = (static_cast<double>(height) + 10.0 - cy) / fy;
    out->lut_step = std::sqrt(x * x + y * y) / static_cast<double>(RTGB_EQUI_LUT_SIZE);
    for (int i = 0; i < RTGB_EQUI_LUT_SIZE; ++i) out->lut[i] = invert_theta_d(out->radial, out->lut_step * static_cast<double>(i));
    return RTGB_OK;
}

rtgb_status rtgb_pack_camera_pose(const double rotation_bc[9], const double translation_bc[3], double rotation_rc[9],
    double translation_rc[3]) {
    if (!rotation_bc || !translation_bc || !rotation_rc || !translation_rc) return RTGB_INVALID_ARGUMENT;
    mat3_mul(kCameraToRenderer, rotation_bc, rotation_rc);
    for (int r = 0; r < 3; ++r) {
        translation_rc[r] = kBodyToRenderer[r * 3] * translation_bc[0] + kBodyToRenderer[r * 3 + 1] * translation_bc[1]
                            + kBodyToRenderer[r * 3 + 2] * translation_bc[2];
    }
    return RTGB_OK;
}

rtgb_status rtgb_default_rig(const char* scene_name, int32_t camera_count, int32_t width, int32_t height, rtgb_camera_rig* rig) {
    if (scene_name == nullptr || rig == nullptr || camera_count < 1 || camera_count > RTGB_MAX_CAMERAS) return RTGB_INVALID_ARGUMENT;
    *rig = rtgb_camera_rig {};
    const std::string n(scene_name);
    rig->active_count = camera_count;
    constexpr double kYaw[4] = {0.0, 90.0, -90.0, 180.0};  // default_viewer_conventions.h:7
    if (n == "cornell_box") {
        // 256x256 pinhole32, fx = fy = 128 / tan(20 deg), eye (278,278,-800) -> (278,278,0)
        for (int i = 0; i < camera_count; ++i) {
            rtgb_camera c = pinhole_camera(width > 0 ? width : 256, height > 0 ? height : 256, 40.0);
            const double f = 0.5 * c.height / std::tan(20.0 * std::numbers::pi / 180.0);
            c.pinhole.fx = f;
            c.pinhole.fy = f;
            const Vec3 eye {278.0, 278.0, -800.0};
            const Vec3 dir = rotate_about({0.0, 0.0, 800.0}, {0.0, 1.0, 0.0}, kYaw[i]);
            look_at(c, eye, {eye[0] + dir[0], eye[1] + dir[1], eye[2] + dir[2]}, {0.0, 1.0, 0.0});
            rig->cameras[i] = c;
        }
        return RTGB_OK;
    }
    if (n == "restir_acceptance") {
        rtgb_camera c {};
        c.enabled = 1;
        c.width = 128;
        c.height = 128;
        c.model = RTGB_CAMERA_PINHOLE32;
        c.pinhole = rtgb_pinhole32 {135.0, 135.0, 64.0, 64.0, 0, 0, 0, 0, 0};
        const double identity[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        const double zero[3] = {0, 0, 0};
        rtgb_pack_camera_pose(identity, zero, c.rotation, c.translation);
        for (int i = 0; i < camera_count; ++i) rig->cameras[i] = c;
        return RTGB_OK;
    }
    if (n == "triangle_terrain" || n == "triangle_terrain_pbr") {
        // mixed rig: 2x pinhole32 640x480 (hfov 90) + 2x equi62_lut1d 1280x1024 (180 deg);
        // a given width/height applies to every camera
        for (int i = 0; i < camera_count; ++i) {
            const bool equi = i >= 2;
            rtgb_camera c = equi ? equi_camera(width > 0 ? width : 1280, height > 0 ? height : 1024, 180.0)
                                 : pinhole_camera(width > 0 ? width : 640, height > 0 ? height : 480, 90.0);
            const Vec3 eye {0.0, 4.0, 0.0};
            const Vec3 dir = rotate_about({0.0, -0.35, 1.0}, {0.0, 1.0, 0.0}, kYaw[i]);
            look_at(c, eye, {eye[0] + dir[0], eye[1] + dir[1], eye[2] + dir[2]}, {0.0, 1.0, 0.0});
            rig->cameras[i] = c;
        }
        return RTGB_OK;
    }
    if (n == "textured_room") {
        // mixed rig at 1920x1080: 2x pinhole32 (hfov 90) + 2x equi62_lut1d (180 deg),
        // on a 9 m circle around the room centre, each looking across the room
        for (int i = 0; i < camera_count; ++i) {
            const bool equi = i % 2 == 1;
            const int w = width > 0 ? width : 1920, h = height > 0 ? height : 1080;
            rtgb_camera c = equi ? equi_camera(w, h, 180.0) : pinhole_camera(w, h, 90.0);
            const Vec3 eye = rotate_about({0.0, 2.2, -9.0}, {0.0, 1.0, 0.0}, 90.0 * i);
            look_at(c, eye, {0.0, 1.2 + 0.4 * (i % 2), 0.0}, {0.0, 1.0, 0.0});
            rig->cameras[i] = c;
        }
        return RTGB_OK;
    }
    // y-up scenes viewed from inside the content with four yawed cameras;
    // legacy z-up scenes (smoke, final_room) convert with legacy_to_world.
    const bool zup = n == "smoke" || n == "final_room";
    Vec3 eye {0.0, 1.0, 0.0}, ahead {0.0, -0.15, 1.0};
    if (n == "bouncing_spheres") {
        eye = {13.0, 2.0, 3.0};
        ahead = {-13.0, -2.0, -3.0};
    } else if (n == "smoke") {
        eye = legacy_to_world({0.0, 0.0, 1.0});
        ahead = legacy_to_world({0.0, 0.0, -1.0});
    } else if (n == "final_room") {
        eye = legacy_to_world({0.0, 1.2, 2.5});
        ahead = legacy_to_world({0.0, -0.1, -1.0});
    }
    const Vec3 up = zup ? Vec3 {0.0, 0.0, 1.0} : Vec3 {0.0, 1.0, 0.0};
    for (int i = 0; i < camera_count; ++i) {
        rtgb_camera c = pinhole_camera(width > 0 ? width : 640, height > 0 ? height : 480, 90.0);
        const Vec3 dir = rotate_about(ahead, up, kYaw[i]);
        look_at(c, eye, {eye[0] + dir[0], eye[1] + dir[1], eye[2] + dir[2]}, up);
        rig->cameras[i] = c;
    }
    return RTGB_OK;
}

rtgb_status rtgb_profile_preset(const char* name, rtgb_render_profile* p) {
    if (name == nullptr || p == nullptr) return RTGB_INVALID_ARGUMENT;
    rtgb_render_profile d {};
    d.samples_per_pixel = 1;
    d.max_bounces = 4;
    d.enable_denoise = 1;
    d.rr_start_bounce = 3;
    d.accumulation_reset_rotation_deg = 2.0;
    d.accumulation_reset_translation = 0.05;
    d.enable_restir_di = 0;
    d.restir_initial_candidates = 4;
    d.restir_temporal_reuse = 1;
    d.restir_max_history_age = 20;
    d.restir_max_temporal_candidates = 64;
    d.restir_spatial_neighbors = 1;
    d.restir_max_spatial_candidates = 4;
    d.restir_bias_correction = 1;
    d.restir_min_analytic_lights = 16;
    const std::string n(name);
    if (n == "quality") {
        d.samples_per_pixel = 4;
        d.max_bounces = 8;
        d.enable_denoise = 0;
        d.rr_start_bounce = 6;
        d.accumulation_reset_rotation_deg = 0.5;
        d.accumulation_reset_translation = 0.01;
    } else if (n == "balanced" || n == "default") {
        d.samples_per_pixel = 2;
        d.max_bounces = 4;
        d.rr_start_bounce = 3;
        d.accumulation_reset_rotation_deg = 1.0;
        d.accumulation_reset_translation = 0.02;
        d.enable_restir_di = 1;
    } else if (n == "realtime") {
        d.samples_per_pixel = 1;
        d.max_bounces = 2;
        d.rr_start_bounce = 2;
        d.enable_restir_di = 1;
    } else {
        return RTGB_INVALID_ARGUMENT;
    }
    *p = d;
    return RTGB_OK;
}

}  // extern "C"
