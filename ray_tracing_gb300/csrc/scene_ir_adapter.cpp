// SceneIR v2 -> packed realtime scene (rtgb_host_scene).
//
// Three compilers the reference splits over three files:
//  * analytic lights: src/scene/analytic_light_compiler.cpp (compile_light
//    :140-238, compile_analytic_lights :242-261, the CDF :15-39) and the float
//    packing of src/realtime/gpu/packed_scene_preparation.cpp:17-37;
//  * OpenPBR surfaces: src/scene/openpbr_core_adapter.cpp:17-101, :133-213;
//  * geometry and textures: src/scene/realtime_scene_adapter.cpp:115-368,
//    :502-581, with the texture / material packing of
//    packed_scene_preparation.cpp:91-190.
// Lights and geometry are computed in double and rounded to float once, at
// packing, as there.
#include <algorithm>
#include <array>
#include <cmath>
#include <filesystem>
#include <numbers>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include "cli/png_reader.h"
#include "host_scene.h"
#include "rtgb_scene_ir_v2.hpp"
#include "scene_ir_math.h"

namespace rtgb::scene {
namespace {

namespace M = math;

// UsdLuxBlackbodyTemperatureAsRgb (OpenUSD pxr/usd/usdLux/blackbody.cpp): a
// Catmull-Rom spline through 22 RGB knots over 1000..10000 K, normalised to
// Rec.709 luminance 1 and clamped at 0. The knot table is OpenUSD's data.
Vec3 blackbody_rgb(double kelvin) {
    static constexpr std::array<std::array<double, 3>, 22> kKnots {{
        {1.000000, 0.027490, 0.000000}, {1.000000, 0.027490, 0.000000}, {1.000000, 0.149664, 0.000000},
        {1.000000, 0.256644, 0.008095}, {1.000000, 0.372033, 0.067450}, {1.000000, 0.476725, 0.153601},
        {1.000000, 0.570376, 0.259196}, {1.000000, 0.653480, 0.377155}, {1.000000, 0.726878, 0.501606},
        {1.000000, 0.791543, 0.628050}, {1.000000, 0.848462, 0.753228}, {1.000000, 0.898581, 0.874905},
        {1.000000, 0.942771, 0.991642}, {0.906947, 0.890456, 1.000000}, {0.828247, 0.841838, 1.000000},
        {0.765791, 0.801896, 1.000000}, {0.715255, 0.768579, 1.000000}, {0.673683, 0.740423, 1.000000},
        {0.638992, 0.716359, 1.000000}, {0.609681, 0.695588, 1.000000}, {0.609681, 0.695588, 1.000000},
        {0.609681, 0.695588, 1.000000},
    }};
    // Catmull-Rom basis rows (cubic, quadratic, linear, constant coefficients)
    static constexpr std::array<std::array<double, 4>, 4> kBasis {{
        {-0.5, 1.5, -1.5, 0.5}, {1.0, -2.5, 2.0, -0.5}, {-0.5, 0.0, 0.5, 0.0}, {0.0, 1.0, 0.0, 0.0}}};
    const double t = std::clamp((kelvin - 1000.0) / 9000.0, 0.0, 1.0);
    const double x = t * static_cast<double>(kKnots.size() - 4);
    const int seg = static_cast<int>(std::floor(x));
    const double u = x - seg;
    Vec3 rgb {};
    for (int ch = 0; ch < 3; ++ch) {
        std::array<double, 4> c {};
        for (int row = 0; row < 4; ++row) {
            const auto& b = kBasis[static_cast<size_t>(row)];
            // ((b0*k0 + b1*k1) + b2*k2) + b3*k3, the order an expression of four scaled vectors evaluates in
            c[static_cast<size_t>(row)] = b[0] * kKnots[static_cast<size_t>(seg)][static_cast<size_t>(ch)] +
                                          b[1] * kKnots[static_cast<size_t>(seg + 1)][static_cast<size_t>(ch)] +
                                          b[2] * kKnots[static_cast<size_t>(seg + 2)][static_cast<size_t>(ch)] +
                                          b[3] * kKnots[static_cast<size_t>(seg + 3)][static_cast<size_t>(ch)];
        }
        rgb[static_cast<size_t>(ch)] = ((c[0] * u + c[1]) * u + c[2]) * u + c[3];
    }
    const double lum = rgb[0] * 0.2126 + rgb[1] * 0.7152 + rgb[2] * 0.0722;
    for (double& v : rgb) v = std::max(v / lum, 0.0);
    return rgb;
}

double rec709(const Vec3& v) { return v[0] * 0.2126 + v[1] * 0.7152 + v[2] * 0.0722; }

// sqrt(trace(L^T L) / 3) when L^T L is that multiple of the identity within
// 1e-6 * max(1, s^2); otherwise the light cannot be represented.
double similarity_scale(const M::Mat3& l, const std::string& path, const char* type) {
    std::array<double, 9> g {};
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += l[static_cast<size_t>(3 * k + r)] * l[static_cast<size_t>(3 * k + c)];
            g[static_cast<size_t>(3 * r + c)] = s;
        }
    }
    const double s2 = (g[0] + g[4] + g[8]) / 3.0;
    if (!std::isfinite(s2) || s2 <= 0.0) throw std::invalid_argument(std::string(type) + " light has a singular transform: " + path);
    const double tol = 1e-6 * std::max(1.0, s2);
    double worst = 0.0;
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) worst = std::max(worst, std::abs(g[static_cast<size_t>(3 * r + c)] - (r == c ? s2 : 0.0)));
    }
    if (worst > tol) {
        throw std::invalid_argument(std::string(type) + " light requires a similarity transform in this backend: " + path);
    }
    return std::sqrt(s2);
}

AnalyticLightType runtime_type(SceneLightType t) {
    switch (t) {
        case SceneLightType::sphere: return AnalyticLightType::sphere;
        case SceneLightType::disk: return AnalyticLightType::disk;
        case SceneLightType::rect: return AnalyticLightType::rect;
        case SceneLightType::cylinder: return AnalyticLightType::cylinder;
        case SceneLightType::distant: return AnalyticLightType::distant;
        case SceneLightType::dome: return AnalyticLightType::dome;
        case SceneLightType::geometry: break;
    }
    throw std::invalid_argument("geometry light is not an intrinsic analytic light");
}

// cone solid-angle factor of a normalised distant light of half-angle theta
double distant_size_factor(double theta) {
    if (theta <= 0.0) return 1.0;
    const double s2 = std::sin(theta) * std::sin(theta);
    return theta <= std::numbers::pi / 2.0 ? std::numbers::pi * s2 : std::numbers::pi * (2.0 - s2);
}

AnalyticLightDesc compile_light(const ScenePrim& prim, const SceneLight& light, const Mat4& world) {
    if (!prim.asset_references.empty()) {
        throw std::invalid_argument("runtime analytic light textures are not supported yet: " + prim.path);
    }
    if (std::abs(light.diffuse - 1.0) > 1e-12 || std::abs(light.specular - 1.0) > 1e-12) {
        throw std::invalid_argument("runtime analytic light diffuse/specular overrides are not supported yet: " + prim.path);
    }
    AnalyticLightDesc out;
    out.type = runtime_type(light.type);
    out.source_path = prim.path;
    out.position = M::translation(world);
    out.local_to_world_linear = M::linear(world);
    out.radius = light.radius;
    out.width = light.width;
    out.height = light.height;
    out.length = light.length;
    out.diffuse = light.diffuse;
    out.specular = light.specular;
    out.treat_as_point = light.treat_as_point;
    out.treat_as_line = light.treat_as_line;
    const M::Mat3& l = out.local_to_world_linear;
    const double plane_scale = M::norm(M::cross(M::column(l, 0), M::column(l, 1)));
    double size = 1.0;
    switch (light.type) {
        case SceneLightType::sphere: {
            const double s = similarity_scale(l, prim.path, "sphere");
            out.world_area = 4.0 * std::numbers::pi * std::pow(light.radius * s, 2.0);
            size = out.world_area;
            break;
        }
        case SceneLightType::disk:
            out.world_area = std::numbers::pi * light.radius * light.radius * plane_scale;
            size = out.world_area;
            break;
        case SceneLightType::rect:
            out.world_area = light.width * light.height * plane_scale;
            size = out.world_area;
            break;
        case SceneLightType::cylinder: {
            const double s = similarity_scale(l, prim.path, "cylinder");
            out.world_area = 2.0 * std::numbers::pi * (light.radius * s) * (light.length * s);
            size = out.world_area;
            break;
        }
        case SceneLightType::distant: {
            const double theta = std::clamp(light.angle_degrees, 0.0, 360.0) * std::numbers::pi / 360.0;
            out.cos_theta_max = std::cos(theta);
            out.delta = theta <= 1e-12;
            size = distant_size_factor(theta);
            break;
        }
        case SceneLightType::dome: break;
        case SceneLightType::geometry: throw std::logic_error("geometry light reached the analytic-light compiler");
    }
    Vec3 color = light.color;
    if (light.enable_color_temperature) {
        const Vec3 bb = blackbody_rgb(light.color_temperature_kelvin);
        for (int i = 0; i < 3; ++i) color[static_cast<size_t>(i)] *= bb[static_cast<size_t>(i)];
    }
    const double scale = scene_light_exposed_intensity(light) / (light.normalize ? size : 1.0);
    for (int i = 0; i < 3; ++i) out.radiance[static_cast<size_t>(i)] = color[static_cast<size_t>(i)] * scale;
    const double lum = std::max(0.0, rec709(out.radiance));
    if (light.type == SceneLightType::dome) {
        out.selection_weight = 4.0 * std::numbers::pi * lum;
    } else if (light.type == SceneLightType::distant) {
        out.selection_weight = (out.delta ? 1.0 : 2.0 * std::numbers::pi * (1.0 - out.cos_theta_max)) * lum;
    } else {
        out.selection_weight = out.world_area * lum;
    }
    return out;
}

}  // namespace

// Selection pmf proportional to the (finite, clamped non-negative) weights;
// the CDF is closed to exactly 1 from the last light with a positive pmf on.
void finalize_analytic_light_distribution(std::vector<AnalyticLightDesc>& lights) {
    double total = 0.0;
    for (AnalyticLightDesc& l : lights) {
        l.selection_weight = std::isfinite(l.selection_weight) ? std::max(0.0, l.selection_weight) : 0.0;
        total += l.selection_weight;
    }
    double cdf = 0.0;
    for (AnalyticLightDesc& l : lights) {
        l.selection_pdf = total > 0.0 ? l.selection_weight / total : 0.0;
        cdf += l.selection_pdf;
        l.cdf = cdf;
    }
    if (total > 0.0) {
        size_t last = lights.size();
        while (last > 0 && !(lights[last - 1].selection_pdf > 0.0)) --last;
        // (none positive happens only when the total overflowed: then nothing is closed)
        for (size_t i = last; i > 0 && i - 1 < lights.size(); ++i) lights[i - 1].cdf = 1.0;
    }
}

std::vector<AnalyticLightDesc> compile_analytic_lights(const SceneIRv2& scene) {
    require_valid_scene_ir_v2(scene);
    std::vector<AnalyticLightDesc> out;
    const double t = scene.stage_metadata().start_time_code.value_or(0.0);
    for (const ScenePrim& p : scene.prims()) {
        if (!p.light || p.light->type == SceneLightType::geometry || !compute_scene_visibility(scene, p.path)) continue;
        const ScenePurpose purpose = compute_scene_purpose(scene, p.path);
        if (purpose == ScenePurpose::proxy || purpose == ScenePurpose::guide) continue;
        out.push_back(compile_light(p, *p.light, compute_scene_world_transform(scene, p.path, t)));
    }
    finalize_analytic_light_distribution(out);
    return out;
}

rtgb_analytic_light pack_analytic_light(const AnalyticLightDesc& l) {
    rtgb_analytic_light o {};
    const auto put = [](float* d, const Vec3& v) {
        for (int i = 0; i < 3; ++i) d[i] = static_cast<float>(v[static_cast<size_t>(i)]);
    };
    o.type = static_cast<int32_t>(l.type);
    put(o.position, l.position);
    put(o.basis_x, M::column(l.local_to_world_linear, 0));
    put(o.basis_y, M::column(l.local_to_world_linear, 1));
    put(o.basis_z, M::column(l.local_to_world_linear, 2));
    put(o.radiance, l.radiance);
    o.radius = static_cast<float>(l.radius);
    o.width = static_cast<float>(l.width);
    o.height = static_cast<float>(l.height);
    o.length = static_cast<float>(l.length);
    o.world_area = static_cast<float>(l.world_area);
    o.cos_theta_max = static_cast<float>(l.cos_theta_max);
    o.selection_pdf = static_cast<float>(l.selection_pdf);
    o.cdf = static_cast<float>(l.cdf);
    o.delta = l.delta ? 1 : 0;
    o.treat_as_point = l.treat_as_point ? 1 : 0;
    o.treat_as_line = l.treat_as_line ? 1 : 0;
    return o;
}

namespace {

void put3(float* d, const Vec3& v) {
    for (int i = 0; i < 3; ++i) d[i] = static_cast<float>(v[static_cast<size_t>(i)]);
}

// What the realtime core of the OpenPBR BSDF implements: no displacement, no
// transmission scattering, default normals and tangents.
void require_core_support(const SceneOpenPbrSurface& m) {
    if (m.displacement.type != SceneMaterialXDisplacementType::none) {
        throw std::invalid_argument("OpenPBR production core does not yet support MaterialX displacement");
    }
    if (M::dot(m.transmission_scatter, m.transmission_scatter) > 0.0 || m.transmission_scatter_anisotropy != 0.0) {
        throw std::invalid_argument("OpenPBR production core does not yet support transmission scattering");
    }
    if (m.geometry_normal_default_geomprop != "Nworld" || m.geometry_tangent_default_geomprop != "Tworld" ||
        m.geometry_coat_normal_default_geomprop != "Nworld" || m.geometry_coat_tangent_default_geomprop != "Tworld") {
        throw std::invalid_argument("OpenPBR production core requires the default base and coat normal/tangent inputs");
    }
}

int32_t source_color_space(SceneColorSpace cs) {
    switch (cs) {
        case SceneColorSpace::raw: return 0;
        case SceneColorSpace::linear_srgb: return 1;
        case SceneColorSpace::srgb_texture: return 2;
        case SceneColorSpace::acescg: break;
    }
    throw std::invalid_argument("OpenPBR production core does not yet support ACEScg source conversion");
}

}  // namespace

namespace detail {

// Binds one connection: RGB colour inputs (base, specular, transmission,
// emission colour) and raw float scalar inputs (base_metalness,
// specular_roughness) are what the core reads from textures.
void bind_connection(rtgb_openpbr_material& out, const SceneMaterialConnection& c, const SceneTexture& tex, int index) {
    static const std::array<std::string_view, 4> kColor {"base_color", "specular_color", "transmission_color", "emission_color"};
    static const std::array<std::string_view, 2> kScalar {"base_metalness", "specular_roughness"};
    const auto color_slot = std::find(kColor.begin(), kColor.end(), c.input_name);
    const auto scalar_slot = std::find(kScalar.begin(), kScalar.end(), c.input_name);
    const bool color = color_slot != kColor.end() && c.input_type == SceneMaterialValueType::color3 &&
                       c.channel == SceneTextureChannel::rgb && tex.output_type == SceneMaterialValueType::color3;
    const bool scalar = scalar_slot != kScalar.end() && c.input_type == SceneMaterialValueType::float_ &&
                        c.channel == SceneTextureChannel::rgb && tex.output_type == SceneMaterialValueType::float_ &&
                        tex.color_space == SceneColorSpace::raw;
    if (!color && !scalar) {
        throw std::invalid_argument(
            "OpenPBR production core supports RGB base/specular/transmission/emission color connections and raw float "
            "base_metalness/specular_roughness connections");
    }
    if (color) {
        const size_t k = static_cast<size_t>(color_slot - kColor.begin());
        out.color_texture[k] = index;
        out.color_space[k] = source_color_space(tex.color_space);
    } else {
        out.scalar_texture[static_cast<size_t>(scalar_slot - kScalar.begin())] = index;
    }
}

}  // namespace detail

rtgb_openpbr_material compile_openpbr_core_material(const SceneOpenPbrSurface& m) {
    require_core_support(m);
    if (!m.connections.empty()) {
        throw std::invalid_argument("connected OpenPBR inputs require a SceneIR v2 texture compilation context");
    }
    rtgb_openpbr_material o {};
    const auto f = [](double v) { return static_cast<float>(v); };
    o.base_weight = f(m.base_weight);
    put3(o.base_color, m.base_color);
    o.base_diffuse_roughness = f(m.base_diffuse_roughness);
    o.base_metalness = f(m.base_metalness);
    o.specular_weight = f(m.specular_weight);
    put3(o.specular_color, m.specular_color);
    o.specular_roughness = f(m.specular_roughness);
    o.specular_ior = f(m.specular_ior);
    o.specular_roughness_anisotropy = f(m.specular_roughness_anisotropy);
    o.transmission_weight = f(m.transmission_weight);
    put3(o.transmission_color, m.transmission_color);
    o.transmission_depth = f(m.transmission_depth);
    o.transmission_dispersion_scale = f(m.transmission_dispersion_scale);
    o.transmission_dispersion_abbe_number = f(m.transmission_dispersion_abbe_number);
    o.subsurface_weight = f(m.subsurface_weight);
    put3(o.subsurface_color, m.subsurface_color);
    o.subsurface_radius = f(m.subsurface_radius);
    put3(o.subsurface_radius_scale, m.subsurface_radius_scale);
    o.subsurface_scatter_anisotropy = f(m.subsurface_scatter_anisotropy);
    o.fuzz_weight = f(m.fuzz_weight);
    put3(o.fuzz_color, m.fuzz_color);
    o.fuzz_roughness = f(m.fuzz_roughness);
    o.coat_weight = f(m.coat_weight);
    put3(o.coat_color, m.coat_color);
    o.coat_roughness = f(m.coat_roughness);
    o.coat_roughness_anisotropy = f(m.coat_roughness_anisotropy);
    o.coat_ior = f(m.coat_ior);
    o.coat_darkening = f(m.coat_darkening);
    o.thin_film_weight = f(m.thin_film_weight);
    o.thin_film_thickness = f(m.thin_film_thickness);
    o.thin_film_ior = f(m.thin_film_ior);
    o.emission_luminance = f(m.emission_luminance);
    put3(o.emission_color, m.emission_color);
    o.geometry_opacity = f(m.geometry_opacity);
    o.geometry_thin_walled = m.geometry_thin_walled ? 1 : 0;
    for (int k = 0; k < 4; ++k) {
        o.color_texture[k] = -1;
        o.color_space[k] = 1;  // linear sRGB, the binding default
    }
    o.scalar_texture[0] = -1;
    o.scalar_texture[1] = -1;
    return o;
}

rtgb_openpbr_material compile_openpbr_core_material(const SceneOpenPbrSurface& m, const SceneIRv2& scene,
    const std::unordered_map<std::string, int>& texture_indices) {
    SceneOpenPbrSurface constants = m;
    constants.connections.clear();
    rtgb_openpbr_material out = compile_openpbr_core_material(constants);
    for (const SceneMaterialConnection& c : m.connections) {
        const ScenePrim* tex = scene.find_prim(c.texture_path);
        if (!tex || !tex->texture) throw std::invalid_argument("OpenPBR connected input does not resolve to a SceneIR v2 texture");
        const auto idx = texture_indices.find(c.texture_path);
        if (idx == texture_indices.end()) {
            throw std::invalid_argument("OpenPBR connected texture has no realtime texture index: " + c.texture_path);
        }
        detail::bind_connection(out, c, *tex->texture, idx->second);
    }
    return out;
}

namespace detail {

// Reads an 8-bit PNG as RGB floats v * float(1/255) (OpenCV's imread +
// convertTo(CV_32FC3, 1/255) of the reference), trying the path and then
// "../" and "../../" before it. Returns false when nothing readable is found;
// the texture then stays 0 x 0, as in the reference.
bool load_png_texels(const std::string& path, int& width, int& height, std::vector<float>& texels) {
    for (const std::string& p : {path, "../" + path, "../../" + path}) {
        std::error_code ec;
        if (!std::filesystem::is_regular_file(p, ec)) continue;
        try {
            const png::Image img = png::read_rgb(p);
            width = img.width;
            height = img.height;
            const float scale = static_cast<float>(1.0 / 255.0);
            texels.reserve(texels.size() + img.rgb.size());
            for (uint8_t v : img.rgb) texels.push_back(static_cast<float>(v) * scale);
            return true;
        } catch (const std::runtime_error&) {
            return false;
        }
    }
    return false;
}

}  // namespace detail

namespace {

rtgb_texture default_texture() {
    rtgb_texture t {};
    t.even_texture = -1;
    t.odd_texture = -1;
    t.u_address_mode = 1;
    t.v_address_mode = 1;
    t.filter_type = 1;
    t.scale = 1.0f;
    return t;
}

std::string image_path(const ScenePrim& prim) {
    for (const SceneAssetReference& a : prim.asset_references) {
        if (!a.resolved_path.empty()) return a.resolved_path;
        if (!a.evaluated_path.empty()) return a.evaluated_path;
        if (!a.authored_path.empty()) return a.authored_path;
    }
    throw std::invalid_argument("SceneIR v2 image texture has no resolved asset: " + prim.path);
}

rtgb_texture adapt_texture(const ScenePrim& prim, const std::unordered_map<std::string, int>& indices,
    rtgb_host_scene& out, const AdaptOptions& opt) {
    const SceneTexture& t = *prim.texture;
    rtgb_texture p = default_texture();
    switch (t.node) {
        case SceneTextureNode::constant_color:
            p.type = RTGB_TEXTURE_CONSTANT;
            put3(p.color, t.value);
            break;
        case SceneTextureNode::checkerboard: {
            const auto even = indices.find(t.even_texture_path), odd = indices.find(t.odd_texture_path);
            if (even == indices.end() || odd == indices.end()) throw std::invalid_argument("SceneIR v2 checker texture input is unresolved");
            p.type = RTGB_TEXTURE_CHECKER;
            p.scale = static_cast<float>(t.scale);
            p.even_texture = even->second;
            p.odd_texture = odd->second;
            break;
        }
        case SceneTextureNode::image: {
            p.type = RTGB_TEXTURE_IMAGE;
            p.u_address_mode = static_cast<int32_t>(t.u_address_mode);  // constant, clamp, periodic, mirror
            p.v_address_mode = static_cast<int32_t>(t.v_address_mode);
            p.filter_type = static_cast<int32_t>(t.filter_type);        // closest, linear, cubic (sampled as linear)
            p.image_offset = static_cast<int32_t>(out.texels.size() / 3);
            const std::string path = image_path(prim);
            int w = 0, h = 0;
            if (opt.load_images && detail::load_png_texels(path, w, h, out.texels)) {
                p.image_width = w;
                p.image_height = h;
            }
            break;
        }
        case SceneTextureNode::noise3d:
            p.type = RTGB_TEXTURE_NOISE;
            p.scale = static_cast<float>(t.scale);
            break;
    }
    return p;
}

// The primvar of a role, preferring the conventional name ("normals", "st").
const ScenePrimvar* find_primvar(const SceneMeshGeometry& mesh, std::string_view name, ScenePrimvarRole role) {
    const ScenePrimvar* first = nullptr;
    for (const ScenePrimvar& p : mesh.primvars) {
        if (p.role != role) continue;
        if (p.name == name) return &p;
        if (!first) first = &p;
    }
    return first;
}

size_t primvar_index(const ScenePrimvar& p, size_t face, size_t corner, size_t point) {
    size_t domain = 0;
    switch (p.interpolation) {
        case ScenePrimvarInterpolation::constant: domain = 0; break;
        case ScenePrimvarInterpolation::uniform: domain = face; break;
        case ScenePrimvarInterpolation::varying:
        case ScenePrimvarInterpolation::vertex: domain = point; break;
        case ScenePrimvarInterpolation::face_varying: domain = corner; break;
    }
    if (p.element_size != 1) throw std::invalid_argument("realtime mesh adapter requires scalar primvar elements");
    if (p.indices.empty()) return domain;
    if (domain >= p.indices.size() || p.indices[domain] < 0) throw std::invalid_argument("SceneIR v2 primvar index is out of range");
    return static_cast<size_t>(p.indices[domain]);
}

template <size_t N, class F, class D>
std::array<double, N> sample_primvar(const ScenePrimvar& p, size_t face, size_t corner, size_t point, const char* what) {
    const size_t i = primvar_index(p, face, corner, point);
    const auto take = [&](const auto& values) {
        if (i >= values.size()) throw std::invalid_argument(std::string("SceneIR v2 vec") + std::to_string(N) + " primvar value is out of range");
        std::array<double, N> out {};
        for (size_t k = 0; k < N; ++k) out[k] = static_cast<double>(values[i][k]);
        return out;
    };
    if (const auto* f = std::get_if<std::vector<F>>(&p.values)) return take(*f);
    if (const auto* d = std::get_if<std::vector<D>>(&p.values)) return take(*d);
    throw std::invalid_argument(what);
}

int material_of(const std::unordered_map<std::string, int>& materials, const std::string& path) {
    const auto it = materials.find(path);
    if (it == materials.end()) throw std::invalid_argument("SceneIR v2 surface material is not realtime-compatible: " + path);
    return it->second;
}

// inverse-transpose of the linear part applied to n, renormalised
Vec3 transform_normal(const M::Mat3& inv_linear, const Vec3& n) {
    const Vec3 t = M::mul3_transposed(inv_linear, n);
    const double len = M::norm(t);
    if (!std::isfinite(len) || len <= 1e-12) throw std::invalid_argument("SceneIR v2 contains a singular or zero-length mesh normal");
    return {t[0] / len, t[1] / len, t[2] / len};
}

void add_mesh(rtgb_host_scene& out, AccelerationIds* ids, const SceneMeshGeometry& mesh, const Mat4& world,
    int fallback, const std::unordered_map<std::string, int>& materials, int prototype, int instance) {
    const ScenePrimvar* normals = find_primvar(mesh, "normals", ScenePrimvarRole::normal);
    const ScenePrimvar* uvs = find_primvar(mesh, "st", ScenePrimvarRole::texcoord);
    std::vector<int> face_material(mesh.face_vertex_counts.size(), fallback);
    for (const SceneMaterialSubset& s : mesh.material_subsets) {
        const int m = material_of(materials, s.material_path);
        for (int32_t f : s.face_indices) {
            if (f < 0 || static_cast<size_t>(f) >= face_material.size()) throw std::invalid_argument("SceneIR v2 material subset face is out of range");
            face_material[static_cast<size_t>(f)] = m;
        }
    }
    const M::Mat3 lin = M::linear(world);
    const bool reverse = (mesh.orientation == SceneMeshOrientation::left_handed) != (M::det(lin) < 0.0);
    const M::Mat3 inv = normals ? M::inverse(lin) : M::Mat3 {};
    size_t offset = 0;
    for (size_t face = 0; face < mesh.face_vertex_counts.size(); ++face) {
        const size_t count = static_cast<size_t>(mesh.face_vertex_counts[face]);
        for (size_t c = 1; c + 1 < count; ++c) {
            std::array<size_t, 3> corner {offset, offset + c, offset + c + 1};
            if (reverse) std::swap(corner[1], corner[2]);
            std::array<size_t, 3> pt {};
            for (size_t k = 0; k < 3; ++k) {
                const int32_t v = mesh.face_vertex_indices[corner[k]];
                if (v < 0 || static_cast<size_t>(v) >= mesh.points.size()) throw std::invalid_argument("SceneIR v2 mesh point index is out of range");
                pt[k] = static_cast<size_t>(v);
            }
            rtgb_triangle t {};
            t.material_index = face_material[face];
            put3(t.p0, M::point(world, mesh.points[pt[0]]));
            put3(t.p1, M::point(world, mesh.points[pt[1]]));
            put3(t.p2, M::point(world, mesh.points[pt[2]]));
            if (normals) {
                float* dst[3] = {t.n0, t.n1, t.n2};
                for (size_t k = 0; k < 3; ++k) {
                    const Vec3 n = sample_primvar<3, Vec3f, Vec3>(*normals, face, corner[k], pt[k],
                        "realtime normal primvar requires float3 or double3 values");
                    put3(dst[k], transform_normal(inv, n));
                }
                t.has_vertex_normals = 1;
            }
            if (uvs) {
                float* dst[3] = {t.uv0, t.uv1, t.uv2};
                for (size_t k = 0; k < 3; ++k) {
                    const Vec2 uv = sample_primvar<2, Vec2f, Vec2>(*uvs, face, corner[k], pt[k],
                        "realtime texcoord primvar requires float2 or double2 values");
                    dst[k][0] = static_cast<float>(uv[0]);
                    dst[k][1] = static_cast<float>(uv[1]);
                }
                t.has_texcoords = 1;
            }
            out.triangles.push_back(t);
            if (ids) {
                ids->triangle_prototype.push_back(prototype);
                ids->triangle_instance.push_back(instance);
            }
        }
        offset += count;
    }
}

// add_mesh's per-prototype half: the fan triangulation, point checks,
// sampled primvars and subset materials, independent of the instance.
MeshInstances::Prototype mesh_prototype(const SceneMeshGeometry& mesh, const std::unordered_map<std::string, int>& materials) {
    MeshInstances::Prototype out;
    const ScenePrimvar* normals = find_primvar(mesh, "normals", ScenePrimvarRole::normal);
    const ScenePrimvar* uvs = find_primvar(mesh, "st", ScenePrimvarRole::texcoord);
    std::vector<int> face_material(mesh.face_vertex_counts.size(), RTGB_INSTANCE_MATERIAL);
    for (const SceneMaterialSubset& s : mesh.material_subsets) {
        const int m = material_of(materials, s.material_path);
        for (int32_t f : s.face_indices) {
            if (f < 0 || static_cast<size_t>(f) >= face_material.size()) throw std::invalid_argument("SceneIR v2 material subset face is out of range");
            face_material[static_cast<size_t>(f)] = m;
        }
    }
    out.points.reserve(3 * mesh.points.size());
    for (const Vec3& p : mesh.points) out.points.insert(out.points.end(), p.begin(), p.end());
    size_t offset = 0;
    for (size_t face = 0; face < mesh.face_vertex_counts.size(); ++face) {
        const size_t count = static_cast<size_t>(mesh.face_vertex_counts[face]);
        for (size_t c = 1; c + 1 < count; ++c) {
            const std::array<size_t, 3> corner {offset, offset + c, offset + c + 1};
            std::array<size_t, 3> pt {};
            for (size_t k = 0; k < 3; ++k) {
                const int32_t v = mesh.face_vertex_indices[corner[k]];
                if (v < 0 || static_cast<size_t>(v) >= mesh.points.size()) throw std::invalid_argument("SceneIR v2 mesh point index is out of range");
                pt[k] = static_cast<size_t>(v);
                out.corner_points.push_back(v);
            }
            for (size_t k = 0; normals && k < 3; ++k) {
                const Vec3 n = sample_primvar<3, Vec3f, Vec3>(*normals, face, corner[k], pt[k],
                    "realtime normal primvar requires float3 or double3 values");
                out.corner_normals.insert(out.corner_normals.end(), n.begin(), n.end());
            }
            for (size_t k = 0; uvs && k < 3; ++k) {
                const Vec2 uv = sample_primvar<2, Vec2f, Vec2>(*uvs, face, corner[k], pt[k],
                    "realtime texcoord primvar requires float2 or double2 values");
                out.corner_texcoords.insert(out.corner_texcoords.end(), uv.begin(), uv.end());
            }
            out.triangle_materials.push_back(face_material[face]);
        }
        offset += count;
    }
    return out;
}

// add_mesh's per-instance half: the transform, its inverse linear part (for
// normals), the bound material and the winding flip.
rtgb_mesh_instance mesh_instance(const SceneMeshGeometry& mesh, const Mat4& world, int material, int prototype,
    bool has_normals) {
    rtgb_mesh_instance in {};
    in.prototype = prototype;
    in.material = material;
    const M::Mat3 lin = M::linear(world);
    in.flip_winding = (mesh.orientation == SceneMeshOrientation::left_handed) != (M::det(lin) < 0.0) ? 1 : 0;
    for (int k = 0; k < 12; ++k) in.world[k] = world[static_cast<size_t>(k)];
    if (has_normals) {
        const M::Mat3 inv = M::inverse(lin);
        for (int k = 0; k < 9; ++k) in.normal_matrix[k] = inv[static_cast<size_t>(k)];
    }
    return in;
}

void add_sphere(rtgb_host_scene& out, AccelerationIds* ids, const SceneSphereGeometry& g, const Mat4& world, int material,
    int prototype, int instance) {
    const M::Mat3 lin = M::linear(world);
    const double sx = M::norm(M::column(lin, 0)), sy = M::norm(M::column(lin, 1)), sz = M::norm(M::column(lin, 2));
    const double scale = (sx + sy + sz) / 3.0;
    const double tol = 1e-6 * std::max(1.0, scale);
    if (std::abs(sx - scale) > tol || std::abs(sy - scale) > tol || std::abs(sz - scale) > tol) {
        throw std::invalid_argument("realtime sphere adapter requires a uniform SceneIR v2 scale");
    }
    rtgb_sphere s {};
    put3(s.center, M::point(world, g.center));
    s.radius = static_cast<float>(g.radius * scale);
    s.material_index = material;
    out.spheres.push_back(s);
    if (ids) {
        ids->sphere_prototype.push_back(prototype);
        ids->sphere_instance.push_back(instance);
    }
}

HostScenePtr adapt(const SceneIRv2& scene, AccelerationIds* ids, const AdaptOptions& opt, MeshInstances* meshes = nullptr) {
    require_valid_scene_ir_v2(scene);
    HostScenePtr result(new rtgb_host_scene);
    rtgb_host_scene& out = *result;

    std::unordered_map<std::string, int> textures;
    for (const ScenePrim& p : scene.prims()) {
        if (p.kind == ScenePrimKind::texture && p.texture) textures.emplace(p.path, static_cast<int>(textures.size()));
    }
    for (const ScenePrim& p : scene.prims()) {
        if (p.kind != ScenePrimKind::texture || !p.texture) continue;
        out.textures.push_back(adapt_texture(p, textures, out, opt));
        if (static_cast<int>(out.textures.size()) - 1 != textures.at(p.path)) {
            throw std::logic_error("SceneIR v2 realtime texture table lost stable ordering");
        }
    }

    std::unordered_map<std::string, int> materials;
    for (const ScenePrim& p : scene.prims()) {
        if (p.kind != ScenePrimKind::material || !p.material) continue;
        const auto* surface = std::get_if<SceneOpenPbrSurface>(&*p.material);
        if (!surface) continue;  // volume materials have no realtime surface
        out.openpbr.push_back(compile_openpbr_core_material(*surface, scene, textures));
        rtgb_material m {};
        m.albedo_texture = -1;
        m.emission_texture = -1;
        m.ior = 1.0f;
        m.type = RTGB_MATERIAL_OPENPBR;
        m.openpbr_index = static_cast<int32_t>(out.openpbr.size()) - 1;
        out.materials.push_back(m);
        materials.emplace(p.path, static_cast<int>(out.materials.size()) - 1);
    }

    const double t = scene.stage_metadata().start_time_code.value_or(0.0);
    std::unordered_map<std::string, int> prototypes;
    std::unordered_map<std::string, int> mesh_prototypes;  // instanced lowering: prototype path -> meshes->prototypes
    int next_instance = 0;
    for (const ScenePrim& p : scene.prims()) {
        if (p.kind != ScenePrimKind::surface || !compute_scene_visibility(scene, p.path)) continue;
        const ScenePurpose purpose = compute_scene_purpose(scene, p.path);
        if (purpose == ScenePurpose::proxy || purpose == ScenePurpose::guide) continue;
        const ScenePrim* proto = p.prototype_path.empty() ? &p : scene.find_prim(p.prototype_path);
        if (!proto || !proto->geometry) throw std::invalid_argument("SceneIR v2 surface has no resolved geometry: " + p.path);
        const int prototype = prototypes.emplace(proto->path, static_cast<int>(prototypes.size())).first->second;
        const int instance = next_instance++;
        const int material = material_of(materials, p.material_path);
        const Mat4 world = compute_scene_world_transform(scene, p.path, t);
        if (const auto* s = std::get_if<SceneSphereGeometry>(&*proto->geometry)) {
            add_sphere(out, ids, *s, world, material, prototype, instance);
        } else if (meshes) {
            const SceneMeshGeometry& mesh = std::get<SceneMeshGeometry>(*proto->geometry);
            auto [it, fresh] = mesh_prototypes.emplace(proto->path, static_cast<int>(meshes->prototypes.size()));
            if (fresh) meshes->prototypes.push_back(mesh_prototype(mesh, materials));
            const bool has_normals = !meshes->prototypes[static_cast<size_t>(it->second)].corner_normals.empty();
            meshes->instances.push_back(mesh_instance(mesh, world, material, it->second, has_normals));
        } else {
            add_mesh(out, ids, std::get<SceneMeshGeometry>(*proto->geometry), world, material, materials, prototype, instance);
        }
    }

    for (const AnalyticLightDesc& l : compile_analytic_lights(scene)) out.analytic.push_back(pack_analytic_light(l));
    return result;
}

}  // namespace

HostScenePtr adapt_scene_ir_v2_to_realtime(const SceneIRv2& scene, const AdaptOptions& options) {
    return adapt(scene, nullptr, options);
}

HostScenePtr adapt_scene_ir_v2_to_realtime(const SceneIRv2& scene, AccelerationIds& ids, const AdaptOptions& options) {
    ids = AccelerationIds {};
    return adapt(scene, &ids, options);
}

HostScenePtr adapt_scene_ir_v2_to_realtime_instanced(const SceneIRv2& scene, MeshInstances& meshes,
    const AdaptOptions& options) {
    meshes = MeshInstances {};
    return adapt(scene, nullptr, options, &meshes);
}

rtgb_mesh_set MeshInstances::view() {
    views_.assign(prototypes.size(), rtgb_mesh_prototype {});
    for (size_t i = 0; i < prototypes.size(); ++i) {
        const Prototype& p = prototypes[i];
        rtgb_mesh_prototype& v = views_[i];
        v.points = p.points.data();
        v.point_count = static_cast<int32_t>(p.points.size() / 3);
        v.triangle_count = static_cast<int32_t>(p.triangle_materials.size());
        v.corner_points = p.corner_points.data();
        v.corner_normals = p.corner_normals.empty() ? nullptr : p.corner_normals.data();
        v.corner_texcoords = p.corner_texcoords.empty() ? nullptr : p.corner_texcoords.data();
        v.triangle_materials = p.triangle_materials.data();
    }
    rtgb_mesh_set set {};
    set.prototypes = views_.data();
    set.prototype_count = static_cast<int32_t>(views_.size());
    set.instances = instances.data();
    set.instance_count = static_cast<int32_t>(instances.size());
    return set;
}

}  // namespace rtgb::scene
