// SceneIR v2 core: the prim table, prim paths, the validator and the
// transform / visibility / purpose resolution the realtime adapter uses.
//
// Follows src/scene/scene_ir_v2.cpp: SceneIRv2::add_prim/find_prim
// (:1057-1074), is_valid_scene_prim_path/parent_scene_prim_path (:1076-1102),
// validate_scene_ir_v2 (:1104-1301) with its helpers (:22-96, :108-322,
// :329-384, :386-783), require_valid_scene_ir_v2 (:1303-1312) and
// sample_scene_local_transform .. scene_light_intensity_unit (:1499-1578).
// The diagnostic codes and their conditions are the reference's, so callers
// that match on codes keep working; the capability report and the legacy
// SceneIR v1 compiler are not part of the realtime path and are not here.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <limits>
#include <optional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>

#include "rtgb_scene_ir_v2.hpp"
#include "scene_ir_math.h"

namespace rtgb::scene {
namespace {

namespace M = math;

bool is_identifier(std::string_view s) {
    if (s.empty()) return false;
    const auto head = [](unsigned char c) { return std::isalpha(c) != 0 || c == '_'; };
    const auto tail = [](unsigned char c) { return std::isalnum(c) != 0 || c == '_'; };
    if (!head(static_cast<unsigned char>(s.front()))) return false;
    return std::all_of(s.begin() + 1, s.end(), [&](char c) { return tail(static_cast<unsigned char>(c)); });
}

// identifiers joined by ':' (a primvar or geometry-property name)
bool is_namespaced_identifier(std::string_view s) {
    if (s.empty()) return false;
    size_t start = 0;
    for (;;) {
        const size_t sep = s.find(':', start);
        if (!is_identifier(s.substr(start, sep == std::string_view::npos ? std::string_view::npos : sep - start))) {
            return false;
        }
        if (sep == std::string_view::npos) return true;
        start = sep + 1;
    }
}

bool affine_last_row(const Mat4& m) {
    return std::abs(m[12]) <= 1e-12 && std::abs(m[13]) <= 1e-12 && std::abs(m[14]) <= 1e-12 &&
           std::abs(m[15] - 1.0) <= 1e-12;
}

using PrimIndex = std::unordered_map<std::string, const ScenePrim*>;

// Collects diagnostics; every check below is one condition of the reference validator.
struct Report {
    std::vector<SceneDiagnostic> out;
    void error(std::string code, std::string_view path, std::string message) {
        out.push_back({SceneDiagnosticSeverity::error, std::move(code), std::string(path), std::move(message)});
    }
    void warning(std::string code, std::string_view path, std::string message) {
        out.push_back({SceneDiagnosticSeverity::warning, std::move(code), std::string(path), std::move(message)});
    }
};

void check_transform(Report& r, const Mat4& m, std::string_view path) {
    if (!M::all_finite(m)) {
        r.error("xform.non_finite", path, "transform contains a non-finite value");
    } else if (!affine_last_row(m)) {
        r.error("xform.non_affine", path, "transform must have affine last row [0, 0, 0, 1]");
    } else if (std::abs(M::det(M::linear(m))) <= 1e-12) {
        r.warning("xform.singular", path, "singular affine transform may be unsupported by rendering backends");
    }
}

size_t primvar_value_count(const ScenePrimvar& p) {
    return std::visit([](const auto& v) { return v.size(); }, p.values);
}

bool primvar_values_finite(const ScenePrimvar& p) {
    return std::visit(
        [](const auto& values) {
            using V = typename std::decay_t<decltype(values)>::value_type;
            if constexpr (std::is_floating_point_v<V>) {
                return std::all_of(values.begin(), values.end(), [](V x) { return std::isfinite(x); });
            } else if constexpr (std::is_same_v<V, Vec2f> || std::is_same_v<V, Vec3f> || std::is_same_v<V, Vec4f> ||
                                 std::is_same_v<V, Vec2> || std::is_same_v<V, Vec3> || std::is_same_v<V, Vec4>) {
                return std::all_of(values.begin(), values.end(), [](const V& x) { return M::all_finite(x); });
            } else {
                return true;
            }
        },
        p.values);
}

template <class... T>
bool holds_any(const ScenePrimvarValues& v) {
    return (std::holds_alternative<std::vector<T>>(v) || ...);
}

bool primvar_role_fits(const ScenePrimvar& p) {
    const bool v2 = holds_any<Vec2f, Vec2>(p.values);
    const bool v3 = holds_any<Vec3f, Vec3>(p.values);
    const bool v4 = holds_any<Vec4f, Vec4>(p.values);
    switch (p.role) {
        case ScenePrimvarRole::none: return true;
        case ScenePrimvarRole::point:
        case ScenePrimvarRole::normal:
        case ScenePrimvarRole::vector: return v3;
        case ScenePrimvarRole::color: return v3 || v4;
        case ScenePrimvarRole::texcoord: return v2;
    }
    return false;
}

size_t primvar_domain(const ScenePrimvar& p, const SceneMeshGeometry& mesh) {
    switch (p.interpolation) {
        case ScenePrimvarInterpolation::constant: return 1;
        case ScenePrimvarInterpolation::uniform: return mesh.face_vertex_counts.size();
        case ScenePrimvarInterpolation::varying:
        case ScenePrimvarInterpolation::vertex: return mesh.points.size();
        case ScenePrimvarInterpolation::face_varying: return mesh.face_vertex_indices.size();
    }
    return 0;
}

void check_primvar(Report& r, const ScenePrimvar& p, const SceneMeshGeometry& mesh, std::string_view path) {
    if (!is_namespaced_identifier(p.name) || p.name.starts_with("primvars:")) {
        r.error("geometry.primvar.name", path, "primvar name must be a valid base name without the primvars: prefix");
    }
    if (p.element_size == 0) {
        r.error("geometry.primvar.element_size", path, "primvar element_size must be positive");
        return;
    }
    const size_t count = primvar_value_count(p);
    if (count == 0) {
        r.error("geometry.primvar.values_empty", path, "primvar values must not be empty");
        return;
    }
    if (!primvar_values_finite(p)) r.error("geometry.primvar.non_finite", path, "numeric primvar values must be finite");
    if (!primvar_role_fits(p)) r.error("geometry.primvar.role_type", path, "primvar role is incompatible with its value type");
    if (p.name == "normals" && p.role != ScenePrimvarRole::normal) {
        r.error("geometry.primvar.normals_role", path, "normals primvar must use the normal role");
    }
    if (p.name == "tangents" && p.role != ScenePrimvarRole::vector) {
        r.error("geometry.primvar.tangents_role", path, "tangents primvar must use the vector role");
    }
    if (count % p.element_size != 0) {
        r.error("geometry.primvar.element_count", path, "primvar value count must be divisible by element_size");
        return;
    }
    const size_t tuples = count / p.element_size;
    const size_t domain = primvar_domain(p, mesh);
    if (p.indices.empty()) {
        if (tuples != domain) {
            r.error("geometry.primvar.domain_size", path, "unindexed primvar value count does not match its interpolation domain");
        }
        return;
    }
    if (p.indices.size() != domain) {
        r.error("geometry.primvar.index_count", path, "indexed primvar index count does not match its interpolation domain");
    }
    if (std::any_of(p.indices.begin(), p.indices.end(), [&](int32_t i) { return i < 0 || static_cast<size_t>(i) >= tuples; })) {
        r.error("geometry.primvar.index_range", path, "primvar index is out of range");
    }
}

bool is_material_prim(const PrimIndex& prims, const std::string& path) {
    const auto it = prims.find(path);
    return it != prims.end() && it->second->kind == ScenePrimKind::material;
}

void check_mesh(Report& r, const SceneMeshGeometry& mesh, std::string_view path, const PrimIndex& prims) {
    if (mesh.points.empty()) {
        r.error("geometry.mesh.points_empty", path, "mesh points must not be empty");
    } else if (!std::all_of(mesh.points.begin(), mesh.points.end(), [](const Vec3& p) { return M::all_finite(p); })) {
        r.error("geometry.mesh.points_non_finite", path, "mesh points must be finite");
    }
    size_t expected = 0;
    bool short_face = false;
    for (int32_t n : mesh.face_vertex_counts) {
        if (n < 3) {
            short_face = true;
        } else {
            expected += static_cast<size_t>(n);
        }
    }
    if (mesh.face_vertex_counts.empty() || short_face) {
        r.error("geometry.mesh.face_counts", path, "mesh faces must each contain at least three vertices");
    }
    if (expected != mesh.face_vertex_indices.size()) {
        r.error("geometry.mesh.topology_size", path, "sum(face_vertex_counts) must equal face_vertex_indices size");
    }
    if (std::any_of(mesh.face_vertex_indices.begin(), mesh.face_vertex_indices.end(),
            [&](int32_t i) { return i < 0 || static_cast<size_t>(i) >= mesh.points.size(); })) {
        r.error("geometry.mesh.vertex_index_range", path, "mesh face-vertex index is out of range");
    }
    if (mesh.subdivision_scheme == SceneSubdivisionScheme::loop &&
        std::any_of(mesh.face_vertex_counts.begin(), mesh.face_vertex_counts.end(), [](int32_t n) { return n != 3; })) {
        r.error("geometry.mesh.loop_non_triangle", path, "Loop subdivision requires triangle topology");
    }
    std::unordered_set<std::string> names;
    for (const ScenePrimvar& p : mesh.primvars) {
        if (!names.insert(p.name).second) r.error("geometry.primvar.duplicate", path, "primvar names must be unique on a mesh");
        check_primvar(r, p, mesh, path);
        if (p.name == "normals" && mesh.subdivision_scheme != SceneSubdivisionScheme::none) {
            r.warning("geometry.mesh.subdivision_authored_normals", path,
                "authored normals on a subdivision mesh may be ignored by OpenUSD renderers");
        }
    }
    std::unordered_set<std::string> subset_names;
    std::unordered_set<int32_t> claimed;
    for (const SceneMaterialSubset& s : mesh.material_subsets) {
        if (!is_identifier(s.name)) {
            r.error("geometry.subset.name", path, "material subset name must be a valid prim identifier");
        } else if (!subset_names.insert(s.name).second) {
            r.error("geometry.subset.duplicate_name", path, "material subset names must be unique");
        }
        if (!is_material_prim(prims, s.material_path)) {
            r.error("geometry.subset.material", path, "material subset path does not resolve to a material");
        }
        if (s.face_indices.empty()) r.error("geometry.subset.faces_empty", path, "material subset must contain at least one face");
        std::unordered_set<int32_t> local;
        for (int32_t f : s.face_indices) {
            if (f < 0 || static_cast<size_t>(f) >= mesh.face_vertex_counts.size()) {
                r.error("geometry.subset.face_range", path, "material subset face index is out of range");
                continue;
            }
            if (!local.insert(f).second) r.error("geometry.subset.duplicate_face", path, "material subset contains a duplicate face index");
            if (!claimed.insert(f).second) r.error("geometry.subset.overlap", path, "materialBind subsets must not overlap");
        }
    }
    if (mesh.material_subset_family_type == SceneMaterialSubsetFamilyType::partition &&
        claimed.size() != mesh.face_vertex_counts.size()) {
        r.error("geometry.subset.partition", path, "partition material subsets must cover every face exactly once");
    }
}

void check_camera(Report& r, const SceneCamera& c, std::string_view path) {
    const auto pos = [](double v) { return std::isfinite(v) && v > 0.0; };
    if (!pos(c.horizontal_aperture) || !pos(c.vertical_aperture) || !pos(c.focal_length)) {
        r.error("camera.filmback", path, "camera apertures and focal length must be finite and positive");
    }
    if (!std::isfinite(c.horizontal_aperture_offset) || !std::isfinite(c.vertical_aperture_offset)) {
        r.error("camera.aperture_offset", path, "camera aperture offsets must be finite");
    }
    if (!pos(c.clipping_range[0]) || !pos(c.clipping_range[1]) || c.clipping_range[0] >= c.clipping_range[1]) {
        r.error("camera.clipping_range", path, "camera clipping range must be finite, positive, and increasing");
    }
    if (!std::isfinite(c.f_stop) || c.f_stop < 0.0) r.error("camera.f_stop", path, "camera f-stop must be finite and non-negative");
    if (!std::isfinite(c.focus_distance) || c.focus_distance < 0.0) {
        r.error("camera.focus_distance", path, "camera focus distance must be finite and non-negative");
    }
    if (!c.renderer_calibration) return;
    const SceneCameraCalibration& k = *c.renderer_calibration;
    if (k.image_width <= 0 || k.image_height <= 0) {
        r.error("camera.calibration.resolution", path, "camera calibration resolution must be positive");
    }
    if (!M::all_finite(k.focal_length_pixels) || k.focal_length_pixels[0] <= 0.0 || k.focal_length_pixels[1] <= 0.0 ||
        !M::all_finite(k.principal_point_pixels)) {
        r.error("camera.calibration.intrinsics", path, "camera pixel intrinsics must be finite with positive focal lengths");
    }
    if (!M::all_finite(k.tangential_distortion) || !M::all_finite(k.radial_distortion)) {
        r.error("camera.calibration.distortion", path, "camera distortion coefficients must be finite");
    }
    if (!M::all_finite(k.camera_to_body) || !affine_last_row(k.camera_to_body)) {
        r.error("camera.calibration.extrinsic", path, "camera-to-body calibration must be a finite affine transform");
    }
}

bool has_control_char(std::string_view s) {
    return std::any_of(s.begin(), s.end(), [](char ch) {
        const unsigned char b = static_cast<unsigned char>(ch);
        return b < 0x20 || b == 0x7f;
    });
}

void check_asset(Report& r, const SceneAssetReference& a, std::string_view path) {
    if (a.authored_path.empty()) r.error("asset.authored_path_empty", path, "asset references must preserve a non-empty authored path");
    if (has_control_char(a.authored_path) || has_control_char(a.evaluated_path) || has_control_char(a.resolved_path)) {
        r.error("asset.path_control_character", path, "asset paths must not contain ASCII control characters");
    }
}

const ScenePrim* texture_prim(const PrimIndex& prims, const std::string& path) {
    const auto it = prims.find(path);
    if (it == prims.end() || it->second->kind != ScenePrimKind::texture || !it->second->texture) return nullptr;
    return it->second;
}

void check_texture_ref(Report& r, const PrimIndex& prims, std::string_view owner, const std::string& target, const char* code) {
    if (!texture_prim(prims, target)) r.error(code, owner, "texture input does not resolve to a texture payload: " + target);
}

std::string_view texture_nodedef(const SceneTexture& t) {
    const bool scalar = t.output_type == SceneMaterialValueType::float_;
    switch (t.node) {
        case SceneTextureNode::constant_color: return scalar ? "ND_constant_float" : "ND_constant_color3";
        case SceneTextureNode::checkerboard: return "ND_checkerboard_color3";
        case SceneTextureNode::image: return scalar ? "ND_image_float" : "ND_image_color3";
        case SceneTextureNode::noise3d: return "ND_noise3d_color3";
    }
    return {};
}

void check_texture(Report& r, const SceneTexture& t, const ScenePrim& prim, const PrimIndex& prims) {
    const bool output_ok = t.output_type == SceneMaterialValueType::color3 ||
                           (t.output_type == SceneMaterialValueType::float_ &&
                               (t.node == SceneTextureNode::constant_color || t.node == SceneTextureNode::image));
    if (!output_ok || t.node_definition != texture_nodedef(t)) {
        r.error("texture.node_definition", prim.path, "SceneIR v2 textures require a supported matching official MaterialX nodedef");
    }
    if (!is_namespaced_identifier(t.texcoord_primvar)) {
        r.error("texture.texcoord_primvar", prim.path, "texture coordinate primvar must be a valid namespaced identifier");
    }
    if (!M::all_finite(t.value) || M::any_negative(t.value)) {
        r.error("texture.value", prim.path, "texture values must be finite and non-negative");
    }
    if (t.output_type == SceneMaterialValueType::float_) {
        // Eigen's isConstant(x, 1e-12): |v - x| <= 1e-12 * min(|v|, |x|) per component
        const auto near = [](double v, double x) { return std::abs(v - x) <= 1e-12 * std::min(std::abs(v), std::abs(x)); };
        const bool replicated = near(t.value[1], t.value[0]) && near(t.value[2], t.value[0]);
        if (!replicated || t.color_space != SceneColorSpace::raw) {
            r.error("texture.scalar_contract", prim.path, "float textures require replicated scalar values and raw color space");
        }
    }
    if (!std::isfinite(t.scale) || t.scale <= 0.0) r.error("texture.scale", prim.path, "texture scale must be finite and positive");
    if (t.node == SceneTextureNode::checkerboard) {
        check_texture_ref(r, prims, prim.path, t.even_texture_path, "texture.checker.even_reference");
        check_texture_ref(r, prims, prim.path, t.odd_texture_path, "texture.checker.odd_reference");
        if (t.even_texture_path == prim.path || t.odd_texture_path == prim.path) {
            r.error("texture.checker.self_reference", prim.path, "checkerboard inputs must not reference the checkerboard itself");
        }
    } else if (!t.even_texture_path.empty() || !t.odd_texture_path.empty()) {
        r.error("texture.input_unexpected", prim.path, "only checkerboard textures may carry even and odd texture inputs");
    }
    if (t.node == SceneTextureNode::image) {
        if (prim.asset_references.size() != 1) {
            r.error("texture.image.asset", prim.path, "MaterialX image textures require exactly one asset reference");
        }
    } else if (!prim.asset_references.empty()) {
        r.error("texture.asset_unexpected", prim.path, "only image textures may carry image asset references");
    }
}

// The inputs of the OpenPBR 1.1.1 surface node definition and their types.
std::optional<SceneMaterialValueType> open_pbr_input_type(std::string_view name) {
    using T = SceneMaterialValueType;
    static const std::unordered_map<std::string_view, T> inputs {
        {"base_weight", T::float_}, {"base_color", T::color3}, {"base_diffuse_roughness", T::float_},
        {"base_metalness", T::float_}, {"specular_weight", T::float_}, {"specular_color", T::color3},
        {"specular_roughness", T::float_}, {"specular_ior", T::float_}, {"specular_roughness_anisotropy", T::float_},
        {"transmission_weight", T::float_}, {"transmission_color", T::color3}, {"transmission_depth", T::float_},
        {"transmission_scatter", T::color3}, {"transmission_scatter_anisotropy", T::float_},
        {"transmission_dispersion_scale", T::float_}, {"transmission_dispersion_abbe_number", T::float_},
        {"subsurface_weight", T::float_}, {"subsurface_color", T::color3}, {"subsurface_radius", T::float_},
        {"subsurface_radius_scale", T::color3}, {"subsurface_scatter_anisotropy", T::float_},
        {"fuzz_weight", T::float_}, {"fuzz_color", T::color3}, {"fuzz_roughness", T::float_},
        {"coat_weight", T::float_}, {"coat_color", T::color3}, {"coat_roughness", T::float_},
        {"coat_roughness_anisotropy", T::float_}, {"coat_ior", T::float_}, {"coat_darkening", T::float_},
        {"thin_film_weight", T::float_}, {"thin_film_thickness", T::float_}, {"thin_film_ior", T::float_},
        {"emission_luminance", T::float_}, {"emission_color", T::color3}, {"geometry_opacity", T::float_},
        {"geometry_normal", T::vector3}, {"geometry_coat_normal", T::vector3}, {"geometry_tangent", T::vector3},
        {"geometry_coat_tangent", T::vector3},
    };
    const auto it = inputs.find(name);
    return it == inputs.end() ? std::nullopt : std::optional<T>(it->second);
}

void check_open_pbr_numbers(Report& r, const SceneOpenPbrSurface& m, std::string_view path) {
    const auto in = [](double v, double lo, double hi) { return std::isfinite(v) && v >= lo && v <= hi; };
    const auto all_in = [&](std::initializer_list<double> vs, double lo, double hi) {
        return std::all_of(vs.begin(), vs.end(), [&](double v) { return in(v, lo, hi); });
    };
    if (!all_in({m.base_weight, m.base_metalness, m.transmission_weight, m.transmission_dispersion_scale,
                    m.subsurface_weight, m.fuzz_weight, m.coat_weight, m.coat_darkening, m.thin_film_weight,
                    m.geometry_opacity},
            0.0, 1.0)) {
        r.error("material.open_pbr.weight", path, "OpenPBR weights, metalness, darkening, and opacity must be in [0, 1]");
    }
    if (!all_in({m.base_diffuse_roughness, m.specular_roughness, m.specular_roughness_anisotropy, m.fuzz_roughness,
                    m.coat_roughness, m.coat_roughness_anisotropy},
            0.0, 1.0)) {
        r.error("material.open_pbr.roughness", path, "OpenPBR roughness and roughness anisotropy must be in [0, 1]");
    }
    if (!all_in({m.transmission_scatter_anisotropy, m.subsurface_scatter_anisotropy}, -1.0, 1.0)) {
        r.error("material.open_pbr.anisotropy", path, "OpenPBR scatter anisotropy must be in [-1, 1]");
    }
    for (const Vec3* c : {&m.base_color, &m.specular_color, &m.transmission_color, &m.transmission_scatter,
             &m.subsurface_color, &m.subsurface_radius_scale, &m.fuzz_color, &m.coat_color, &m.emission_color}) {
        if (!M::all_finite(*c) || M::any_negative(*c)) {
            r.error("material.open_pbr.color", path, "OpenPBR colors must be finite and non-negative; emission may be HDR");
            break;
        }
    }
    const double inf = std::numeric_limits<double>::infinity();
    if (!all_in({m.specular_weight, m.transmission_depth, m.subsurface_radius, m.thin_film_thickness, m.emission_luminance},
            0.0, inf)) {
        r.error("material.open_pbr.nonnegative", path,
            "OpenPBR unbounded weights, depths, radii, and luminance must be finite and non-negative");
    }
    for (double v : {m.specular_ior, m.transmission_dispersion_abbe_number, m.coat_ior, m.thin_film_ior}) {
        if (!std::isfinite(v) || v <= 0.0) {
            r.error("material.open_pbr.positive", path, "OpenPBR IOR and Abbe number inputs must be finite and positive");
            break;
        }
    }
}

void check_connections(Report& r, const SceneOpenPbrSurface& m, std::string_view path, const PrimIndex& prims) {
    std::unordered_set<std::string> seen;
    for (const SceneMaterialConnection& c : m.connections) {
        const std::optional<SceneMaterialValueType> want = open_pbr_input_type(c.input_name);
        if (!want) {
            r.error("material.connection.input_name", path, "connection does not name an OpenPBR 1.1.1 input: " + c.input_name);
            continue;
        }
        if (!seen.insert(c.input_name).second) {
            r.error("material.connection.duplicate", path, "an OpenPBR input may have at most one texture connection");
        }
        if (c.input_type != *want) {
            r.error("material.connection.input_type", path, "connected input type does not match the official OpenPBR node definition");
        }
        const ScenePrim* tex = texture_prim(prims, c.texture_path);
        if (!tex) {
            check_texture_ref(r, prims, path, c.texture_path, "material.connection.texture_reference");
            continue;
        }
        const SceneMaterialValueType out = tex->texture->output_type;
        const bool direct = out == c.input_type && c.channel == SceneTextureChannel::rgb;
        const bool extract = c.input_type == SceneMaterialValueType::float_ && out == SceneMaterialValueType::color3 &&
                             c.channel != SceneTextureChannel::rgb;
        if (!direct && !extract) {
            r.error("material.connection.output_type", path, "texture output and selected channel do not match the connected input");
        }
    }
}

void check_material(Report& r, const SceneMaterial& material, std::string_view path, const PrimIndex& prims) {
    if (const auto* m = std::get_if<SceneOpenPbrSurface>(&material)) {
        if (m->version != kOpenPbrVersion) {
            r.error("material.open_pbr.version", path, "SceneIR v2 currently requires the OpenPBR 1.1.1 contract");
        }
        check_open_pbr_numbers(r, *m, path);
        for (const std::string* g : {&m->geometry_normal_default_geomprop, &m->geometry_coat_normal_default_geomprop,
                 &m->geometry_tangent_default_geomprop, &m->geometry_coat_tangent_default_geomprop}) {
            if (!is_namespaced_identifier(*g)) {
                r.error("material.open_pbr.geometry_default", path,
                    "OpenPBR normal and tangent defaults must name valid geometry properties");
                break;
            }
        }
        check_connections(r, *m, path, prims);
        const SceneMaterialXDisplacement& d = m->displacement;
        if (!std::isfinite(d.scale) || !std::isfinite(d.scalar_value) || !M::all_finite(d.vector_value)) {
            r.error("material.displacement.value", path, "MaterialX displacement values and scale must be finite");
        }
        if (d.type == SceneMaterialXDisplacementType::none) {
            if (!d.texture_path.empty()) {
                r.error("material.displacement.unexpected_texture", path,
                    "a disabled displacement shader must not have a texture input");
            }
        } else if (!d.texture_path.empty()) {
            check_texture_ref(r, prims, path, d.texture_path, "material.displacement.texture_reference");
        }
    } else {
        const auto& v = std::get<SceneIsotropicVolumeMaterial>(material);
        if (!M::all_finite(v.scattering_color) || M::any_negative(v.scattering_color)) {
            r.error("material.volume.scattering_color", path, "volume scattering color must be finite and non-negative");
        }
        if (!std::isfinite(v.scattering_anisotropy) || v.scattering_anisotropy < -1.0 || v.scattering_anisotropy > 1.0) {
            r.error("material.volume.anisotropy", path, "volume scattering anisotropy must be in [-1, 1]");
        }
        if (!v.scattering_color_texture_path.empty()) {
            check_texture_ref(r, prims, path, v.scattering_color_texture_path, "material.volume.texture_reference");
        }
    }
}

void check_light(Report& r, const SceneLight& l, std::string_view path) {
    if (!M::all_finite(l.color) || M::any_negative(l.color)) {
        r.error("light.color", path, "light color must be finite and non-negative in the rendering color space");
    }
    if (!std::isfinite(l.intensity) || l.intensity < 0.0) r.error("light.intensity", path, "light intensity must be finite and non-negative");
    if (!std::isfinite(l.exposure)) r.error("light.exposure", path, "light exposure must be finite");
    if (std::isfinite(l.intensity) && std::isfinite(l.exposure) && !std::isfinite(scene_light_exposed_intensity(l))) {
        r.error("light.exposed_intensity", path, "light intensity multiplied by exp2(exposure) must remain finite");
    }
    if (!std::isfinite(l.color_temperature_kelvin) || l.color_temperature_kelvin < 1000.0 || l.color_temperature_kelvin > 10000.0) {
        r.error("light.color_temperature", path, "light color temperature must be between 1000 and 10000 kelvin");
    }
    if (!std::isfinite(l.diffuse) || l.diffuse < 0.0 || !std::isfinite(l.specular) || l.specular < 0.0) {
        r.error("light.response_multiplier", path, "light diffuse and specular multipliers must be finite and non-negative");
    }
    const auto pos = [](double v) { return std::isfinite(v) && v > 0.0; };
    using L = SceneLightType;
    if ((l.type == L::sphere || l.type == L::disk || l.type == L::cylinder) && !pos(l.radius)) {
        r.error("light.radius", path, "sphere, disk, and cylinder light radius must be finite and positive");
    }
    if (l.type == L::rect && (!pos(l.width) || !pos(l.height))) {
        r.error("light.rect_size", path, "rect light width and height must be finite and positive");
    }
    if (l.type == L::cylinder && !pos(l.length)) r.error("light.cylinder_length", path, "cylinder light length must be finite and positive");
    if (l.type == L::distant && !std::isfinite(l.angle_degrees)) r.error("light.distant_angle", path, "distant light angle must be finite");
    if (l.treat_as_point && l.type != L::sphere) r.error("light.treat_as_point", path, "only sphere lights may be treated as point lights");
    if (l.treat_as_line && l.type != L::cylinder) r.error("light.treat_as_line", path, "only cylinder lights may be treated as line lights");
}

const ScenePrim& require_prim(const SceneIRv2& scene, std::string_view path) {
    const ScenePrim* p = scene.find_prim(path);
    if (!p) throw std::out_of_range("scene prim not found: " + std::string(path));
    return *p;
}

}  // namespace

std::size_t SceneIRv2::add_prim(ScenePrim prim) {
    const std::size_t index = prims_.size();
    first_prim_by_path_.try_emplace(prim.path, index);
    prims_.push_back(std::move(prim));
    return index;
}

const ScenePrim* SceneIRv2::find_prim(std::string_view path) const {
    const auto it = first_prim_by_path_.find(std::string(path));
    return it == first_prim_by_path_.end() ? nullptr : &prims_[it->second];
}

// "/A/B_1": absolute, '/'-separated identifiers, no trailing separator
bool is_valid_scene_prim_path(std::string_view path) {
    if (path.size() < 2 || path.front() != '/' || path.back() == '/') return false;
    size_t start = 1;
    for (;;) {
        const size_t sep = path.find('/', start);
        const size_t end = sep == std::string_view::npos ? path.size() : sep;
        if (!is_identifier(path.substr(start, end - start))) return false;
        if (sep == std::string_view::npos) return true;
        start = sep + 1;
    }
}

std::string parent_scene_prim_path(std::string_view path) {
    if (!is_valid_scene_prim_path(path)) throw std::invalid_argument("invalid scene prim path: " + std::string(path));
    const size_t sep = path.find_last_of('/');
    return sep == 0 ? "/" : std::string(path.substr(0, sep));
}

std::vector<SceneDiagnostic> validate_scene_ir_v2(const SceneIRv2& scene) {
    Report r;
    const SceneStageMetadata& st = scene.stage_metadata();
    const auto pos = [](double v) { return std::isfinite(v) && v > 0.0; };
    if (!pos(st.meters_per_unit)) r.error("stage.meters_per_unit", {}, "meters_per_unit must be finite and positive");
    if (!st.right_handed) r.error("stage.handedness", {}, "OpenUSD geometry stages use right-handed coordinates");
    if (!pos(st.time_codes_per_second)) r.error("stage.time_codes_per_second", {}, "time_codes_per_second must be finite and positive");
    if (!pos(st.frames_per_second)) r.error("stage.frames_per_second", {}, "frames_per_second must be finite and positive");
    if (st.start_time_code && !std::isfinite(*st.start_time_code)) r.error("stage.start_time_code", {}, "start_time_code must be finite");
    if (st.end_time_code && !std::isfinite(*st.end_time_code)) r.error("stage.end_time_code", {}, "end_time_code must be finite");
    if (st.start_time_code && st.end_time_code && *st.start_time_code > *st.end_time_code) {
        r.error("stage.time_range", {}, "start_time_code must not exceed end_time_code");
    }

    PrimIndex prims;
    for (const ScenePrim& p : scene.prims()) {
        if (!is_valid_scene_prim_path(p.path)) {
            r.error("prim.path.invalid", p.path, "prim path must be an absolute ASCII prim path");
        } else if (!prims.emplace(p.path, &p).second) {
            r.error("prim.path.duplicate", p.path, "prim path must be unique");
        }
    }
    if (!is_valid_scene_prim_path(st.default_prim_path)) {
        r.error("stage.default_prim_path", st.default_prim_path, "default prim must be an absolute prim path");
    } else {
        if (parent_scene_prim_path(st.default_prim_path) != "/") {
            r.error("stage.default_prim_not_root", st.default_prim_path, "default prim must be a root prim");
        }
        if (!prims.contains(st.default_prim_path)) {
            r.error("stage.default_prim_missing", st.default_prim_path, "default prim path does not resolve");
        }
    }

    for (const ScenePrim& p : scene.prims()) {
        if (!is_valid_scene_prim_path(p.path)) continue;
        const std::string parent = parent_scene_prim_path(p.path);
        if (parent != "/" && !prims.contains(parent)) r.error("prim.parent.missing", p.path, "parent prim does not exist: " + parent);
        check_transform(r, p.local_to_parent, p.path);
        std::optional<double> prev;
        for (const SceneTransformSample& s : p.transform_samples) {
            if (!std::isfinite(s.time_code)) {
                r.error("xform.sample_time.non_finite", p.path, "transform sample time must be finite");
            } else if (prev && s.time_code <= *prev) {
                r.error("xform.sample_time.order", p.path, "transform sample times must be strictly increasing");
            }
            prev = s.time_code;
            check_transform(r, s.local_to_parent, p.path);
        }

        if (p.kind == ScenePrimKind::geometry_prototype) {
            if (!p.geometry) {
                r.error("geometry.payload_missing", p.path, "geometry prototype requires a geometry payload");
            } else if (const auto* sphere = std::get_if<SceneSphereGeometry>(&*p.geometry)) {
                if (!M::all_finite(sphere->center) || !std::isfinite(sphere->radius) || sphere->radius <= 0.0) {
                    r.error("geometry.sphere.invalid", p.path,
                        "sphere center must be finite and radius must be finite and positive");
                }
            } else {
                check_mesh(r, std::get<SceneMeshGeometry>(*p.geometry), p.path, prims);
            }
        } else if (p.geometry) {
            r.error("geometry.payload_unexpected", p.path, "only geometry prototype prims may carry geometry payloads");
        }

        if (p.kind == ScenePrimKind::camera) {
            if (!p.camera) {
                r.error("camera.payload_missing", p.path, "camera prim requires a camera payload");
            } else {
                check_camera(r, *p.camera, p.path);
            }
        } else if (p.camera) {
            r.error("camera.payload_unexpected", p.path, "only camera prims may carry camera payloads");
        }

        if (p.kind == ScenePrimKind::light) {
            if (!p.light) {
                r.error("light.payload_missing", p.path, "light prim requires a light payload");
            } else if (p.light->type == SceneLightType::geometry) {
                r.error("light.payload_kind", p.path, "geometry light payloads must be applied to surface prims");
            }
        } else if (p.kind == ScenePrimKind::surface && p.light) {
            if (p.light->type != SceneLightType::geometry) {
                r.error("light.payload_kind", p.path, "surface prims may only carry geometry light payloads");
            }
        } else if (p.light) {
            r.error("light.payload_unexpected", p.path, "only light and surface prims may carry light payloads");
        }
        if (p.light) check_light(r, *p.light, p.path);

        if (p.kind == ScenePrimKind::texture) {
            if (!p.texture) {
                r.error("texture.payload_missing", p.path, "texture prim requires a MaterialX texture payload");
            } else {
                check_texture(r, *p.texture, p, prims);
            }
        } else if (p.texture) {
            r.error("texture.payload_unexpected", p.path, "only texture prims may carry texture payloads");
        }

        if (p.kind == ScenePrimKind::material) {
            if (!p.material) {
                r.error("material.payload_missing", p.path, "material prim requires an OpenPBR or volume payload");
            } else {
                check_material(r, *p.material, p.path, prims);
            }
        } else if (p.material) {
            r.error("material.payload_unexpected", p.path, "only material prims may carry material payloads");
        }

        for (const SceneAssetReference& a : p.asset_references) check_asset(r, a, p.path);

        if (p.kind == ScenePrimKind::surface || p.kind == ScenePrimKind::volume) {
            const auto proto = prims.find(p.prototype_path);
            if (proto == prims.end() || proto->second->kind != ScenePrimKind::geometry_prototype) {
                r.error("reference.prototype", p.path, "surface or volume prototype path does not resolve to a geometry prototype");
            }
            if (!is_material_prim(prims, p.material_path)) {
                r.error("reference.material", p.path, "surface or volume material path does not resolve to a material");
            }
        }
        if (p.kind == ScenePrimKind::volume && (!p.volume_density || !pos(*p.volume_density))) {
            r.error("volume.density", p.path, "volume density must be finite and positive");
        }
    }
    return std::move(r.out);
}

void require_valid_scene_ir_v2(const SceneIRv2& scene) {
    for (const SceneDiagnostic& d : validate_scene_ir_v2(scene)) {
        if (d.severity == SceneDiagnosticSeverity::error) throw std::invalid_argument(d.code + ": " + d.message);
    }
}

bool has_scene_diagnostic(const std::vector<SceneDiagnostic>& diagnostics, std::string_view code) {
    return std::any_of(diagnostics.begin(), diagnostics.end(), [&](const SceneDiagnostic& d) { return d.code == code; });
}

// Time samples are sorted by time code: before the first or after the last,
// the end sample; between two, the lower one (held) or the component-wise
// blend with the last row reset to [0 0 0 1] (linear).
Mat4 sample_scene_local_transform(const ScenePrim& prim, double time_code, SceneTimeInterpolation interpolation) {
    const auto& s = prim.transform_samples;
    if (s.empty()) return prim.local_to_parent;
    const auto hi = std::lower_bound(s.begin(), s.end(), time_code,
        [](const SceneTransformSample& x, double t) { return x.time_code < t; });
    if (hi == s.begin()) return hi->local_to_parent;
    if (hi == s.end()) return s.back().local_to_parent;
    if (hi->time_code == time_code) return hi->local_to_parent;
    const SceneTransformSample& lo = *(hi - 1);
    if (interpolation == SceneTimeInterpolation::held) return lo.local_to_parent;
    const double a = (time_code - lo.time_code) / (hi->time_code - lo.time_code);
    Mat4 m {};
    for (size_t i = 0; i < 16; ++i) m[i] = (1.0 - a) * lo.local_to_parent[i] + a * hi->local_to_parent[i];
    m[12] = 0.0;
    m[13] = 0.0;
    m[14] = 0.0;
    m[15] = 1.0;
    return m;
}

// Root-to-leaf product of the local transforms; a prim with reset_xform_stack
// starts over from its own.
Mat4 compute_scene_world_transform(const SceneIRv2& scene, std::string_view prim_path, double time_code) {
    std::vector<const ScenePrim*> chain;
    for (std::string path(prim_path); path != "/"; path = parent_scene_prim_path(path)) chain.push_back(&require_prim(scene, path));
    Mat4 world = kIdentity4;
    for (auto it = chain.rbegin(); it != chain.rend(); ++it) {
        const Mat4 local = sample_scene_local_transform(**it, time_code, scene.stage_metadata().interpolation);
        world = (*it)->reset_xform_stack ? local : M::mul(world, local);
    }
    return world;
}

bool compute_scene_visibility(const SceneIRv2& scene, std::string_view prim_path) {
    for (std::string path(prim_path); path != "/"; path = parent_scene_prim_path(path)) {
        if (require_prim(scene, path).visibility == SceneVisibility::invisible) return false;
    }
    return true;
}

ScenePurpose compute_scene_purpose(const SceneIRv2& scene, std::string_view prim_path) {
    for (std::string path(prim_path); path != "/"; path = parent_scene_prim_path(path)) {
        const ScenePrim& p = require_prim(scene, path);
        if (p.authored_purpose) return *p.authored_purpose;
    }
    return ScenePurpose::default_;
}

double scene_light_exposed_intensity(const SceneLight& light) { return light.intensity * std::exp2(light.exposure); }

SceneLightIntensityUnit scene_light_intensity_unit(const SceneLight& light) {
    return light.type == SceneLightType::distant && light.normalize ? SceneLightIntensityUnit::lux : SceneLightIntensityUnit::nit;
}

}  // namespace rtgb::scene
