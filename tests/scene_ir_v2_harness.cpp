// Self-checking C++ cases of the SceneIR v2 layer (include/rtgb_scene_ir_v2.hpp)
// and of the SceneIR v1 compatibility adapter (include/rtgb_scene_ir.hpp),
// linked against librtgb.so; run by tests/test_scene_ir_v2.py.
//
// The reference's own expectations come first: tests/test_realtime_scene_adapter.cpp:43-131
// (a textured OpenPBR panel with two material subsets) and
// tests/test_analytic_light_compiler.cpp:35-219 (every light type, normalisation,
// exposure, colour temperature and the rejected cases). The remaining cases
// cover the validator's codes, time-sampled and reset transforms,
// visibility/purpose inheritance, winding, normal transformation and the
// scene file round trip.
//
// `harness DIR` runs the cases; `harness DIR --write-scene FILE` also lowers
// the parity scene (meshes, spheres, instances, subsets, checker / image /
// constant textures bound to OpenPBR inputs, all analytic light types) and
// writes it with rtgb_host_scene_save for the GPU parity test;
// `harness DIR --instanced-gpu` (needs a GPU) also prepares the scene through
// rtgb_prepare_scene_instanced and compares it with the flat lowering.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <functional>
#include <numbers>
#include <stdexcept>
#include <string>
#include <vector>

#include "cli/png_writer.h"
#include "rtgb_scene_ir.hpp"
#include "rtgb_scene_ir_v2.hpp"

using namespace rtgb::scene;

static int g_failures = 0;
static int g_checks = 0;

#define CHECK(cond, what)                                                        \
    do {                                                                         \
        ++g_checks;                                                              \
        if (!(cond)) {                                                           \
            ++g_failures;                                                        \
            std::fprintf(stderr, "FAILED %s:%d %s\n", __FILE__, __LINE__, what); \
        }                                                                        \
    } while (0)

static bool near(double a, double b, double tol) { return std::abs(a - b) <= tol; }

static bool near3(const float* a, const Vec3& b, double tol) {
    return near(a[0], b[0], tol) && near(a[1], b[1], tol) && near(a[2], b[2], tol);
}

static bool near3(const Vec3& a, const Vec3& b, double tol) {
    return near(a[0], b[0], tol) && near(a[1], b[1], tol) && near(a[2], b[2], tol);
}

// expects fn() to throw std::invalid_argument whose message contains `fragment`
static void expect_invalid(const std::function<void()>& fn, const std::string& fragment, const char* what) {
    ++g_checks;
    try {
        fn();
    } catch (const std::invalid_argument& e) {
        if (std::string(e.what()).find(fragment) != std::string::npos) return;
        std::fprintf(stderr, "FAILED %s: message '%s' lacks '%s'\n", what, e.what(), fragment.c_str());
        ++g_failures;
        return;
    }
    std::fprintf(stderr, "FAILED %s: no std::invalid_argument\n", what);
    ++g_failures;
}

static rtgb_scene view_of(const HostScenePtr& s) {
    rtgb_scene v {};
    rtgb_host_scene_view(s.get(), &v);
    return v;
}

static Mat4 translate(double x, double y, double z) {
    Mat4 m = kIdentity4;
    m[3] = x;
    m[7] = y;
    m[11] = z;
    return m;
}

static Mat4 scale_translate(const Vec3& s, const Vec3& t = {0.0, 0.0, 0.0}) {
    Mat4 m = kIdentity4;
    m[0] = s[0];
    m[5] = s[1];
    m[10] = s[2];
    m[3] = t[0];
    m[7] = t[1];
    m[11] = t[2];
    return m;
}

static ScenePrim prim(std::string path, ScenePrimKind kind = ScenePrimKind::scope) {
    ScenePrim p;
    p.path = std::move(path);
    p.kind = kind;
    return p;
}

// tests/test_realtime_scene_adapter.cpp:43-131
static void reference_adapter_case() {
    SceneIRv2 s;
    s.add_prim(prim("/World"));
    ScenePrim tex = prim("/World/BaseTexture", ScenePrimKind::texture);
    tex.texture = SceneTexture {};
    tex.texture->value = {0.2, 0.4, 0.8};
    s.add_prim(tex);
    SceneOpenPbrSurface blue;
    blue.connections.push_back({"base_color", SceneMaterialValueType::color3, "/World/BaseTexture", SceneTextureChannel::rgb});
    ScenePrim mb = prim("/World/Blue", ScenePrimKind::material);
    mb.material = SceneMaterial {blue};
    s.add_prim(mb);
    SceneOpenPbrSurface metal;
    metal.base_metalness = 1.0;
    ScenePrim mm = prim("/World/Metal", ScenePrimKind::material);
    mm.material = SceneMaterial {metal};
    s.add_prim(mm);
    s.add_prim(prim("/World/Prototypes"));
    SceneMeshGeometry panel;
    panel.points = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {1.0, 1.0, 0.0}, {0.0, 1.0, 0.0}};
    panel.face_vertex_counts = {3, 3};
    panel.face_vertex_indices = {0, 1, 2, 0, 2, 3};
    ScenePrimvar normals;
    normals.name = "normals";
    normals.interpolation = ScenePrimvarInterpolation::face_varying;
    normals.role = ScenePrimvarRole::normal;
    normals.values = std::vector<Vec3f>(6, Vec3f {0.0f, 0.0f, 1.0f});
    ScenePrimvar st;
    st.name = "st";
    st.interpolation = ScenePrimvarInterpolation::face_varying;
    st.role = ScenePrimvarRole::texcoord;
    st.values = std::vector<Vec2f> {{0.0f, 0.0f}, {1.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, 1.0f}};
    panel.primvars = {normals, st};
    panel.material_subset_family_type = SceneMaterialSubsetFamilyType::partition;
    panel.material_subsets = {{"blue", {0}, "/World/Blue"}, {"metal", {1}, "/World/Metal"}};
    ScenePrim proto = prim("/World/Prototypes/Panel", ScenePrimKind::geometry_prototype);
    proto.geometry = SceneGeometry {panel};
    s.add_prim(proto);
    ScenePrim surf = prim("/World/Panel", ScenePrimKind::surface);
    surf.local_to_parent = translate(2.0, 0.0, 0.0);
    surf.prototype_path = "/World/Prototypes/Panel";
    surf.material_path = "/World/Blue";
    s.add_prim(surf);

    const HostScenePtr packed = adapt_scene_ir_v2_to_realtime(s);
    const rtgb_scene v = view_of(packed);
    CHECK(v.texture_count == 1, "native v2 texture table");
    CHECK(v.material_count == 2, "native v2 material table");
    CHECK(v.triangle_count == 2, "native v2 mesh triangulation");
    CHECK(v.triangles[0].material_index == 0, "native v2 fallback subset material");
    CHECK(v.triangles[1].material_index == 1, "native v2 second subset material");
    CHECK(near(v.triangles[0].p0[0], 2.0, 1e-9), "native v2 world transform");
    CHECK(v.triangles[0].has_vertex_normals == 1, "native v2 vertex normals");
    CHECK(v.triangles[0].has_texcoords == 1, "native v2 texcoords");
    CHECK(near(v.triangles[0].uv2[1], 1.0, 1e-9), "native v2 face-varying uv");
    CHECK(v.materials[0].type == RTGB_MATERIAL_OPENPBR && v.materials[0].openpbr_index == 0, "OpenPBR material record");
    CHECK(v.openpbr_materials[0].color_texture[0] == 0, "native v2 connected OpenPBR texture binding");
    CHECK(v.openpbr_materials[0].color_space[0] == 1, "linear sRGB source colour space");
    CHECK(v.openpbr_materials[1].base_metalness == 1.0f && v.openpbr_materials[1].color_texture[0] == -1, "metal constants");
    CHECK(v.textures[0].type == RTGB_TEXTURE_CONSTANT && near3(v.textures[0].color, {0.2, 0.4, 0.8}, 1e-7), "constant texture");
    CHECK(near3(v.triangles[0].n1, {0.0, 0.0, 1.0}, 0.0), "face-varying normal");
}

static ScenePrim light_prim(std::string path, const SceneLight& l, const Mat4& m = kIdentity4) {
    ScenePrim p = prim(std::move(path), ScenePrimKind::light);
    p.local_to_parent = m;
    p.light = l;
    return p;
}

static SceneLight light_of(SceneLightType t) {
    SceneLight l;
    l.type = t;
    return l;
}

// tests/test_analytic_light_compiler.cpp:35-219
static void reference_light_case() {
    const double pi = std::numbers::pi;
    SceneIRv2 s;
    s.add_prim(prim("/World"));
    SceneLight sphere = light_of(SceneLightType::sphere);
    sphere.radius = 0.5;
    sphere.intensity = 4.0;
    sphere.normalize = true;
    s.add_prim(light_prim("/World/Sphere", sphere, scale_translate({2.0, 2.0, 2.0}, {1.0, 2.0, 3.0})));
    SceneLight disk = light_of(SceneLightType::disk);
    disk.radius = 1.0;
    disk.intensity = 6.0 * pi;
    disk.normalize = true;
    s.add_prim(light_prim("/World/Disk", disk, scale_translate({2.0, 3.0, 1.0})));
    SceneLight rect = light_of(SceneLightType::rect);
    rect.width = 2.0;
    rect.height = 3.0;
    rect.intensity = 6.0;
    rect.normalize = true;
    s.add_prim(light_prim("/World/Rect", rect));
    SceneLight cyl = light_of(SceneLightType::cylinder);
    cyl.radius = 1.0;
    cyl.length = 2.0;
    cyl.intensity = 16.0 * pi;
    cyl.normalize = true;
    s.add_prim(light_prim("/World/Cylinder", cyl, scale_translate({2.0, 2.0, 2.0})));
    SceneLight distant = light_of(SceneLightType::distant);
    distant.angle_degrees = 60.0;
    distant.intensity = pi / 4.0;
    distant.normalize = true;
    s.add_prim(light_prim("/World/Distant", distant));
    SceneLight dome = light_of(SceneLightType::dome);
    dome.intensity = 2.0;
    dome.exposure = 1.0;
    s.add_prim(light_prim("/World/Dome", dome));
    ScenePrim hidden = light_prim("/World/Hidden", light_of(SceneLightType::sphere));
    hidden.visibility = SceneVisibility::invisible;
    s.add_prim(hidden);
    ScenePrim proxy = light_prim("/World/Proxy", light_of(SceneLightType::sphere));
    proxy.authored_purpose = ScenePurpose::proxy;
    s.add_prim(proxy);

    const std::vector<AnalyticLightDesc> lights = compile_analytic_lights(s);
    CHECK(lights.size() == 6, "only visible render-purpose intrinsic lights compile");
    if (lights.size() != 6) return;
    CHECK(lights[0].type == AnalyticLightType::sphere, "sphere type");
    CHECK(near3(lights[0].position, {1.0, 2.0, 3.0}, 1e-12), "sphere world position");
    CHECK(near(lights[0].world_area, 4.0 * pi, 1e-12), "sphere world-space area");
    CHECK(near3(lights[0].radiance, {1.0 / pi, 1.0 / pi, 1.0 / pi}, 1e-12), "normalized sphere radiance");
    CHECK(near(lights[1].world_area, 6.0 * pi, 1e-12), "affine disk world-space area");
    CHECK(near3(lights[1].radiance, {1.0, 1.0, 1.0}, 1e-12), "normalized disk radiance");
    CHECK(near(lights[2].world_area, 6.0, 1e-12), "rect world-space area");
    CHECK(near(lights[3].world_area, 16.0 * pi, 1e-12), "cylinder lateral area excludes end caps");
    CHECK(near(lights[4].cos_theta_max, std::cos(pi / 6.0), 1e-12), "distant angular radius");
    CHECK(near3(lights[4].radiance, {1.0, 1.0, 1.0}, 1e-12), "normalized distant radiance");
    CHECK(near3(lights[5].radiance, {4.0, 4.0, 4.0}, 1e-12), "dome exposure radiance");
    double sum = 0.0;
    for (const AnalyticLightDesc& l : lights) {
        CHECK(l.selection_pdf > 0.0, "compiled light has positive selection PDF");
        sum += l.selection_pdf;
    }
    CHECK(near(sum, 1.0, 1e-12), "analytic-light selection PDFs normalize");
    CHECK(near(lights.back().cdf, 1.0, 1e-12), "analytic-light CDF closes exactly");

    // the packed table of the realtime scene
    const HostScenePtr packed = adapt_scene_ir_v2_to_realtime(s);
    const rtgb_scene v = view_of(packed);
    CHECK(v.analytic_light_count == 6, "realtime scene carries the analytic-light table");
    CHECK(near(v.analytic_lights[0].world_area, lights[0].world_area, 1e-5), "packed sphere area");
    CHECK(near(v.analytic_lights[4].cos_theta_max, lights[4].cos_theta_max, 1e-6), "packed distant cone");
    CHECK(v.analytic_lights[5].cdf == 1.0f, "packed analytic CDF closes exactly");
    CHECK(near3(v.analytic_lights[1].basis_x, {2.0, 0.0, 0.0}, 0.0) && near3(v.analytic_lights[1].basis_y, {0.0, 3.0, 0.0}, 0.0),
        "packed basis = columns of the light's linear transform");
    CHECK(v.analytic_lights[4].delta == 0 && v.analytic_lights[4].type == RTGB_ANALYTIC_DISTANT, "distant light record");

    SceneIRv2 warm_scene;
    warm_scene.add_prim(prim("/World"));
    SceneLight warm = light_of(SceneLightType::sphere);
    warm.enable_color_temperature = true;
    warm.color_temperature_kelvin = 3200.0;
    warm_scene.add_prim(light_prim("/World/Warm", warm));
    const Vec3 r = compile_analytic_lights(warm_scene).front().radiance;
    CHECK(r[0] > r[1] && r[1] > r[2], "OpenUSD blackbody color temperature warms red over blue");
    CHECK(near(r[0] * 0.2126 + r[1] * 0.7152 + r[2] * 0.0722, 1.0, 1e-6), "blackbody preserves luminance");

    const auto fails = [](ScenePrim p, const std::string& fragment, const char* what) {
        SceneIRv2 f;
        f.add_prim(prim("/World"));
        f.add_prim(std::move(p));
        expect_invalid([&] { (void)compile_analytic_lights(f); }, fragment, what);
    };
    ScenePrim textured = light_prim("/World/Textured", light_of(SceneLightType::dome));
    textured.asset_references.push_back({"studio.exr", "", ""});
    fails(textured, "textures are not supported yet", "textured dome rejected");
    fails(light_prim("/World/Stretched", light_of(SceneLightType::sphere), scale_translate({1.0, 2.0, 1.0})),
        "similarity transform", "stretched sphere rejected");
    SceneLight response = light_of(SceneLightType::rect);
    response.diffuse = 0.5;
    fails(light_prim("/World/Response", response), "diffuse/specular overrides", "response override rejected");

    // a delta distant light and the 6500 K white point
    SceneIRv2 d;
    d.add_prim(prim("/World"));
    SceneLight sun = light_of(SceneLightType::distant);
    sun.angle_degrees = 0.0;
    sun.intensity = 3.0;
    d.add_prim(light_prim("/World/Sun", sun));
    const AnalyticLightDesc sd = compile_analytic_lights(d).front();
    CHECK(sd.delta && sd.cos_theta_max == 1.0 && near(sd.selection_weight, 3.0, 1e-12), "delta distant light weight = luminance");
}

static bool has_code(const SceneIRv2& s, const char* code) { return has_scene_diagnostic(validate_scene_ir_v2(s), code); }

static SceneMeshGeometry quad_mesh() {
    SceneMeshGeometry m;
    m.points = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {1.0, 1.0, 0.0}, {0.0, 1.0, 0.0}};
    m.face_vertex_counts = {4};
    m.face_vertex_indices = {0, 1, 2, 3};
    return m;
}

// One prototype, one OpenPBR material and a surface instancing it.
static SceneIRv2 base_scene(const SceneMeshGeometry& mesh, const Mat4& xf = kIdentity4) {
    SceneIRv2 s;
    s.add_prim(prim("/World"));
    ScenePrim m = prim("/World/Mat", ScenePrimKind::material);
    m.material = SceneMaterial {SceneOpenPbrSurface {}};
    s.add_prim(m);
    ScenePrim g = prim("/World/Geo", ScenePrimKind::geometry_prototype);
    g.geometry = SceneGeometry {mesh};
    s.add_prim(g);
    ScenePrim surf = prim("/World/Surf", ScenePrimKind::surface);
    surf.local_to_parent = xf;
    surf.prototype_path = "/World/Geo";
    surf.material_path = "/World/Mat";
    s.add_prim(surf);
    return s;
}

static void validator_case() {
    CHECK(validate_scene_ir_v2(base_scene(quad_mesh())).empty(), "a well-formed scene has no diagnostics");
    {
        SceneIRv2 s = base_scene(quad_mesh());
        s.add_prim(prim("/World/Mat"));
        s.add_prim(prim("World/Bad"));
        s.add_prim(prim("/Orphan/Child"));
        s.stage_metadata().meters_per_unit = 0.0;
        CHECK(has_code(s, "prim.path.duplicate"), "prim.path.duplicate");
        CHECK(has_code(s, "prim.path.invalid"), "prim.path.invalid");
        CHECK(has_code(s, "prim.parent.missing"), "prim.parent.missing");
        CHECK(has_code(s, "stage.meters_per_unit"), "stage.meters_per_unit");
    }
    {
        SceneMeshGeometry m = quad_mesh();
        m.face_vertex_counts = {2, 2};
        SceneIRv2 s = base_scene(m);
        CHECK(has_code(s, "geometry.mesh.face_counts"), "geometry.mesh.face_counts");
        m = quad_mesh();
        m.face_vertex_indices = {0, 1, 2, 7};
        CHECK(has_code(base_scene(m), "geometry.mesh.vertex_index_range"), "geometry.mesh.vertex_index_range");
        m = quad_mesh();
        m.face_vertex_indices = {0, 1, 2};
        CHECK(has_code(base_scene(m), "geometry.mesh.topology_size"), "geometry.mesh.topology_size");
        m = quad_mesh();
        ScenePrimvar st;
        st.name = "st";
        st.role = ScenePrimvarRole::texcoord;
        st.interpolation = ScenePrimvarInterpolation::vertex;
        st.values = std::vector<Vec2f>(3, Vec2f {0.0f, 0.0f});
        m.primvars = {st};
        CHECK(has_code(base_scene(m), "geometry.primvar.domain_size"), "geometry.primvar.domain_size");
        m.primvars[0].values = std::vector<Vec3f>(4, Vec3f {0.0f, 0.0f, 0.0f});
        CHECK(has_code(base_scene(m), "geometry.primvar.role_type"), "geometry.primvar.role_type");
        m.primvars[0].values = std::vector<Vec2f>(2, Vec2f {0.0f, 0.0f});
        m.primvars[0].indices = {0, 1, 5, 0};
        CHECK(has_code(base_scene(m), "geometry.primvar.index_range"), "geometry.primvar.index_range");
        m = quad_mesh();
        m.material_subsets = {{"a", {0}, "/World/Mat"}, {"b", {0}, "/World/Nope"}};
        SceneIRv2 s2 = base_scene(m);
        CHECK(has_code(s2, "geometry.subset.overlap") && has_code(s2, "geometry.subset.material"), "subset overlap and material");
    }
    {
        SceneIRv2 s = base_scene(quad_mesh());
        ScenePrim t = prim("/World/Tex", ScenePrimKind::texture);
        t.texture = SceneTexture {};
        t.texture->node = SceneTextureNode::checkerboard;
        t.texture->node_definition = "ND_checkerboard_color3";
        t.texture->even_texture_path = "/World/Tex";
        t.texture->odd_texture_path = "/World/Missing";
        s.add_prim(t);
        CHECK(has_code(s, "texture.checker.self_reference"), "texture.checker.self_reference");
        CHECK(has_code(s, "texture.checker.odd_reference"), "texture.checker.odd_reference");
        ScenePrim img = prim("/World/Img", ScenePrimKind::texture);
        img.texture = SceneTexture {};
        img.texture->node = SceneTextureNode::image;
        img.texture->node_definition = "ND_image_color3";
        s.add_prim(img);
        CHECK(has_code(s, "texture.image.asset"), "texture.image.asset");
    }
    {
        SceneIRv2 s = base_scene(quad_mesh());
        SceneOpenPbrSurface bad;
        bad.base_weight = 1.5;
        bad.specular_ior = 0.0;
        bad.connections.push_back({"base_colour", SceneMaterialValueType::color3, "/World/Mat", SceneTextureChannel::rgb});
        bad.connections.push_back({"specular_roughness", SceneMaterialValueType::color3, "/World/Nope", SceneTextureChannel::rgb});
        ScenePrim m = prim("/World/Bad", ScenePrimKind::material);
        m.material = SceneMaterial {bad};
        s.add_prim(m);
        CHECK(has_code(s, "material.open_pbr.weight"), "material.open_pbr.weight");
        CHECK(has_code(s, "material.open_pbr.positive"), "material.open_pbr.positive");
        CHECK(has_code(s, "material.connection.input_name"), "material.connection.input_name");
        CHECK(has_code(s, "material.connection.input_type"), "material.connection.input_type");
        CHECK(has_code(s, "material.connection.texture_reference"), "material.connection.texture_reference");
        expect_invalid([&] { (void)adapt_scene_ir_v2_to_realtime(s); }, "material.open_pbr.weight", "adapter validates first");
    }
    {
        SceneIRv2 s = base_scene(quad_mesh());
        SceneLight l = light_of(SceneLightType::rect);
        l.width = -1.0;
        l.treat_as_point = true;
        s.add_prim(light_prim("/World/L", l));
        ScenePrim sl = prim("/World/Surf2", ScenePrimKind::surface);
        sl.prototype_path = "/World/Geo";
        sl.material_path = "/World/Geo";
        sl.light = light_of(SceneLightType::sphere);
        s.add_prim(sl);
        CHECK(has_code(s, "light.rect_size") && has_code(s, "light.treat_as_point"), "light shape codes");
        CHECK(has_code(s, "light.payload_kind") && has_code(s, "reference.material"), "surface light kind and material ref");
    }
    {
        Mat4 m = kIdentity4;
        m[12] = 1.0;
        SceneIRv2 s = base_scene(quad_mesh(), m);
        CHECK(has_code(s, "xform.non_affine"), "xform.non_affine");
        SceneIRv2 z = base_scene(quad_mesh(), scale_translate({0.0, 1.0, 1.0}));
        const auto d = validate_scene_ir_v2(z);
        CHECK(has_scene_diagnostic(d, "xform.singular") && d[0].severity == SceneDiagnosticSeverity::warning,
            "a singular transform is a warning");
    }
}

static void transform_case() {
    // time samples at t = 0 and 10 on the parent; held and linear lookups, ends clamp
    ScenePrim p = prim("/World");
    p.transform_samples = {{0.0, translate(0.0, 0.0, 0.0)}, {10.0, translate(10.0, 0.0, 0.0)}};
    CHECK(sample_scene_local_transform(p, 2.5, SceneTimeInterpolation::linear)[3] == 2.5, "linear sample");
    CHECK(sample_scene_local_transform(p, 2.5, SceneTimeInterpolation::held)[3] == 0.0, "held sample");
    CHECK(sample_scene_local_transform(p, -5.0, SceneTimeInterpolation::linear)[3] == 0.0, "before the first sample");
    CHECK(sample_scene_local_transform(p, 50.0, SceneTimeInterpolation::linear)[3] == 10.0, "after the last sample");
    CHECK(sample_scene_local_transform(p, 10.0, SceneTimeInterpolation::held)[3] == 10.0, "exact sample");

    SceneIRv2 s;
    s.add_prim(p);
    s.stage_metadata().start_time_code = 5.0;
    ScenePrim child = prim("/World/A");
    child.local_to_parent = translate(0.0, 1.0, 0.0);
    s.add_prim(child);
    ScenePrim reset = prim("/World/A/B");
    reset.local_to_parent = translate(0.0, 0.0, 3.0);
    reset.reset_xform_stack = true;
    s.add_prim(reset);
    ScenePrim leaf = prim("/World/A/B/C");
    leaf.local_to_parent = translate(1.0, 0.0, 0.0);
    leaf.visibility = SceneVisibility::inherited;
    s.add_prim(leaf);
    const Mat4 wa = compute_scene_world_transform(s, "/World/A", 5.0);
    CHECK(wa[3] == 5.0 && wa[7] == 1.0, "parent x child");
    const Mat4 wc = compute_scene_world_transform(s, "/World/A/B/C", 5.0);
    CHECK(wc[3] == 1.0 && wc[7] == 0.0 && wc[11] == 3.0, "reset_xform_stack drops the ancestors");

    SceneIRv2 v;
    v.add_prim(prim("/World"));
    ScenePrim hid = prim("/World/Hidden");
    hid.visibility = SceneVisibility::invisible;
    hid.authored_purpose = ScenePurpose::guide;
    v.add_prim(hid);
    v.add_prim(prim("/World/Hidden/Child"));
    CHECK(!compute_scene_visibility(v, "/World/Hidden/Child"), "invisibility inherits");
    CHECK(compute_scene_purpose(v, "/World/Hidden/Child") == ScenePurpose::guide, "purpose inherits");
    CHECK(compute_scene_purpose(v, "/World") == ScenePurpose::default_, "default purpose");
    CHECK(parent_scene_prim_path("/World") == "/" && parent_scene_prim_path("/World/A") == "/World", "parent paths");
    CHECK(!is_valid_scene_prim_path("/World/") && !is_valid_scene_prim_path("/9x") && is_valid_scene_prim_path("/_a/b9"),
        "prim path grammar");
}

static void geometry_case() {
    // quad fan: 2 triangles (0,1,2), (0,2,3); a mirror flips the winding back
    {
        const HostScenePtr h = adapt_scene_ir_v2_to_realtime(base_scene(quad_mesh()));
        const rtgb_scene v = view_of(h);
        CHECK(v.triangle_count == 2 && near3(v.triangles[1].p1, {1.0, 1.0, 0.0}, 0.0), "fan triangulation");
        const HostScenePtr m = adapt_scene_ir_v2_to_realtime(base_scene(quad_mesh(), scale_translate({-1.0, 1.0, 1.0})));
        const rtgb_scene w = view_of(m);
        CHECK(near3(w.triangles[0].p1, {-1.0, 1.0, 0.0}, 0.0) && near3(w.triangles[0].p2, {-1.0, 0.0, 0.0}, 0.0),
            "negative determinant reverses the winding");
        SceneMeshGeometry lh = quad_mesh();
        lh.orientation = SceneMeshOrientation::left_handed;
        const HostScenePtr l = adapt_scene_ir_v2_to_realtime(base_scene(lh));
        CHECK(near3(view_of(l).triangles[0].p1, {1.0, 1.0, 0.0}, 0.0), "left-handed mesh reverses the winding");
    }
    // normals go through the inverse transpose: a 45-degree normal under scale (2, 1, 1)
    {
        SceneMeshGeometry m = quad_mesh();
        ScenePrimvar n;
        n.name = "normals";
        n.role = ScenePrimvarRole::normal;
        n.interpolation = ScenePrimvarInterpolation::constant;
        n.values = std::vector<Vec3> {{1.0, 0.0, 1.0}};
        m.primvars = {n};
        const HostScenePtr h = adapt_scene_ir_v2_to_realtime(base_scene(m, scale_translate({2.0, 1.0, 1.0})));
        const double len = std::sqrt(0.25 + 1.0);
        CHECK(near3(view_of(h).triangles[0].n0, {0.5 / len, 0.0, 1.0 / len}, 1e-7), "inverse-transpose normal");
        m.primvars[0].values = std::vector<Vec3> {{0.0, 0.0, 0.0}};
        expect_invalid([&] { (void)adapt_scene_ir_v2_to_realtime(base_scene(m)); }, "zero-length mesh normal", "zero normal");
        m.primvars[0].element_size = 3;
        m.primvars[0].values = std::vector<Vec3> {{0.0, 0.0, 1.0}, {0.0, 0.0, 1.0}, {0.0, 0.0, 1.0}};
        expect_invalid([&] { (void)adapt_scene_ir_v2_to_realtime(base_scene(m)); }, "scalar primvar elements", "element size");
    }
    // spheres: uniform scale folds into the radius; a stretched sphere is rejected
    {
        SceneIRv2 s = base_scene(quad_mesh());
        ScenePrim g = prim("/World/Ball", ScenePrimKind::geometry_prototype);
        g.geometry = SceneGeometry {SceneSphereGeometry {{0.0, 1.0, 0.0}, 0.5}};
        s.add_prim(g);
        ScenePrim b = prim("/World/B1", ScenePrimKind::surface);
        b.prototype_path = "/World/Ball";
        b.material_path = "/World/Mat";
        b.local_to_parent = scale_translate({3.0, 3.0, 3.0}, {1.0, 0.0, 0.0});
        s.add_prim(b);
        ScenePrim hidden = b;
        hidden.path = "/World/B2";
        hidden.visibility = SceneVisibility::invisible;
        s.add_prim(hidden);
        ScenePrim guide = b;
        guide.path = "/World/B3";
        guide.authored_purpose = ScenePurpose::guide;
        s.add_prim(guide);
        AccelerationIds ids;
        const HostScenePtr h = adapt_scene_ir_v2_to_realtime(s, ids);
        const rtgb_scene v = view_of(h);
        CHECK(v.sphere_count == 1 && v.spheres[0].radius == 1.5f && near3(v.spheres[0].center, {1.0, 3.0, 0.0}, 0.0),
            "sphere instance: scaled radius, transformed centre, hidden and guide instances skipped");
        CHECK(ids.sphere_prototype == std::vector<int> {1} && ids.sphere_instance == std::vector<int> {1} &&
                  ids.triangle_prototype == std::vector<int> ({0, 0}),
            "acceleration prototype / instance ids");
        s.add_prim([&] {
            ScenePrim st = b;
            st.path = "/World/B4";
            st.local_to_parent = scale_translate({1.0, 2.0, 1.0});
            return st;
        }());
        expect_invalid([&] { (void)adapt_scene_ir_v2_to_realtime(s); }, "uniform SceneIR v2 scale", "stretched sphere");
    }
    // a volume material is not a realtime surface material
    {
        SceneIRv2 s = base_scene(quad_mesh());
        ScenePrim vm = prim("/World/Fog", ScenePrimKind::material);
        vm.material = SceneMaterial {SceneIsotropicVolumeMaterial {}};
        s.add_prim(vm);
        ScenePrim surf = prim("/World/S2", ScenePrimKind::surface);
        surf.prototype_path = "/World/Geo";
        surf.material_path = "/World/Fog";
        s.add_prim(surf);
        expect_invalid([&] { (void)adapt_scene_ir_v2_to_realtime(s); }, "not realtime-compatible", "volume material on a surface");
    }
}

static ScenePrim texture_prim(const char* path, SceneTexture t) {
    ScenePrim p = prim(path, ScenePrimKind::texture);
    p.texture = std::move(t);
    return p;
}

static ScenePrim material_prim(const char* path, const SceneOpenPbrSurface& m) {
    ScenePrim p = prim(path, ScenePrimKind::material);
    p.material = SceneMaterial {m};
    return p;
}

static ScenePrim surface(const char* path, const char* proto, const char* material, const Mat4& xf) {
    ScenePrim p = prim(path, ScenePrimKind::surface);
    p.prototype_path = proto;
    p.material_path = material;
    p.local_to_parent = xf;
    return p;
}

static Mat4 yaw(double deg, const Vec3& s, const Vec3& t) {
    const double a = deg * std::numbers::pi / 180.0, c = std::cos(a), sn = std::sin(a);
    Mat4 m = kIdentity4;
    m[0] = c * s[0];
    m[2] = sn * s[2];
    m[5] = s[1];
    m[8] = -sn * s[0];
    m[10] = c * s[2];
    m[3] = t[0];
    m[7] = t[1];
    m[11] = t[2];
    return m;
}

// unit cube [-0.5, 0.5]^3 as six quads with face-varying st and two subsets
static SceneMeshGeometry cube_mesh() {
    SceneMeshGeometry m;
    for (int i = 0; i < 8; ++i) m.points.push_back({(i & 1) ? 0.5 : -0.5, (i & 2) ? 0.5 : -0.5, (i & 4) ? 0.5 : -0.5});
    // counter-clockwise seen from outside
    m.face_vertex_indices = {0, 4, 6, 2, 1, 3, 7, 5, 0, 1, 5, 4, 2, 6, 7, 3, 0, 2, 3, 1, 4, 5, 7, 6};
    m.face_vertex_counts = {4, 4, 4, 4, 4, 4};
    ScenePrimvar st;
    st.name = "st";
    st.role = ScenePrimvarRole::texcoord;
    st.interpolation = ScenePrimvarInterpolation::face_varying;
    std::vector<Vec2f> uv;
    for (int f = 0; f < 6; ++f) uv.insert(uv.end(), {{0.0f, 0.0f}, {1.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, 1.0f}});
    st.values = uv;
    m.primvars = {st};
    m.material_subsets = {{"top", {3}, "/World/Looks/Gold"}};
    return m;
}

// The GPU parity scene: every SceneIR v2 feature the realtime path lowers.
// `lights`: bit k keeps light k (sphere, rect, disk, tube, sun, dome); `textures`
// binds the checker and image textures; `normals` authors the pentagon's normals.
static SceneIRv2 parity_scene(const std::string& image_path, unsigned lights = 0x3f, bool textures = true,
    bool normals = true) {
    SceneIRv2 s;
    s.add_prim(prim("/World"));
    s.add_prim(prim("/World/Tex"));
    SceneTexture red, white, check, img;
    red.value = {0.8, 0.25, 0.2};
    white.value = {0.9, 0.9, 0.85};
    check.node = SceneTextureNode::checkerboard;
    check.node_definition = "ND_checkerboard_color3";
    check.scale = 2.0;
    check.even_texture_path = "/World/Tex/Red";
    check.odd_texture_path = "/World/Tex/White";
    img.node = SceneTextureNode::image;
    img.node_definition = "ND_image_color3";
    img.color_space = SceneColorSpace::srgb_texture;
    s.add_prim(texture_prim("/World/Tex/Red", red));
    s.add_prim(texture_prim("/World/Tex/White", white));
    s.add_prim(texture_prim("/World/Tex/Check", check));
    ScenePrim ip = texture_prim("/World/Tex/Img", img);
    ip.asset_references.push_back({"grid.png", "", image_path});
    s.add_prim(ip);

    s.add_prim(prim("/World/Looks"));
    SceneOpenPbrSurface floor, gold, glass, pic, emit, coat;
    floor.specular_roughness = 0.6;
    if (textures) floor.connections.push_back({"base_color", SceneMaterialValueType::color3, "/World/Tex/Check", SceneTextureChannel::rgb});
    gold.base_metalness = 1.0;
    gold.base_color = {1.0, 0.78, 0.34};
    gold.specular_roughness = 0.3;
    glass.transmission_weight = 1.0;
    glass.specular_roughness = 0.0;
    glass.base_color = {1.0, 1.0, 1.0};
    if (textures) pic.connections.push_back({"base_color", SceneMaterialValueType::color3, "/World/Tex/Img", SceneTextureChannel::rgb});
    emit.base_color = {0.0, 0.0, 0.0};
    emit.emission_luminance = 4.0;
    emit.emission_color = {1.0, 0.9, 0.7};
    coat.base_color = {0.1, 0.3, 0.7};
    coat.coat_weight = 1.0;
    coat.coat_roughness = 0.05;
    s.add_prim(material_prim("/World/Looks/Floor", floor));
    s.add_prim(material_prim("/World/Looks/Gold", gold));
    s.add_prim(material_prim("/World/Looks/Glass", glass));
    s.add_prim(material_prim("/World/Looks/Picture", pic));
    s.add_prim(material_prim("/World/Looks/Emit", emit));
    s.add_prim(material_prim("/World/Looks/Coat", coat));

    s.add_prim(prim("/World/Proto"));
    {
        SceneMeshGeometry f;
        // 1 cm below y = 0: the checker's cells are floor(p / scale) per axis, so
        // on the plane y = 0 a hit's cell would hang on the last bit of its position
        f.points = {{-6.0, -0.01, -6.0}, {6.0, -0.01, -6.0}, {6.0, -0.01, 6.0}, {-6.0, -0.01, 6.0}};
        f.face_vertex_counts = {4};
        f.face_vertex_indices = {0, 3, 2, 1};  // facing +y
        ScenePrimvar st;
        st.name = "st";
        st.role = ScenePrimvarRole::texcoord;
        st.interpolation = ScenePrimvarInterpolation::vertex;
        st.values = std::vector<Vec2> {{0.0, 0.0}, {6.0, 0.0}, {6.0, 6.0}, {0.0, 6.0}};
        f.primvars = {st};
        ScenePrim p = prim("/World/Proto/Floor", ScenePrimKind::geometry_prototype);
        p.geometry = SceneGeometry {f};
        s.add_prim(p);
    }
    {
        ScenePrim p = prim("/World/Proto/Cube", ScenePrimKind::geometry_prototype);
        p.geometry = SceneGeometry {cube_mesh()};
        s.add_prim(p);
        ScenePrim b = prim("/World/Proto/Ball", ScenePrimKind::geometry_prototype);
        b.geometry = SceneGeometry {SceneSphereGeometry {{0.0, 0.0, 0.0}, 0.5}};
        s.add_prim(b);
        // a pentagon (n-gon fan) with an indexed vertex-normal primvar
        SceneMeshGeometry g;
        for (int i = 0; i < 5; ++i) {
            const double a = 2.0 * std::numbers::pi * i / 5.0;
            g.points.push_back({std::cos(a), std::sin(a), 0.0});
        }
        g.face_vertex_counts = {5};
        g.face_vertex_indices = {0, 1, 2, 3, 4};
        ScenePrimvar n;
        n.name = "normals";
        n.role = ScenePrimvarRole::normal;
        n.interpolation = ScenePrimvarInterpolation::vertex;
        n.values = std::vector<Vec3f> {{0.0f, 0.0f, 1.0f}, {0.2f, 0.0f, 1.0f}};
        n.indices = {0, 1, 0, 1, 0};
        if (normals) g.primvars = {n};
        ScenePrim pg = prim("/World/Proto/Pentagon", ScenePrimKind::geometry_prototype);
        pg.geometry = SceneGeometry {g};
        s.add_prim(pg);
    }

    s.add_prim(surface("/World/Floor", "/World/Proto/Floor", "/World/Looks/Floor", kIdentity4));
    s.add_prim(prim("/World/Props"));
    s.add_prim(surface("/World/Props/CubeA", "/World/Proto/Cube", "/World/Looks/Picture", yaw(30.0, {1.0, 1.0, 1.0}, {-1.5, 0.5, 1.0})));
    s.add_prim(surface("/World/Props/CubeB", "/World/Proto/Cube", "/World/Looks/Coat", yaw(-15.0, {0.6, 1.6, 0.6}, {1.6, 0.8, 0.2})));
    {
        // an animated instance, sampled at the stage's start time code
        ScenePrim c = surface("/World/Props/CubeC", "/World/Proto/Cube", "/World/Looks/Picture", kIdentity4);
        c.transform_samples = {{0.0, translate(0.0, 0.4, -3.0)}, {48.0, translate(4.0, 0.4, -3.0)}};
        c.local_to_parent = translate(0.0, 0.4, -3.0);
        s.add_prim(c);
    }
    s.add_prim(surface("/World/Props/Gold", "/World/Proto/Ball", "/World/Looks/Gold", scale_translate({1.2, 1.2, 1.2}, {0.0, 0.6, 2.5})));
    s.add_prim(surface("/World/Props/Glass", "/World/Proto/Ball", "/World/Looks/Glass", scale_translate({1.4, 1.4, 1.4}, {-0.2, 0.7, -0.8})));
    s.add_prim(surface("/World/Props/Pentagon", "/World/Proto/Pentagon", "/World/Looks/Coat", yaw(90.0, {0.8, 0.8, 0.8}, {-3.0, 1.2, -1.0})));
    s.add_prim(surface("/World/Props/Lamp", "/World/Proto/Cube", "/World/Looks/Emit", scale_translate({1.5, 0.05, 1.5}, {0.0, 4.0, 0.0})));
    {
        ScenePrim hidden = surface("/World/Props/Hidden", "/World/Proto/Ball", "/World/Looks/Gold", translate(0.0, 1.0, 4.0));
        hidden.visibility = SceneVisibility::invisible;
        s.add_prim(hidden);
    }
    s.stage_metadata().start_time_code = 12.0;

    s.add_prim(prim("/World/Lights"));
    SceneLight sph = light_of(SceneLightType::sphere), rect = light_of(SceneLightType::rect), disk = light_of(SceneLightType::disk),
               cyl = light_of(SceneLightType::cylinder), sun = light_of(SceneLightType::distant), dome = light_of(SceneLightType::dome);
    sph.radius = 0.2;
    sph.intensity = 30.0;
    sph.color = {1.0, 0.85, 0.7};
    rect.width = 1.0;
    rect.height = 0.5;
    rect.intensity = 12.0;
    rect.normalize = true;
    disk.radius = 0.3;
    disk.intensity = 15.0;
    disk.enable_color_temperature = true;
    disk.color_temperature_kelvin = 4000.0;
    cyl.radius = 0.05;
    cyl.length = 1.5;
    cyl.intensity = 20.0;
    sun.angle_degrees = 4.0;
    sun.intensity = 2.0;
    sun.normalize = true;
    dome.intensity = 0.15;
    dome.color = {0.6, 0.7, 1.0};
    if (lights & 1) s.add_prim(light_prim("/World/Lights/Sphere", sph, translate(2.5, 2.5, 2.0)));
    // rect / disk lights face -(basis_x x basis_y), local -z: a rotation about x
    // taking local -z onto world -y points them at the floor
    Mat4 down = kIdentity4;
    down[5] = 0.0;
    down[6] = 1.0;
    down[9] = -1.0;
    down[10] = 0.0;
    Mat4 rect_xf = down;
    rect_xf[3] = -2.0;
    rect_xf[7] = 3.0;
    rect_xf[11] = 0.5;
    if (lights & 2) s.add_prim(light_prim("/World/Lights/Rect", rect, rect_xf));
    Mat4 disk_xf = down;
    disk_xf[3] = 1.0;
    disk_xf[7] = 3.2;
    disk_xf[11] = -1.5;
    if (lights & 4) s.add_prim(light_prim("/World/Lights/Disk", disk, disk_xf));
    if (lights & 8) s.add_prim(light_prim("/World/Lights/Tube", cyl, translate(0.0, 2.2, -1.8)));
    Mat4 sun_xf = kIdentity4;  // tilt the sun about x
    const double a = 0.9;
    sun_xf[5] = std::cos(a);
    sun_xf[6] = -std::sin(a);
    sun_xf[9] = std::sin(a);
    sun_xf[10] = std::cos(a);
    if (lights & 16) s.add_prim(light_prim("/World/Lights/Sun", sun, sun_xf));
    if (lights & 32) s.add_prim(light_prim("/World/Lights/Dome", dome));
    return s;
}

static void file_case(const std::filesystem::path& dir) {
    const HostScenePtr a = adapt_scene_ir_v2_to_realtime(parity_scene((dir / "grid.png").string()));
    const std::string path = (dir / "roundtrip.rtgbscene").string();
    CHECK(rtgb_host_scene_save(a.get(), path.c_str()) == RTGB_OK, "save");
    rtgb_host_scene* raw = nullptr;
    CHECK(rtgb_host_scene_load(path.c_str(), &raw) == RTGB_OK && raw, "load");
    if (!raw) return;
    const HostScenePtr b(raw);
    const rtgb_scene va = view_of(a), vb = view_of(b);
    const auto same = [](const void* x, const void* y, size_t n) { return n == 0 || std::memcmp(x, y, n) == 0; };
    CHECK(va.triangle_count == vb.triangle_count && same(va.triangles, vb.triangles, sizeof(rtgb_triangle) * static_cast<size_t>(va.triangle_count)),
        "triangles survive the file");
    CHECK(va.analytic_light_count == vb.analytic_light_count &&
              same(va.analytic_lights, vb.analytic_lights, sizeof(rtgb_analytic_light) * static_cast<size_t>(va.analytic_light_count)),
        "lights survive the file");
    CHECK(va.image_texel_count == vb.image_texel_count && same(va.image_texels, vb.image_texels, 12 * static_cast<size_t>(va.image_texel_count)),
        "texels survive the file");
    CHECK(same(va.openpbr_materials, vb.openpbr_materials, sizeof(rtgb_openpbr_material) * static_cast<size_t>(va.openpbr_material_count)),
        "OpenPBR blocks survive the file");
    rtgb_host_scene* copy = nullptr;
    CHECK(rtgb_host_scene_from_view(&va, &copy) == RTGB_OK, "from_view");
    const HostScenePtr c(copy);
    CHECK(view_of(c).sphere_count == va.sphere_count && view_of(c).texture_count == va.texture_count, "from_view copies");
    // a truncated file is refused, not half-read
    {
        std::FILE* f = std::fopen(path.c_str(), "rb+");
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fclose(f);
        std::filesystem::resize_file(path, static_cast<uintmax_t>(n / 2));
        rtgb_host_scene* bad = nullptr;
        CHECK(rtgb_host_scene_load(path.c_str(), &bad) != RTGB_OK && bad == nullptr, "truncated file refused");
    }
}

// SceneIR v1: tests/test_realtime_scene_adapter.cpp:9-30 (one triangle), then
// the Cornell box of shared_scene_builders.cpp:101-139 built through the IR,
// which must pack to the builtin "cornell_box" scene's arrays byte for byte.
static void scene_ir_v1_case() {
    SceneIR tri;
    const int white = tri.add_texture(ConstantColorTextureDesc {{1.0, 1.0, 1.0}});
    const int matte = tri.add_material(DiffuseMaterial {white});
    const int mesh = tri.add_shape(TriangleMeshShape {{{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}}, {{0, 1, 2}}, {}, {}, {}, {}, {}, {}});
    tri.add_instance(SurfaceInstance {mesh, matte, Transform::identity()});
    CHECK(view_of(adapt_to_realtime(tri)).triangle_count == 1, "realtime adapter emits triangle primitive");

    SceneIR c;
    auto diffuse = [&](const Vec3& col) { return c.add_material(DiffuseMaterial {c.add_texture(ConstantColorTextureDesc {col})}); };
    const int red = diffuse({0.65, 0.05, 0.05}), whitem = diffuse({0.73, 0.73, 0.73}), green = diffuse({0.12, 0.45, 0.15});
    const int light = c.add_material(EmissiveMaterial {c.add_texture(ConstantColorTextureDesc {{15.0, 15.0, 15.0}})});
    auto quad = [&](int m, const Vec3& o, const Vec3& u, const Vec3& v) {
        c.add_instance(SurfaceInstance {c.add_shape(QuadShape {o, u, v}), m, Transform::identity()});
    };
    quad(green, {555, 0, 0}, {0, 555, 0}, {0, 0, 555});
    quad(red, {0, 0, 0}, {0, 555, 0}, {0, 0, 555});
    quad(light, {343, 554, 332}, {-130, 0, 0}, {0, 0, -105});
    quad(whitem, {0, 0, 0}, {555, 0, 0}, {0, 0, 555});
    quad(whitem, {555, 555, 555}, {-555, 0, 0}, {0, 0, -555});
    quad(whitem, {0, 0, 555}, {555, 0, 0}, {0, 555, 0});
    auto box = [&](const Vec3& mx, const Vec3& t, double deg) {
        const double a = deg * std::numbers::pi / 180.0, co = std::cos(a), si = std::sin(a);
        Transform xf;
        xf.translation = t;
        xf.rotation = {co, 0.0, si, 0.0, 1.0, 0.0, -si, 0.0, co};
        c.add_instance(SurfaceInstance {c.add_shape(BoxShape {{0, 0, 0}, mx}), whitem, xf});
    };
    box({165, 330, 165}, {265, 0, 295}, 15.0);
    box({165, 165, 165}, {130, 0, 65}, -18.0);
    const HostScenePtr ir = adapt_to_realtime(c);
    rtgb_host_scene* raw = nullptr;
    CHECK(rtgb_host_scene_create("cornell_box", 0, 0, &raw) == RTGB_OK, "builtin cornell_box");
    const HostScenePtr builtin(raw);
    const rtgb_scene a = view_of(ir), b = view_of(builtin);
    const auto same = [](const void* x, const void* y, size_t n) { return n == 0 || std::memcmp(x, y, n) == 0; };
    CHECK(a.quad_count == 18 && a.quad_count == b.quad_count &&
              same(a.quads, b.quads, sizeof(rtgb_quad) * static_cast<size_t>(a.quad_count)),
        "Cornell quads through SceneIR v1 = the builtin scene's");
    CHECK(a.material_count == b.material_count && same(a.materials, b.materials, sizeof(rtgb_material) * 4) &&
              a.texture_count == b.texture_count && same(a.textures, b.textures, sizeof(rtgb_texture) * 4),
        "Cornell materials and textures through SceneIR v1 = the builtin scene's");

    // media: a box of fog with an isotropic material; rows are world -> local
    SceneIR fog;
    const int t0 = fog.add_texture(ConstantColorTextureDesc {{1.0, 1.0, 1.0}});
    const int iso = fog.add_material(IsotropicVolumeMaterial {t0});
    const int diff = fog.add_material(DiffuseMaterial {t0});
    const int cube = fog.add_shape(BoxShape {{-1, -1, -1}, {1, 1, 1}});
    fog.add_instance(SurfaceInstance {fog.add_shape(SphereShape {{0, 0, 0}, 0.5}), diff, Transform::identity()});
    Transform spin;
    spin.rotation = {0.0, -1.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0};  // +90 deg about z
    spin.translation = {3.0, 0.0, 0.0};
    fog.add_medium(MediumInstance {cube, iso, 0.25, spin});
    const HostScenePtr f = adapt_to_realtime(fog);
    const rtgb_scene fv = view_of(f);
    CHECK(fv.medium_count == 1 && fv.media[0].boundary_type == 1 && fv.media[0].density == 0.25f &&
              fv.media[0].rotation_row0[1] == 1.0f && fv.media[0].rotation_row1[0] == -1.0f && fv.media[0].translation[0] == 3.0f,
        "medium: box boundary, density, world-to-local rows, translation");
    fog.add_medium(MediumInstance {cube, diff, 0.25, spin});
    expect_invalid([&] { (void)adapt_to_realtime(fog); }, "isotropic volume material", "medium with a surface material");
    SceneIR bad;
    bad.add_instance(SurfaceInstance {0, 0, Transform::identity()});
    ++g_checks;
    try {
        (void)adapt_to_realtime(bad);
        ++g_failures;
        std::fprintf(stderr, "FAILED: a dangling shape index was accepted\n");
    } catch (const std::out_of_range&) {
    }
}

// adapt_to_realtime_openpbr (realtime_scene_adapter.cpp:488-500): the
// compatibility surface material becomes the OpenPBR block its SceneIR v2
// material prim names, the volume stays a volume, the v2 lights come along.
static void openpbr_compatibility_case() {
    SceneIR compat;
    const int tex = compat.add_texture(ConstantColorTextureDesc {{0.4, 0.5, 0.6}});
    const int surf = compat.add_material(DiffuseMaterial {tex});
    const int fogm = compat.add_material(IsotropicVolumeMaterial {tex});
    compat.add_instance(SurfaceInstance {compat.add_shape(SphereShape {{0, 1, 0}, 1.0}), surf, Transform::identity()});
    compat.add_medium(MediumInstance {compat.add_shape(SphereShape {{0, 0, 0}, 3.0}), fogm, 0.1, Transform::identity()});
    SceneIRv2 v2;
    v2.add_prim(prim("/World"));
    ScenePrim t = prim("/World/Tex", ScenePrimKind::texture);
    t.texture = SceneTexture {};
    t.texture->value = {0.4, 0.5, 0.6};
    t.compatibility_source_index = 0;
    v2.add_prim(t);
    SceneOpenPbrSurface pbr;
    pbr.specular_roughness = 0.2;
    pbr.connections.push_back({"base_color", SceneMaterialValueType::color3, "/World/Tex", SceneTextureChannel::rgb});
    ScenePrim m0 = prim("/World/M0", ScenePrimKind::material);
    m0.material = SceneMaterial {pbr};
    m0.compatibility_source_index = 0;
    v2.add_prim(m0);
    ScenePrim m1 = prim("/World/M1", ScenePrimKind::material);
    m1.material = SceneMaterial {SceneIsotropicVolumeMaterial {}};
    m1.compatibility_source_index = 1;
    v2.add_prim(m1);
    v2.add_prim(light_prim("/World/Key", light_of(SceneLightType::sphere), translate(0.0, 4.0, 0.0)));
    const HostScenePtr h = adapt_to_realtime_openpbr(compat, v2);
    const rtgb_scene v = view_of(h);
    CHECK(v.material_count == 2 && v.materials[0].type == RTGB_MATERIAL_OPENPBR && v.materials[1].type == RTGB_MATERIAL_ISOTROPIC,
        "surface material replaced by OpenPBR, volume kept");
    CHECK(v.openpbr_material_count == 1 && v.openpbr_materials[0].color_texture[0] == 0 &&
              v.openpbr_materials[0].specular_roughness == 0.2f,
        "compatibility texture index bound to base_color");
    CHECK(v.analytic_light_count == 1 && v.sphere_count == 1 && v.medium_count == 1, "v2 lights, v1 geometry and media");
    SceneIRv2 missing;
    missing.add_prim(prim("/World"));
    missing.add_prim(m0);
    missing.add_prim(t);
    expect_invalid([&] { (void)adapt_to_realtime_openpbr(compat, missing); }, "missing a compatibility material for index 1",
        "every compatibility material must be named");
    SceneIRv2 swap;
    swap.add_prim(prim("/World"));
    swap.add_prim(t);
    ScenePrim s0 = m0, s1 = m1;
    s0.compatibility_source_index = 1;
    s1.compatibility_source_index = 0;
    swap.add_prim(s0);
    swap.add_prim(s1);
    expect_invalid([&] { (void)adapt_to_realtime_openpbr(compat, swap); }, "compatibility surface must compile to OpenPBR",
        "a surface material must get an OpenPBR block");
    SceneIR only_fog;
    const int ft = only_fog.add_texture(ConstantColorTextureDesc {{1.0, 1.0, 1.0}});
    const int fm = only_fog.add_material(IsotropicVolumeMaterial {ft});
    only_fog.add_instance(SurfaceInstance {only_fog.add_shape(SphereShape {{0, 0, 0}, 1.0}), fm, Transform::identity()});
    SceneIRv2 pbr_for_fog;
    pbr_for_fog.add_prim(prim("/World"));
    pbr_for_fog.add_prim(t);
    pbr_for_fog.add_prim(m0);
    expect_invalid([&] { (void)adapt_to_realtime_openpbr(only_fog, pbr_for_fog); }, "cannot replace a compatibility volume",
        "an OpenPBR surface cannot replace a volume");
}

// The instanced lowering on the CPU: the same scene with every mesh triangle
// carried by a prototype / instance instead of the host scene's triangles.
static void instanced_case(const std::string& img) {
    const SceneIRv2 ir = parity_scene(img);
    const HostScenePtr flat = adapt_scene_ir_v2_to_realtime(ir);
    MeshInstances mi;
    const HostScenePtr base = adapt_scene_ir_v2_to_realtime_instanced(ir, mi);
    const rtgb_scene f = view_of(flat), b = view_of(base);
    CHECK(b.triangle_count == 0 && b.sphere_count == f.sphere_count && b.material_count == f.material_count,
        "instanced lowering keeps everything but the mesh triangles");
    const rtgb_mesh_set set = mi.view();
    long long tris = 0;
    for (int i = 0; i < set.instance_count; ++i) tris += set.prototypes[set.instances[i].prototype].triangle_count;
    CHECK(tris == f.triangle_count, "instances flatten to the flat lowering's triangle count");
    CHECK(set.prototype_count < set.instance_count, "instanced cubes share one prototype");
}

// rtgb_prepare_scene_instanced against rtgb_prepare_scene on a GB300: the
// device-flattened triangles, the light table and a rendered frame must be
// identical bytes to the flat lowering's, for each variant of the scene.
static void instanced_gpu_case(const std::string& img) {
    const std::vector<SceneIRv2> variants = {parity_scene(img), parity_scene(img, 0x3f, true, false),
        parity_scene(img, 0x3f, false)};
    for (size_t k = 0; k < variants.size(); ++k) {
        const HostScenePtr flat = adapt_scene_ir_v2_to_realtime(variants[k]);
        MeshInstances mi;
        const HostScenePtr base = adapt_scene_ir_v2_to_realtime_instanced(variants[k], mi);
        const rtgb_scene fv = view_of(flat), bv = view_of(base);
        const rtgb_mesh_set set = mi.view();
        rtgb_create_info info {};
        info.use_cuda_graph = 1;
        rtgb_handle a = nullptr, c = nullptr;
        CHECK(rtgb_create(&info, &a) == RTGB_OK && rtgb_create(&info, &c) == RTGB_OK, "create two renderers");
        CHECK(rtgb_prepare_scene(a, &fv) == RTGB_OK, "prepare the flat lowering");
        CHECK(rtgb_prepare_scene_instanced(c, &bv, &set) == RTGB_OK, "prepare the instanced lowering");
        int32_t na = 0, nc = 0;
        rtgb_download_triangles(a, nullptr, 0, &na);
        rtgb_download_triangles(c, nullptr, 0, &nc);
        std::vector<rtgb_triangle> ta(static_cast<size_t>(na)), tc(static_cast<size_t>(nc));
        rtgb_download_triangles(a, ta.data(), na, &na);
        rtgb_download_triangles(c, tc.data(), nc, &nc);
        CHECK(na == fv.triangle_count && nc == na, "triangle counts");
        CHECK(std::memcmp(ta.data(), tc.data(), ta.size() * sizeof(rtgb_triangle)) == 0,
            "device-flattened triangles equal the host lowering's bit for bit");
        int32_t la = 0, lc = 0;
        rtgb_download_light_table(a, nullptr, 0, &la, nullptr, nullptr, nullptr);
        rtgb_download_light_table(c, nullptr, 0, &lc, nullptr, nullptr, nullptr);
        std::vector<uint8_t> lta(static_cast<size_t>(la) * 16), ltc(static_cast<size_t>(lc) * 16);
        rtgb_download_light_table(a, lta.data(), la, &la, nullptr, nullptr, nullptr);
        rtgb_download_light_table(c, ltc.data(), lc, &lc, nullptr, nullptr, nullptr);
        CHECK(la == lc && lta == ltc, "light tables equal");
        rtgb_camera_rig rig {};
        rtgb_render_profile prof {};
        CHECK(rtgb_default_rig("cornell_box", 1, 64, 48, &rig) == RTGB_OK && rtgb_profile_preset("balanced", &prof) == RTGB_OK,
            "rig and profile");
        prof.samples_per_pixel = 2;
        prof.enable_denoise = 0;
        std::vector<float> ba(64 * 48 * 4), bc(64 * 48 * 4);
        for (rtgb_handle h : {a, c}) {
            rtgb_frame_views views {};
            CHECK(rtgb_render_frame(h, &rig, &prof, 1, &views) == RTGB_OK, "render a frame");
        }
        rtgb_download_frame(a, 0, ba.data(), nullptr, nullptr, nullptr, nullptr);
        rtgb_download_frame(c, 0, bc.data(), nullptr, nullptr, nullptr, nullptr);
        CHECK(ba == bc, "rendered frames equal");
        rtgb_destroy(a);
        rtgb_destroy(c);
        std::printf("instanced variant %zu: %d triangles from %d prototypes / %d instances\n", k, nc,
            set.prototype_count, set.instance_count);
    }
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s DIR [--write-scene FILE | --write-variants DIR | --instanced-gpu]\n", argv[0]);
        return 2;
    }
    const std::filesystem::path dir = argv[1];
    // an 8 x 8 sRGB grid image for the image-texture binding
    std::vector<uint8_t> rgb(8 * 8 * 3);
    for (int y = 0; y < 8; ++y) {
        for (int x = 0; x < 8; ++x) {
            uint8_t* p = &rgb[static_cast<size_t>((y * 8 + x) * 3)];
            p[0] = static_cast<uint8_t>(32 * x + 8);
            p[1] = static_cast<uint8_t>(32 * y + 8);
            p[2] = static_cast<uint8_t>(((x ^ y) & 1) ? 230 : 40);
        }
    }
    rtgb::png::write_rgb(dir / "grid.png", 8, 8, rgb.data());
    try {
        reference_adapter_case();
        scene_ir_v1_case();
        openpbr_compatibility_case();
        reference_light_case();
        validator_case();
        transform_case();
        geometry_case();
        file_case(dir);
        instanced_case((dir / "grid.png").string());
        if (argc >= 3 && std::string(argv[2]) == "--instanced-gpu") instanced_gpu_case((dir / "grid.png").string());
        {
            const HostScenePtr h = adapt_scene_ir_v2_to_realtime(parity_scene((dir / "grid.png").string()));
            const rtgb_scene v = view_of(h);
            CHECK(v.texture_count == 4 && v.textures[3].type == RTGB_TEXTURE_IMAGE && v.textures[3].image_width == 8 &&
                      v.image_texel_count == 64,
                "image texture loaded from the asset's resolved path");
            CHECK(v.image_texels[0] == 8.0f * static_cast<float>(1.0 / 255.0), "texels scaled by 1/255");
            CHECK(v.sphere_count == 2 && v.analytic_light_count == 6 && v.material_count == 6, "parity scene counts");
            // fans: floor 2 + 4 cubes x 12 + pentagon 3
            CHECK(v.triangle_count == 2 + 4 * 12 + 3, "parity scene triangles");
            // CubeC (triangles 26..37) sampled at t = 12 between x = 0 (t = 0) and x = 4 (t = 48)
            CHECK(near3(v.triangles[26].p0, {0.5, -0.1, -3.5}, 1e-6), "time-sampled instance at the start time code");
            if (argc >= 4 && std::string(argv[2]) == "--write-scene") {
                CHECK(rtgb_host_scene_save(h.get(), argv[3]) == RTGB_OK, "write the parity scene");
            }
            if (argc >= 4 && std::string(argv[2]) == "--write-variants") {
                // one scene per feature, for locating a parity difference
                const std::string img = (dir / "grid.png").string();
                const auto save = [&](const SceneIRv2& ir, const std::string& name) {
                    const HostScenePtr v2 = adapt_scene_ir_v2_to_realtime(ir);
                    CHECK(rtgb_host_scene_save(v2.get(), (std::filesystem::path(argv[3]) / name).string().c_str()) == RTGB_OK,
                        "write a variant");
                };
                for (unsigned k = 0; k < 6; ++k) save(parity_scene(img, 1u << k), "light" + std::to_string(k) + ".rtgbscene");
                save(parity_scene(img, 0), "nolights.rtgbscene");
                save(parity_scene(img, 0x3f, false), "notex.rtgbscene");
                save(parity_scene(img, 0x3f, true, false), "nonormals.rtgbscene");
            }
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "FAILED: uncaught %s\n", e.what());
        return 1;
    }
    std::printf("scene_ir_v2 checks=%d failures=%d\n", g_checks, g_failures);
    return g_failures == 0 ? 0 : 1;
}
