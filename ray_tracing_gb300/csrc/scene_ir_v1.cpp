// SceneIR (v1) -> packed realtime scene: the compatibility path of
// src/scene/realtime_scene_adapter.cpp:371-486 (adapt_to_realtime) after the
// index checks of src/scene/scene_ir_validator.cpp:98-130. Geometry is
// transformed in double (rotation * p + translation) and rounded to float at
// packing; boxes expand to six quads in the adapter's face order (:76-110);
// media pack their world-to-local rotation (the transposed instance rotation)
// as packed_scene_preparation.cpp:78-91 does.
#include <stdexcept>
#include <string>

#include "host_scene.h"
#include "rtgb_scene_ir.hpp"

namespace rtgb::scene {
namespace {

template <class T>
void require_index(const std::vector<T>& items, int index, const std::string& label) {
    if (index < 0 || static_cast<size_t>(index) >= items.size()) throw std::out_of_range(label + " index out of range");
}

// per-corner attribute indices (normals, tangents, texcoords) against their values
template <class V>
void require_attribute(const TriangleMeshShape& mesh, const char* label, const std::vector<V>& values,
    const std::vector<Vec3i>& indices) {
    const std::string l(label);
    if (indices.empty()) {
        if (!values.empty() && values.size() != mesh.positions.size()) {
            throw std::invalid_argument("triangle mesh " + l + " count must match positions without indices");
        }
        return;
    }
    if (values.empty()) throw std::invalid_argument("triangle mesh " + l + " indices require values");
    if (indices.size() != mesh.triangles.size()) throw std::invalid_argument("triangle mesh " + l + " index count mismatch");
    for (const Vec3i& t : indices) {
        for (int i : t) {
            if (i < 0 || static_cast<size_t>(i) >= values.size()) throw std::out_of_range("triangle mesh " + l + " index out of range");
        }
    }
}

Vec3 rotate(const Transform& t, const Vec3& v) {
    const auto& r = t.rotation;
    return {r[0] * v[0] + r[1] * v[1] + r[2] * v[2], r[3] * v[0] + r[4] * v[1] + r[5] * v[2],
        r[6] * v[0] + r[7] * v[1] + r[8] * v[2]};
}

Vec3 place(const Transform& t, const Vec3& p) {
    const Vec3 r = rotate(t, p);
    return {r[0] + t.translation[0], r[1] + t.translation[1], r[2] + t.translation[2]};
}

Vec3 minus(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }

void put3(float* d, const Vec3& v) {
    for (int i = 0; i < 3; ++i) d[i] = static_cast<float>(v[static_cast<size_t>(i)]);
}

void add_quad(rtgb_host_scene& out, int material, const Vec3& origin, const Vec3& eu, const Vec3& ev) {
    rtgb_quad q {};
    put3(q.origin, origin);
    put3(q.edge_u, eu);
    put3(q.edge_v, ev);
    q.material_index = material;
    out.quads.push_back(q);
}

// add_box_quads: the six faces, each an origin corner and two edges, rotated then placed
void add_box(rtgb_host_scene& out, int material, const BoxShape& box, const Transform& t) {
    const Vec3& a = box.min_corner;
    const Vec3& b = box.max_corner;
    const Vec3 p000 {a[0], a[1], a[2]}, p001 {a[0], a[1], b[2]}, p010 {a[0], b[1], a[2]}, p011 {a[0], b[1], b[2]};
    const Vec3 p100 {b[0], a[1], a[2]}, p101 {b[0], a[1], b[2]}, p110 {b[0], b[1], a[2]}, p111 {b[0], b[1], b[2]};
    const auto face = [&](const Vec3& o, const Vec3& eu, const Vec3& ev) {
        add_quad(out, material, place(t, o), rotate(t, eu), rotate(t, ev));
    };
    face(p001, minus(p101, p001), minus(p011, p001));
    face(p100, minus(p000, p100), minus(p110, p100));
    face(p000, minus(p001, p000), minus(p010, p000));
    face(p101, minus(p100, p101), minus(p111, p101));
    face(p010, minus(p110, p010), minus(p011, p010));
    face(p000, minus(p100, p000), minus(p001, p000));
}

rtgb_texture pack_texture(const TextureDesc& desc, rtgb_host_scene& out, const AdaptOptions& opt) {
    rtgb_texture t {};
    t.even_texture = -1;
    t.odd_texture = -1;
    t.u_address_mode = 1;
    t.v_address_mode = 1;
    t.filter_type = 1;
    t.scale = 1.0f;
    if (const auto* c = std::get_if<ConstantColorTextureDesc>(&desc)) {
        t.type = RTGB_TEXTURE_CONSTANT;
        put3(t.color, c->color);
    } else if (const auto* k = std::get_if<CheckerTextureDesc>(&desc)) {
        t.type = RTGB_TEXTURE_CHECKER;
        t.scale = static_cast<float>(k->scale);
        t.even_texture = k->even_texture;
        t.odd_texture = k->odd_texture;
    } else if (const auto* img = std::get_if<ImageTextureDesc>(&desc)) {
        // rt::ImageTextureDesc defaults: clamp / clamp, closest
        t.type = RTGB_TEXTURE_IMAGE;
        t.u_address_mode = 1;
        t.v_address_mode = 1;
        t.filter_type = 0;
        t.image_offset = static_cast<int32_t>(out.texels.size() / 3);
        int w = 0, h = 0;
        if (opt.load_images && detail::load_png_texels(img->path, w, h, out.texels)) {
            t.image_width = w;
            t.image_height = h;
        }
    } else {
        t.type = RTGB_TEXTURE_NOISE;
        t.scale = static_cast<float>(std::get<NoiseTextureDesc>(desc).scale);
    }
    return t;
}

rtgb_material pack_material(const MaterialDesc& desc) {
    rtgb_material m {};
    m.albedo_texture = -1;
    m.emission_texture = -1;
    m.ior = 1.0f;
    m.openpbr_index = -1;
    if (const auto* d = std::get_if<DiffuseMaterial>(&desc)) {
        m.type = RTGB_MATERIAL_LAMBERTIAN;
        m.albedo_texture = d->albedo_texture;
    } else if (const auto* mt = std::get_if<MetalMaterial>(&desc)) {
        m.type = RTGB_MATERIAL_METAL;
        m.albedo_texture = mt->albedo_texture;
        m.fuzz = static_cast<float>(mt->fuzz);
    } else if (const auto* di = std::get_if<DielectricMaterial>(&desc)) {
        m.type = RTGB_MATERIAL_DIELECTRIC;
        m.ior = static_cast<float>(di->ior);
    } else if (const auto* e = std::get_if<EmissiveMaterial>(&desc)) {
        m.type = RTGB_MATERIAL_DIFFUSE_LIGHT;
        m.emission_texture = e->emission_texture;
    } else {
        m.type = RTGB_MATERIAL_ISOTROPIC;
        m.albedo_texture = std::get<IsotropicVolumeMaterial>(desc).albedo_texture;
    }
    return m;
}

}  // namespace

void validate_scene_ir(const SceneIR& scene) {
    const auto& textures = scene.textures();
    const auto& materials = scene.materials();
    const auto& shapes = scene.shapes();
    for (const TextureDesc& t : textures) {
        if (const auto* k = std::get_if<CheckerTextureDesc>(&t)) {
            require_index(textures, k->even_texture, "checker even texture");
            require_index(textures, k->odd_texture, "checker odd texture");
        }
    }
    for (const MaterialDesc& m : materials) {
        if (const auto* d = std::get_if<DiffuseMaterial>(&m)) require_index(textures, d->albedo_texture, "diffuse albedo texture");
        if (const auto* mt = std::get_if<MetalMaterial>(&m)) require_index(textures, mt->albedo_texture, "metal albedo texture");
        if (const auto* e = std::get_if<EmissiveMaterial>(&m)) require_index(textures, e->emission_texture, "emissive texture");
        if (const auto* v = std::get_if<IsotropicVolumeMaterial>(&m)) require_index(textures, v->albedo_texture, "isotropic albedo texture");
    }
    for (const ShapeDesc& s : shapes) {
        const auto* mesh = std::get_if<TriangleMeshShape>(&s);
        if (!mesh) continue;
        for (const Vec3i& t : mesh->triangles) {
            for (int i : t) {
                if (i < 0 || static_cast<size_t>(i) >= mesh->positions.size()) throw std::out_of_range("triangle mesh vertex index out of range");
            }
        }
        require_attribute(*mesh, "normal", mesh->normals, mesh->normal_indices);
        require_attribute(*mesh, "tangent", mesh->tangents, mesh->tangent_indices);
        require_attribute(*mesh, "texcoord", mesh->texcoords, mesh->texcoord_indices);
    }
    for (const SurfaceInstance& i : scene.surface_instances()) {
        require_index(shapes, i.shape_index, "surface shape");
        require_index(materials, i.material_index, "surface material");
    }
    for (const MediumInstance& m : scene.media()) {
        if (m.density <= 0.0) throw std::invalid_argument("medium density must be positive");
        require_index(shapes, m.shape_index, "medium shape");
        require_index(materials, m.material_index, "medium material");
        if (!std::holds_alternative<IsotropicVolumeMaterial>(materials[static_cast<size_t>(m.material_index)])) {
            throw std::invalid_argument("medium requires isotropic volume material");
        }
    }
}

std::vector<std::optional<rtgb_openpbr_material>> compile_openpbr_core_material_table(const SceneIRv2& scene,
    std::size_t material_count, std::size_t texture_count) {
    require_valid_scene_ir_v2(scene);
    std::vector<std::optional<rtgb_openpbr_material>> table(material_count);
    std::vector<bool> seen(material_count, false);
    for (const ScenePrim& prim : scene.prims()) {
        if (prim.kind != ScenePrimKind::material || !prim.compatibility_source_index) continue;
        const std::size_t index = *prim.compatibility_source_index;
        if (index >= material_count) throw std::invalid_argument("SceneIR v2 material compatibility index is out of range");
        if (seen[index]) throw std::invalid_argument("SceneIR v2 material compatibility index is duplicated");
        if (!prim.material) throw std::invalid_argument("SceneIR v2 material prim has no material payload");
        seen[index] = true;
        const auto* surface = std::get_if<SceneOpenPbrSurface>(&*prim.material);
        if (!surface) continue;
        SceneOpenPbrSurface constants = *surface;
        constants.connections.clear();
        rtgb_openpbr_material compiled = compile_openpbr_core_material(constants);
        for (const SceneMaterialConnection& c : surface->connections) {
            const ScenePrim* tex = scene.find_prim(c.texture_path);
            if (!tex || !tex->texture) throw std::invalid_argument("OpenPBR connected input does not resolve to a SceneIR v2 texture");
            if (!tex->compatibility_source_index) {
                throw std::invalid_argument("OpenPBR connected texture requires a compatibility texture index");
            }
            if (*tex->compatibility_source_index >= texture_count) {
                throw std::invalid_argument("OpenPBR connected texture compatibility index is out of range");
            }
            detail::bind_connection(compiled, c, *tex->texture, static_cast<int>(*tex->compatibility_source_index));
        }
        table[index] = compiled;
    }
    for (std::size_t i = 0; i < seen.size(); ++i) {
        if (!seen[i]) throw std::invalid_argument("SceneIR v2 is missing a compatibility material for index " + std::to_string(i));
    }
    return table;
}

namespace {

HostScenePtr adapt_impl(const SceneIR& scene, const std::vector<std::optional<rtgb_openpbr_material>>* openpbr,
    const AdaptOptions& options) {
    validate_scene_ir(scene);
    HostScenePtr result(new rtgb_host_scene);
    rtgb_host_scene& out = *result;
    for (const TextureDesc& t : scene.textures()) out.textures.push_back(pack_texture(t, out, options));
    for (size_t i = 0; i < scene.materials().size(); ++i) {
        const MaterialDesc& m = scene.materials()[i];
        const bool volume = std::holds_alternative<IsotropicVolumeMaterial>(m);
        if (openpbr && (*openpbr)[i]) {
            if (volume) throw std::invalid_argument("SceneIR v2 surface material cannot replace a compatibility volume");
            out.openpbr.push_back(*(*openpbr)[i]);
            rtgb_material r {};
            r.albedo_texture = -1;
            r.emission_texture = -1;
            r.ior = 1.0f;
            r.type = RTGB_MATERIAL_OPENPBR;
            r.openpbr_index = static_cast<int32_t>(out.openpbr.size()) - 1;
            out.materials.push_back(r);
            continue;
        }
        if (openpbr && !volume) throw std::invalid_argument("SceneIR v2 compatibility surface must compile to OpenPBR");
        out.materials.push_back(pack_material(m));
    }
    const auto& shapes = scene.shapes();
    for (const SurfaceInstance& inst : scene.surface_instances()) {
        const ShapeDesc& shape = shapes[static_cast<size_t>(inst.shape_index)];
        const Transform& t = inst.transform;
        if (const auto* sp = std::get_if<SphereShape>(&shape)) {
            rtgb_sphere s {};
            put3(s.center, place(t, sp->center));
            s.radius = static_cast<float>(sp->radius);
            s.material_index = inst.material_index;
            out.spheres.push_back(s);
        } else if (const auto* q = std::get_if<QuadShape>(&shape)) {
            add_quad(out, inst.material_index, place(t, q->origin), rotate(t, q->edge_u), rotate(t, q->edge_v));
        } else if (const auto* box = std::get_if<BoxShape>(&shape)) {
            add_box(out, inst.material_index, *box, t);
        } else {
            const auto& mesh = std::get<TriangleMeshShape>(shape);
            for (const Vec3i& tri : mesh.triangles) {
                rtgb_triangle tr {};
                put3(tr.p0, place(t, mesh.positions[static_cast<size_t>(tri[0])]));
                put3(tr.p1, place(t, mesh.positions[static_cast<size_t>(tri[1])]));
                put3(tr.p2, place(t, mesh.positions[static_cast<size_t>(tri[2])]));
                tr.material_index = inst.material_index;
                out.triangles.push_back(tr);
            }
        }
    }
    for (const MediumInstance& m : scene.media()) {
        const ShapeDesc& shape = shapes[static_cast<size_t>(m.shape_index)];
        rtgb_medium p {};
        p.material_index = m.material_index;
        p.density = static_cast<float>(m.density);
        put3(p.translation, m.transform.translation);
        const auto& r = m.transform.rotation;  // world-to-local = rotation^T: its rows are the columns of r
        for (int k = 0; k < 3; ++k) {
            p.rotation_row0[k] = static_cast<float>(r[static_cast<size_t>(3 * k + 0)]);
            p.rotation_row1[k] = static_cast<float>(r[static_cast<size_t>(3 * k + 1)]);
            p.rotation_row2[k] = static_cast<float>(r[static_cast<size_t>(3 * k + 2)]);
        }
        if (const auto* sp = std::get_if<SphereShape>(&shape)) {
            p.boundary_type = 0;
            put3(p.local_center_or_min, sp->center);
            p.radius = static_cast<float>(sp->radius);
        } else if (const auto* box = std::get_if<BoxShape>(&shape)) {
            p.boundary_type = 1;
            put3(p.local_center_or_min, box->min_corner);
            put3(p.local_max, box->max_corner);
        } else if (std::holds_alternative<QuadShape>(shape)) {
            throw std::invalid_argument("quad boundaries are unsupported for homogeneous media");
        } else {
            throw std::invalid_argument("triangle mesh boundaries are unsupported for homogeneous media");
        }
        out.media.push_back(p);
    }
    return result;
}

}  // namespace

HostScenePtr adapt_to_realtime(const SceneIR& scene, const AdaptOptions& options) {
    return adapt_impl(scene, nullptr, options);
}

HostScenePtr adapt_to_realtime_openpbr(const SceneIR& compatibility_scene, const SceneIRv2& scene_v2,
    const AdaptOptions& options) {
    const auto table = compile_openpbr_core_material_table(scene_v2, compatibility_scene.materials().size(),
        compatibility_scene.textures().size());
    HostScenePtr result = adapt_impl(compatibility_scene, &table, options);
    for (const AnalyticLightDesc& l : compile_analytic_lights(scene_v2)) result->analytic.push_back(pack_analytic_light(l));
    return result;
}

}  // namespace rtgb::scene
