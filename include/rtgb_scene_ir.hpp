// SceneIR (v1) input for the realtime path (C++23, host only).
//
// The compatibility scene description of the reference
// (src/scene/shared_scene_ir.h: texture / material / shape tables and
// instances referring to them by index) and its lowering to the packed arrays
// of rtgb.h:
//
//   validate_scene_ir     src/scene/scene_ir_validator.cpp:98-130
//   adapt_to_realtime     src/scene/realtime_scene_adapter.cpp:371-486 (with
//                         the box-to-quads expansion :76-110 and the material /
//                         texture / medium packing of
//                         src/realtime/gpu/packed_scene_preparation.cpp:78-190)
//
// Names and defaults are the reference's; Eigen vectors become std::array
// (Vec3 / Vec2 / Vec3i) and the transform's rotation a row-major 3x3 array.
// Errors are the reference's exceptions (std::out_of_range for a bad index,
// std::invalid_argument for a bad value).
#pragma once

#include <array>
#include <optional>
#include <string>
#include <variant>
#include <vector>

#include "rtgb_scene_ir_v2.hpp"

namespace rtgb::scene {

using Vec3i = std::array<int, 3>;

struct ConstantColorTextureDesc {
    Vec3 color {0.0, 0.0, 0.0};
};

struct CheckerTextureDesc {
    double scale = 1.0;
    int even_texture = -1;
    int odd_texture = -1;
};

struct ImageTextureDesc {
    std::string authored_path;
    std::string path;
};

struct NoiseTextureDesc {
    double scale = 1.0;
};

using TextureDesc = std::variant<ConstantColorTextureDesc, CheckerTextureDesc, ImageTextureDesc, NoiseTextureDesc>;

struct DiffuseMaterial {
    int albedo_texture = -1;
};

struct MetalMaterial {
    int albedo_texture = -1;
    double fuzz = 0.0;
};

struct DielectricMaterial {
    double ior = 1.0;
};

struct EmissiveMaterial {
    int emission_texture = -1;
};

struct IsotropicVolumeMaterial {
    int albedo_texture = -1;
};

using MaterialDesc = std::variant<DiffuseMaterial, MetalMaterial, DielectricMaterial, EmissiveMaterial, IsotropicVolumeMaterial>;

struct SphereShape {
    Vec3 center {0.0, 0.0, 0.0};
    double radius = 1.0;
};

struct QuadShape {
    Vec3 origin {0.0, 0.0, 0.0};
    Vec3 edge_u {0.0, 0.0, 0.0};
    Vec3 edge_v {0.0, 0.0, 0.0};
};

struct BoxShape {
    Vec3 min_corner {0.0, 0.0, 0.0};
    Vec3 max_corner {0.0, 0.0, 0.0};
};

// Vertex attributes beyond positions are validated but, as in the reference's
// realtime adapter, only positions reach the packed triangles.
struct TriangleMeshShape {
    std::vector<Vec3> positions;
    std::vector<Vec3i> triangles;
    std::vector<Vec3> normals;
    std::vector<Vec3i> normal_indices;
    std::vector<Vec3> tangents;
    std::vector<Vec3i> tangent_indices;
    std::vector<Vec2> texcoords;
    std::vector<Vec3i> texcoord_indices;
};

using ShapeDesc = std::variant<SphereShape, QuadShape, BoxShape, TriangleMeshShape>;

struct Transform {
    Vec3 translation {0.0, 0.0, 0.0};
    std::array<double, 9> rotation {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};  // row-major
    static Transform identity() { return Transform {}; }
};

struct SurfaceInstance {
    int shape_index = -1;
    int material_index = -1;
    Transform transform = Transform::identity();
};

struct MediumInstance {
    int shape_index = -1;
    int material_index = -1;
    double density = 0.0;
    Transform transform = Transform::identity();
};

class SceneIR {
public:
    int add_texture(const TextureDesc& texture) { return push(textures_, texture); }
    int add_material(const MaterialDesc& material) { return push(materials_, material); }
    int add_shape(const ShapeDesc& shape) { return push(shapes_, shape); }
    void add_instance(const SurfaceInstance& instance) { surface_instances_.push_back(instance); }
    void add_medium(const MediumInstance& medium) { media_.push_back(medium); }

    const std::vector<TextureDesc>& textures() const { return textures_; }
    const std::vector<MaterialDesc>& materials() const { return materials_; }
    const std::vector<ShapeDesc>& shapes() const { return shapes_; }
    const std::vector<SurfaceInstance>& surface_instances() const { return surface_instances_; }
    const std::vector<MediumInstance>& media() const { return media_; }

private:
    template <class T, class V>
    static int push(std::vector<T>& v, const V& x) {
        v.push_back(x);
        return static_cast<int>(v.size()) - 1;
    }
    std::vector<TextureDesc> textures_;
    std::vector<MaterialDesc> materials_;
    std::vector<ShapeDesc> shapes_;
    std::vector<SurfaceInstance> surface_instances_;
    std::vector<MediumInstance> media_;
};

void validate_scene_ir(const SceneIR& scene);

// Textures, then materials, then one primitive per surface instance in
// instance order (a box becomes six quads), then the media; the background is
// black and there are no analytic lights (the compatibility IR has none).
HostScenePtr adapt_to_realtime(const SceneIR& scene, const AdaptOptions& options = {});

// openpbr_core_adapter.cpp:215-254: the OpenPBR block of every SceneIR v2
// material prim that names a compatibility material (its
// compatibility_source_index), indexed by that material; texture connections
// bind the compatibility texture index of their texture prim. Prims with a
// volume payload leave their entry empty. Every compatibility material must
// be named exactly once.
std::vector<std::optional<rtgb_openpbr_material>> compile_openpbr_core_material_table(const SceneIRv2& scene,
    std::size_t compatibility_material_count, std::size_t compatibility_texture_count);

// realtime_scene_adapter.cpp:488-500: the compatibility scene with each
// surface material replaced by its OpenPBR block from `scene_v2` (a volume
// material must stay a volume), then the analytic lights of `scene_v2`.
HostScenePtr adapt_to_realtime_openpbr(const SceneIR& compatibility_scene, const SceneIRv2& scene_v2,
    const AdaptOptions& options = {});

}  // namespace rtgb::scene
