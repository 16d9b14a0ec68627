// SceneIR v2 input for the realtime path (C++23, host only).
//
// The scene description the reference's realtime renderer consumes
// (src/scene/scene_ir_v2.h: prims addressed by absolute paths, each carrying
// an optional geometry / material / texture / light / camera payload) and the
// functions that lower it to the packed arrays of rtgb.h:
//
//   validate_scene_ir_v2 / require_valid_scene_ir_v2      scene_ir_v2.cpp:1104-1311
//   compute_scene_world_transform / _visibility / _purpose scene_ir_v2.cpp:1499-1569
//   compile_openpbr_core_material                          openpbr_core_adapter.cpp:133-213
//   compile_analytic_lights                                analytic_light_compiler.cpp:240-261
//   adapt_scene_ir_v2_to_realtime                          realtime_scene_adapter.cpp:502-581
//
// Type, field and enumerator names and defaults are the reference's, so code
// that builds a SceneIRv2 ports by swapping the vector types: Eigen vectors
// become std::array (Vec2/Vec3/Vec4 in double, Vec2f/Vec3f/Vec4f in float)
// and Eigen::Matrix4d becomes Mat4, row-major (m[4 * row + col]), the same
// element order Eigen's (row, col) accessor names. Errors are the reference's
// exceptions: std::invalid_argument for a scene the path cannot take.
//
// The adapter's result is an rtgb_host_scene, the packed scene of the C ABI:
// rtgb_host_scene_view() gives the rtgb_scene for rtgb_prepare_scene(), and
// rtgb_host_scene_destroy() frees it.
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <string>
#include <string_view>
#include <unordered_map>
#include <variant>
#include <vector>

#include "rtgb.h"

namespace rtgb::scene {

using Vec2 = std::array<double, 2>;
using Vec3 = std::array<double, 3>;
using Vec4 = std::array<double, 4>;
using Vec2f = std::array<float, 2>;
using Vec3f = std::array<float, 3>;
using Vec4f = std::array<float, 4>;
using Mat4 = std::array<double, 16>;  // row-major affine matrix, column vectors: p' = M p

inline constexpr Mat4 kIdentity4 {1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0};

enum class SceneUpAxis { y, z };
enum class SceneTimeInterpolation { held, linear };
enum class SceneVisibility { inherited, invisible };
enum class ScenePurpose { default_, render, proxy, guide };
enum class ScenePrimKind { scope, texture, material, geometry_prototype, surface, volume, camera, light };
enum class SceneCameraProjection { perspective, orthographic };
enum class SceneCameraCalibrationModel { pinhole32, equi62_lut1d };

struct SceneCameraCalibration {
    SceneCameraCalibrationModel model = SceneCameraCalibrationModel::pinhole32;
    int image_width = 0;
    int image_height = 0;
    Vec2 focal_length_pixels {0.0, 0.0};
    Vec2 principal_point_pixels {0.0, 0.0};
    std::vector<double> radial_distortion;
    Vec2 tangential_distortion {0.0, 0.0};
    Mat4 camera_to_body = kIdentity4;
    bool compatibility_pose_fallback = false;
};

struct SceneCamera {
    SceneCameraProjection projection = SceneCameraProjection::perspective;
    // filmback and focal values in tenths of a scene unit (OpenUSD convention)
    double horizontal_aperture = 20.955;
    double vertical_aperture = 15.2908;
    double horizontal_aperture_offset = 0.0;
    double vertical_aperture_offset = 0.0;
    double focal_length = 50.0;
    Vec2 clipping_range {1.0, 1'000'000.0};
    double f_stop = 0.0;
    double focus_distance = 0.0;
    std::optional<SceneCameraCalibration> renderer_calibration;
};

struct SceneAssetReference {
    std::string authored_path;
    std::string evaluated_path;
    std::string resolved_path;
};

inline constexpr std::string_view kOpenPbrMaterialXNodeDef = "ND_open_pbr_surface_surfaceshader";
inline constexpr std::string_view kOpenPbrVersion = "1.1.1";

enum class SceneMaterialValueType { float_, color3, vector3 };
enum class SceneColorSpace { raw, linear_srgb, srgb_texture, acescg };
enum class SceneTextureNode { constant_color, checkerboard, image, noise3d };
enum class SceneTextureAddressMode { constant, clamp, periodic, mirror };
enum class SceneTextureFilterType { closest, linear, cubic };

struct SceneTexture {
    SceneTextureNode node = SceneTextureNode::constant_color;
    std::string node_definition = "ND_constant_color3";
    SceneMaterialValueType output_type = SceneMaterialValueType::color3;
    SceneColorSpace color_space = SceneColorSpace::linear_srgb;
    Vec3 value {0.0, 0.0, 0.0};
    double scale = 1.0;
    std::string even_texture_path;
    std::string odd_texture_path;
    std::string texcoord_primvar = "st";
    SceneTextureAddressMode u_address_mode = SceneTextureAddressMode::periodic;
    SceneTextureAddressMode v_address_mode = SceneTextureAddressMode::periodic;
    SceneTextureFilterType filter_type = SceneTextureFilterType::linear;
};

enum class SceneTextureChannel { rgb, red, green, blue, alpha, luminance };

struct SceneMaterialConnection {
    std::string input_name;  // OpenPBR input, e.g. "base_color"
    SceneMaterialValueType input_type = SceneMaterialValueType::color3;
    std::string texture_path;
    SceneTextureChannel channel = SceneTextureChannel::rgb;
};

enum class SceneMaterialXDisplacementType { none, scalar, vector3 };

struct SceneMaterialXDisplacement {
    SceneMaterialXDisplacementType type = SceneMaterialXDisplacementType::none;
    double scalar_value = 0.0;
    Vec3 vector_value {0.0, 0.0, 0.0};
    double scale = 1.0;
    std::string texture_path;
};

enum class SceneMaterialEnergyPolicy { open_pbr_layered_energy_conserving };

struct SceneOpenPbrSurface {
    std::string version = std::string {kOpenPbrVersion};

    double base_weight = 1.0;
    Vec3 base_color {0.8, 0.8, 0.8};
    double base_diffuse_roughness = 0.0;
    double base_metalness = 0.0;

    double specular_weight = 1.0;
    Vec3 specular_color {1.0, 1.0, 1.0};
    double specular_roughness = 0.3;
    double specular_ior = 1.5;
    double specular_roughness_anisotropy = 0.0;

    double transmission_weight = 0.0;
    Vec3 transmission_color {1.0, 1.0, 1.0};
    double transmission_depth = 0.0;
    Vec3 transmission_scatter {0.0, 0.0, 0.0};
    double transmission_scatter_anisotropy = 0.0;
    double transmission_dispersion_scale = 0.0;
    double transmission_dispersion_abbe_number = 20.0;

    double subsurface_weight = 0.0;
    Vec3 subsurface_color {0.8, 0.8, 0.8};
    double subsurface_radius = 1.0;
    Vec3 subsurface_radius_scale {1.0, 0.5, 0.25};
    double subsurface_scatter_anisotropy = 0.0;

    double fuzz_weight = 0.0;
    Vec3 fuzz_color {1.0, 1.0, 1.0};
    double fuzz_roughness = 0.5;

    double coat_weight = 0.0;
    Vec3 coat_color {1.0, 1.0, 1.0};
    double coat_roughness = 0.0;
    double coat_roughness_anisotropy = 0.0;
    double coat_ior = 1.6;
    double coat_darkening = 1.0;

    double thin_film_weight = 0.0;
    double thin_film_thickness = 0.5;
    double thin_film_ior = 1.4;

    double emission_luminance = 0.0;
    Vec3 emission_color {1.0, 1.0, 1.0};

    double geometry_opacity = 1.0;
    bool geometry_thin_walled = false;
    std::string geometry_normal_default_geomprop = "Nworld";
    std::string geometry_coat_normal_default_geomprop = "Nworld";
    std::string geometry_tangent_default_geomprop = "Tworld";
    std::string geometry_coat_tangent_default_geomprop = "Tworld";

    std::vector<SceneMaterialConnection> connections;
    SceneMaterialXDisplacement displacement;
    SceneMaterialEnergyPolicy energy_policy = SceneMaterialEnergyPolicy::open_pbr_layered_energy_conserving;
};

struct SceneIsotropicVolumeMaterial {
    Vec3 scattering_color {1.0, 1.0, 1.0};
    std::string scattering_color_texture_path;
    double scattering_anisotropy = 0.0;
};

using SceneMaterial = std::variant<SceneOpenPbrSurface, SceneIsotropicVolumeMaterial>;

enum class SceneLightType { geometry, sphere, disk, rect, cylinder, distant, dome };
enum class SceneLightMaterialSyncMode { material_glow_tints_light, independent, no_material_response };
enum class SceneLightIntensityUnit { nit, lux };

struct SceneLight {
    SceneLightType type = SceneLightType::sphere;
    Vec3 color {1.0, 1.0, 1.0};
    double intensity = 1.0;  // nits at exposure 0 (lux for a normalized distant light)
    double exposure = 0.0;   // stops: intensity * exp2(exposure)
    bool normalize = false;
    bool enable_color_temperature = false;
    double color_temperature_kelvin = 6500.0;
    double diffuse = 1.0;
    double specular = 1.0;
    SceneLightMaterialSyncMode material_sync_mode = SceneLightMaterialSyncMode::no_material_response;
    double radius = 0.5;
    double width = 1.0;
    double height = 1.0;
    double length = 1.0;
    double angle_degrees = 0.53;
    bool treat_as_point = false;
    bool treat_as_line = false;
};

enum class SceneMeshOrientation { right_handed, left_handed };
enum class SceneSubdivisionScheme { none, catmull_clark, loop, bilinear };
enum class ScenePrimvarInterpolation { constant, uniform, varying, vertex, face_varying };
enum class ScenePrimvarRole { none, point, normal, vector, color, texcoord };

using ScenePrimvarValues = std::variant<std::vector<std::int32_t>, std::vector<float>, std::vector<double>,
    std::vector<Vec2f>, std::vector<Vec3f>, std::vector<Vec4f>, std::vector<Vec2>, std::vector<Vec3>,
    std::vector<Vec4>, std::vector<std::string>>;

struct ScenePrimvar {
    std::string name;  // base name ("st"), without the "primvars:" prefix
    ScenePrimvarInterpolation interpolation = ScenePrimvarInterpolation::constant;
    ScenePrimvarRole role = ScenePrimvarRole::none;
    std::size_t element_size = 1;
    ScenePrimvarValues values;
    std::vector<std::int32_t> indices;
};

enum class SceneMaterialSubsetFamilyType { non_overlapping, partition };

struct SceneMaterialSubset {
    std::string name;
    std::vector<std::int32_t> face_indices;
    std::string material_path;
};

struct SceneSphereGeometry {
    Vec3 center {0.0, 0.0, 0.0};
    double radius = 1.0;
};

struct SceneMeshGeometry {
    std::vector<Vec3> points;
    std::vector<std::int32_t> face_vertex_counts;
    std::vector<std::int32_t> face_vertex_indices;
    SceneMeshOrientation orientation = SceneMeshOrientation::right_handed;
    SceneSubdivisionScheme subdivision_scheme = SceneSubdivisionScheme::none;
    std::vector<ScenePrimvar> primvars;
    SceneMaterialSubsetFamilyType material_subset_family_type = SceneMaterialSubsetFamilyType::non_overlapping;
    std::vector<SceneMaterialSubset> material_subsets;
};

using SceneGeometry = std::variant<SceneSphereGeometry, SceneMeshGeometry>;

struct SceneStageMetadata {
    double meters_per_unit = 0.01;
    SceneUpAxis up_axis = SceneUpAxis::y;
    bool right_handed = true;
    double time_codes_per_second = 24.0;
    double frames_per_second = 24.0;
    std::optional<double> start_time_code;
    std::optional<double> end_time_code;
    SceneTimeInterpolation interpolation = SceneTimeInterpolation::linear;
    std::string default_prim_path = "/World";
};

struct SceneTransformSample {
    double time_code = 0.0;
    Mat4 local_to_parent = kIdentity4;
};

struct ScenePrim {
    std::string path;
    ScenePrimKind kind = ScenePrimKind::scope;
    Mat4 local_to_parent = kIdentity4;
    bool reset_xform_stack = false;
    SceneVisibility visibility = SceneVisibility::inherited;
    std::optional<ScenePurpose> authored_purpose;
    std::vector<SceneTransformSample> transform_samples;

    std::string prototype_path;
    std::string material_path;
    std::optional<double> volume_density;
    std::optional<SceneGeometry> geometry;
    std::optional<SceneCamera> camera;
    std::optional<SceneLight> light;  // kind=light, or a geometry light on a surface
    std::optional<SceneTexture> texture;
    std::optional<SceneMaterial> material;
    std::vector<SceneAssetReference> asset_references;
    std::optional<std::size_t> compatibility_source_index;
    std::optional<std::string> compatibility_source_name;
};

class SceneIRv2 {
public:
    SceneStageMetadata& stage_metadata() { return stage_metadata_; }
    const SceneStageMetadata& stage_metadata() const { return stage_metadata_; }

    // Appends a prim; find_prim resolves a path to its first prim.
    std::size_t add_prim(ScenePrim prim);
    const std::vector<ScenePrim>& prims() const { return prims_; }
    const ScenePrim* find_prim(std::string_view path) const;

private:
    SceneStageMetadata stage_metadata_;
    std::vector<ScenePrim> prims_;
    std::unordered_map<std::string, std::size_t> first_prim_by_path_;
};

enum class SceneDiagnosticSeverity { warning, error };

struct SceneDiagnostic {
    SceneDiagnosticSeverity severity = SceneDiagnosticSeverity::error;
    std::string code;  // the reference validator's code, e.g. "geometry.mesh.face_counts"
    std::string prim_path;
    std::string message;
};

bool is_valid_scene_prim_path(std::string_view path);
std::string parent_scene_prim_path(std::string_view path);

std::vector<SceneDiagnostic> validate_scene_ir_v2(const SceneIRv2& scene);
void require_valid_scene_ir_v2(const SceneIRv2& scene);
bool has_scene_diagnostic(const std::vector<SceneDiagnostic>& diagnostics, std::string_view code);

Mat4 sample_scene_local_transform(const ScenePrim& prim, double time_code, SceneTimeInterpolation interpolation);
Mat4 compute_scene_world_transform(const SceneIRv2& scene, std::string_view prim_path, double time_code);
bool compute_scene_visibility(const SceneIRv2& scene, std::string_view prim_path);
ScenePurpose compute_scene_purpose(const SceneIRv2& scene, std::string_view prim_path);

double scene_light_exposed_intensity(const SceneLight& light);
SceneLightIntensityUnit scene_light_intensity_unit(const SceneLight& light);

// AnalyticLightDesc (src/common/analytic_light.h:19-39): one compiled light in
// double precision before packing into rtgb_analytic_light.
enum class AnalyticLightType : int { sphere = 0, disk = 1, rect = 2, cylinder = 3, distant = 4, dome = 5 };

struct AnalyticLightDesc {
    AnalyticLightType type = AnalyticLightType::sphere;
    std::string source_path;
    Vec3 position {0.0, 0.0, 0.0};
    std::array<double, 9> local_to_world_linear {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};  // row-major
    Vec3 radiance {0.0, 0.0, 0.0};
    double radius = 0.5;
    double width = 1.0;
    double height = 1.0;
    double length = 1.0;
    double world_area = 0.0;
    double cos_theta_max = 1.0;
    double diffuse = 1.0;
    double specular = 1.0;
    double selection_weight = 0.0;
    double selection_pdf = 0.0;
    double cdf = 0.0;
    bool delta = false;
    bool treat_as_point = false;
    bool treat_as_line = false;
};

void finalize_analytic_light_distribution(std::vector<AnalyticLightDesc>& lights);
std::vector<AnalyticLightDesc> compile_analytic_lights(const SceneIRv2& scene);
rtgb_analytic_light pack_analytic_light(const AnalyticLightDesc& light);

// OpenPBR surface -> the compiled parameter block. Without a scene, connected
// inputs are rejected; with one, each connection binds the realtime texture
// index of its texture prim (texture_indices: prim path -> index).
rtgb_openpbr_material compile_openpbr_core_material(const SceneOpenPbrSurface& material);
rtgb_openpbr_material compile_openpbr_core_material(const SceneOpenPbrSurface& material, const SceneIRv2& scene,
    const std::unordered_map<std::string, int>& texture_indices);

struct HostSceneDeleter {
    void operator()(rtgb_host_scene* scene) const { rtgb_host_scene_destroy(scene); }
};
using HostScenePtr = std::unique_ptr<rtgb_host_scene, HostSceneDeleter>;

// Options of the lowering that the reference takes from its environment.
struct AdaptOptions {
    // Image textures: files are read as 8-bit PNG (grey, RGB or RGBA), texels
    // scaled by 1/255 (OpenCV imread + convertTo(1/255) in the reference). A
    // path that does not open leaves the texture with zero size, as there.
    bool load_images = true;
};

// realtime_scene_adapter.cpp:502-581: texture prims in prim order, then each
// OpenPBR material prim, then every visible render/default-purpose surface
// (spheres need a uniform scale; meshes are fan-triangulated with winding,
// normals, texcoords and material subsets), then the analytic lights.
HostScenePtr adapt_scene_ir_v2_to_realtime(const SceneIRv2& scene, const AdaptOptions& options = {});

// Per-primitive BLAS bookkeeping of the adapter (prototype and instance ids,
// one entry per sphere / triangle in packed order): the reference keeps these
// on each primitive for its instanced acceleration structures. This path
// flattens instances, so they are reported, not packed.
struct AccelerationIds {
    std::vector<int> sphere_prototype, sphere_instance, triangle_prototype, triangle_instance;
};
HostScenePtr adapt_scene_ir_v2_to_realtime(const SceneIRv2& scene, AccelerationIds& ids,
    const AdaptOptions& options = {});

// The mesh half of the lowering left instanced, for the device flattening of
// rtgb_prepare_scene_instanced: each mesh prototype fan-triangulated with its
// primvars sampled once (corner order before any winding flip, subset
// materials or RTGB_INSTANCE_MATERIAL), each visible mesh surface one
// instance (world transform, inverse linear part, bound material, winding
// flip), in the order the flat lowering appends their triangles.
struct MeshInstances {
    struct Prototype {
        std::vector<double> points;             // xyz per point
        std::vector<int32_t> corner_points;     // 3 per triangle
        std::vector<double> corner_normals;     // 9 per triangle; empty without a normals primvar
        std::vector<double> corner_texcoords;   // 6 per triangle; empty without an st primvar
        std::vector<int32_t> triangle_materials;
    };
    std::vector<Prototype> prototypes;
    std::vector<rtgb_mesh_instance> instances;

    // A view of the arrays above, valid until this object changes.
    rtgb_mesh_set view();

private:
    std::vector<rtgb_mesh_prototype> views_;
};

// adapt_scene_ir_v2_to_realtime with the meshes in `meshes` instead of the
// host scene's triangles; rtgb_prepare_scene_instanced(handle, &scene view,
// &meshes.view()) then prepares the same scene as the flat lowering.
HostScenePtr adapt_scene_ir_v2_to_realtime_instanced(const SceneIRv2& scene, MeshInstances& meshes,
    const AdaptOptions& options = {});

}  // namespace rtgb::scene
