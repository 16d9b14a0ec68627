/*
 * rtgb.h — C ABI of the GB300 wavefront path tracer.
 *
 * This is the drop-in boundary for the realtime per-pixel radiance path of
 * elegracer/ray_tracing. The reference exposes that path only as C++ classes;
 * every entry point below names the reference member it replaces (file:line,
 * relative to the reference project root).
 *
 * Conventions
 *   - Plain C: POD structs, raw pointers and sizes, status codes. No C++
 *     exceptions cross this boundary; rtgb_last_error() returns the message
 *     the reference would have thrown.
 *   - One thread per handle. A handle owns its CUDA stream, its device scene,
 *     all frame/history buffers and its CUDA graphs.
 *   - Device views returned by rtgb_render_frame() stay valid until the next
 *     rtgb_render_frame()/rtgb_prepare_scene()/rtgb_destroy() on that handle
 *     (the reference states the same contract at
 *     src/realtime/gpu/optix_renderer.h:84).
 */
#ifndef RTGB_H
#define RTGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTGB_ABI_VERSION 1
#define RTGB_MAX_CAMERAS 4          /* PackedCameraRig slots, src/realtime/camera_rig.h:27-30 */
#define RTGB_EQUI_LUT_SIZE 1024     /* Equi62Lut1DParams::lut, src/realtime/camera_models.h:30-40 */

typedef enum rtgb_status {
    RTGB_OK = 0,
    RTGB_INVALID_ARGUMENT = 1,   /* reference: std::invalid_argument / request validation */
    RTGB_RUNTIME_ERROR = 2,      /* reference: std::runtime_error (CUDA failure, capacity) */
    RTGB_NOT_PREPARED = 3,       /* render before rtgb_prepare_scene */
    RTGB_DEVICE_FAULT_FLAG = 4,  /* a bounded device loop gave up and set the error word */
    RTGB_UNSUPPORTED = 5
} rtgb_status;

/* ------------------------------------------------------------------------ */
/* Scene: the packed (post prepare_gpu_scene) form of PackedScene.          */
/* Mirrors src/realtime/gpu/launch_params.h:135-237 and                     */
/* src/common/light_sampling.h:44-62, with Eigen members replaced by float. */
/* ------------------------------------------------------------------------ */

typedef enum rtgb_material_type {
    RTGB_MATERIAL_LAMBERTIAN = 0,
    RTGB_MATERIAL_METAL = 1,
    RTGB_MATERIAL_DIELECTRIC = 2,
    RTGB_MATERIAL_DIFFUSE_LIGHT = 3,
    RTGB_MATERIAL_ISOTROPIC = 4,
    RTGB_MATERIAL_OPENPBR = 5
} rtgb_material_type;

typedef enum rtgb_texture_type {
    RTGB_TEXTURE_CONSTANT = 0,
    RTGB_TEXTURE_CHECKER = 1,
    RTGB_TEXTURE_IMAGE = 2,
    RTGB_TEXTURE_NOISE = 3
} rtgb_texture_type;

typedef enum rtgb_analytic_light_type {
    RTGB_ANALYTIC_SPHERE = 0,
    RTGB_ANALYTIC_DISK = 1,
    RTGB_ANALYTIC_RECT = 2,
    RTGB_ANALYTIC_CYLINDER = 3,
    RTGB_ANALYTIC_DISTANT = 4,
    RTGB_ANALYTIC_DOME = 5
} rtgb_analytic_light_type;

/* PackedTexture, launch_params.h:226-237 */
typedef struct rtgb_texture {
    int32_t type;
    int32_t even_texture;
    int32_t odd_texture;
    int32_t image_offset;   /* first texel in rtgb_scene::image_texels */
    int32_t image_width;
    int32_t image_height;
    int32_t u_address_mode; /* 0 constant, 1 clamp, 2 periodic, 3 mirror */
    int32_t v_address_mode;
    int32_t filter_type;    /* 0 closest, 1 linear */
    float scale;
    float color[3];
} rtgb_texture;

/* MaterialSample, launch_params.h:216-223 */
typedef struct rtgb_material {
    int32_t albedo_texture;
    int32_t emission_texture;
    float ior;
    float fuzz;
    int32_t type;           /* rtgb_material_type */
    int32_t openpbr_index;
} rtgb_material;

/* OpenPbrCompiledMaterial, src/common/openpbr_core.h:33-122: the OpenPBR
 * parameter block (OpenPbrCoreMaterial, field for field) followed by the
 * texture bindings. A texture index < 0 means "use the parameter". Color
 * bindings carry the source color space (0 raw, 1 linear sRGB, 2 sRGB
 * texture: decoded with the sRGB transfer curve). */
typedef struct rtgb_openpbr_material {
    float base_weight;
    float base_color[3];
    float base_diffuse_roughness;
    float base_metalness;
    float specular_weight;
    float specular_color[3];
    float specular_roughness;
    float specular_ior;
    float specular_roughness_anisotropy;
    float transmission_weight;
    float transmission_color[3];
    float transmission_depth;
    float transmission_dispersion_scale;
    float transmission_dispersion_abbe_number;
    float subsurface_weight;
    float subsurface_color[3];
    float subsurface_radius;
    float subsurface_radius_scale[3];
    float subsurface_scatter_anisotropy;
    float fuzz_weight;
    float fuzz_color[3];
    float fuzz_roughness;
    float coat_weight;
    float coat_color[3];
    float coat_roughness;
    float coat_roughness_anisotropy;
    float coat_ior;
    float coat_darkening;
    float thin_film_weight;
    float thin_film_thickness;      /* micrometres */
    float thin_film_ior;
    float emission_luminance;
    float emission_color[3];
    float geometry_opacity;
    int32_t geometry_thin_walled;
    /* color bindings: base, specular, transmission, emission */
    int32_t color_texture[4];
    int32_t color_space[4];
    /* scalar bindings: base_metalness, specular_roughness (texture's red channel) */
    int32_t scalar_texture[2];
} rtgb_openpbr_material;

/* PackedSphere, launch_params.h:135-141 */
typedef struct rtgb_sphere {
    float center[3];
    float radius;
    int32_t material_index;
} rtgb_sphere;

/* PackedQuad, launch_params.h:143-152 */
typedef struct rtgb_quad {
    float origin[3];
    float edge_u[3];
    float edge_v[3];
    int32_t material_index;
} rtgb_quad;

/* PackedTriangle, launch_params.h:154-175 */
typedef struct rtgb_triangle {
    float p0[3];
    float p1[3];
    float p2[3];
    float n0[3];
    float n1[3];
    float n2[3];
    float uv0[2];
    float uv1[2];
    float uv2[2];
    int32_t material_index;
    int32_t has_vertex_normals;
    int32_t has_texcoords;
} rtgb_triangle;

/* PackedMedium, launch_params.h:201-214 (rotation rows are world->local) */
typedef struct rtgb_medium {
    float local_center_or_min[3];
    float radius;
    float local_max[3];
    float density;
    float rotation_row0[3];
    float rotation_row1[3];
    float rotation_row2[3];
    float translation[3];
    int32_t material_index;
    int32_t boundary_type;  /* 0 sphere, 1 box */
} rtgb_medium;

/* PackedAnalyticLight, src/common/light_sampling.h:44-62 */
typedef struct rtgb_analytic_light {
    int32_t type;           /* rtgb_analytic_light_type */
    float position[3];
    float basis_x[3];
    float basis_y[3];
    float basis_z[3];
    float radiance[3];
    float radius;
    float width;
    float height;
    float length;
    float world_area;
    float cos_theta_max;
    float selection_pdf;
    float cdf;
    int32_t delta;
    int32_t treat_as_point;
    int32_t treat_as_line;
} rtgb_analytic_light;

/* PackedScene (src/realtime/scene_description.h:130-146) after
 * prepare_gpu_scene (src/realtime/gpu/packed_scene_preparation.cpp:306-348).
 * The emissive-geometry light CDF (build_light_distribution, :265-302) is
 * computed by the library; the analytic-light CDF is the caller's (it comes
 * from finalize_analytic_light_distribution, src/scene/analytic_light_compiler.cpp:15-39). */
typedef struct rtgb_scene {
    const rtgb_texture* textures;
    int32_t texture_count;
    const float* image_texels;          /* RGB float triplets */
    int32_t image_texel_count;          /* number of triplets */
    const rtgb_material* materials;
    int32_t material_count;
    const rtgb_sphere* spheres;
    int32_t sphere_count;
    const rtgb_quad* quads;
    int32_t quad_count;
    const rtgb_triangle* triangles;
    int32_t triangle_count;
    const rtgb_medium* media;
    int32_t medium_count;
    const rtgb_analytic_light* analytic_lights;
    int32_t analytic_light_count;
    float background[3];
    const rtgb_openpbr_material* openpbr_materials;   /* rtgb_material::openpbr_index */
    int32_t openpbr_material_count;
} rtgb_scene;

/* Instanced meshes flattened on the device (rtgb_prepare_scene_instanced): the
 * mesh half of the SceneIR v2 lowering (add_v2_mesh,
 * src/scene/realtime_scene_adapter.cpp:289-346), with each prototype
 * triangulated and its primvars sampled once on the host and every instance's
 * triangles (transformed points and normals, winding, materials) produced by
 * a kernel. */
#define RTGB_INSTANCE_MATERIAL (-2147483647 - 1)  /* triangle_materials entry: use the instance's material */

typedef struct rtgb_mesh_prototype {
    const double* points;              /* xyz per point */
    int32_t point_count;
    int32_t triangle_count;            /* fan triangles of the mesh's faces, in face order */
    const int32_t* corner_points;      /* 3 point indices per triangle (fan order, before any winding flip) */
    const double* corner_normals;      /* 9 per triangle: the normals primvar at the 3 corners, or NULL */
    const double* corner_texcoords;    /* 6 per triangle: the st primvar at the 3 corners, or NULL */
    const int32_t* triangle_materials; /* per triangle: a material index (subsets) or RTGB_INSTANCE_MATERIAL */
} rtgb_mesh_prototype;

typedef struct rtgb_mesh_instance {
    int32_t prototype;
    int32_t material;                  /* the surface's bound material */
    int32_t flip_winding;              /* swap corners 1 and 2 (orientation against the transform's handedness) */
    int32_t reserved;
    double world[12];                  /* row-major 3 x 4 affine transform */
    double normal_matrix[9];           /* inverse of the linear part; normals transform by its transpose */
} rtgb_mesh_instance;

typedef struct rtgb_mesh_set {
    const rtgb_mesh_prototype* prototypes;
    int32_t prototype_count;
    const rtgb_mesh_instance* instances; /* flattened in this order after the scene's own triangles */
    int32_t instance_count;
} rtgb_mesh_set;

/* ------------------------------------------------------------------------ */
/* Cameras: PackedCamera / PackedCameraRig, src/realtime/camera_rig.h:15-30  */
/* ------------------------------------------------------------------------ */

typedef enum rtgb_camera_model {
    RTGB_CAMERA_PINHOLE32 = 0,
    RTGB_CAMERA_EQUI62_LUT1D = 1
} rtgb_camera_model;

/* Pinhole32Params, src/realtime/camera_models.h:14-24 */
typedef struct rtgb_pinhole32 {
    double fx, fy, cx, cy, k1, k2, k3, p1, p2;
} rtgb_pinhole32;

/* Equi62Lut1DParams, src/realtime/camera_models.h:26-37 */
typedef struct rtgb_equi62_lut1d {
    int32_t width;
    int32_t height;
    double fx, fy, cx, cy;
    double radial[6];
    double tangential[2];
    double lut[RTGB_EQUI_LUT_SIZE];
    double lut_step;
} rtgb_equi62_lut1d;

/* PackedCamera. T_rc maps camera coordinates (x right, y down, z forward)
 * into renderer/world coordinates: rotation is row-major 3x3. */
typedef struct rtgb_camera {
    int32_t enabled;
    int32_t width;
    int32_t height;
    int32_t model;          /* rtgb_camera_model */
    double rotation[9];
    double translation[3];
    rtgb_pinhole32 pinhole;
    rtgb_equi62_lut1d equi;
} rtgb_camera;

typedef struct rtgb_camera_rig {
    int32_t active_count;
    rtgb_camera cameras[RTGB_MAX_CAMERAS];
} rtgb_camera_rig;

/* RenderProfile, src/realtime/render_profile.h:10-25 */
typedef struct rtgb_render_profile {
    int32_t samples_per_pixel;
    int32_t max_bounces;
    int32_t enable_denoise;
    int32_t rr_start_bounce;
    double accumulation_reset_rotation_deg;
    double accumulation_reset_translation;
    int32_t enable_restir_di;
    int32_t restir_initial_candidates;
    int32_t restir_temporal_reuse;
    int32_t restir_max_history_age;
    int32_t restir_max_temporal_candidates;
    int32_t restir_spatial_neighbors;
    int32_t restir_max_spatial_candidates;
    int32_t restir_bias_correction;   /* 0 off, 1 basic (src/common/restir_di.h:16-19) */
    int32_t restir_min_analytic_lights;
    /* No reference counterpart (0 keeps the reference's behaviour). 1: ReSTIR DI
     * resamples the emissive-geometry lights (the light list NEE samples,
     * packed_scene_preparation.cpp:265-302) instead of the analytic lights:
     * bounce-0 receivers that are not emitters take their emissive direct
     * light from the reservoir (candidates, temporal and spatial reuse, BASIC
     * bias correction as for analytic lights) in place of the one-sample
     * emissive NEE, and analytic lights, if any, get the plain analytic NEE.
     * The reference's ReSTIR covers analytic lights only (programs.cu:1915-1924). */
    int32_t restir_emissive;
} rtgb_render_profile;

/* ------------------------------------------------------------------------ */
/* Renderer                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct rtgb_renderer* rtgb_handle;

typedef struct rtgb_create_info {
    int32_t device;            /* CUDA ordinal (the reference hard-codes 0: optix_renderer.cpp:120) */
    int32_t use_cuda_graph;    /* capture each frame's launch sequence as a CUDA graph */
    int32_t debug_path_records;/* record per-path hit codes and radiance (parity tests) */
    int32_t stage_timing;      /* record CUDA events between the frame's launches (rtgb_stage_times) */
    int32_t shade_order;       /* shade each bounce's paths bucketed by hit material: 0 automatic (from
                                  bounce 0 when the scene has OpenPBR materials or more than 8
                                  materials), 2 always from bounce 0, 1 from bounce 1, -1 never;
                                  results do not depend on it */
    int32_t debug_traversal_limit; /* node visits per BVH traversal before the loop gives up; 0 = 2^24.
                                      No reference counterpart: the reference's traversal loop is unbounded
                                      (programs.cu:1632-1650). A loop that gives up makes the frame return
                                      RTGB_DEVICE_FAULT_FLAG; small values exist to test that path. */
    int32_t debug_rejection_limit; /* draws of the rejection sampler (random_in_unit_sphere,
                                      programs.cu:125-133, unbounded there) before it gives up; 0 = 10^6 */
} rtgb_create_info;

/* DeviceRadianceFrameView (src/realtime/gpu/device_radiance_frame_view.h) plus
 * the remaining DeviceFrameBuffers AOVs (launch_params.h:25-34) and
 * RadianceTiming (optix_renderer.h:27-31). Pointers are device pointers. */
typedef struct rtgb_camera_frame_view {
    int32_t camera_index;
    int32_t width;
    int32_t height;
    const void* beauty;           /* float4 per pixel */
    const void* normal;           /* float4, [0,1]-encoded world normal */
    const void* denoiser_normal;  /* float4, camera-space normal */
    const void* albedo;           /* float4 */
    const void* depth;            /* float */
    const void* flow;             /* float2 */
    const void* flow_trustworthiness; /* float */
    float render_ms;
    float denoise_ms;
    float download_ms;
} rtgb_camera_frame_view;

typedef struct rtgb_frame_views {
    int32_t camera_count;
    rtgb_camera_frame_view cameras[RTGB_MAX_CAMERAS];
    float frame_render_ms;        /* whole-frame CUDA-event time (all cameras, one launch sequence) */
    uint32_t sample_stream;       /* stream used for this frame */
    uint64_t rays_traced;         /* primary+extension+shadow+ReSTIR visibility rays */
    uint64_t primary_rays;
    uint64_t extension_rays;
    uint64_t shadow_rays;
    uint64_t restir_visibility_rays;
    uint64_t h2d_bytes;           /* bytes this frame copied host -> device (frame parameters, camera tables) */
    uint64_t active_paths[64];    /* paths entering each bounce (wavefront queue lengths) */
    uint64_t restir_pixels;       /* bounce-0 paths that ran ReSTIR DI */
    uint64_t shadow_per_bounce[64]; /* shadow rays traced at each bounce */
} rtgb_frame_views;

/* RestirDiagnostics, optix_renderer.h:43-51 */
typedef struct rtgb_restir_stats {
    int32_t pixel_count;
    int32_t active_reservoir_count;
    int32_t temporal_reuse_count;
    int32_t spatial_reuse_count;
    int32_t bias_corrected_count;
    int32_t max_candidate_count;
    int32_t max_age;
} rtgb_restir_stats;

/* AccelerationUpdateStats-like summary of the device LBVH. */
typedef struct rtgb_acceleration_info {
    int32_t primitive_count;      /* spheres + quads + triangles */
    int32_t node_count;           /* internal BVH2 nodes */
    int32_t analytic_light_node_count;
    int32_t analytic_bvh_light_count; /* finite, non-point analytic lights in the light BVH */
    float build_ms;               /* device build time (Morton, sort, hierarchy, bounds) */
    int32_t traversal_stack_overflows; /* count since the last prepare; always reported, never silent */
    /* AccelerationUpdateKind of the last rtgb_prepare_scene (gpu_scene_acceleration.cpp:247-295):
     * 0 reuse (nothing changed), 1 update (non-geometry data changed),
     * 2 refit (same primitive counts, geometry changed: node boxes refitted
     * over the kept hierarchy), 3 rebuild */
    int32_t update_kind;
    int32_t generation;           /* incremented by every update, refit and rebuild */
    int32_t wide_node_count;      /* nodes of the 4-wide BVH the rays traverse (rtgb_download_bvh4) */
} rtgb_acceleration_info;

/* Replaces OptixRenderer::OptixRenderer + RendererPool(int) (optix_renderer.cpp:104-109,
 * renderer_pool.cpp:111-116): one handle serves every camera of a rig. */
rtgb_status rtgb_create(const rtgb_create_info* info, rtgb_handle* out_handle);
void rtgb_destroy(rtgb_handle handle);

/* Last error message of this handle ("" if none). */
const char* rtgb_last_error(rtgb_handle handle);

/* Replaces OptixRenderer::prepare_scene / RendererPool::prepare_scene
 * (optix_renderer.cpp:440-456, renderer_pool.cpp:120): packs the scene,
 * builds the light CDF, uploads it and builds the device LBVH. Resets the
 * sample stream to 0 and the temporal history, like use_prepared_scene. */
rtgb_status rtgb_prepare_scene(rtgb_handle handle, const rtgb_scene* scene);

/* rtgb_prepare_scene with instanced meshes: the scene's own primitives, then
 * every instance of `meshes` flattened on the device into triangles appended
 * after the scene's triangles, bit for bit the triangles the host lowering
 * (add_v2_mesh, realtime_scene_adapter.cpp:289-346) appends. A normal whose
 * transformed length is not finite or at most 1e-12 fails the call with the
 * reference's message. Reuse / update / refit / rebuild as rtgb_prepare_scene,
 * with the mesh set part of the geometry. */
rtgb_status rtgb_prepare_scene_instanced(rtgb_handle handle, const rtgb_scene* scene, const rtgb_mesh_set* meshes);

/* The device triangle array of the prepared scene (the scene's triangles, then
 * the flattened instances): up to `capacity` records into `out` (may be NULL)
 * and the total in *count. */
rtgb_status rtgb_download_triangles(rtgb_handle handle, rtgb_triangle* out, int32_t capacity, int32_t* count);

/* OptixRenderer::reset_sequence (optix_renderer.cpp:178-181). */
rtgb_status rtgb_reset_sequence(rtgb_handle handle, uint32_t sample_stream);

/* OptixRenderer::reset_accumulation (optix_renderer.cpp:173-176). */
rtgb_status rtgb_reset_accumulation(rtgb_handle handle);

/* Replaces RendererPool::render_device_frame / render_frame
 * (renderer_pool.cpp:160-185) and OptixRenderer::render_prepared_device
 * (optix_renderer.cpp:434-457): all `active_cameras` leading slots of the rig
 * render in ONE launch sequence on the handle's stream, then the frame's
 * sample stream advances by one. Returns device views and timings. The call
 * is asynchronous except for reading back the frame's ray counters. */
rtgb_status rtgb_render_frame(rtgb_handle handle, const rtgb_camera_rig* rig,
    const rtgb_render_profile* profile, int32_t active_cameras, rtgb_frame_views* out_views);

/* rtgb_render_frame without the final wait: the frame is enqueued on the
 * handle's stream and the call returns. Views and statistics of the last
 * enqueued frame come from rtgb_frame_stats(). */
rtgb_status rtgb_render_frame_async(rtgb_handle handle, const rtgb_camera_rig* rig,
    const rtgb_render_profile* profile, int32_t active_cameras);

/* Waits for the last enqueued frame and fills its views, timing and ray counts. */
rtgb_status rtgb_frame_stats(rtgb_handle handle, rtgb_frame_views* out_views);

/* Per-launch device times (ms) of the last frame, in launch order:
 * raygen, then per bounce trace / shade (+ ReSTIR DI at bounce 0) / shadow,
 * then finalize and resolve (3 * max_bounces + 3 entries). Needs
 * rtgb_create_info::stage_timing. */
rtgb_status rtgb_stage_times(rtgb_handle handle, float* out_ms, int32_t capacity, int32_t* out_count);

/* Changes the debug loop bounds of rtgb_create_info on a live handle (0 keeps
 * the default). No reference counterpart. Frames after the call use the new
 * bounds; a frame in which a bounded loop gave up returns
 * RTGB_DEVICE_FAULT_FLAG with the count in rtgb_last_error, and the handle
 * stays usable. */
rtgb_status rtgb_set_debug_limits(rtgb_handle handle, int32_t traversal_limit, int32_t rejection_limit);

/* Launch shape of each wavefront launch slot the handle uses now (persistent
 * sizes, or the autotuner's choice): grid size in blocks and threads per
 * block (`blocks` may be NULL). No reference counterpart (OptiX picks its own
 * launch shapes). Fills min(capacity, count) entries; *count = number of slots. */
rtgb_status rtgb_launch_grids(rtgb_handle handle, int32_t* grids, int32_t* blocks, int32_t capacity, int32_t* count);

/* Launch-shape autotuner (no reference counterpart; the reference leaves
 * launch shapes to OptiX). Renders `frames` (1..64) frames of this rig and
 * profile with every wavefront launch at each of RTGB_TUNE_CANDIDATES shapes:
 * grid scales 0.5, 1, 2, 4 of the persistent size (SMs x resident blocks) with
 * the kernels' own block size, then the same four with half-size blocks (and
 * twice the blocks, so the same threads); times every stage with events, and
 * keeps per stage group (raygen, trace, shade with ReSTIR and material
 * bucketing, shadow, finalize + resolve) the fastest shape for the handle's
 * later frames. Results never depend on the shapes (the kernels loop
 * grid-stride over their queues). The tuning frames are discarded:
 * accumulation and history restart. Call after prepare_scene. */
#define RTGB_TUNE_CANDIDATES 8
#define RTGB_TUNE_GROUPS 5
typedef struct rtgb_launch_tuning {
    float scales[RTGB_TUNE_CANDIDATES];                   /* grid scales tried (of the persistent grid at that block size) */
    int32_t block_halved[RTGB_TUNE_CANDIDATES];           /* 1: the candidate uses half-size blocks */
    float group_ms[RTGB_TUNE_CANDIDATES][RTGB_TUNE_GROUPS];/* per frame: raygen, trace, shade, shadow, finalize+resolve */
    float frame_ms[RTGB_TUNE_CANDIDATES];                 /* whole frame at each candidate */
    int32_t chosen[RTGB_TUNE_GROUPS];                     /* index into the candidates, per group */
    float tuned_frame_ms;                                 /* whole frame with the chosen shapes */
} rtgb_launch_tuning;
rtgb_status rtgb_autotune_launches(rtgb_handle handle, const rtgb_camera_rig* rig,
    const rtgb_render_profile* profile, int32_t active_cameras, int32_t frames, rtgb_launch_tuning* out);

/* Rays traced since the scene was prepared: primary, extension, shadow and
 * ReSTIR visibility (waits for the stream). */
rtgb_status rtgb_ray_totals(rtgb_handle handle, uint64_t totals[4]);

/* Replaces download_radiance_frame_profiled (optix_renderer.cpp:283-326):
 * copies the last frame's AOVs of one camera into caller-owned host memory.
 * Any pointer may be NULL. Sizes are width*height*4 floats (rgba) and
 * width*height floats (depth). Returns the copy time in *download_ms. */
rtgb_status rtgb_download_frame(rtgb_handle handle, int32_t camera_index, float* beauty_rgba,
    float* normal_rgba, float* albedo_rgba, float* depth, float* download_ms);

/* Pipelined form of rtgb_download_frame (no counterpart in the reference,
 * whose download waits for its copies): enqueues the same copies of the last
 * frame's buffers on the handle's copy stream, after that frame's kernels, and
 * returns without waiting, so the copies overlap the next frame's rendering.
 * Page-locked host memory (cudaHostAlloc / cudaHostRegister) is needed for the
 * overlap; with other memory the copies are still correct but the call waits
 * for them. The host buffers must stay valid and unread until
 * rtgb_wait_downloads returns. The frame after next, which reuses the frame's
 * device buffers, waits for these copies on the device. Any pointer may be
 * NULL. */
rtgb_status rtgb_download_frame_async(rtgb_handle handle, int32_t camera_index, float* beauty_rgba,
    float* normal_rgba, float* albedo_rgba, float* depth);

/* Waits until the copies of rtgb_download_frame_async have landed in host
 * memory: all of them (keep_latest == 0), or all but those of the most
 * recently downloaded frame (keep_latest != 0; the double-buffered loop
 * render(i), download_async(i), wait_downloads(1) -> frame i-1 is on the host). */
rtgb_status rtgb_wait_downloads(rtgb_handle handle, int32_t keep_latest);

/* The emissive light table of the prepared scene, built on the device
 * (build_light_distribution, packed_scene_preparation.cpp:265-302): `lights`
 * receives up to `capacity` 16-byte records {int32 type (0 sphere, 1 quad,
 * 2 triangle, 3 environment), int32 primitive_index, float selection_pdf,
 * float cdf} (the reference's PackedLight, light_sampling.h:15-27) and
 * *light_count the table's length; each non-NULL map receives one int32 per
 * sphere / quad / triangle of the scene: the primitive's light index or -1.
 * lights may be NULL to query the count. */
rtgb_status rtgb_download_light_table(rtgb_handle handle, void* lights, int32_t capacity, int32_t* light_count,
    int32_t* sphere_light, int32_t* quad_light, int32_t* triangle_light);

/* Copies any device frame buffer of one camera (flow, trust, denoiser normal)
 * to host: which = 0 beauty (the path tracer's, before denoising), 1 normal,
 * 2 denoiser_normal, 3 albedo, 4 depth, 5 flow, 6 flow_trustworthiness,
 * 8 denoised beauty (only after a denoised frame). `bytes` must equal the
 * buffer size. */
rtgb_status rtgb_download_buffer(rtgb_handle handle, int32_t camera_index, int32_t which,
    void* host, size_t bytes);

/* OptixRenderer::restir_diagnostics (optix_renderer.cpp:183-215), per camera. */
rtgb_status rtgb_restir_diagnostics(rtgb_handle handle, int32_t camera_index,
    rtgb_restir_stats* out);

/* Copies the last frame's reservoirs of one camera (84 bytes each, the
 * RestirReservoir layout of src/common/restir_di.h:36-48). */
rtgb_status rtgb_download_reservoirs(rtgb_handle handle, int32_t camera_index, void* host,
    size_t bytes);

/* OptixRenderer::render_direction_debug (optix_renderer.cpp:156-162 ->
 * programs.cu:1807-1826): RGBA8 encoding of world ray directions. */
rtgb_status rtgb_render_direction_debug(rtgb_handle handle, const rtgb_camera_rig* rig,
    int32_t camera_index, uint8_t* host_rgba);

/* Headless tone map of a camera's beauty into RGBA8 host memory, the
 * arithmetic of src/realtime/viewer/cuda_gl_presenter.cu:23-38. */
rtgb_status rtgb_tonemap_rgba8(rtgb_handle handle, int32_t camera_index, uint8_t* host_rgba);

rtgb_status rtgb_acceleration_info_get(rtgb_handle handle, rtgb_acceleration_info* out);

/* Device identity, toolkit versions and device-global memory use (the
 * RunEnvironment / GPU memory fields of the reference's benchmark report,
 * utils/render_realtime.cpp:55-134). */
typedef struct rtgb_device_info {
    char name[256];
    int32_t device;
    int32_t major, minor;            /* compute capability */
    int32_t multiprocessors;
    int32_t driver_version;          /* cudaDriverGetVersion */
    int32_t runtime_version;         /* cudaRuntimeGetVersion */
    uint64_t total_bytes;
    uint64_t used_bytes;             /* total - free (all processes) */
} rtgb_device_info;

rtgb_status rtgb_device_info_get(rtgb_handle handle, rtgb_device_info* out);

/* The CUDA stream (cudaStream_t) every launch of this handle is issued on. */
void* rtgb_stream(rtgb_handle handle);

/* Parity support (only with rtgb_create_info::debug_path_records).
 * Per path (pixel-major, then sample) and bounce: hit code
 *   -1 miss, (k << 28) | (decisions << 22) | index with k = 0 sphere, 1 quad,
 *   2 triangle, 4 medium, 5 analytic light; decisions: bit 0 emissive NEE
 *   visible, bit 1 analytic/ReSTIR NEE visible, bits 2-5 the OpenPBR scatter
 *   event (1-9, 10 = random-walk scattering inside the medium); indexes of
 *   2^22 and above share bits with the decisions. And the path's final
 *   radiance (float3).
 * `paths` must equal the frame's total path count. */
rtgb_status rtgb_download_path_records(rtgb_handle handle, int32_t camera_index,
    int32_t* hit_codes, int32_t max_bounces, float* radiance_rgb, int64_t paths);

/* LBVH parity: sorted Morton codes, the primitive order they induce and the
 * Karras hierarchy (per internal node: left, right child; a negative child c
 * is the leaf of sorted slot ~c). Arrays sized primitive_count and
 * primitive_count-1 respectively. */
rtgb_status rtgb_download_lbvh(rtgb_handle handle, uint32_t* sorted_morton,
    int32_t* sorted_primitive, int32_t* node_children /* 2 per node */);

/* The internal nodes' child boxes, 12 floats per node (left lo.xyz, left
 * hi.xyz, right lo.xyz, right hi.xyz), primitive_count-1 nodes: what a refit
 * (rtgb_acceleration_info::update_kind 2) rewrites
 * (GpuSceneAcceleration::refit, gpu_scene_acceleration.cpp:347-365). */
rtgb_status rtgb_download_lbvh_boxes(rtgb_handle handle, float* child_boxes);

/* The 4-wide BVH every ray traverses, collapsed breadth-first from the binary
 * LBVH (same leaves): per node 4 child indices (>= 0 a node, < 0 the leaf of
 * sorted slot ~c, INT32_MIN unused) and 24 floats of child boxes (lo.x[4],
 * lo.y[4], lo.z[4], hi.x[4], hi.y[4], hi.z[4]); wide_node_count nodes, node 0
 * the root. No counterpart in the reference (its BVH is binary). */
rtgb_status rtgb_download_bvh4(rtgb_handle handle, int32_t* children, float* child_boxes);

/* ------------------------------------------------------------------------ */
/* Host-side authoring helpers (C++23 host code in the same library).        */
/* ------------------------------------------------------------------------ */

typedef struct rtgb_host_scene rtgb_host_scene;

/* Builtin and procedural scenes. Names:
 *   "cornell_box"        shared_scene_builders.cpp:101-139, :348-356
 *   "smoke"              shared_scene_builders.cpp:475-487
 *   "final_room"         shared_scene_builders.cpp:489-552
 *   "bouncing_spheres"   shared_scene_builders.cpp:241-264
 *   "restir_acceptance"  utils/render_restir_acceptance.cpp:41-93
 *   "random_spheres"     seeded 22x22 sphere field + emissive rect lights
 *   "triangle_terrain"   seeded displaced-grid terrain + icosphere instances
 *   "triangle_terrain_pbr"  the same with constant OpenPBR materials
 *   "openpbr_gallery"    one sphere per OpenPBR feature + analytic sphere lights
 *   "textured_room"      4 M-triangle room, checker / noise textured OpenPBR,
 *                        600 icosphere props, 4096 emissive triangles
 * `detail` scales the procedural scenes (light count / triangle budget);
 * 0 selects the default size. */
rtgb_status rtgb_host_scene_create(const char* name, uint32_t seed, int64_t detail,
    rtgb_host_scene** out_scene);
void rtgb_host_scene_destroy(rtgb_host_scene* scene);
/* A view of the scene's arrays (owned by the host scene). */
rtgb_status rtgb_host_scene_view(const rtgb_host_scene* scene, rtgb_scene* out_view);

/* Scene files: the packed arrays of a host scene (from a builtin builder or
 * from the SceneIR v2 adapter of rtgb_scene_ir_v2.hpp) written to / read from
 * disk, so a scene compiled once renders from any caller of this ABI. Format:
 * "RTGBSCN1", a version word, the byte size of each record type (a file from
 * a build with other record layouts is refused), then per array a 64-bit
 * count and the records, all little-endian. No reference counterpart (its
 * packed scenes live only in memory). */
rtgb_status rtgb_host_scene_save(const rtgb_host_scene* scene, const char* path);
rtgb_status rtgb_host_scene_load(const char* path, rtgb_host_scene** out_scene);
/* A host scene holding copies of a view's arrays (the view is not kept). */
rtgb_status rtgb_host_scene_from_view(const rtgb_scene* view, rtgb_host_scene** out_scene);

/* make_equi62_lut1d_params (src/realtime/camera_models.cpp:228-248). */
rtgb_status rtgb_make_equi62_lut1d(int32_t width, int32_t height, double fx, double fy,
    double cx, double cy, const double radial[6], const double tangential[2],
    rtgb_equi62_lut1d* out);

/* CameraRig::pack for a body pose T_bc (row-major rotation, translation):
 * T_rc = (camera_to_renderer * R_bc, body_to_renderer * t_bc), camera_rig.cpp:73-97. */
rtgb_status rtgb_pack_camera_pose(const double rotation_bc[9], const double translation_bc[3],
    double rotation_rc[9], double translation_rc[3]);

/* Default rig of a scene (the viewer's four yawed cameras, or the configured
 * mixed pinhole/equi rig of the procedural scenes). */
rtgb_status rtgb_default_rig(const char* scene_name, int32_t camera_count, int32_t width,
    int32_t height, rtgb_camera_rig* out_rig);

/* RenderProfile::quality/balanced/realtime (render_profile.h:27-63). */
rtgb_status rtgb_profile_preset(const char* name, rtgb_render_profile* out_profile);

/* ------------------------------------------------------------------------ */
/* Learned denoiser: OptixDenoiserWrapper::run (denoiser.cpp:111-185) is      */
/* replaced by a BF16 U-Net on the tensor cores. With parameters set, frames */
/* rendered with rtgb_render_profile::enable_denoise != 0 are denoised after */
/* the resolve pass; the frame views and rtgb_download_frame then return the  */
/* denoised beauty and denoise_ms its device time. Without parameters the    */
/* plain accumulated beauty is returned (the reference's no-denoiser path).  */
/* ------------------------------------------------------------------------ */

/* Loads the parameters from a file of exactly rtgb_denoiser_param_count()
 * little-endian BF16 values (ray_tracing_gb300/weights/denoiser_unet.bf16). */
rtgb_status rtgb_load_denoiser_file(rtgb_handle handle, const char* path);

/* Number of network parameters rtgb_set_denoiser_params expects. */
int64_t rtgb_denoiser_param_count(void);

/* Parameters in layer order, each layer's conv weight (out x in x 3 x 3, as
 * PyTorch's conv2d) then its bias; NULL clears them (plain path). */
rtgb_status rtgb_set_denoiser_params(rtgb_handle handle, const float* params, int64_t count);

/* ------------------------------------------------------------------------ */
/* Denoiser layer primitive (replaces the closed OptiX denoiser's network,   */
/* src/realtime/gpu/denoiser.cpp:111-185, with this library's U-Net).       */
/* ------------------------------------------------------------------------ */

/* Packs PyTorch conv2d weights (c_out x c_in_used x 3 x 3, float) into the
 * BF16 layout rtgb_conv3x3_bf16 reads: [tap = dy*3+dx][c_in/8][c_out][8],
 * input channels past c_in_used zero. `packed` holds 9 * c_in * c_out values. */
rtgb_status rtgb_conv3x3_pack_weights(const float* weight_oihw, int32_t c_out, int32_t c_in_used,
    int32_t c_in, uint16_t* packed);

/* y[n, y_channel_offset + o, y, x] = act(bias[o] + sum conv3x3(x)) on the
 * tensor cores (tcgen05, TMA halo tiles, FP32 accumulation), zero padding 1,
 * stride 1. Tensors are channel-blocked BF16, [n][c/8][h][w][8]: channel c of
 * pixel (x, y) of image n at ((n * C/8 + c/8) * h + y) * w * 8 + x * 8 + c % 8.
 * x has c_in channels (multiple of 16, <= 128); c_out a multiple of 16,
 * <= 64; y has y_channels channels (multiple of 8) and the output starts at
 * block y_channel_offset / 8 (offset a multiple of 8).
 * act = ReLU when relu != 0. device_error (device int, may be null) receives a
 * non-zero code if a bounded wait inside the kernel ran out. Asynchronous on
 * `stream` (a cudaStream_t). */
rtgb_status rtgb_conv3x3_bf16(const void* x, int32_t n, int32_t h, int32_t w, int32_t c_in,
    const void* packed_weight, const float* bias, int32_t c_out, int32_t relu, void* y,
    int32_t y_channels, int32_t y_channel_offset, int32_t* device_error, void* stream,
    char* message, size_t message_size);

/* Weight and bias gradients of rtgb_conv3x3_bf16 (the training backward pass;
 * the input gradient is rtgb_conv3x3_bf16 itself with the weights flipped and
 * transposed): dweight[o][i][dy][dx] = sum over pixels of dy[o] * x[i] at the
 * offset (dy - 1, dx - 1) with zero padding, dbias[o] = sum of dy[o]; both
 * FP32 and overwritten. x (c_in channels, multiple of 16, <= 128) and dy
 * (c_out channels, multiple of 16, <= 64) are channel-blocked BF16 of the
 * same n x h x w. Tensor cores (tcgen05, MN-major operands straight from the
 * blocked tiles), FP32 accumulation. Asynchronous on `stream`. */
rtgb_status rtgb_conv3x3_wgrad_bf16(const void* x, int32_t n, int32_t h, int32_t w, int32_t c_in,
    const void* dy, int32_t c_out, float* dweight, float* dbias, int32_t* device_error, void* stream,
    char* message, size_t message_size);

/* Native training of the denoiser U-Net (the reference's denoiser is closed
 * and has no training): forward, log-space L1 loss, backward (input
 * gradients by rtgb_conv3x3_bf16's kernel with flipped, transposed weights,
 * weight gradients by rtgb_conv3x3_wgrad_bf16's) and Adam (beta 0.9 / 0.999,
 * eps 1e-8) on FP32 master parameters, for batches of n crops of h x w (h, w
 * multiples of 4). Parameters in rtgb_set_denoiser_params order. */
typedef struct rtgb_trainer_s* rtgb_trainer;
rtgb_status rtgb_trainer_create(int32_t n, int32_t h, int32_t w, const float* params, int64_t count,
    rtgb_trainer* out_trainer);
void rtgb_trainer_destroy(rtgb_trainer trainer);
/* input: device, channel-blocked BF16, 16 channels (the network input of
 * denoiser.py's make_input, channels 10..15 zero); target: device FP32
 * n x h x w x 3, log1p radiance. learning_rate 0 computes the gradients only.
 * *loss (host, may be null) receives the mean L1 loss of the forward pass. */
rtgb_status rtgb_trainer_step(rtgb_trainer trainer, const void* input, const float* target, float learning_rate,
    float* loss);
/* Parameter gradients of the last step and the current parameters (host, count values). */
rtgb_status rtgb_trainer_gradients(rtgb_trainer trainer, float* grads);
rtgb_status rtgb_trainer_params(rtgb_trainer trainer, float* params);
const char* rtgb_trainer_last_error(rtgb_trainer trainer);

/* ------------------------------------------------------------------------ */
/* Allocation-free LBVH build. No counterpart in the reference.              */
/* ------------------------------------------------------------------------ */
#define RTGB_STATIC_LBVH_MAX_PRIMITIVES 131072

/* The device LBVH build of rtgb_prepare_scene over caller-owned boxes, with all
 * scratch carved from one fixed device array compiled into the library, so
 * the call never allocates device or host memory. Same outputs as
 * rtgb_download_lbvh for the same boxes.
 *   aabb_lo/aabb_hi   device, 4 floats per primitive (x, y, z, unused), 16-byte aligned
 *   sorted_morton     device, primitive_count words
 *   sorted_primitive  device, primitive_count words (sorted slot -> input index)
 *   node_children     device, 2 per internal node (a negative child c is sorted slot ~c)
 *   nodes             device, 16 floats per internal node (child boxes inline), 16-byte aligned
 *   stream            cudaStream_t of `device` (0: legacy default stream)
 *   message           optional caller buffer for the error text
 * 2 <= primitive_count <= RTGB_STATIC_LBVH_MAX_PRIMITIVES, else RTGB_INVALID_ARGUMENT.
 * The first call on a device looks up the array's address there; make it
 * before any stream capture. The address is cached for the life of the
 * process: after cudaDeviceReset of that device the entry point must not be
 * called for it again. Calls overlapping in time share the one array and
 * race: serialise them. Asynchronous on `stream`. */
rtgb_status rtgb_build_lbvh_static(int32_t device, const float* aabb_lo, const float* aabb_hi,
    int32_t primitive_count, uint32_t* sorted_morton, int32_t* sorted_primitive, int32_t* node_children,
    float* nodes, void* stream, char* message, size_t message_size);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* RTGB_H */
