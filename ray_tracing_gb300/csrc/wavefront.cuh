// Wavefront state, frame buffers and launch entry points.
#pragma once

#include "device_common.cuh"

namespace rtgb {

// Frame-wide AOV buffers: every active camera's pixels back to back
// (camera c starts at CameraDev::pixel_offset). DeviceFrameBuffers of
// src/realtime/gpu/launch_params.h:25-34.
struct FrameBufs {
    float4* beauty;
    float4* normal;
    float4* dnormal;
    float4* albedo;
    float* depth;
    float2* flow;
    float* trust;
    ReservoirRec* reservoirs;   // 96-byte sector-ordered records (device_common.cuh)
    float4* denoised;           // denoiser output radiance (written when the frame is denoised)
};

// Structure-of-arrays path streams, one slot per path (pixel-major, sample-minor).
struct Paths {
    float4* ray_o;      // origin.xyz
    float4* ray_d;      // direction.xyz
    float4* thr;        // throughput.xyz, w = previous BSDF pdf
    float4* rad;        // radiance.xyz
    float4* prev_pos;   // previous scatter position.xyz, w = flags (1 valid, 2 delta) as int bits
    float4* prev_nrm;   // previous scatter normal.xyz, w = previous material type as int bits
    int2* prev_prim;    // previous primitive type, index
    uint32_t* rng;
    float4* aux_n;      // bounce-0 shading normal.xyz, w = depth
    float4* aux_a;      // bounce-0 albedo.xyz, w = 1 when captured
    float4* hit;        // x = t, y = surface/medium code bits (-1 miss), z = analytic light index bits
    float4* sh_o[2];    // shadow ray origin.xyz, w = tmax
    float4* sh_d[2];    // shadow ray direction.xyz
    float4* sh_c[2];    // contribution (throughput * direct).xyz, w = 1 when pending
    ReservoirRec* res_scratch;  // per path reservoir when spp > 1 (ReSTIR)
    int* res_written;        // per path: 1 when the path wrote res_scratch
    int* queue[2];
    int* shadow_queue;
    int* restir_queue;       // bounce-0 surfaces waiting for ReSTIR DI
    int* codes;              // optional parity record [path][max_bounces]
    int* sss_mat;            // OpenPBR material whose random-walk medium the path is inside, -1 outside
    float4* sss_ext;         // that medium's extinction.xyz, w = Henyey-Greenstein anisotropy
    float4* sss_alb;         // its single-scattering albedo.xyz
    int2* res_src;           // ReSTIR reuse sources [source][path] (9 sources): history pixel, multiplicity
    float* res_src_t;        // their bias-correction targets [source][path]
    long long src_stride;    // paths per source row of res_src / res_src_t (the path capacity)
    int* res_meta;           // per path: source count, selected source + 1, canonical M
    int* vis_queue;          // (path << 4) | source of each bias-correction ray
    int* sort_key;           // material bucket of each shade-queue slot (shade_sort.cu)
    int* sorted;             // the shade queue in bucket order
    int* sort_hist;          // [kSortBins] bucket sizes (zero between bounces)
    int* sort_cursor;        // [kSortBins] bucket fill positions
    int* scatter_queue;      // paths whose BSDF sampling runs in k_scatter (split OpenPBR shading)
};

struct Counters {
    int active[2];
    int shadow;
    int error;
    unsigned long long rays[4];  // primary, extension, shadow, restir visibility
    int overflow;
    int denoise_error;                // a denoiser kernel's bounded wait ran out
    int gave_up;                      // this frame's loops that reached their bound (LoopBounds)
    int pad;
    unsigned long long cum_rays[4];  // running totals since the counters were last cleared
    int bounce_active[64];           // paths entering each bounce of the last frame
    unsigned long long restir_pixels; // paths that ran ReSTIR DI in the last frame
    int restir;                       // ReSTIR queue length
    int vis;                          // bias-correction ray queue length
    unsigned long long shadow_bounce[64];  // shadow rays traced per bounce
    int scatter;                      // scatter queue length (split OpenPBR shading)
};

struct FrameParams {
    CameraDev cam[RTGB_MAX_CAMERAS];
    CameraDev prev[RTGB_MAX_CAMERAS];
    int prev_valid[RTGB_MAX_CAMERAS];
    int history_length[RTGB_MAX_CAMERAS];
    int cam_count;
    int spp;
    int max_bounces;
    int rr_start;
    long long total_pixels;
    long long total_paths;
    uint32_t stream;
    int restir_enabled;
    int restir_candidates;
    int restir_temporal;
    int restir_max_age;
    int restir_max_temporal;
    int restir_spatial;
    int restir_max_spatial;
    int restir_bias;
    int restir_emissive;   // 1: ReSTIR DI resamples the emissive-geometry lights (opt-in; no reference counterpart)
    int record_paths;
    int sort_from_bounce;  // shade in material-bucket order from this bounce on (INT_MAX: never)
    FrameBufs cur;      // this frame's buffers
    FrameBufs hist;     // the previous frame's (ping-pong)
};

constexpr int kSortBins = 1024;  // material buckets of the shading order (one scan block)
constexpr int kBucketMaterials = 8;  // automatic bucketing needs more materials than this (or OpenPBR)

struct LaunchShape {
    int grid;
    int block;
};

// Kernel launchers (wavefront.cu). All are asynchronous on `stream`.
void launch_analytic_hot(DeviceScene scene, float4* out, cudaStream_t stream);
void launch_camera_dirs(const CameraDev& cam, float4* out, cudaStream_t stream);
void launch_raygen(const FrameParams* fp, Paths paths, Counters* counters, LaunchShape shape, cudaStream_t stream);
void launch_trace(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, cudaStream_t stream);
// `scatter_shape`: the grid of k_scatter, which the OpenPBR instance runs after k_shade.
void launch_shade(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, LaunchShape scatter_shape, cudaStream_t stream);
// Buckets the bounce's shade queue by hit material into Paths::sorted (a no-op
// below FrameParams::sort_from_bounce); shade_sort.cu.
void launch_shade_sort(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce, int grid,
    cudaStream_t stream);
void launch_shadow(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce, LaunchShape shape,
    cudaStream_t stream);
// The three ReSTIR passes (RIS + merges, bias-correction rays, finalisation);
// `shapes` is the full array filled by query_launch_shapes.
void launch_restir(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters,
    const LaunchShape* shapes, cudaStream_t stream);
void launch_finalize(const FrameParams* fp, Paths paths, Counters* counters, LaunchShape shape, cudaStream_t stream);
void launch_resolve(const FrameParams* fp, LaunchShape shape, cudaStream_t stream);
void launch_direction_debug(const CameraDev& cam, uint8_t* rgba, cudaStream_t stream);
void launch_reset_counters(Counters* counters, int bounce, cudaStream_t stream);
// Persistent grid sizes: SM count x resident blocks per SM for raygen, trace,
// shade, shadow, finalize, resolve and restir.
// shapes[0..6]: raygen, trace, shade, shadow, finalize, resolve, restir;
// shapes[7..8]: the OpenPBR instances of shade and restir; [9..10]: restir RIS
// and visibility passes; [11..12]: their OpenPBR instances; [13]: k_scatter
// (OpenPBR BSDF sampling after k_shade); [14..15]: the deep-hierarchy
// instances of trace and shadow (deep_bvh).
void query_launch_shapes(int sm_count, LaunchShape* shapes);
constexpr int kLaunchShapes = 16;

// Scenes whose wide BVH has at least this many nodes (4 MB) trace with the
// 80-register instances of k_trace / k_shadow, six blocks per SM: their node
// fetches miss the L1 and wait on L2 / DRAM, and more warps in flight hide
// that (the 4 M-triangle room: trace 27.8 against 30.3 ms, shadow 20.7 against
// 22.5 ms per frame); shallow ones keep the 90-register instances, whose
// traversal is cache-resident and slower with spills (the benchmark frame:
// 0.588 against 0.600 ms of trace).
constexpr int kDeepBvhNodes4 = 1 << 15;
inline bool deep_bvh(const DeviceScene& s) { return s.node4_count >= kDeepBvhNodes4; }

// Reuse sources kept per path by the ReSTIR passes: temporal + up to 8 spatial.
constexpr int kMaxReuseSources = 9;

// OpenPBR instances of the shade stage (shade_pbr.cu, restir_pbr.cu);
// launch_shade and launch_restir forward to them when the scene has OpenPBR
// materials.
void launch_shade_pbr(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, LaunchShape scatter_shape, cudaStream_t stream);
void launch_restir_pbr(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters,
    const LaunchShape* shapes, cudaStream_t stream);
LaunchShape query_shade_pbr_shape(int sm_count);
LaunchShape query_scatter_pbr_shape(int sm_count);
void query_restir_pbr_shapes(int sm_count, LaunchShape* shapes);
void launch_tonemap(const float4* beauty, uint8_t* rgba, long long pixels, cudaStream_t stream);

// Scene preparation kernels (scene_prep.cu).
void launch_prim_records(const DeviceScene& scene, PrimRecord* records, float4* aabb_lo, float4* aabb_hi, float pad,
    cudaStream_t stream);
void launch_gather_records(const PrimRecord* in, const int* order, PrimRecord* out, int n, cudaStream_t stream);

}  // namespace rtgb
