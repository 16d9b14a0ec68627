// Renderer: the C ABI of include/rtgb.h over the wavefront kernels.
//
// One handle replaces the reference's RendererPool + one OptixRenderer per
// camera (src/realtime/gpu/renderer_pool.cpp, optix_renderer.cpp): the scene
// is uploaded once, every active camera renders in one launch sequence on one
// stream, frame and history buffers ping-pong instead of being copied
// (device_frame_buffers.cpp:153-164), and the per-frame sequence is captured
// once as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "denoiser.cuh"
#include "lbvh.cuh"
#include "light_table.cuh"
#include "mesh_flatten.cuh"
#include "openpbr.h"
#include "wavefront.cuh"

namespace rtgb {

// scene_prep: leaf records and padded boxes for every surface primitive
// (spheres, then quads, then triangles).
__global__ void k_prim_records(DeviceScene s, PrimRecord* records, float4* aabb_lo, float4* aabb_hi, float pad) {
    const int n = s.sphere_count + s.quad_count + s.triangle_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        PrimRecord r;
        float3 lo, hi;
        int code;
        if (i < s.sphere_count) {
            const rtgb_sphere sp = s.spheres[i];
            const float3 c = ld3(sp.center);
            const float rr = fabsf(sp.radius);
            r.q[0] = make_float4(c.x, c.y, c.z, sp.radius);
            r.q[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            r.q[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            lo = f3(c.x - rr, c.y - rr, c.z - rr);
            hi = f3(c.x + rr, c.y + rr, c.z + rr);
            code = (0 << 28) | i;
            r.q[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else if (i < s.sphere_count + s.quad_count) {
            const int k = i - s.sphere_count;
            const rtgb_quad q = s.quads[k];
            const float3 o = ld3(q.origin), eu = ld3(q.edge_u), ev = ld3(q.edge_v);
            const float3 n3 = cross(eu, ev);
            const float nls = len_sq(n3);
            float3 normal = f3(0.0f, 0.0f, 0.0f), w = f3(0.0f, 0.0f, 0.0f);
            if (nls > 1e-12f) {  // degenerate quads keep a zero normal and never hit
                normal = divs(n3, sqrtf(nls));
                w = divs(n3, nls);
            }
            r.q[0] = make_float4(o.x, o.y, o.z, normal.x);
            r.q[1] = make_float4(eu.x, eu.y, eu.z, normal.y);
            r.q[2] = make_float4(ev.x, ev.y, ev.z, normal.z);
            r.q[3] = make_float4(w.x, w.y, w.z, 0.0f);
            const float3 p1 = add(o, eu), p2 = add(o, ev), p3 = add(add(o, eu), ev);
            lo = f3(fminf(fminf(o.x, p1.x), fminf(p2.x, p3.x)), fminf(fminf(o.y, p1.y), fminf(p2.y, p3.y)),
                fminf(fminf(o.z, p1.z), fminf(p2.z, p3.z)));
            hi = f3(fmaxf(fmaxf(o.x, p1.x), fmaxf(p2.x, p3.x)), fmaxf(fmaxf(o.y, p1.y), fmaxf(p2.y, p3.y)),
                fmaxf(fmaxf(o.z, p1.z), fmaxf(p2.z, p3.z)));
            code = (1 << 28) | k;
        } else {
            const int k = i - s.sphere_count - s.quad_count;
            const rtgb_triangle t = s.triangles[k];
            const float3 p0 = ld3(t.p0), p1 = ld3(t.p1), p2 = ld3(t.p2);
            const float3 e1 = sub(p1, p0), e2 = sub(p2, p0);
            r.q[0] = make_float4(p0.x, p0.y, p0.z, 0.0f);
            r.q[1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
            r.q[2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
            r.q[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            lo = f3(fminf(fminf(p0.x, p1.x), p2.x), fminf(fminf(p0.y, p1.y), p2.y), fminf(fminf(p0.z, p1.z), p2.z));
            hi = f3(fmaxf(fmaxf(p0.x, p1.x), p2.x), fmaxf(fmaxf(p0.y, p1.y), p2.y), fmaxf(fmaxf(p0.z, p1.z), p2.z));
            code = (2 << 28) | k;
        }
        r.q[3].w = __int_as_float(code);
        records[i] = r;
        aabb_lo[i] = make_float4(lo.x - pad, lo.y - pad, lo.z - pad, 0.0f);
        aabb_hi[i] = make_float4(hi.x + pad, hi.y + pad, hi.z + pad, 0.0f);
    }
}

__global__ void k_gather_records(const PrimRecord* __restrict__ in, const int* __restrict__ order, PrimRecord* out,
    int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[order[i]];
}

void launch_prim_records(const DeviceScene& scene, PrimRecord* records, float4* aabb_lo, float4* aabb_hi, float pad,
    cudaStream_t stream) {
    const int n = scene.sphere_count + scene.quad_count + scene.triangle_count;
    k_prim_records<<<std::min((n + 255) / 256, 8192), 256, 0, stream>>>(scene, records, aabb_lo, aabb_hi, pad);
}

void launch_gather_records(const PrimRecord* in, const int* order, PrimRecord* out, int n, cudaStream_t stream) {
    k_gather_records<<<std::min((n + 255) / 256, 8192), 256, 0, stream>>>(in, order, out, n);
}

namespace {

struct CudaFailure {
    cudaError_t err;
    const char* expr;
};

#define RTGB_CHECK(expr)                                      \
    do {                                                      \
        const cudaError_t rtgb_err_ = (expr);                 \
        if (rtgb_err_ != cudaSuccess) throw CudaFailure{rtgb_err_, #expr}; \
    } while (0)

struct Invalid {
    std::string message;
};

// A device allocation that grows on demand.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void* ensure(size_t need) {
        if (need <= bytes && p) return p;
        release();
        if (need == 0) need = 256;
        RTGB_CHECK(cudaMalloc(&p, need));
        bytes = need;
        return p;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// A build-time scratch buffer freed when it leaves scope (cudaFree waits for
// the work that uses it), also when the build throws.
struct ScopedBuf : DevBuf {
    ScopedBuf() = default;
    ScopedBuf(const ScopedBuf&) = delete;
    ScopedBuf& operator=(const ScopedBuf&) = delete;
    ~ScopedBuf() { release(); }
};

// Timing events destroyed on every exit path.
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        RTGB_CHECK(cudaEventCreate(&a));
        RTGB_CHECK(cudaEventCreate(&b));
    }
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

template <typename T>
T* upload(DevBuf& buf, const T* host, size_t count, cudaStream_t stream) {
    buf.ensure(std::max<size_t>(count, 1) * sizeof(T));
    if (count > 0) RTGB_CHECK(cudaMemcpyAsync(buf.p, host, count * sizeof(T), cudaMemcpyHostToDevice, stream));
    return buf.as<T>();
}

// Per camera slot: device LUT and per-pixel direction table for one set of
// intrinsics. Two per slot, so the previous frame's camera stays valid while
// the current one changes.
struct CameraRes {
    DevBuf lut;
    DevBuf dirs;
    bool valid = false;
    int width = 0, height = 0, model = 0;
    rtgb_pinhole32 pinhole{};
    rtgb_equi62_lut1d equi{};
    int monotone = 1;
};

bool same_intrinsics(const CameraRes& r, const rtgb_camera& c) {
    if (!r.valid || r.width != c.width || r.height != c.height || r.model != c.model) return false;
    if (c.model == RTGB_CAMERA_PINHOLE32) return std::memcmp(&r.pinhole, &c.pinhole, sizeof(rtgb_pinhole32)) == 0;
    return std::memcmp(&r.equi, &c.equi, sizeof(rtgb_equi62_lut1d)) == 0;
}

float luminance(float r, float g, float b) { return std::max(0.0f, 0.2126f * r + 0.7152f * g + 0.0722f * b); }

}  // namespace
}  // namespace rtgb

using namespace rtgb;

struct rtgb_renderer {
    int device = 0;
    bool use_graph = true;
    bool record = false;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    LaunchShape shapes[kLaunchShapes]{};
    std::string error;

    // scene
    bool prepared = false;
    DeviceScene scene{};
    DevBuf openpbr, analytic_hot;
    // learned denoiser (replaces OptixDenoiserWrapper, denoiser.cpp:111-185)
    UNet* unet = nullptr;
    bool last_denoised = false;
    bool denoise_this_frame = false;
    float last_denoise_ms = 0.0f;
    cudaEvent_t ev_dn0 = nullptr, ev_dn1 = nullptr;
    DevBuf light_guide, analytic_guide;  // CDF guide tables of the NEE searches (sample_cdf_guided)
    DevBuf material_lum, light_counts;   // light table inputs; its counts (+ the LBVH scale word)
    // device copy of an instanced mesh set (rtgb_prepare_scene_instanced, mesh_flatten.cu)
    DevBuf mesh_points, mesh_corners, mesh_normals, mesh_texcoords, mesh_materials, mesh_protos, mesh_insts;
    DevBuf spheres, quads, triangles, media, materials, textures, texels, lights, light_cdf, sphere_light, quad_light,
        triangle_light, analytic, analytic_cdf, analytic_nodes, analytic_leaf, infinite_analytic, prims, nodes,
        sorted_keys, sorted_vals;
    int prim_count = 0;
    int analytic_bvh_count = 0;
    float build_ms = 0.0f;
    // acceleration lifecycle (GpuSceneAcceleration, gpu_scene_acceleration.cpp:247-295):
    // the hierarchy's children/parent survive so a geometry change with the
    // same primitive counts refits the boxes instead of rebuilding
    DevBuf bvh_children, bvh_parent;
    // wide BVH traversed by every ray: nodes and the collapse (children, box
    // references into the binary nodes) kept for refits
    DevBuf nodes4, child4, ref4;
    int node4_count = 0;
    bool accel_valid = false;
    int accel_counts[3] = {-1, -1, -1};
    uint64_t geometry_sig = 0, scene_sig = 0;
    int update_kind = 3;
    int generation = 0;

    // frame state
    uint32_t sample_stream = 0;
    CameraRes cam_res[RTGB_MAX_CAMERAS][2];
    int cam_cur[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    CameraDev prev[RTGB_MAX_CAMERAS]{};
    int prev_valid[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int history_length[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int layout_w[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int layout_h[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int layout_count = 0;
    long long total_pixels = 0;
    long long total_paths = 0;
    DevBuf frame_mem[2];
    FrameBufs frames[2]{};
    int cur = 0;
    int last = -1;  // frame index holding the last rendered frame
    long long last_pixel_offset[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int last_w[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int last_h[RTGB_MAX_CAMERAS] = {0, 0, 0, 0};
    int last_count = 0;
    int last_spp = 1;
    int last_bounces = 1;
    DevBuf path_mem;
    long long path_capacity = 0;
    int path_record_bounces = 0;
    Paths paths{};
    DevBuf counters_mem, fp_mem, debug_rgba;
    Counters* d_counters = nullptr;
    Counters* h_counters = nullptr;  // pinned
    FrameParams* d_fp = nullptr;
    FrameParams h_fp{};
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    // pipelined downloads (rtgb_download_frame_async): copies of a frame's
    // buffers run on copy_stream while the next frame renders on `stream`;
    // the frame that reuses a buffer set waits for that set's copies
    // (copied[slot]) on the device
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_ready = nullptr;        // end of the frame being downloaded, on `stream`
    cudaEvent_t ev_copied[2]{};            // last copy enqueued from frames[slot]
    cudaEvent_t ev_older_copied = nullptr; // every copy of frames before the latest downloaded one
    bool copy_pending[2] = {false, false};
    uint64_t frame_serial = 0;             // frames rendered
    uint64_t download_serial = 0;          // frame_serial of the frame last downloaded asynchronously
    bool stage_timing = false;
    int shade_order = 0;  // rtgb_create_info::shade_order
    // device loop bounds (rtgb_create_info debug fields, rtgb_set_debug_limits)
    int traversal_limit = kDefaultTraversalLimit;
    int rejection_limit = kDefaultRejectionLimit;
    std::vector<cudaEvent_t> stage_events;
    int stage_count = 0;
    uint64_t frame_h2d = 0;
    // graph
    cudaGraphExec_t graph_exec = nullptr;
    long long graph_key[5] = {-1, -1, -1, -1, -1};
    long long unet_generation = 0;

    void fail_cuda(const CudaFailure& f) {
        error = std::string("CUDA failure at ") + f.expr + ": " + cudaGetErrorString(f.err);
    }

    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
        graph_key[0] = -1;
    }

    // Loop bounds of the device code: 0 (or less) keeps the default. The scene
    // struct is baked into captured graphs, so the graph is dropped.
    void set_limits(int traversal, int rejection) {
        traversal_limit = traversal > 0 ? traversal : kDefaultTraversalLimit;
        rejection_limit = rejection > 0 ? rejection : kDefaultRejectionLimit;
        scene.bounds = loop_bounds();
        drop_graph();
    }

    LoopBounds loop_bounds() const { return LoopBounds{traversal_limit, rejection_limit, &d_counters->gave_up}; }

    void set_denoiser(const float* params, long long count) {
        RTGB_CHECK(cudaSetDevice(device));
        RTGB_CHECK(cudaStreamSynchronize(stream));
        if (!unet) unet = unet_create();
        std::string err;
        if (!unet_set_params(unet, params, count, err)) throw Invalid{err};
        ++unet_generation;
        drop_graph();
    }

    ~rtgb_renderer() {
        if (stream) cudaStreamSynchronize(stream);
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        drop_graph();
        unet_destroy(unet);
        if (ev_dn0) cudaEventDestroy(ev_dn0);
        if (ev_dn1) cudaEventDestroy(ev_dn1);
        for (cudaEvent_t e : {ev_ready, ev_copied[0], ev_copied[1], ev_older_copied}) {
            if (e) cudaEventDestroy(e);
        }
        if (copy_stream) cudaStreamDestroy(copy_stream);
        DevBuf* bufs[] = {&spheres, &quads, &triangles, &media, &materials, &textures, &texels, &lights, &light_cdf,
            &sphere_light, &quad_light, &triangle_light, &analytic, &analytic_cdf, &analytic_nodes, &analytic_leaf,
            &infinite_analytic, &prims, &nodes, &sorted_keys, &sorted_vals, &frame_mem[0], &frame_mem[1], &path_mem,
            &counters_mem, &fp_mem, &debug_rgba, &openpbr, &analytic_hot, &bvh_children, &bvh_parent, &nodes4, &child4, &ref4,
            &light_guide, &analytic_guide, &material_lum, &light_counts, &mesh_points, &mesh_corners, &mesh_normals,
            &mesh_texcoords, &mesh_materials, &mesh_protos, &mesh_insts};
        for (DevBuf* b : bufs) b->release();
        for (auto& slot : cam_res) {
            for (auto& r : slot) {
                r.lut.release();
                r.dirs.release();
            }
        }
        if (h_counters) cudaFreeHost(h_counters);
        for (cudaEvent_t e : stage_events) cudaEventDestroy(e);
        if (ev_start) cudaEventDestroy(ev_start);
        if (ev_stop) cudaEventDestroy(ev_stop);
        if (stream) cudaStreamDestroy(stream);
    }

    void init(const rtgb_create_info& info) {
        device = info.device;
        use_graph = info.use_cuda_graph != 0;
        record = info.debug_path_records != 0;
        stage_timing = info.stage_timing != 0;
        shade_order = info.shade_order;
        RTGB_CHECK(cudaSetDevice(device));
        RTGB_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        RTGB_CHECK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
        query_launch_shapes(sm_count, shapes);
        RTGB_CHECK(cudaGetLastError());
        d_counters = static_cast<Counters*>(counters_mem.ensure(sizeof(Counters)));
        RTGB_CHECK(cudaMemsetAsync(d_counters, 0, sizeof(Counters), stream));
        d_fp = static_cast<FrameParams*>(fp_mem.ensure(sizeof(FrameParams)));
        set_limits(info.debug_traversal_limit, info.debug_rejection_limit);
        RTGB_CHECK(cudaMallocHost(reinterpret_cast<void**>(&h_counters), sizeof(Counters)));
        std::memset(h_counters, 0, sizeof(Counters));
        RTGB_CHECK(cudaEventCreate(&ev_start));
        RTGB_CHECK(cudaEventCreate(&ev_stop));
        RTGB_CHECK(cudaStreamSynchronize(stream));
    }

    // ---- scene: packed_scene_preparation.cpp:191-348 + device LBVH --------------

    std::vector<float> scene_texels_;

    float average_texture_lum_r(const rtgb_scene& s, int index, int depth, float out[3]) const {
        out[0] = out[1] = out[2] = 0.0f;
        if (index < 0 || index >= s.texture_count || depth >= 8) return 0.0f;
        const rtgb_texture& t = s.textures[index];
        if (t.type == 0) {
            for (int k = 0; k < 3; ++k) out[k] = std::max(t.color[k], 0.0f);
        } else if (t.type == 1) {
            float e[3], o[3];
            average_texture_lum_r(s, t.even_texture, depth + 1, e);
            average_texture_lum_r(s, t.odd_texture, depth + 1, o);
            for (int k = 0; k < 3; ++k) out[k] = 0.5f * (e[k] + o[k]);
        } else if (t.type == 2 && t.image_width > 0 && t.image_height > 0) {
            const int count = t.image_width * t.image_height;
            if (t.image_offset < 0 || t.image_offset + count > s.image_texel_count) return 0.0f;
            float sum[3] = {0.0f, 0.0f, 0.0f};
            for (int i = 0; i < count; ++i)
                for (int k = 0; k < 3; ++k) sum[k] += s.image_texels[3 * static_cast<size_t>(t.image_offset + i) + k];
            for (int k = 0; k < 3; ++k) out[k] = std::max(sum[k] / static_cast<float>(count), 0.0f);
        } else if (t.type == 3) {
            out[0] = out[1] = out[2] = 0.5f;
        }
        return 0.0f;
    }

    // material_emission_luminance, packed_scene_preparation.cpp:227-251
    float emission_lum(const rtgb_scene& s, int mi) const {
        if (mi < 0 || mi >= s.material_count) return 0.0f;
        const rtgb_material& m = s.materials[mi];
        float c[3];
        if (m.type == 3) {
            average_texture_lum_r(s, m.emission_texture, 0, c);
            return luminance(c[0], c[1], c[2]);
        }
        if (m.type != 5 || m.openpbr_index < 0 || m.openpbr_index >= s.openpbr_material_count) return 0.0f;
        const rtgb_openpbr_material& om = s.openpbr_materials[m.openpbr_index];
        pbr::Mat params;
        std::memcpy(&params, &om, sizeof params);
        if (om.color_texture[3] >= 0) {
            average_texture_lum_r(s, om.color_texture[3], 0, c);
            pbr::apply_color(params, 3, pbr::V3{c[0], c[1], c[2]}, om.color_space[3]);
        }
        return pbr::luminance(pbr::emission(params));
    }

    void validate_scene(const rtgb_scene& s, long long mesh_triangles = 0) {
        auto check = [&](const void* p, int n, const char* what) {
            if (n < 0 || (n > 0 && p == nullptr)) throw Invalid{std::string("scene ") + what + " array is invalid"};
        };
        check(s.textures, s.texture_count, "texture");
        check(s.image_texels, s.image_texel_count, "image texel");
        check(s.materials, s.material_count, "material");
        check(s.spheres, s.sphere_count, "sphere");
        check(s.quads, s.quad_count, "quad");
        check(s.triangles, s.triangle_count, "triangle");
        check(s.media, s.medium_count, "medium");
        check(s.analytic_lights, s.analytic_light_count, "analytic light");
        check(s.openpbr_materials, s.openpbr_material_count, "OpenPBR material");
        const long long surfaces = static_cast<long long>(s.sphere_count) + s.quad_count + s.triangle_count + mesh_triangles;
        if (surfaces == 0) throw Invalid{"render_radiance requires at least one surface primitive"};
        if (surfaces >= (1ll << 28)) throw Invalid{"scene exceeds 2^28 surface primitives"};
    }

    // FNV-1a over 64-bit words, the tail byte by byte. It detects changes the
    // way the geometry and scene signatures of gpu_scene_acceleration.cpp:116-135
    // do, eight bytes per step: each step is a bijection of the running hash,
    // so inputs differing in one word always hash differently.
    static uint64_t fnv_words(uint64_t h, const void* data, size_t bytes) {
        constexpr uint64_t kPrime = 1099511628211ull;
        const unsigned char* p = static_cast<const unsigned char*>(data);
        size_t i = 0;
        for (; i + 8 <= bytes; i += 8) {
            uint64_t w;
            std::memcpy(&w, p + i, 8);
            h = (h ^ w) * kPrime;
        }
        for (; i < bytes; ++i) h = (h ^ p[i]) * kPrime;
        return h;
    }

    template <typename T>
    static uint64_t fnv_array(uint64_t h, const T* data, long long count) {
        const long long n = count > 0 && data ? count : 0;
        h = fnv_words(h, &n, sizeof n);
        return n > 0 ? fnv_words(h, data, static_cast<size_t>(n) * sizeof(T)) : h;
    }

    static uint64_t geometry_signature(const rtgb_scene& s) {
        uint64_t h = 14695981039346656037ull;
        h = fnv_array(h, s.spheres, s.sphere_count);
        h = fnv_array(h, s.quads, s.quad_count);
        return fnv_array(h, s.triangles, s.triangle_count);
    }

    // The mesh set's contribution to the geometry signature: every prototype
    // array and every instance record.
    static uint64_t mesh_signature(uint64_t h, const rtgb_mesh_set& m) {
        for (int i = 0; i < m.prototype_count; ++i) {
            const rtgb_mesh_prototype& p = m.prototypes[i];
            const long long t = p.triangle_count;
            h = fnv_array(h, p.points, 3ll * p.point_count);
            h = fnv_array(h, p.corner_points, 3 * t);
            h = fnv_array(h, p.corner_normals, p.corner_normals ? 9 * t : 0);
            h = fnv_array(h, p.corner_texcoords, p.corner_texcoords ? 6 * t : 0);
            h = fnv_array(h, p.triangle_materials, t);
        }
        return fnv_array(h, m.instances, m.instance_count);
    }

    // Checks a mesh set as add_v2_mesh checks a mesh; returns the number of
    // triangles its instances flatten to.
    static long long validate_meshes(const rtgb_mesh_set& m) {
        if (m.prototype_count < 0 || m.instance_count < 0 || (m.prototype_count > 0 && m.prototypes == nullptr)
            || (m.instance_count > 0 && m.instances == nullptr)) {
            throw Invalid{"mesh set arrays are invalid"};
        }
        for (int i = 0; i < m.prototype_count; ++i) {
            const rtgb_mesh_prototype& p = m.prototypes[i];
            if (p.point_count < 0 || p.triangle_count < 0 || (p.point_count > 0 && p.points == nullptr)
                || (p.triangle_count > 0 && (p.corner_points == nullptr || p.triangle_materials == nullptr))) {
                throw Invalid{"mesh prototype arrays are invalid"};
            }
            for (long long c = 0; c < 3ll * p.triangle_count; ++c) {
                if (p.corner_points[c] < 0 || p.corner_points[c] >= p.point_count) {
                    throw Invalid{"SceneIR v2 mesh point index is out of range"};
                }
            }
        }
        long long n = 0;
        for (int i = 0; i < m.instance_count; ++i) {
            const int proto = m.instances[i].prototype;
            if (proto < 0 || proto >= m.prototype_count) throw Invalid{"mesh instance prototype is out of range"};
            n += m.prototypes[proto].triangle_count;
        }
        return n;
    }

    // Appends the mesh set's instances to d's triangles (the buffer holds the
    // scene's own d.triangle_count and room for the instances) on the device.
    void flatten_meshes(const rtgb_mesh_set& m, DeviceScene& d) {
        std::vector<double> points, normals, texcoords;
        std::vector<int> corners, mats;
        std::vector<MeshProtoDev> protos(static_cast<size_t>(m.prototype_count));
        for (int i = 0; i < m.prototype_count; ++i) {
            const rtgb_mesh_prototype& p = m.prototypes[i];
            const size_t t = static_cast<size_t>(p.triangle_count);
            MeshProtoDev& q = protos[static_cast<size_t>(i)];
            q.point_offset = static_cast<long long>(points.size() / 3);
            q.tri_offset = static_cast<long long>(mats.size());
            q.tri_count = p.triangle_count;
            q.has_normals = p.corner_normals != nullptr;
            q.has_texcoords = p.corner_texcoords != nullptr;
            points.insert(points.end(), p.points, p.points + 3 * static_cast<size_t>(p.point_count));
            corners.insert(corners.end(), p.corner_points, p.corner_points + 3 * t);
            mats.insert(mats.end(), p.triangle_materials, p.triangle_materials + t);
            // per-triangle arrays stay aligned with mats: zeros where a prototype has none
            if (p.corner_normals) normals.insert(normals.end(), p.corner_normals, p.corner_normals + 9 * t);
            else normals.resize(normals.size() + 9 * t, 0.0);
            if (p.corner_texcoords) texcoords.insert(texcoords.end(), p.corner_texcoords, p.corner_texcoords + 6 * t);
            else texcoords.resize(texcoords.size() + 6 * t, 0.0);
        }
        std::vector<MeshInstDev> insts(static_cast<size_t>(m.instance_count));
        long long out = d.triangle_count;
        for (int i = 0; i < m.instance_count; ++i) {
            const rtgb_mesh_instance& src = m.instances[i];
            MeshInstDev& q = insts[static_cast<size_t>(i)];
            q.out_offset = out;
            q.prototype = src.prototype;
            q.material = src.material;
            q.flip = src.flip_winding != 0;
            std::memcpy(q.world, src.world, sizeof q.world);
            std::memcpy(q.normal_matrix, src.normal_matrix, sizeof q.normal_matrix);
            out += m.prototypes[src.prototype].triangle_count;
        }
        MeshSetDev set{};
        set.points = upload(mesh_points, points.data(), points.size(), stream);
        set.corners = upload(mesh_corners, corners.data(), corners.size(), stream);
        set.normals = upload(mesh_normals, normals.data(), normals.size(), stream);
        set.texcoords = upload(mesh_texcoords, texcoords.data(), texcoords.size(), stream);
        set.materials = upload(mesh_materials, mats.data(), mats.size(), stream);
        set.prototypes = upload(mesh_protos, protos.data(), protos.size(), stream);
        set.instances = upload(mesh_insts, insts.data(), insts.size(), stream);
        set.instance_count = m.instance_count;
        set.first_out = d.triangle_count;
        set.end_out = out;
        int* bad = static_cast<int*>(light_counts.ensure(4 * sizeof(int))) + 3;
        RTGB_CHECK(cudaMemsetAsync(bad, 0, sizeof(int), stream));
        RTGB_CHECK(launch_flatten_meshes(set, const_cast<rtgb_triangle*>(d.triangles), bad, sm_count, stream));
        int h_bad = 0;
        RTGB_CHECK(cudaMemcpyAsync(&h_bad, bad, sizeof h_bad, cudaMemcpyDeviceToHost, stream));
        RTGB_CHECK(cudaStreamSynchronize(stream));
        if (h_bad != 0) throw Invalid{"SceneIR v2 contains a singular or zero-length mesh normal"};
        d.triangle_count = static_cast<int>(out);
    }

    // Everything prepare uploads besides geometry (the packed light list is a
    // function of geometry and materials, so it needs no hash of its own).
    static uint64_t scene_signature(const rtgb_scene& s, uint64_t geometry) {
        uint64_t h = fnv_words(geometry, s.background, sizeof s.background);
        h = fnv_array(h, s.media, s.medium_count);
        h = fnv_array(h, s.textures, s.texture_count);
        h = fnv_array(h, s.image_texels, 3ll * s.image_texel_count);
        h = fnv_array(h, s.materials, s.material_count);
        h = fnv_array(h, s.openpbr_materials, s.openpbr_material_count);
        return fnv_array(h, s.analytic_lights, s.analytic_light_count);
    }

    // GpuSceneAcceleration::update + use_prepared_scene: reuse when nothing
    // changed, update (re-upload, keep the hierarchy) when only non-geometry
    // data changed, refit when the primitive counts are unchanged, else
    // rebuild. Every kind restarts the sample stream and drops history.
    void prepare(const rtgb_scene& s, const rtgb_mesh_set* meshes = nullptr) {
        const long long extra = meshes ? validate_meshes(*meshes) : 0;
        validate_scene(s, extra);
        RTGB_CHECK(cudaSetDevice(device));
        RTGB_CHECK(cudaStreamSynchronize(stream));
        const uint64_t geo = meshes ? mesh_signature(geometry_signature(s), *meshes) : geometry_signature(s);
        const uint64_t sig = scene_signature(s, geo);
        const long long tri_total = s.triangle_count + extra;
        const bool topology_changed = accel_counts[0] != s.sphere_count || accel_counts[1] != s.quad_count
                                      || accel_counts[2] != tri_total;
        int kind = 0;
        if (topology_changed || !accel_valid || !prepared) kind = 3;
        else if (geo != geometry_sig) kind = 2;
        else if (sig != scene_sig) kind = 1;
        if (kind != 0) {
            drop_graph();
            prepared = false;
            accel_valid = false;
            upload_scene(s, kind, meshes);
            accel_valid = true;
            accel_counts[0] = s.sphere_count;
            accel_counts[1] = s.quad_count;
            accel_counts[2] = static_cast<int>(tri_total);
            geometry_sig = geo;
            scene_sig = sig;
            ++generation;
        } else {
            build_ms = 0.0f;
        }
        update_kind = kind;
        prepared = true;
        // use_prepared_scene: the sample stream restarts and history is dropped
        sample_stream = 0;
        reset_accumulation();
        std::memset(h_counters, 0, sizeof(Counters));
        RTGB_CHECK(cudaMemsetAsync(d_counters, 0, sizeof(Counters), stream));
        RTGB_CHECK(cudaStreamSynchronize(stream));
    }

    // guide[j] = first i with j / kGuide < cdf[i], by the same bisection the
    // kernels use, guide[kGuide] = the count: sample_cdf_guided then returns
    // exactly sample_cdf's index from one bucket.
    static std::vector<int> cdf_guide(const std::vector<float>& cdf) {
        const int n = static_cast<int>(cdf.size());
        std::vector<int> g(static_cast<size_t>(kGuide) + 1);
        for (int j = 0; j < kGuide; ++j) {
            const float t = static_cast<float>(j) * (1.0f / static_cast<float>(kGuide));
            int lo = 0, hi = n;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (t < cdf[static_cast<size_t>(mid)]) hi = mid;
                else lo = mid + 1;
            }
            g[static_cast<size_t>(j)] = lo;
        }
        g[static_cast<size_t>(kGuide)] = n;
        return g;
    }

    // Uploads the scene for update kind 1 (non-geometry data; the primitives,
    // records and hierarchy stay), 2 (refit) or 3 (rebuild).
    void upload_scene(const rtgb_scene& s, int kind, const rtgb_mesh_set* meshes) {
        DeviceScene d = kind == 1 ? scene : DeviceScene{};
        if (kind >= 2) {
            d.spheres = upload(spheres, s.spheres, static_cast<size_t>(s.sphere_count), stream);
            d.quads = upload(quads, s.quads, static_cast<size_t>(s.quad_count), stream);
            // the scene's triangles, then room for the flattened instances
            long long extra = 0;
            for (int i = 0; meshes && i < meshes->instance_count; ++i) {
                extra += meshes->prototypes[meshes->instances[i].prototype].triangle_count;
            }
            rtgb_triangle* tris = static_cast<rtgb_triangle*>(
                triangles.ensure(std::max<size_t>(static_cast<size_t>(s.triangle_count + extra), 1) * sizeof(rtgb_triangle)));
            if (s.triangle_count > 0) {
                RTGB_CHECK(cudaMemcpyAsync(tris, s.triangles, static_cast<size_t>(s.triangle_count) * sizeof(rtgb_triangle),
                    cudaMemcpyHostToDevice, stream));
            }
            d.triangles = tris;
            d.triangle_count = s.triangle_count;
            if (meshes) flatten_meshes(*meshes, d);
        }
        d.media = upload(media, s.media, static_cast<size_t>(s.medium_count), stream);
        d.materials = upload(materials, s.materials, static_cast<size_t>(s.material_count), stream);
        d.openpbr = s.openpbr_material_count > 0
                        ? upload(openpbr, s.openpbr_materials, static_cast<size_t>(s.openpbr_material_count), stream)
                        : nullptr;
        d.openpbr_count = s.openpbr_material_count;
        d.textures = upload(textures, s.textures, static_cast<size_t>(s.texture_count), stream);
        d.texels = s.image_texel_count > 0 ? upload(texels, s.image_texels, 3 * static_cast<size_t>(s.image_texel_count), stream) : nullptr;
        d.sphere_count = s.sphere_count;
        d.quad_count = s.quad_count;
        d.medium_count = s.medium_count;
        d.material_count = s.material_count;
        d.texture_count = s.texture_count;
        d.texel_count = s.image_texel_count;
        std::memcpy(d.background, s.background, sizeof d.background);

        // build_light_distribution (packed_scene_preparation.cpp:265-302) on
        // the device (light_table.cu): the emission luminance once per material
        // here; each primitive's weight, the order-keeping compaction, the
        // sequential normalisation and the guide table there. A primitive is
        // at most one light, so the maps answer find_packed_light.
        {
            std::vector<float> mat_lum(static_cast<size_t>(s.material_count));
            for (int m = 0; m < s.material_count; ++m) mat_lum[static_cast<size_t>(m)] = emission_lum(s, m);
            constexpr float kPiF = 3.14159265358979323846f;
            const LightSources src{d.spheres, d.quads, d.triangles, d.sphere_count, d.quad_count, d.triangle_count,
                upload(material_lum, mat_lum.data(), mat_lum.size(), stream), s.material_count,
                4.0f * kPiF * luminance(s.background[0], s.background[1], s.background[2])};
            const size_t prims = static_cast<size_t>(d.sphere_count) + d.quad_count + d.triangle_count;
            auto ints = [](DevBuf& b, size_t n) { return static_cast<int*>(b.ensure(std::max<size_t>(n, 1) * sizeof(int))); };
            const LightTable lt{static_cast<PackedLight*>(lights.ensure((prims + 1) * sizeof(PackedLight))),
                static_cast<float*>(light_cdf.ensure((prims + 1) * sizeof(float))), ints(light_guide, kGuide + 1),
                ints(sphere_light, static_cast<size_t>(d.sphere_count)), ints(quad_light, static_cast<size_t>(d.quad_count)),
                ints(triangle_light, static_cast<size_t>(d.triangle_count)), ints(light_counts, 4)};
            ScopedBuf scratch;
            scratch.ensure(light_table_scratch_bytes(static_cast<long long>(prims)));
            RTGB_CHECK(launch_light_table(src, lt, scratch.p, stream));
            int counts[2] = {0, -1};
            RTGB_CHECK(cudaMemcpyAsync(counts, lt.counts, sizeof counts, cudaMemcpyDeviceToHost, stream));
            RTGB_CHECK(cudaStreamSynchronize(stream));
            d.lights = lt.lights;
            d.light_cdf = lt.cdf;
            d.light_guide = lt.guide;
            d.light_count = counts[0];
            d.environment_light = counts[1];
            d.sphere_light = lt.sphere_light;
            d.quad_light = lt.quad_light;
            d.triangle_light = lt.triangle_light;
        }

        // analytic lights: CDF array, infinite list and a BVH over finite ones
        const int na = s.analytic_light_count;
        d.analytic = upload(analytic, s.analytic_lights, static_cast<size_t>(na), stream);
        d.analytic_count = na;
        d.analytic_hot = na > 0 ? static_cast<const float4*>(
                                      analytic_hot.ensure(static_cast<size_t>(na) * kAnalyticHot * sizeof(float4)))
                                : nullptr;
        launch_analytic_hot(d, const_cast<float4*>(d.analytic_hot), stream);
        RTGB_CHECK(cudaGetLastError());
        std::vector<float> acdf(static_cast<size_t>(na));
        std::vector<int> inf, finite;
        for (int i = 0; i < na; ++i) {
            const rtgb_analytic_light& l = s.analytic_lights[i];
            acdf[static_cast<size_t>(i)] = l.cdf;
            if (l.type == 4 || l.type == 5) inf.push_back(i);
            if ((l.type >= 0 && l.type <= 3) && l.treat_as_point == 0) finite.push_back(i);
        }
        d.analytic_cdf = upload(analytic_cdf, acdf.data(), acdf.size(), stream);
        const std::vector<int> aguide = cdf_guide(acdf);
        d.analytic_guide = upload(analytic_guide, aguide.data(), aguide.size(), stream);
        d.infinite_analytic = upload(infinite_analytic, inf.data(), inf.size(), stream);
        d.infinite_analytic_count = static_cast<int>(inf.size());

        EventPair ev;
        RTGB_CHECK(cudaEventRecord(ev.a, stream));
        if (kind >= 2) build_scene_bvh(d, kind);
        build_analytic_bvh(s, finite, d);
        RTGB_CHECK(cudaEventRecord(ev.b, stream));
        RTGB_CHECK(cudaStreamSynchronize(stream));
        RTGB_CHECK(cudaGetLastError());
        RTGB_CHECK(cudaEventElapsedTime(&build_ms, ev.a, ev.b));
        d.bounds = loop_bounds();
        scene = d;
    }

    // Scene LBVH: a full device build (kind 3) that keeps children/parent, or
    // a refit (kind 2) of the kept hierarchy to the new primitive boxes.
    void build_scene_bvh(DeviceScene& d, int kind) {
        const int n = d.sphere_count + d.quad_count + d.triangle_count;
        // the largest coordinate magnitude of any primitive (launch_scene_scale)
        unsigned* scale_bits = static_cast<unsigned*>(light_counts.ensure(4 * sizeof(int))) + 2;
        RTGB_CHECK(launch_scene_scale(d, scale_bits, sm_count, stream));
        unsigned bits = 0;
        RTGB_CHECK(cudaMemcpyAsync(&bits, scale_bits, sizeof bits, cudaMemcpyDeviceToHost, stream));
        RTGB_CHECK(cudaStreamSynchronize(stream));
        float scale;
        std::memcpy(&scale, &bits, sizeof scale);
        const float pad = 1e-5f + 1e-5f * scale;
        d.prim_count = n;
        prim_count = n;
        ScopedBuf scratch, unsorted;
        unsorted.ensure(static_cast<size_t>(n) * sizeof(PrimRecord));
        scratch.ensure(lbvh_scratch_bytes(n));
        LbvhScratch ls = lbvh_carve(scratch.p, n);
        PrimRecord* recs = static_cast<PrimRecord*>(prims.ensure(static_cast<size_t>(n) * sizeof(PrimRecord)));
        launch_prim_records(d, unsorted.as<PrimRecord>(), ls.aabb_lo, ls.aabb_hi, pad, stream);
        RTGB_CHECK(cudaGetLastError());
        if (n >= 2 && kind == 2) {
            // same counts: the kept leaf order and hierarchy, boxes refitted bottom-up
            BvhNode* nd = nodes.as<BvhNode>();
            RTGB_CHECK(lbvh_refit(ls, n, sorted_vals.as<int>(), bvh_children.as<int>(), bvh_parent.as<int>(), nd, stream));
            launch_gather_records(unsorted.as<PrimRecord>(), sorted_vals.as<int>(), recs, n, stream);
            RTGB_CHECK(cudaGetLastError());
            RTGB_CHECK(fill_bvh4(nd, child4.as<int>(), ref4.as<int>(), node4_count, nodes4.as<float4>(), stream));
            d.nodes = nd;
            d.node_count = n - 1;
        } else if (n >= 2) {
            BvhNode* nd = static_cast<BvhNode*>(nodes.ensure(static_cast<size_t>(n - 1) * sizeof(BvhNode)));
            int* svals = nullptr;
            uint32_t* skeys = nullptr;
            RTGB_CHECK(lbvh_build(ls, n, nd, &svals, &skeys, stream));
            launch_gather_records(unsorted.as<PrimRecord>(), svals, recs, n, stream);
            RTGB_CHECK(cudaGetLastError());
            sorted_keys.ensure(static_cast<size_t>(n) * sizeof(uint32_t));
            sorted_vals.ensure(static_cast<size_t>(n) * sizeof(int));
            bvh_children.ensure(2 * static_cast<size_t>(n - 1) * sizeof(int));
            bvh_parent.ensure((2 * static_cast<size_t>(n) - 1) * sizeof(int));
            RTGB_CHECK(cudaMemcpyAsync(sorted_keys.p, skeys, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToDevice, stream));
            RTGB_CHECK(cudaMemcpyAsync(sorted_vals.p, svals, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToDevice, stream));
            RTGB_CHECK(cudaMemcpyAsync(bvh_children.p, ls.children, 2 * static_cast<size_t>(n - 1) * sizeof(int),
                cudaMemcpyDeviceToDevice, stream));
            RTGB_CHECK(cudaMemcpyAsync(bvh_parent.p, ls.parent, (2 * static_cast<size_t>(n) - 1) * sizeof(int),
                cudaMemcpyDeviceToDevice, stream));
            // the wide BVH: collapse the binary hierarchy on the host, boxes filled on the device
            std::vector<int> children2(2 * static_cast<size_t>(n - 1)), c4, r4;
            RTGB_CHECK(cudaMemcpyAsync(children2.data(), ls.children, children2.size() * sizeof(int), cudaMemcpyDeviceToHost,
                stream));
            RTGB_CHECK(cudaStreamSynchronize(stream));
            node4_count = collapse_bvh4(children2.data(), n, c4, r4);
            RTGB_CHECK(cudaMemcpyAsync(child4.ensure(c4.size() * sizeof(int)), c4.data(), c4.size() * sizeof(int),
                cudaMemcpyHostToDevice, stream));
            RTGB_CHECK(cudaMemcpyAsync(ref4.ensure(r4.size() * sizeof(int)), r4.data(), r4.size() * sizeof(int),
                cudaMemcpyHostToDevice, stream));
            nodes4.ensure(static_cast<size_t>(node4_count) * kNode4 * sizeof(float4));
            RTGB_CHECK(fill_bvh4(nd, child4.as<int>(), ref4.as<int>(), node4_count, nodes4.as<float4>(), stream));
            RTGB_CHECK(cudaStreamSynchronize(stream));  // the host vectors leave scope
            d.nodes = nd;
            d.node_count = n - 1;
        } else {
            RTGB_CHECK(cudaMemcpyAsync(recs, unsorted.p, sizeof(PrimRecord), cudaMemcpyDeviceToDevice, stream));
            d.nodes = nullptr;
            d.node_count = 0;
            node4_count = 0;
        }
        d.nodes4 = node4_count > 0 ? nodes4.as<float4>() : nullptr;
        d.node4_count = node4_count;
        d.prims = recs;
        RTGB_CHECK(cudaStreamSynchronize(stream));
    }

    // Analytic-light BVH over the finite lights (host boxes, device build).
    void build_analytic_bvh(const rtgb_scene& s, const std::vector<int>& finite, DeviceScene& d) {
        const int nf = static_cast<int>(finite.size());
        d.analytic_bvh_count = nf;
        analytic_bvh_count = nf;
        d.analytic_nodes = nullptr;
        d.analytic_node_count = 0;
        if (nf > 0) {
            std::vector<float4> lo(static_cast<size_t>(nf)), hi(static_cast<size_t>(nf));
            float lscale = 0.0f;
            for (int k = 0; k < nf; ++k) {
                const rtgb_analytic_light& l = s.analytic_lights[finite[static_cast<size_t>(k)]];
                float e[3];
                const float bxl = std::sqrt(l.basis_x[0] * l.basis_x[0] + l.basis_x[1] * l.basis_x[1] + l.basis_x[2] * l.basis_x[2]);
                for (int a = 0; a < 3; ++a) {
                    const float bx = std::fabs(l.basis_x[a]), by = std::fabs(l.basis_y[a]), bz = std::fabs(l.basis_z[a]);
                    if (l.type == 0) e[a] = std::fabs(l.radius) * bxl;
                    else if (l.type == 1) e[a] = std::fabs(l.radius) * (bx + by);
                    else if (l.type == 2) e[a] = 0.5f * (std::fabs(l.width) * bx + std::fabs(l.height) * by);
                    else e[a] = std::fabs(l.radius) * (bx + by) + 0.5f * std::fabs(l.length) * bz;
                    lscale = std::max(lscale, std::fabs(l.position[a]) + e[a]);
                }
                lo[static_cast<size_t>(k)] = make_float4(l.position[0] - e[0], l.position[1] - e[1], l.position[2] - e[2], 0.0f);
                hi[static_cast<size_t>(k)] = make_float4(l.position[0] + e[0], l.position[1] + e[1], l.position[2] + e[2], 0.0f);
            }
            const float lpad = 1e-5f + 1e-5f * lscale;
            for (int k = 0; k < nf; ++k) {
                lo[static_cast<size_t>(k)].x -= lpad; lo[static_cast<size_t>(k)].y -= lpad; lo[static_cast<size_t>(k)].z -= lpad;
                hi[static_cast<size_t>(k)].x += lpad; hi[static_cast<size_t>(k)].y += lpad; hi[static_cast<size_t>(k)].z += lpad;
            }
            std::vector<int> leaf(static_cast<size_t>(nf));
            if (nf >= 2) {
                ScopedBuf ascratch;
                ascratch.ensure(lbvh_scratch_bytes(nf));
                LbvhScratch as = lbvh_carve(ascratch.p, nf);
                RTGB_CHECK(cudaMemcpyAsync(as.aabb_lo, lo.data(), lo.size() * sizeof(float4), cudaMemcpyHostToDevice, stream));
                RTGB_CHECK(cudaMemcpyAsync(as.aabb_hi, hi.data(), hi.size() * sizeof(float4), cudaMemcpyHostToDevice, stream));
                BvhNode* an = static_cast<BvhNode*>(analytic_nodes.ensure(static_cast<size_t>(nf - 1) * sizeof(BvhNode)));
                int* svals = nullptr;
                uint32_t* skeys = nullptr;
                RTGB_CHECK(lbvh_build(as, nf, an, &svals, &skeys, stream));
                std::vector<int> order(static_cast<size_t>(nf));
                RTGB_CHECK(cudaMemcpyAsync(order.data(), svals, order.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
                RTGB_CHECK(cudaStreamSynchronize(stream));
                for (int k = 0; k < nf; ++k) leaf[static_cast<size_t>(k)] = finite[static_cast<size_t>(order[static_cast<size_t>(k)])];
                d.analytic_nodes = an;
                d.analytic_node_count = nf - 1;
            } else {
                leaf[0] = finite[0];
            }
            d.analytic_leaf = upload(analytic_leaf, leaf.data(), leaf.size(), stream);
        } else {
            d.analytic_leaf = nullptr;
        }
    }

    void reset_accumulation() {
        for (int c = 0; c < RTGB_MAX_CAMERAS; ++c) {
            history_length[c] = 0;
            prev_valid[c] = 0;
        }
    }

    // ---- frames -------------------------------------------------------------

    void validate_request(const rtgb_camera_rig& rig, const rtgb_render_profile& profile, int active) {
        // validate_render_pool_request (render_request_validation.cpp)
        if (rig.active_count < 1 || rig.active_count > RTGB_MAX_CAMERAS) throw Invalid{"render_frame rig.active_count out of range"};
        if (active < 1 || active > RTGB_MAX_CAMERAS) throw Invalid{"render_frame active_cameras out of range"};
        if (active > rig.active_count) throw Invalid{"render_frame active_cameras exceeds rig.active_count"};
        for (int c = 0; c < active; ++c) {
            const rtgb_camera& cam = rig.cameras[c];
            if (cam.enabled == 0) throw Invalid{"render_frame leading camera slot disabled at index " + std::to_string(c)};
            if (cam.width <= 0 || cam.height <= 0) throw Invalid{"render_frame leading camera slot has invalid resolution at index " + std::to_string(c)};
            if (cam.model != RTGB_CAMERA_PINHOLE32 && cam.model != RTGB_CAMERA_EQUI62_LUT1D) throw Invalid{"render_frame unknown camera model"};
            if (cam.model == RTGB_CAMERA_PINHOLE32 && (cam.pinhole.fx == 0.0 || cam.pinhole.fy == 0.0)) throw Invalid{"pinhole32 focal length is zero"};
            if (cam.model == RTGB_CAMERA_EQUI62_LUT1D && (cam.equi.fx == 0.0 || cam.equi.fy == 0.0)) throw Invalid{"equi62_lut1d focal length is zero"};
        }
        if (profile.samples_per_pixel > 4096 || profile.max_bounces > 64) throw Invalid{"render profile exceeds spp 4096 / 64 bounces"};
    }

    void ensure_frames(long long pixels) {
        // beauty, normal, dnormal, albedo, denoised float4; depth, trust float; flow float2; reservoir record 96 B
        const size_t per = 5 * 16 + 4 + 4 + 8 + sizeof(ReservoirRec);
        for (int f = 0; f < 2; ++f) {
            if (frame_mem[f].bytes >= static_cast<size_t>(pixels) * per + 2304 && frame_mem[f].p) continue;
            drop_graph();
            // asynchronous downloads may still read the old buffers
            if (copy_stream) RTGB_CHECK(cudaStreamSynchronize(copy_stream));
            copy_pending[f] = false;
            char* p = static_cast<char*>(frame_mem[f].ensure(static_cast<size_t>(pixels) * per + 2304));
            auto take = [&](size_t bytes) {
                char* r = p;
                p += (bytes + 255) & ~size_t(255);
                return r;
            };
            FrameBufs& b = frames[f];
            b.beauty = reinterpret_cast<float4*>(take(pixels * 16));
            b.normal = reinterpret_cast<float4*>(take(pixels * 16));
            b.dnormal = reinterpret_cast<float4*>(take(pixels * 16));
            b.albedo = reinterpret_cast<float4*>(take(pixels * 16));
            b.depth = reinterpret_cast<float*>(take(pixels * 4));
            b.flow = reinterpret_cast<float2*>(take(pixels * 8));
            b.trust = reinterpret_cast<float*>(take(pixels * 4));
            b.reservoirs = reinterpret_cast<ReservoirRec*>(take(pixels * sizeof(ReservoirRec)));
            b.denoised = reinterpret_cast<float4*>(take(pixels * 16));
        }
    }

    void ensure_paths(long long n, int spp, int bounces) {
        const bool need_records = record;
        if (n <= path_capacity && (!need_records || path_record_bounces >= bounces) && path_mem.p) return;
        drop_graph();
        const size_t align = 256;
        auto sz = [&](size_t b) { return (b + align - 1) & ~(align - 1); };
        const size_t f4 = sz(static_cast<size_t>(n) * 16), i1 = sz(static_cast<size_t>(n) * 4), i2 = sz(static_cast<size_t>(n) * 8);
        const size_t src2 = sz(static_cast<size_t>(n) * 8 * kMaxReuseSources);
        const size_t src1 = sz(static_cast<size_t>(n) * 4 * kMaxReuseSources);
        const size_t bins = sz(static_cast<size_t>(kSortBins) * 4);
        size_t total = f4 * 17 + i2 + i1 * 11 + src2 + 2 * src1 + 2 * bins;
        const bool scratch = true;
        if (scratch) total += sz(static_cast<size_t>(n) * sizeof(ReservoirRec));
        if (need_records) total += sz(static_cast<size_t>(n) * 4 * bounces);
        char* p = static_cast<char*>(path_mem.ensure(total));
        auto take = [&](size_t b) {
            char* r = p;
            p += b;
            return r;
        };
        Paths P{};
        P.ray_o = reinterpret_cast<float4*>(take(f4));
        P.ray_d = reinterpret_cast<float4*>(take(f4));
        P.thr = reinterpret_cast<float4*>(take(f4));
        P.rad = reinterpret_cast<float4*>(take(f4));
        P.prev_pos = reinterpret_cast<float4*>(take(f4));
        P.prev_nrm = reinterpret_cast<float4*>(take(f4));
        P.aux_n = reinterpret_cast<float4*>(take(f4));
        P.aux_a = reinterpret_cast<float4*>(take(f4));
        P.hit = reinterpret_cast<float4*>(take(f4));
        for (int k = 0; k < 2; ++k) {
            P.sh_o[k] = reinterpret_cast<float4*>(take(f4));
            P.sh_d[k] = reinterpret_cast<float4*>(take(f4));
            P.sh_c[k] = reinterpret_cast<float4*>(take(f4));
        }
        P.prev_prim = reinterpret_cast<int2*>(take(i2));
        P.rng = reinterpret_cast<uint32_t*>(take(i1));
        P.queue[0] = reinterpret_cast<int*>(take(i1));
        P.queue[1] = reinterpret_cast<int*>(take(i1));
        P.shadow_queue = reinterpret_cast<int*>(take(i1));
        P.restir_queue = reinterpret_cast<int*>(take(i1));
        P.res_written = reinterpret_cast<int*>(take(i1));
        P.sss_mat = reinterpret_cast<int*>(take(i1));
        P.sss_ext = reinterpret_cast<float4*>(take(f4));
        P.sss_alb = reinterpret_cast<float4*>(take(f4));
        P.res_meta = reinterpret_cast<int*>(take(i1));
        P.res_src = reinterpret_cast<int2*>(take(src2));
        P.res_src_t = reinterpret_cast<float*>(take(src1));
        P.src_stride = n;  // source-major: one source of consecutive paths is contiguous
        P.vis_queue = reinterpret_cast<int*>(take(src1));
        P.sort_key = reinterpret_cast<int*>(take(i1));
        P.sorted = reinterpret_cast<int*>(take(i1));
        P.scatter_queue = reinterpret_cast<int*>(take(i1));
        P.sort_hist = reinterpret_cast<int*>(take(bins));
        P.sort_cursor = reinterpret_cast<int*>(take(bins));
        RTGB_CHECK(cudaMemsetAsync(P.sort_hist, 0, bins, stream));  // k_sort_scan re-zeroes it after each use
        P.res_scratch = reinterpret_cast<ReservoirRec*>(take(sz(static_cast<size_t>(n) * sizeof(ReservoirRec))));
        P.codes = need_records ? reinterpret_cast<int*>(take(sz(static_cast<size_t>(n) * 4 * bounces))) : nullptr;
        paths = P;
        path_capacity = n;
        path_record_bounces = need_records ? bounces : 0;
        (void)spp;
    }

    // Binds a slot's device LUT and direction table for these intrinsics;
    // returns true when the table has to be (re)computed.
    bool bind_camera(int slot, const rtgb_camera& c, CameraDev& d) {
        CameraRes* res = &cam_res[slot][cam_cur[slot]];
        bool fresh = false;
        if (!same_intrinsics(*res, c)) {
            cam_cur[slot] ^= 1;
            res = &cam_res[slot][cam_cur[slot]];
            res->valid = true;
            res->width = c.width;
            res->height = c.height;
            res->model = c.model;
            res->pinhole = c.pinhole;
            res->equi = c.equi;
            res->monotone = 1;
            for (int i = 0; i + 1 < RTGB_EQUI_LUT_SIZE; ++i) {
                if (!(c.equi.lut[i] <= c.equi.lut[i + 1])) res->monotone = 0;
            }
            upload(res->lut, c.equi.lut, RTGB_EQUI_LUT_SIZE, stream);
            res->dirs.ensure(static_cast<size_t>(c.width) * c.height * sizeof(float4));
            fresh = true;
        }
        d.lut_monotone = res->monotone;
        d.lut = res->lut.as<double>();
        d.dirs = res->dirs.as<float4>();
        return fresh;
    }

    // make_device_active_camera (radiance_launch_setup.cpp:19-64)
    static CameraDev camera_dev(const rtgb_camera& c, long long pixel_offset, long long path_offset) {
        CameraDev d{};
        d.width = c.width;
        d.height = c.height;
        d.model = c.model;
        d.pixel_offset = pixel_offset;
        d.path_offset = path_offset;
        for (int r = 0; r < 3; ++r) {
            d.origin[r] = c.translation[r];
            d.bx[r] = c.rotation[r * 3 + 0];
            d.by[r] = c.rotation[r * 3 + 1];
            d.bz[r] = c.rotation[r * 3 + 2];
            d.origin_f[r] = static_cast<float>(d.origin[r]);
            d.bx_f[r] = static_cast<float>(d.bx[r]);
            d.by_f[r] = static_cast<float>(d.by[r]);
            d.bz_f[r] = static_cast<float>(d.bz[r]);
        }
        const rtgb_pinhole32& ph = c.pinhole;
        const double pin[9] = {ph.fx, ph.fy, ph.cx, ph.cy, ph.k1, ph.k2, ph.k3, ph.p1, ph.p2};
        std::memcpy(d.pin, pin, sizeof pin);
        d.eq_fx = c.equi.fx;
        d.eq_fy = c.equi.fy;
        d.eq_cx = c.equi.cx;
        d.eq_cy = c.equi.cy;
        d.eq_tan[0] = c.equi.tangential[0];
        d.eq_tan[1] = c.equi.tangential[1];
        d.lut_step = c.equi.lut_step;
        d.lut_monotone = 1;
        return d;
    }

    // Stage events are recorded as external event nodes, so they also time
    // each launch inside the replayed graph.
    void mark(int& k) {
        if (!stage_timing) return;
        RTGB_CHECK(cudaEventRecordWithFlags(stage_events[static_cast<size_t>(k)], stream, cudaEventRecordExternal));
        ++k;
    }

    void enqueue_frame_kernels() {
        const int mb = h_fp.max_bounces;
        if (stage_timing) {
            const size_t need = static_cast<size_t>(3 * mb + 4);
            while (stage_events.size() < need) {
                cudaEvent_t e;
                RTGB_CHECK(cudaEventCreate(&e));
                stage_events.push_back(e);
            }
        }
        // Grids: the persistent size (SMs x resident blocks), but no more blocks
        // than the frame's paths need (small frames then launch few, cheap blocks).
        LaunchShape sh[kLaunchShapes];
        for (int i = 0; i < kLaunchShapes; ++i) {
            sh[i] = shapes[i];
            const long long need = (total_paths + sh[i].block - 1) / (sh[i].block > 0 ? sh[i].block : 1);
            if (need > 0 && need < sh[i].grid) sh[i].grid = static_cast<int>(need);
        }
        int k = 0;
        mark(k);
        launch_raygen(d_fp, paths, d_counters, sh[0], stream);
        mark(k);
        for (int b = 0; b < mb; ++b) {
            launch_trace(d_fp, scene, paths, d_counters, b, sh[deep_bvh(scene) ? 14 : 1], stream);
            mark(k);
            launch_reset_counters(d_counters, b, stream);
            const bool pbr_scene = scene.openpbr_count > 0;
            if (h_fp.sort_from_bounce <= b) launch_shade_sort(d_fp, scene, paths, d_counters, b, sh[1].grid, stream);
            launch_shade(d_fp, scene, paths, d_counters, b, sh[pbr_scene ? 7 : 2], sh[13], stream);
            if (b == 0) launch_restir(d_fp, scene, paths, d_counters, sh, stream);
            mark(k);
            launch_shadow(d_fp, scene, paths, d_counters, b, sh[deep_bvh(scene) ? 15 : 3], stream);
            mark(k);
        }
        launch_finalize(d_fp, paths, d_counters, sh[4], stream);
        mark(k);
        launch_resolve(d_fp, sh[5], stream);
        mark(k);
        stage_count = stage_timing ? k - 1 : 0;
        if (denoise_this_frame) enqueue_denoise();
    }

    // Denoises every run of consecutive equal-size cameras as one batch into
    // the frame's `denoised` buffer, between two external events (denoise_ms).
    void enqueue_denoise() {
        RTGB_CHECK(cudaEventRecordWithFlags(ev_dn0, stream, cudaEventRecordExternal));
        const FrameParams& fp = h_fp;
        int c = 0;
        while (c < fp.cam_count) {
            int e = c + 1;
            while (e < fp.cam_count && fp.cam[e].width == fp.cam[c].width && fp.cam[e].height == fp.cam[c].height) ++e;
            RTGB_CHECK(unet_run(unet, d_fp, fp.cam[c].pixel_offset, e - c, fp.cam[c].height, fp.cam[c].width,
                &d_counters->denoise_error, sm_count, stream));
            c = e;
        }
        RTGB_CHECK(cudaEventRecordWithFlags(ev_dn1, stream, cudaEventRecordExternal));
    }

    int render(const rtgb_camera_rig& rig, const rtgb_render_profile& profile, int active, bool sync,
        rtgb_frame_views* out) {
        if (!prepared) {
            error = "render_frame requires prepare_scene() first";
            return RTGB_NOT_PREPARED;
        }
        validate_request(rig, profile, active);
        RTGB_CHECK(cudaSetDevice(device));
        const int spp = profile.samples_per_pixel > 0 ? profile.samples_per_pixel : 1;
        const int mb = profile.max_bounces > 0 ? profile.max_bounces : 1;
        // layout: cameras back to back; a change of any resolution drops history
        bool layout_changed = active != layout_count;
        for (int c = 0; c < active; ++c) layout_changed |= rig.cameras[c].width != layout_w[c] || rig.cameras[c].height != layout_h[c];
        long long pixels = 0;
        long long offsets[RTGB_MAX_CAMERAS];
        for (int c = 0; c < active; ++c) {
            offsets[c] = pixels;
            pixels += static_cast<long long>(rig.cameras[c].width) * rig.cameras[c].height;
        }
        if (pixels * spp >= (1ll << 31)) throw Invalid{"frame exceeds 2^31 paths"};
        // the bias-correction ray queue packs (path << 4) | source into an int
        if (profile.enable_restir_di != 0 && pixels * spp >= (1ll << 27)) {
            throw Invalid{"ReSTIR DI frames are limited to 2^27 paths"};
        }
        if (layout_changed) {
            // resize_history -> reset_history (device_frame_buffers.cpp:80-98)
            for (int c = 0; c < RTGB_MAX_CAMERAS; ++c) {
                history_length[c] = 0;
                prev_valid[c] = 0;
                layout_w[c] = c < active ? rig.cameras[c].width : 0;
                layout_h[c] = c < active ? rig.cameras[c].height : 0;
            }
            layout_count = active;
        }
        total_pixels = pixels;
        total_paths = pixels * spp;
        ensure_frames(pixels);
        ensure_paths(total_paths, spp, mb);
        // asynchronous downloads of the frame that last used frames[cur] finish
        // before this frame's kernels overwrite it
        if (copy_pending[cur]) {
            RTGB_CHECK(cudaStreamWaitEvent(stream, ev_copied[cur], 0));
            copy_pending[cur] = false;
        }
        denoise_this_frame = profile.enable_denoise != 0 && unet_ready(unet);
        if (denoise_this_frame) {
            if (!ev_dn0) {
                RTGB_CHECK(cudaEventCreate(&ev_dn0));
                RTGB_CHECK(cudaEventCreate(&ev_dn1));
            }
            for (int c = 0; c < active;) {
                int e = c + 1;
                while (e < active && rig.cameras[e].width == rig.cameras[c].width &&
                       rig.cameras[e].height == rig.cameras[c].height) {
                    ++e;
                }
                if (!unet_prepare(unet, e - c, rig.cameras[c].height, rig.cameras[c].width)) {
                    throw CudaFailure{cudaErrorMemoryAllocation, "denoiser activations / tensor maps (unet_prepare)"};
                }
                c = e;
            }
        }

        FrameParams& fp = h_fp;
        std::memset(&fp, 0, sizeof fp);
        frame_h2d = sizeof(FrameParams);
        for (int c = 0; c < active; ++c) {
            fp.cam[c] = camera_dev(rig.cameras[c], offsets[c], offsets[c] * spp);
            if (bind_camera(c, rig.cameras[c], fp.cam[c])) {
                launch_camera_dirs(fp.cam[c], const_cast<float4*>(fp.cam[c].dirs), stream);
                frame_h2d += RTGB_EQUI_LUT_SIZE * sizeof(double);
            }
            fp.prev[c] = prev[c];
            fp.prev_valid[c] = prev_valid[c];
            fp.history_length[c] = history_length[c];
        }
        RTGB_CHECK(cudaGetLastError());
        fp.cam_count = active;
        fp.spp = spp;
        fp.max_bounces = mb;
        fp.rr_start = profile.rr_start_bounce;
        fp.total_pixels = total_pixels;
        fp.total_paths = total_paths;
        fp.stream = sample_stream;
        const int min_lights = profile.restir_min_analytic_lights > 0 ? profile.restir_min_analytic_lights : 1;
        // ReSTIR over emissive geometry (opt-in) needs an emissive light list; the
        // reference's ReSTIR needs restir_min_analytic_lights analytic lights
        fp.restir_emissive = profile.enable_restir_di != 0 && profile.restir_emissive != 0 && scene.light_count > 0 ? 1 : 0;
        fp.restir_enabled = fp.restir_emissive != 0 ||
                            (profile.enable_restir_di != 0 && scene.analytic_count >= min_lights) ? 1 : 0;
        fp.restir_candidates = profile.restir_initial_candidates;
        fp.restir_temporal = profile.restir_temporal_reuse;
        fp.restir_max_age = profile.restir_max_history_age;
        fp.restir_max_temporal = profile.restir_max_temporal_candidates;
        fp.restir_spatial = profile.restir_spatial_neighbors;
        fp.restir_max_spatial = profile.restir_max_spatial_candidates;
        fp.restir_bias = profile.restir_bias_correction;
        fp.record_paths = record ? 1 : 0;
        // material-bucketed shading (shade_sort.cu) keeps a warp's paths on one
        // material's branches. Automatic: on where there is divergence to remove
        // (OpenPBR materials, or more than kBucketMaterials materials); a scene of
        // a handful of materials (the Cornell box) only pays the three launches.
        const bool bucket = shade_order > 0 ||
            (shade_order == 0 && (scene.openpbr_count > 0 || scene.material_count > kBucketMaterials));
        fp.sort_from_bounce = !bucket ? INT_MAX : (shade_order == 1 ? 1 : 0);
        fp.cur = frames[cur];
        fp.hist = frames[cur ^ 1];
        // Pageable source: the copy is staged before the call returns, so the
        // host struct can be rewritten for the next frame immediately.
        RTGB_CHECK(cudaMemcpyAsync(d_fp, &fp, sizeof fp, cudaMemcpyHostToDevice, stream));

        RTGB_CHECK(cudaEventRecord(ev_start, stream));
        // the captured launches depend on the bucketing switch too (the sort kernels are in or out)
        const long long key[5] = {total_paths, mb,
            static_cast<long long>(paths.ray_o != nullptr) | (fp.sort_from_bounce != INT_MAX ? 2ll : 0ll),
            reinterpret_cast<long long>(scene.prims), (denoise_this_frame ? 1ll : 0ll) | (static_cast<long long>(unet_generation) << 1)};
        if (use_graph) {
            if (!graph_exec || std::memcmp(key, graph_key, sizeof key) != 0) {
                drop_graph();
                cudaGraph_t graph;
                RTGB_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                enqueue_frame_kernels();
                RTGB_CHECK(cudaStreamEndCapture(stream, &graph));
                const cudaError_t inst = cudaGraphInstantiate(&graph_exec, graph, 0);
                cudaGraphDestroy(graph);
                RTGB_CHECK(inst);
                std::memcpy(graph_key, key, sizeof key);
            }
            RTGB_CHECK(cudaGraphLaunch(graph_exec, stream));
        } else {
            enqueue_frame_kernels();
        }
        RTGB_CHECK(cudaGetLastError());
        RTGB_CHECK(cudaEventRecord(ev_stop, stream));
        RTGB_CHECK(cudaMemcpyAsync(h_counters, d_counters, sizeof(Counters), cudaMemcpyDeviceToHost, stream));

        // capture_launch_history (radiance_launch_setup.cpp:122-136); the
        // frame buffers swap instead of copying into history.
        for (int c = 0; c < active; ++c) {
            prev[c] = fp.cam[c];
            prev_valid[c] = 1;
            history_length[c] = history_length[c] == 0 ? 1 : history_length[c] + 1;
            last_pixel_offset[c] = offsets[c];
            last_w[c] = rig.cameras[c].width;
            last_h[c] = rig.cameras[c].height;
        }
        last_count = active;
        last_denoised = denoise_this_frame;
        last_spp = spp;
        last_bounces = mb;
        last = cur;
        cur ^= 1;
        ++frame_serial;
        const uint32_t used_stream = sample_stream++;
        if (out) {
            std::memset(out, 0, sizeof *out);
            out->camera_count = active;
            out->sample_stream = used_stream;
            for (int c = 0; c < active; ++c) fill_view(c, out->cameras[c]);
        }
        if (sync) {
            RTGB_CHECK(cudaStreamSynchronize(stream));
            if (out) fill_stats(out);
            if (h_counters->error != 0) {
                error = "device reported " + std::to_string(h_counters->error) + " inconsistent hit records";
                return RTGB_DEVICE_FAULT_FLAG;
            }
            if (h_counters->denoise_error != 0) {
                error = "a denoiser kernel gave up waiting (code " + std::to_string(h_counters->denoise_error) + ")";
                return RTGB_DEVICE_FAULT_FLAG;
            }
            if (h_counters->gave_up != 0) {
                error = gave_up_message();
                return RTGB_DEVICE_FAULT_FLAG;
            }
        }
        return RTGB_OK;
    }

    std::string gave_up_message() const {
        return std::to_string(h_counters->gave_up) + " device loops reached their bound this frame (traversal " +
               std::to_string(traversal_limit) + " node visits, rejection sampling " + std::to_string(rejection_limit) +
               " draws); the frame's results are incomplete";
    }

    void fill_view(int c, rtgb_camera_frame_view& v) const {
        const FrameBufs& f = frames[last];
        const long long o = last_pixel_offset[c];
        v.camera_index = c;
        v.width = last_w[c];
        v.height = last_h[c];
        v.beauty = last_denoised ? f.denoised + o : f.beauty + o;
        v.normal = f.normal + o;
        v.denoiser_normal = f.dnormal + o;
        v.albedo = f.albedo + o;
        v.depth = f.depth + o;
        v.flow = f.flow + o;
        v.flow_trustworthiness = f.trust + o;
    }

    void fill_stats(rtgb_frame_views* out) {
        float ms = 0.0f;
        RTGB_CHECK(cudaEventElapsedTime(&ms, ev_start, ev_stop));
        out->frame_render_ms = ms;
        float dn = 0.0f;
        if (last_denoised) RTGB_CHECK(cudaEventElapsedTime(&dn, ev_dn0, ev_dn1));
        last_denoise_ms = dn;
        // per camera, the reference's RadianceTiming: render and denoise are separate stages
        for (int c = 0; c < out->camera_count; ++c) {
            out->cameras[c].render_ms = ms - dn;
            out->cameras[c].denoise_ms = dn;
        }
        const Counters& k = *h_counters;
        out->primary_rays = k.rays[0];
        out->extension_rays = k.rays[1];
        out->shadow_rays = k.rays[2];
        out->restir_visibility_rays = k.rays[3];
        out->rays_traced = k.rays[0] + k.rays[1] + k.rays[2] + k.rays[3];
        out->h2d_bytes = frame_h2d;
        out->restir_pixels = k.restir_pixels;
        for (int b = 0; b < last_bounces && b < 64; ++b) out->shadow_per_bounce[b] = k.shadow_bounce[b];
        for (int b = 0; b < last_bounces && b < 64; ++b) out->active_paths[b] = static_cast<uint64_t>(k.bounce_active[b]);
    }

    void check_camera(int c) const {
        if (last < 0) throw Invalid{"no frame has been rendered"};
        if (c < 0 || c >= last_count) throw Invalid{"camera_index out of range: camera_index=" + std::to_string(c) + ", active_count=" + std::to_string(last_count)};
    }

    void download(int c, float* beauty, float* normal, float* albedo, float* depth, float* ms) {
        check_camera(c);
        const size_t n = static_cast<size_t>(last_w[c]) * last_h[c];
        const FrameBufs& f = frames[last];
        const long long o = last_pixel_offset[c];
        RTGB_CHECK(cudaEventRecord(ev_start, stream));
        enqueue_copies(f, o, n, beauty, normal, albedo, depth, stream);
        RTGB_CHECK(cudaEventRecord(ev_stop, stream));
        RTGB_CHECK(cudaStreamSynchronize(stream));
        if (ms) RTGB_CHECK(cudaEventElapsedTime(ms, ev_start, ev_stop));
    }

    // beauty (denoised when the frame was), normal, albedo and depth of one camera
    void enqueue_copies(const FrameBufs& f, long long o, size_t n, float* beauty, float* normal, float* albedo,
        float* depth, cudaStream_t s) const {
        const float4* bsrc = last_denoised ? f.denoised + o : f.beauty + o;
        if (beauty) RTGB_CHECK(cudaMemcpyAsync(beauty, bsrc, n * 16, cudaMemcpyDeviceToHost, s));
        if (normal) RTGB_CHECK(cudaMemcpyAsync(normal, f.normal + o, n * 16, cudaMemcpyDeviceToHost, s));
        if (albedo) RTGB_CHECK(cudaMemcpyAsync(albedo, f.albedo + o, n * 16, cudaMemcpyDeviceToHost, s));
        if (depth) RTGB_CHECK(cudaMemcpyAsync(depth, f.depth + o, n * 4, cudaMemcpyDeviceToHost, s));
    }

    // rtgb_download_frame_async: the copies of the last frame's buffers go on
    // copy_stream after that frame's kernels; the call does not wait for them.
    void download_async(int c, float* beauty, float* normal, float* albedo, float* depth) {
        check_camera(c);
        if (!copy_stream) {
            RTGB_CHECK(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
            for (cudaEvent_t* e : {&ev_ready, &ev_copied[0], &ev_copied[1], &ev_older_copied}) {
                RTGB_CHECK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
            }
        }
        if (download_serial != frame_serial) {
            // first download of a newer frame: mark where the older frames' copies end
            RTGB_CHECK(cudaEventRecord(ev_older_copied, copy_stream));
            download_serial = frame_serial;
        }
        RTGB_CHECK(cudaEventRecord(ev_ready, stream));
        RTGB_CHECK(cudaStreamWaitEvent(copy_stream, ev_ready, 0));
        const size_t n = static_cast<size_t>(last_w[c]) * last_h[c];
        enqueue_copies(frames[last], last_pixel_offset[c], n, beauty, normal, albedo, depth, copy_stream);
        RTGB_CHECK(cudaEventRecord(ev_copied[last], copy_stream));
        copy_pending[last] = true;
    }

    // rtgb_wait_downloads: every asynchronous download, or all but those of
    // the most recently downloaded frame, has landed in host memory
    void wait_downloads(bool keep_latest) {
        if (!copy_stream) return;
        if (keep_latest) {
            RTGB_CHECK(cudaEventSynchronize(ev_older_copied));
        } else {
            RTGB_CHECK(cudaStreamSynchronize(copy_stream));
        }
    }

    void download_buffer(int c, int which, void* host, size_t bytes) {
        check_camera(c);
        const size_t n = static_cast<size_t>(last_w[c]) * last_h[c];
        const FrameBufs& f = frames[last];
        const long long o = last_pixel_offset[c];
        const void* src = nullptr;
        size_t need = 0;
        switch (which) {
            case 0: src = f.beauty + o; need = n * 16; break;
            case 1: src = f.normal + o; need = n * 16; break;
            case 2: src = f.dnormal + o; need = n * 16; break;
            case 3: src = f.albedo + o; need = n * 16; break;
            case 4: src = f.depth + o; need = n * 4; break;
            case 5: src = f.flow + o; need = n * 8; break;
            case 6: src = f.trust + o; need = n * 4; break;
            case 7: {
                // the reference's 84-byte RestirReservoir records, converted from the device records
                need = n * sizeof(Reservoir);
                if (bytes != need) throw Invalid{"buffer size mismatch: expected " + std::to_string(need) + " bytes"};
                std::vector<ReservoirRec> recs(n);
                RTGB_CHECK(cudaMemcpyAsync(recs.data(), f.reservoirs + o, n * sizeof(ReservoirRec),
                    cudaMemcpyDeviceToHost, stream));
                RTGB_CHECK(cudaStreamSynchronize(stream));
                Reservoir* out = static_cast<Reservoir*>(host);
                for (size_t i = 0; i < n; ++i) out[i] = load_reservoir(&recs[i]);
                return;
            }
            case 8:
                if (!last_denoised) throw Invalid{"the last frame was not denoised"};
                src = f.denoised + o;
                need = n * 16;
                break;
            default: throw Invalid{"unknown frame buffer"};
        }
        if (bytes != need) throw Invalid{"buffer size mismatch: expected " + std::to_string(need) + " bytes"};
        RTGB_CHECK(cudaMemcpyAsync(host, src, need, cudaMemcpyDeviceToHost, stream));
        RTGB_CHECK(cudaStreamSynchronize(stream));
    }
};

namespace {

template <typename F>
rtgb_status guarded(rtgb_handle h, F&& fn) {
    try {
        if (h) h->error.clear();
        return static_cast<rtgb_status>(fn());
    } catch (const Invalid& e) {
        if (h) h->error = e.message;
        return RTGB_INVALID_ARGUMENT;
    } catch (const CudaFailure& f) {
        if (h) h->fail_cuda(f);
        return RTGB_RUNTIME_ERROR;
    } catch (const std::bad_alloc&) {
        if (h) h->error = "host allocation failed";
        return RTGB_RUNTIME_ERROR;
    }
}

}  // namespace

extern "C" {

rtgb_status rtgb_create(const rtgb_create_info* info, rtgb_handle* out) {
    if (out == nullptr) return RTGB_INVALID_ARGUMENT;
    *out = nullptr;
    rtgb_create_info defaults{0, 1, 0, 0};
    auto* h = new (std::nothrow) rtgb_renderer();
    if (!h) return RTGB_RUNTIME_ERROR;
    try {
        h->init(info ? *info : defaults);
    } catch (const CudaFailure&) {
        delete h;
        return RTGB_RUNTIME_ERROR;
    }
    *out = h;
    return RTGB_OK;
}

void rtgb_destroy(rtgb_handle h) { delete h; }

const char* rtgb_last_error(rtgb_handle h) { return h ? h->error.c_str() : "null handle"; }

rtgb_status rtgb_prepare_scene(rtgb_handle h, const rtgb_scene* scene) {
    if (!h || !scene) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->prepare(*scene);
        return RTGB_OK;
    });
}

rtgb_status rtgb_prepare_scene_instanced(rtgb_handle h, const rtgb_scene* scene, const rtgb_mesh_set* meshes) {
    if (!h || !scene || !meshes) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->prepare(*scene, meshes);
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_triangles(rtgb_handle h, rtgb_triangle* out, int32_t capacity, int32_t* count) {
    if (!h || capacity < 0) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->prepared) {
            h->error = "download_triangles requires prepare_scene() first";
            return RTGB_NOT_PREPARED;
        }
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        const int n = std::min(capacity, h->scene.triangle_count);
        if (count) *count = h->scene.triangle_count;
        if (out && n > 0) {
            RTGB_CHECK(cudaMemcpy(out, h->scene.triangles, static_cast<size_t>(n) * sizeof(rtgb_triangle), cudaMemcpyDeviceToHost));
        }
        return RTGB_OK;
    });
}

rtgb_status rtgb_reset_sequence(rtgb_handle h, uint32_t s) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    h->sample_stream = s;
    h->reset_accumulation();
    return RTGB_OK;
}

rtgb_status rtgb_reset_accumulation(rtgb_handle h) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    h->reset_accumulation();
    return RTGB_OK;
}

rtgb_status rtgb_render_frame(rtgb_handle h, const rtgb_camera_rig* rig, const rtgb_render_profile* profile,
    int32_t active, rtgb_frame_views* out) {
    if (!h || !rig || !profile) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] { return h->render(*rig, *profile, active, true, out); });
}

rtgb_status rtgb_render_frame_async(rtgb_handle h, const rtgb_camera_rig* rig, const rtgb_render_profile* profile,
    int32_t active) {
    if (!h || !rig || !profile) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] { return h->render(*rig, *profile, active, false, nullptr); });
}

rtgb_status rtgb_frame_stats(rtgb_handle h, rtgb_frame_views* out) {
    if (!h || !out) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (h->last < 0) throw Invalid{"no frame has been rendered"};
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        std::memset(out, 0, sizeof *out);
        out->camera_count = h->last_count;
        out->sample_stream = h->sample_stream - 1;
        for (int c = 0; c < h->last_count; ++c) h->fill_view(c, out->cameras[c]);
        h->fill_stats(out);
        if (h->h_counters->gave_up != 0) h->error = h->gave_up_message();
        return h->h_counters->error != 0 || h->h_counters->denoise_error != 0 || h->h_counters->gave_up != 0
                   ? RTGB_DEVICE_FAULT_FLAG
                   : RTGB_OK;
    });
}

rtgb_status rtgb_stage_times(rtgb_handle h, float* out, int32_t capacity, int32_t* count) {
    if (!h || !out || !count) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->stage_timing) throw Invalid{"stage times need rtgb_create_info::stage_timing"};
        if (h->last < 0) throw Invalid{"no frame has been rendered"};
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        const int n = std::min(h->stage_count, capacity);
        for (int i = 0; i < n; ++i) {
            RTGB_CHECK(cudaEventElapsedTime(out + i, h->stage_events[static_cast<size_t>(i)],
                h->stage_events[static_cast<size_t>(i + 1)]));
        }
        *count = h->stage_count;
        return RTGB_OK;
    });
}

rtgb_status rtgb_set_debug_limits(rtgb_handle h, int32_t traversal_limit, int32_t rejection_limit) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        RTGB_CHECK(cudaSetDevice(h->device));
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        h->set_limits(traversal_limit, rejection_limit);
        return RTGB_OK;
    });
}

rtgb_status rtgb_launch_grids(rtgb_handle h, int32_t* grids, int32_t* blocks, int32_t capacity, int32_t* count) {
    if (!h || !count || capacity < 0 || (capacity > 0 && !grids)) return RTGB_INVALID_ARGUMENT;
    for (int i = 0; i < capacity && i < kLaunchShapes; ++i) {
        grids[i] = h->shapes[i].grid;
        if (blocks) blocks[i] = h->shapes[i].block;
    }
    *count = kLaunchShapes;
    return RTGB_OK;
}

// Launch-shape autotuner: the wavefront kernels loop grid-stride over the
// bounce's queue, so any grid size is correct; which one is fastest depends on
// the scene and the rig (tail balance against per-block setup such as the BVH
// node staging of k_trace / k_shadow). Each candidate scale of the persistent
// grids (SMs x resident blocks) is rendered for `frames` frames with stage
// events; per stage group the fastest scale wins. The frames rendered while
// tuning are discarded: accumulation and history restart afterwards.
rtgb_status rtgb_autotune_launches(rtgb_handle h, const rtgb_camera_rig* rig, const rtgb_render_profile* profile,
    int32_t active, int32_t frames, rtgb_launch_tuning* out) {
    if (!h || !rig || !profile || !out || frames < 1 || frames > 64) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        constexpr int kCandidates = RTGB_TUNE_CANDIDATES;
        // four grid scales at the kernels' block size, then the same with half-size blocks
        constexpr float kScales[kCandidates] = {0.5f, 1.0f, 2.0f, 4.0f, 0.5f, 1.0f, 2.0f, 4.0f};
        constexpr int kHalved[kCandidates] = {0, 0, 0, 0, 1, 1, 1, 1};
        // shape slots of each stage group (rtgb_launch_tuning::group_ms order)
        static const std::vector<int> kGroups[RTGB_TUNE_GROUPS] = {{0}, {1, 14}, {2, 6, 7, 8, 9, 10, 11, 12, 13}, {3, 15}, {4, 5}};
        *out = rtgb_launch_tuning {};
        LaunchShape base[kLaunchShapes];
        query_launch_shapes(h->sm_count, base);
        // Every exit that does not reach the end (a failed render, a CUDA
        // error thrown out of here) puts back the shapes and the stage-timing
        // switch the handle had before, drops the graph captured with a
        // candidate's grids and restarts accumulation.
        struct Restore {
            rtgb_renderer* h;
            LaunchShape shapes[kLaunchShapes];
            bool had_timing;
            bool done = false;
            ~Restore() {
                if (done) return;
                std::memcpy(h->shapes, shapes, sizeof shapes);
                h->stage_timing = had_timing;
                h->drop_graph();
                h->reset_accumulation();
            }
        } restore{h, {}, h->stage_timing};
        std::memcpy(restore.shapes, h->shapes, sizeof restore.shapes);
        const bool had_timing = h->stage_timing;
        h->stage_timing = true;
        // a half-size block keeps the threads in flight with twice the blocks
        auto apply = [&](const int* candidate_of_group) {
            for (int g = 0; g < RTGB_TUNE_GROUPS; ++g) {
                const int c = candidate_of_group[g];
                for (int slot : kGroups[g]) {
                    h->shapes[slot] = base[slot];
                    const int half = kHalved[c] != 0 ? 2 : 1;
                    h->shapes[slot].block = base[slot].block / half;
                    h->shapes[slot].grid =
                        std::max(1, static_cast<int>(static_cast<float>(base[slot].grid * half) * kScales[c]));
                }
            }
            h->drop_graph();
        };
        rtgb_frame_views views {};
        std::vector<float> st(256);
        for (int c = 0; c < kCandidates; ++c) {
            int cand[RTGB_TUNE_GROUPS];
            for (int& x : cand) x = c;
            apply(cand);
            out->scales[c] = kScales[c];
            out->block_halved[c] = kHalved[c];
            if (const int st0 = h->render(*rig, *profile, active, true, &views); st0 != RTGB_OK) return static_cast<rtgb_status>(st0);  // warm
            double frame = 0.0;
            for (int f = 0; f < frames; ++f) {
                if (const int st1 = h->render(*rig, *profile, active, true, &views); st1 != RTGB_OK) return static_cast<rtgb_status>(st1);
                frame += views.frame_render_ms;
                RTGB_CHECK(cudaStreamSynchronize(h->stream));
                const int n = h->stage_count;
                for (int i = 0; i < n && i < 256; ++i) {
                    RTGB_CHECK(cudaEventElapsedTime(&st[static_cast<size_t>(i)], h->stage_events[static_cast<size_t>(i)],
                        h->stage_events[static_cast<size_t>(i + 1)]));
                }
                // stage order: raygen, (trace, shade, shadow) per bounce, finalize, resolve
                const int mb = (n - 3) / 3;
                float* g = out->group_ms[c];
                g[0] += st[0] / static_cast<float>(frames);
                for (int b = 0; b < mb; ++b) {
                    g[1] += st[static_cast<size_t>(1 + 3 * b)] / static_cast<float>(frames);
                    g[2] += st[static_cast<size_t>(2 + 3 * b)] / static_cast<float>(frames);
                    g[3] += st[static_cast<size_t>(3 + 3 * b)] / static_cast<float>(frames);
                }
                g[4] += (st[static_cast<size_t>(n - 2)] + st[static_cast<size_t>(n - 1)]) / static_cast<float>(frames);
            }
            out->frame_ms[c] = static_cast<float>(frame / frames);
        }
        int best[RTGB_TUNE_GROUPS];
        for (int g = 0; g < RTGB_TUNE_GROUPS; ++g) {
            int pick = 1;  // the persistent shape unless another is faster
            for (int c = 0; c < kCandidates; ++c) {
                if (out->group_ms[c][g] < out->group_ms[pick][g]) pick = c;
            }
            out->chosen[g] = pick;
            best[g] = pick;
        }
        apply(best);
        if (const int st2 = h->render(*rig, *profile, active, true, &views); st2 != RTGB_OK) return static_cast<rtgb_status>(st2);
        double tuned = 0.0;
        for (int f = 0; f < frames; ++f) {
            if (const int st3 = h->render(*rig, *profile, active, true, &views); st3 != RTGB_OK) return static_cast<rtgb_status>(st3);
            tuned += views.frame_render_ms;
        }
        out->tuned_frame_ms = static_cast<float>(tuned / frames);
        h->stage_timing = had_timing;
        h->drop_graph();
        h->reset_accumulation();
        restore.done = true;
        return RTGB_OK;
    });
}

rtgb_status rtgb_ray_totals(rtgb_handle h, uint64_t totals[4]) {
    if (!h || !totals) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        Counters k;
        RTGB_CHECK(cudaMemcpy(&k, h->d_counters, sizeof k, cudaMemcpyDeviceToHost));
        for (int i = 0; i < 4; ++i) totals[i] = k.cum_rays[i];
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_frame(rtgb_handle h, int32_t c, float* beauty, float* normal, float* albedo, float* depth,
    float* ms) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->download(c, beauty, normal, albedo, depth, ms);
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_frame_async(rtgb_handle h, int32_t c, float* beauty, float* normal, float* albedo,
    float* depth) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->download_async(c, beauty, normal, albedo, depth);
        return RTGB_OK;
    });
}

rtgb_status rtgb_wait_downloads(rtgb_handle h, int32_t keep_latest) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->wait_downloads(keep_latest != 0);
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_light_table(rtgb_handle h, void* lights, int32_t capacity, int32_t* light_count,
    int32_t* sphere_light, int32_t* quad_light, int32_t* triangle_light) {
    if (!h || capacity < 0) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->prepared) {
            h->error = "download_light_table requires prepare_scene() first";
            return RTGB_NOT_PREPARED;
        }
        const DeviceScene& d = h->scene;
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        if (light_count) *light_count = d.light_count;
        const int n = std::min(capacity, d.light_count);
        if (lights && n > 0) RTGB_CHECK(cudaMemcpy(lights, d.lights, static_cast<size_t>(n) * sizeof(PackedLight), cudaMemcpyDeviceToHost));
        auto map = [](int32_t* dst, const int* src, int count) {
            if (dst && count > 0) RTGB_CHECK(cudaMemcpy(dst, src, static_cast<size_t>(count) * sizeof(int), cudaMemcpyDeviceToHost));
        };
        map(sphere_light, d.sphere_light, d.sphere_count);
        map(quad_light, d.quad_light, d.quad_count);
        map(triangle_light, d.triangle_light, d.triangle_count);
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_buffer(rtgb_handle h, int32_t c, int32_t which, void* host, size_t bytes) {
    if (!h || !host) return RTGB_INVALID_ARGUMENT;
    if (which < 0 || which > 8 || which == 7) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->download_buffer(c, which, host, bytes);
        return RTGB_OK;
    });
}

rtgb_status rtgb_set_denoiser_params(rtgb_handle h, const float* params, int64_t count) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->set_denoiser(params, count);
        return RTGB_OK;
    });
}

int64_t rtgb_denoiser_param_count(void) { return rtgb::unet_param_count(); }

rtgb_status rtgb_load_denoiser_file(rtgb_handle h, const char* path) {
    if (!h || !path) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        FILE* f = std::fopen(path, "rb");
        if (!f) throw Invalid{std::string("cannot open denoiser weights: ") + path};
        const long long n = rtgb::unet_param_count();
        std::vector<uint16_t> bits(static_cast<size_t>(n));
        const size_t got = std::fread(bits.data(), 2, bits.size(), f);
        const int extra = std::fgetc(f);
        std::fclose(f);
        if (got != bits.size() || extra != EOF) {
            throw Invalid{std::string("denoiser weights must hold exactly ") + std::to_string(n) + " BF16 values: " + path};
        }
        std::vector<float> params(bits.size());
        for (size_t i = 0; i < bits.size(); ++i) {
            const uint32_t u = static_cast<uint32_t>(bits[i]) << 16;
            std::memcpy(&params[i], &u, 4);
        }
        h->set_denoiser(params.data(), n);
        return RTGB_OK;
    });
}

rtgb_status rtgb_device_info_get(rtgb_handle h, rtgb_device_info* out) {
    if (!h || !out) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        *out = rtgb_device_info{};
        RTGB_CHECK(cudaSetDevice(h->device));
        cudaDeviceProp prop{};
        RTGB_CHECK(cudaGetDeviceProperties(&prop, h->device));
        std::snprintf(out->name, sizeof out->name, "%s", prop.name);
        out->device = h->device;
        out->major = prop.major;
        out->minor = prop.minor;
        out->multiprocessors = prop.multiProcessorCount;
        RTGB_CHECK(cudaDriverGetVersion(&out->driver_version));
        RTGB_CHECK(cudaRuntimeGetVersion(&out->runtime_version));
        size_t free_b = 0, total_b = 0;
        RTGB_CHECK(cudaMemGetInfo(&free_b, &total_b));
        out->total_bytes = total_b;
        out->used_bytes = total_b - free_b;
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_reservoirs(rtgb_handle h, int32_t c, void* host, size_t bytes) {
    if (!h || !host) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->download_buffer(c, 7, host, bytes);
        return RTGB_OK;
    });
}

rtgb_status rtgb_restir_diagnostics(rtgb_handle h, int32_t c, rtgb_restir_stats* out) {
    if (!h || !out) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->check_camera(c);
        const size_t n = static_cast<size_t>(h->last_w[c]) * h->last_h[c];
        std::vector<Reservoir> r(n);
        h->download_buffer(c, 7, r.data(), n * sizeof(Reservoir));
        rtgb_restir_stats d{};
        d.pixel_count = static_cast<int32_t>(n);
        for (const Reservoir& x : r) {
            if (x.valid == 0) continue;
            ++d.active_reservoir_count;
            if (x.temporal_candidate_count > 0) ++d.temporal_reuse_count;
            if (x.spatial_candidate_count > 0) ++d.spatial_reuse_count;
            if (x.bias_correction_source_count > 0) ++d.bias_corrected_count;
            d.max_candidate_count = std::max(d.max_candidate_count, x.candidate_count);
            d.max_age = std::max(d.max_age, x.age);
        }
        *out = d;
        return RTGB_OK;
    });
}

rtgb_status rtgb_render_direction_debug(rtgb_handle h, const rtgb_camera_rig* rig, int32_t c, uint8_t* host) {
    if (!h || !rig || !host) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (rig->active_count < 1 || rig->active_count > RTGB_MAX_CAMERAS) throw Invalid{"render_radiance requires rig.active_count in [1, 4]"};
        if (c < 0 || c >= rig->active_count) throw Invalid{"render_radiance camera_index out of range"};
        const rtgb_camera& cam = rig->cameras[c];
        if (cam.enabled == 0 || cam.width <= 0 || cam.height <= 0) throw Invalid{"render_radiance camera slot is disabled or invalid"};
        RTGB_CHECK(cudaSetDevice(h->device));
        CameraRes tmp;
        tmp.valid = false;
        // a private camera resource so the frame's camera tables stay untouched
        upload(tmp.lut, cam.equi.lut, RTGB_EQUI_LUT_SIZE, h->stream);
        tmp.dirs.ensure(static_cast<size_t>(cam.width) * cam.height * sizeof(float4));
        CameraDev d = rtgb_renderer::camera_dev(cam, 0, 0);
        d.lut = tmp.lut.as<double>();
        d.dirs = tmp.dirs.as<float4>();
        launch_camera_dirs(d, tmp.dirs.as<float4>(), h->stream);
        const size_t n = static_cast<size_t>(cam.width) * cam.height;
        h->debug_rgba.ensure(n * 4);
        launch_direction_debug(d, h->debug_rgba.as<uint8_t>(), h->stream);
        RTGB_CHECK(cudaGetLastError());
        RTGB_CHECK(cudaMemcpyAsync(host, h->debug_rgba.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        tmp.lut.release();
        tmp.dirs.release();
        return RTGB_OK;
    });
}

rtgb_status rtgb_tonemap_rgba8(rtgb_handle h, int32_t c, uint8_t* host) {
    if (!h || !host) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        h->check_camera(c);
        const size_t n = static_cast<size_t>(h->last_w[c]) * h->last_h[c];
        h->debug_rgba.ensure(n * 4);
        const FrameBufs& f = h->frames[h->last];
        const float4* src = h->last_denoised ? f.denoised : f.beauty;
        launch_tonemap(src + h->last_pixel_offset[c], h->debug_rgba.as<uint8_t>(), static_cast<long long>(n), h->stream);
        RTGB_CHECK(cudaGetLastError());
        RTGB_CHECK(cudaMemcpyAsync(host, h->debug_rgba.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        return RTGB_OK;
    });
}

rtgb_status rtgb_acceleration_info_get(rtgb_handle h, rtgb_acceleration_info* out) {
    if (!h || !out) return RTGB_INVALID_ARGUMENT;
    rtgb_acceleration_info a{};
    a.primitive_count = h->prim_count;
    a.node_count = h->scene.node_count;
    a.analytic_light_node_count = h->scene.analytic_node_count;
    a.analytic_bvh_light_count = h->analytic_bvh_count;
    a.build_ms = h->build_ms;
    a.traversal_stack_overflows = h->h_counters ? h->h_counters->overflow : 0;
    a.update_kind = h->update_kind;
    a.generation = h->generation;
    a.wide_node_count = h->scene.node4_count;
    *out = a;
    return RTGB_OK;
}

void* rtgb_stream(rtgb_handle h) { return h ? static_cast<void*>(h->stream) : nullptr; }

rtgb_status rtgb_download_path_records(rtgb_handle h, int32_t c, int32_t* codes, int32_t max_bounces, float* radiance,
    int64_t paths) {
    if (!h || !codes || !radiance) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->record || h->paths.codes == nullptr) throw Invalid{"path records need rtgb_create_info::debug_path_records"};
        h->check_camera(c);
        const long long n = static_cast<long long>(h->last_w[c]) * h->last_h[c] * h->last_spp;
        if (paths != n || max_bounces != h->last_bounces) throw Invalid{"path record shape mismatch"};
        const long long first = h->last_pixel_offset[c] * h->last_spp;
        RTGB_CHECK(cudaMemcpyAsync(codes, h->paths.codes + first * max_bounces, static_cast<size_t>(n) * max_bounces * 4,
            cudaMemcpyDeviceToHost, h->stream));
        std::vector<float4> rad(static_cast<size_t>(n));
        RTGB_CHECK(cudaMemcpyAsync(rad.data(), h->paths.rad + first, static_cast<size_t>(n) * 16, cudaMemcpyDeviceToHost, h->stream));
        RTGB_CHECK(cudaStreamSynchronize(h->stream));
        for (long long i = 0; i < n; ++i) {
            radiance[3 * i] = rad[static_cast<size_t>(i)].x;
            radiance[3 * i + 1] = rad[static_cast<size_t>(i)].y;
            radiance[3 * i + 2] = rad[static_cast<size_t>(i)].z;
        }
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_lbvh(rtgb_handle h, uint32_t* sorted_morton, int32_t* sorted_primitive, int32_t* children) {
    if (!h) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->prepared) throw Invalid{"no scene prepared"};
        const int n = h->prim_count;
        if (n < 2) throw Invalid{"the scene has fewer than two primitives and no hierarchy"};
        if (sorted_morton) RTGB_CHECK(cudaMemcpy(sorted_morton, h->sorted_keys.p, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost));
        if (sorted_primitive) RTGB_CHECK(cudaMemcpy(sorted_primitive, h->sorted_vals.p, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost));
        if (children) {
            std::vector<BvhNode> nodes(static_cast<size_t>(n - 1));
            RTGB_CHECK(cudaMemcpy(nodes.data(), h->nodes.p, nodes.size() * sizeof(BvhNode), cudaMemcpyDeviceToHost));
            for (int i = 0; i < n - 1; ++i) {
                int c0, c1;
                std::memcpy(&c0, &nodes[static_cast<size_t>(i)].a.w, 4);
                std::memcpy(&c1, &nodes[static_cast<size_t>(i)].b.w, 4);
                children[2 * i] = c0;
                children[2 * i + 1] = c1;
            }
        }
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_bvh4(rtgb_handle h, int32_t* children, float* child_boxes) {
    if (!h || !children || !child_boxes) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->prepared) throw Invalid{"no scene prepared"};
        const int n4 = h->scene.node4_count;
        if (n4 <= 0) throw Invalid{"the scene has fewer than two primitives and no hierarchy"};
        std::vector<float4> q(static_cast<size_t>(n4) * kNode4);
        RTGB_CHECK(cudaMemcpy(q.data(), h->scene.nodes4, q.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        for (int i = 0; i < n4; ++i) {
            const float4* n = q.data() + static_cast<size_t>(i) * kNode4;
            for (int k = 0; k < 6; ++k) {
                const float v[4] = {n[k].x, n[k].y, n[k].z, n[k].w};
                for (int c = 0; c < 4; ++c) child_boxes[24 * static_cast<size_t>(i) + 4 * k + c] = v[c];
            }
            const float w[4] = {n[6].x, n[6].y, n[6].z, n[6].w};
            std::memcpy(children + 4 * static_cast<size_t>(i), w, sizeof w);
        }
        return RTGB_OK;
    });
}

rtgb_status rtgb_download_lbvh_boxes(rtgb_handle h, float* child_boxes) {
    if (!h || !child_boxes) return RTGB_INVALID_ARGUMENT;
    return guarded(h, [&] {
        if (!h->prepared) throw Invalid{"no scene prepared"};
        const int n = h->prim_count;
        if (n < 2) throw Invalid{"the scene has fewer than two primitives and no hierarchy"};
        std::vector<BvhNode> nodes(static_cast<size_t>(n - 1));
        RTGB_CHECK(cudaMemcpy(nodes.data(), h->nodes.p, nodes.size() * sizeof(BvhNode), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nodes.size(); ++i) {
            const float4 q[4] = {nodes[i].a, nodes[i].b, nodes[i].c, nodes[i].d};
            for (int k = 0; k < 4; ++k) {
                child_boxes[12 * i + 3 * k] = q[k].x;
                child_boxes[12 * i + 3 * k + 1] = q[k].y;
                child_boxes[12 * i + 3 * k + 2] = q[k].z;
            }
        }
        return RTGB_OK;
    });
}

}  // extern "C"
