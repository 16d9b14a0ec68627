// C++23 call surface of the reference's realtime renderer over the C ABI
// (header only): OptixRenderer (src/realtime/gpu/optix_renderer.h:69-128) and
// RendererPool (src/realtime/gpu/renderer_pool.h:30-53) with their frame
// types (frame_types.h:9-22), so C++ callers of the reference switch by
// changing the namespace and the scene type. Failures throw what the
// reference throws, with the handle's rtgb_last_error as the message:
// std::runtime_error for a rejected render request (active camera count, rig
// slots, camera index: validate_render_pool_request and
// validate_render_camera_request, src/realtime/gpu/render_request_validation.cpp:15-62)
// and for CUDA failures; std::invalid_argument where the reference uses it,
// for a scene without surfaces (gpu_scene_acceleration.cpp:335) and a bad
// denoiser input.
//
// One handle renders all cameras of a frame in one launch sequence, so the
// pool's N renderers are one handle here; RendererPool(n) only bounds the
// active camera count as the reference's constructor does (1..4).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rtgb.h"

namespace rtgb {

struct DirectionDebugFrame {
    int width = 0;
    int height = 0;
    std::vector<std::uint8_t> rgba;
};

struct RadianceFrame {
    int width = 0;
    int height = 0;
    double average_luminance = 0.0;
    std::vector<float> beauty_rgba;
    std::vector<float> normal_rgba;
    std::vector<float> albedo_rgba;
    std::vector<float> depth;
};

struct RadianceTiming {
    double render_ms = 0.0;
    double denoise_ms = 0.0;
    double download_ms = 0.0;
};

struct ProfiledRadianceFrame {
    RadianceFrame frame;
    RadianceTiming timing;
};

// Device view of one camera's beauty (valid until the next launch on the renderer).
struct ProfiledDeviceRadianceFrame {
    const void* beauty = nullptr;  // float4 per pixel, device memory
    int width = 0;
    int height = 0;
    RadianceTiming timing;
};

struct CameraRenderResult {
    int camera_index = 0;
    RadianceFrame frame;
    RadianceTiming timing;
};

struct CameraDeviceRenderResult {
    int camera_index = 0;
    ProfiledDeviceRadianceFrame frame;
};

namespace detail {

inline std::string message(rtgb_handle h, const char* what) {
    std::string msg = what;
    if (h) {
        const char* e = rtgb_last_error(h);
        if (e && *e) msg += std::string(": ") + e;
    }
    return msg;
}

// Scene and set-up calls: a rejected argument is std::invalid_argument.
inline void check(rtgb_status st, rtgb_handle h, const char* what) {
    if (st == RTGB_OK) return;
    if (st == RTGB_INVALID_ARGUMENT) throw std::invalid_argument(message(h, what));
    throw std::runtime_error(message(h, what));
}

// Render requests: the reference's request validation throws std::runtime_error.
inline void check_request(rtgb_status st, rtgb_handle h, const char* what) {
    if (st != RTGB_OK) throw std::runtime_error(message(h, what));
}

inline double luminance(const std::vector<float>& rgba) {
    const size_t n = rgba.size() / 4;
    double sum = 0.0;
    for (size_t i = 0; i < n; ++i) sum += 0.2126 * rgba[4 * i] + 0.7152 * rgba[4 * i + 1] + 0.0722 * rgba[4 * i + 2];
    return n ? sum / static_cast<double>(n) : 0.0;
}

}  // namespace detail

class OptixRenderer {
public:
    explicit OptixRenderer(int device = 0) {
        rtgb_create_info info {};
        info.device = device;
        info.use_cuda_graph = 1;
        detail::check(rtgb_create(&info, &h_), nullptr, "rtgb_create");
    }
    ~OptixRenderer() { rtgb_destroy(h_); }
    OptixRenderer(const OptixRenderer&) = delete;
    OptixRenderer& operator=(const OptixRenderer&) = delete;

    rtgb_handle handle() const { return h_; }

    void prepare_scene(const rtgb_scene& scene) { detail::check(rtgb_prepare_scene(h_, &scene), h_, "prepare_scene"); }
    // use_prepared_scene: the prepare step reuses an unchanged scene (acceleration kind "reuse")
    void use_prepared_scene(const rtgb_scene& scene) { prepare_scene(scene); }
    void reset_accumulation() { detail::check(rtgb_reset_accumulation(h_), h_, "reset_accumulation"); }
    void reset_sequence(std::uint32_t sample_stream) {
        detail::check(rtgb_reset_sequence(h_, sample_stream), h_, "reset_sequence");
    }

    rtgb_restir_stats restir_diagnostics(int camera_index = 0) const {
        rtgb_restir_stats s {};
        detail::check_request(rtgb_restir_diagnostics(h_, camera_index, &s), h_, "restir_diagnostics");
        return s;
    }
    rtgb_acceleration_info acceleration_diagnostics() const {
        rtgb_acceleration_info a {};
        detail::check(rtgb_acceleration_info_get(h_, &a), h_, "acceleration_diagnostics");
        return a;
    }

    DirectionDebugFrame render_direction_debug(const rtgb_camera_rig& rig, int camera_index = 0) {
        if (camera_index < 0 || camera_index >= RTGB_MAX_CAMERAS) {
            throw std::runtime_error("render_direction_debug camera_index out of range");
        }
        DirectionDebugFrame f;
        f.width = rig.cameras[camera_index].width;
        f.height = rig.cameras[camera_index].height;
        f.rgba.resize(static_cast<size_t>(f.width) * static_cast<size_t>(f.height) * 4);
        detail::check_request(rtgb_render_direction_debug(h_, &rig, camera_index, f.rgba.data()), h_,
            "render_direction_debug");
        return f;
    }

    // render_prepared_radiance: renders the rig's cameras up to camera_index
    // and downloads that camera
    ProfiledRadianceFrame render_prepared_radiance(const rtgb_camera_rig& rig, const rtgb_render_profile& profile,
        int camera_index) {
        const rtgb_frame_views v = render(rig, profile, camera_index + 1);
        return download(v, camera_index);
    }
    ProfiledDeviceRadianceFrame render_prepared_device(const rtgb_camera_rig& rig, const rtgb_render_profile& profile,
        int camera_index) {
        const rtgb_frame_views v = render(rig, profile, camera_index + 1);
        return device_view(v, camera_index);
    }
    RadianceFrame render_radiance(const rtgb_scene& scene, const rtgb_camera_rig& rig, const rtgb_render_profile& profile,
        int camera_index) {
        prepare_scene(scene);
        return render_prepared_radiance(rig, profile, camera_index).frame;
    }
    ProfiledRadianceFrame render_radiance_profiled(const rtgb_scene& scene, const rtgb_camera_rig& rig,
        const rtgb_render_profile& profile, int camera_index) {
        prepare_scene(scene);
        return render_prepared_radiance(rig, profile, camera_index);
    }

    // every active camera of one frame (RendererPool::render_frame's work)
    rtgb_frame_views render(const rtgb_camera_rig& rig, const rtgb_render_profile& profile, int active) {
        rtgb_frame_views v {};
        detail::check_request(rtgb_render_frame(h_, &rig, &profile, active, &v), h_, "render_frame");
        return v;
    }
    ProfiledRadianceFrame download(const rtgb_frame_views& v, int camera_index) {
        if (camera_index < 0 || camera_index >= v.camera_count) throw std::runtime_error("camera_index out of range");
        const rtgb_camera_frame_view& c = v.cameras[camera_index];
        ProfiledRadianceFrame out;
        RadianceFrame& f = out.frame;
        f.width = c.width;
        f.height = c.height;
        const size_t px = static_cast<size_t>(c.width) * static_cast<size_t>(c.height);
        f.beauty_rgba.resize(px * 4);
        f.normal_rgba.resize(px * 4);
        f.albedo_rgba.resize(px * 4);
        f.depth.resize(px);
        float dl = 0.0f;
        detail::check_request(rtgb_download_frame(h_, camera_index, f.beauty_rgba.data(), f.normal_rgba.data(),
                                  f.albedo_rgba.data(), f.depth.data(), &dl),
            h_, "download_frame");
        f.average_luminance = detail::luminance(f.beauty_rgba);
        out.timing = {c.render_ms, c.denoise_ms, dl};
        return out;
    }
    ProfiledDeviceRadianceFrame device_view(const rtgb_frame_views& v, int camera_index) const {
        if (camera_index < 0 || camera_index >= v.camera_count) throw std::runtime_error("camera_index out of range");
        const rtgb_camera_frame_view& c = v.cameras[camera_index];
        return {c.beauty, c.width, c.height, {c.render_ms, c.denoise_ms, 0.0}};
    }

private:
    rtgb_handle h_ = nullptr;
};

class RendererPool {
public:
    explicit RendererPool(int renderer_count, int device = 0) : count_(renderer_count), renderer_(checked(renderer_count, device)) {}
    RendererPool(const RendererPool&) = delete;
    RendererPool& operator=(const RendererPool&) = delete;

    void prepare_scene(const rtgb_scene& scene) { renderer_.prepare_scene(scene); }
    void reset_accumulation() { renderer_.reset_accumulation(); }
    void reset_sequence(std::uint32_t sample_stream) { renderer_.reset_sequence(sample_stream); }

    std::vector<CameraRenderResult> render_frame(const rtgb_camera_rig& rig, const rtgb_render_profile& profile,
        int active_cameras) {
        require_active(active_cameras);
        const rtgb_frame_views v = renderer_.render(rig, profile, active_cameras);
        std::vector<CameraRenderResult> out;
        for (int c = 0; c < active_cameras; ++c) {
            ProfiledRadianceFrame f = renderer_.download(v, c);
            out.push_back({c, std::move(f.frame), f.timing});
        }
        return out;  // sorted by camera_index, as the reference returns them
    }
    std::vector<CameraDeviceRenderResult> render_device_frame(const rtgb_camera_rig& rig, const rtgb_render_profile& profile,
        int active_cameras) {
        require_active(active_cameras);
        const rtgb_frame_views v = renderer_.render(rig, profile, active_cameras);
        std::vector<CameraDeviceRenderResult> out;
        for (int c = 0; c < active_cameras; ++c) out.push_back({c, renderer_.device_view(v, c)});
        return out;
    }
    OptixRenderer& renderer() { return renderer_; }

private:
    static int checked(int n, int device) {
        // renderer_pool.cpp:112-114 throws runtime_error for this
        if (n < 1 || n > RTGB_MAX_CAMERAS) throw std::runtime_error("RendererPool requires renderer_count in [1, 4]");
        return device;
    }
    void require_active(int active) const {
        // validate_render_pool_request (render_request_validation.cpp:43-46)
        if (active < 1 || active > count_) throw std::runtime_error("RendererPool::render_frame active_cameras out of range");
    }
    int count_;
    OptixRenderer renderer_;
};

}  // namespace rtgb
