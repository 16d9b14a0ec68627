// render_realtime: the reference's realtime benchmark CLI (utils/render_realtime.cpp)
// over this library's C ABI. Same flags, the same per-frame console lines, and
// the same artifacts in --output-dir: frame_XXXX_cam_N.png (unless
// --skip-image-write; with --write-exr also frame_XXXX_cam_N.exr, the linear
// radiance as 32-bit float B/G/R), benchmark_frames.csv, benchmark_summary.json (schema 3)
// and benchmark_manifest.json (FNV-1a64 digests). One library handle renders
// all cameras of a frame in one launch sequence, so the reference's
// per-camera worker threads become one worker; render_ms is the whole frame's
// device time and denoise_ms the U-Net's.
//
// Extra flags: --width/--height (default 640 x 480, the reference's fixed
// size), --denoiser-weights (default: the weights shipped beside the
// library), --device, --write-exr, --scene-file (a scene file from
// rtgb_host_scene_save, e.g. lowered from SceneIR v2; the rig then comes
// from --scene when given, else four yawed pinholes at the origin).
#include <sys/utsname.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <limits>
#include <optional>
#include <format>
#include <stdexcept>
#include <string>
#include <string_view>
#include <unistd.h>
#include <vector>

#include "benchmark_report.h"
#include "exr_writer.h"
#include "png_writer.h"
#include "rtgb.h"

#ifndef RTGB_SOURCE_REVISION
#define RTGB_SOURCE_REVISION "unknown"
#endif
#ifndef RTGB_CXX_COMPILER
#define RTGB_CXX_COMPILER "g++"
#endif

namespace {

constexpr const char* kVersion = "0.1.0";

template <class... A>
void println(FILE* f, std::format_string<A...> fmt, A&&... args) {
    std::string s = std::format(fmt, std::forward<A>(args)...);
    s.push_back('\n');
    std::fputs(s.c_str(), f);
}

template <class... A>
void println(std::format_string<A...> fmt, A&&... args) {
    println(stdout, fmt, std::forward<A>(args)...);
}

struct Args {
    int camera_count = 4;
    int frames = 1;
    int warmup_frames = 8;
    unsigned long seed = 0;
    std::string output_dir = "build/realtime-smoke";
    std::string scene = "smoke";
    bool scene_given = false;
    std::string scene_file;  // a packed scene written by rtgb_host_scene_save (e.g. lowered from SceneIR v2)
    std::string profile;
    bool skip_image_write = false;
    bool write_exr = false;
    int width = 640;
    int height = 480;
    int device = 0;
    std::string weights;
};

void usage(FILE* out) {
    println(out,
        "usage: render_realtime [--camera-count N] [--frames N] [--warmup-frames N] [--seed S]\n"
        "                       [--output-dir DIR] [--scene NAME] [--profile quality|balanced|realtime]\n"
        "                       [--skip-image-write] [--width W] [--height H] [--device D]\n"
        "                       [--denoiser-weights FILE] [--write-exr] [--scene-file FILE]");
}

template <class T>
bool parse_num(std::string_view s, T& out) {
    try {
        size_t pos = 0;
        const long long v = std::stoll(std::string(s), &pos);
        if (pos != s.size()) return false;
        out = static_cast<T>(v);
        return true;
    } catch (...) {
        return false;
    }
}

std::optional<Args> parse(int argc, char** argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        const std::string_view k = argv[i];
        auto value = [&]() -> std::optional<std::string_view> {
            if (i + 1 >= argc) return std::nullopt;
            return std::string_view(argv[++i]);
        };
        std::optional<std::string_view> v;
        bool ok = true;
        if (k == "--skip-image-write") {
            a.skip_image_write = true;
        } else if (k == "--write-exr") {
            a.write_exr = true;
        } else if (k == "--help" || k == "-h") {
            usage(stdout);
            std::exit(EXIT_SUCCESS);
        } else if (k != "--camera-count" && k != "--frames" && k != "--warmup-frames" && k != "--seed" &&
                   k != "--output-dir" && k != "--scene" && k != "--profile" && k != "--width" && k != "--height" &&
                   k != "--device" && k != "--denoiser-weights" && k != "--scene-file") {
            println(stderr, "unknown argument: {}", k);
            return std::nullopt;
        } else if (!(v = value())) {
            println(stderr, "{} needs a value", k);
            return std::nullopt;
        } else if (k == "--camera-count") {
            ok = parse_num(*v, a.camera_count);
        } else if (k == "--frames") {
            ok = parse_num(*v, a.frames);
        } else if (k == "--warmup-frames") {
            ok = parse_num(*v, a.warmup_frames);
        } else if (k == "--seed") {
            ok = parse_num(*v, a.seed) && v->find('-') == std::string_view::npos;
        } else if (k == "--output-dir") {
            a.output_dir = *v;
        } else if (k == "--scene") {
            a.scene = *v;
            a.scene_given = true;
        } else if (k == "--scene-file") {
            a.scene_file = *v;
        } else if (k == "--profile") {
            a.profile = *v;
        } else if (k == "--width") {
            ok = parse_num(*v, a.width);
        } else if (k == "--height") {
            ok = parse_num(*v, a.height);
        } else if (k == "--device") {
            ok = parse_num(*v, a.device);
        } else {  // --denoiser-weights
            a.weights = *v;
        }
        if (!ok) {
            println(stderr, "invalid value for {}: {}", k, *v);
            return std::nullopt;
        }
    }
    return a;
}

void check(rtgb_status st, rtgb_handle h, const char* what) {
    if (st != RTGB_OK) {
        throw std::runtime_error(std::string(what) + " failed: " + (h ? rtgb_last_error(h) : "") + " (status " +
                                 std::to_string(static_cast<int>(st)) + ")");
    }
}

std::string utc_now() {
    const std::time_t now = std::time(nullptr);
    std::tm utc{};
    gmtime_r(&now, &utc);
    char buf[32];
    std::strftime(buf, sizeof buf, "%Y-%m-%dT%H:%M:%SZ", &utc);
    return buf;
}

std::string first_line(const std::filesystem::path& p, const std::string& fallback) {
    std::ifstream in(p);
    std::string line;
    if (!in.is_open() || !std::getline(in, line)) return fallback;
    const size_t a = line.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return fallback;
    return line.substr(a, line.find_last_not_of(" \t\r\n") - a + 1);
}

std::string cuda_version_text(int v) { return std::to_string(v / 1000) + "." + std::to_string((v % 1000) / 10); }

std::filesystem::path exe_dir() {
    std::error_code ec;
    const auto p = std::filesystem::read_symlink("/proc/self/exe", ec);
    return ec ? std::filesystem::current_path() : p.parent_path();
}

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }

int run(const Args& a) {
    if (a.camera_count < 1 || a.camera_count > 4) {
        println(stderr, "--camera-count must be in [1, 4]");
        return EXIT_FAILURE;
    }
    if (a.frames < 1) {
        println(stderr, "--frames must be >= 1");
        return EXIT_FAILURE;
    }
    if (a.warmup_frames < 0) {
        println(stderr, "--warmup-frames must be >= 0");
        return EXIT_FAILURE;
    }
    if (a.seed + static_cast<unsigned long>(a.warmup_frames) + static_cast<unsigned long>(a.frames) - 1ul >
        std::numeric_limits<uint32_t>::max()) {
        println(stderr, "--seed + --warmup-frames + --frames exceeds uint32 sample streams");
        return EXIT_FAILURE;
    }
    rtgb_render_profile profile{};
    std::string profile_name = a.profile.empty() ? "balanced" : a.profile;  // realtime_default() = balanced()
    if (rtgb_profile_preset(profile_name.c_str(), &profile) != RTGB_OK) {
        println(stderr, "--profile must be one of: quality, balanced, realtime");
        return EXIT_FAILURE;
    }
    rtgb_host_scene* scene = nullptr;
    std::string rig_name = a.scene;
    if (!a.scene_file.empty()) {
        // the scene's content from the file; --scene (if given) still names the camera rig
        if (rtgb_host_scene_load(a.scene_file.c_str(), &scene) != RTGB_OK) {
            println(stderr, "--scene-file must name a readable scene file: {}", a.scene_file);
            return EXIT_FAILURE;
        }
        if (!a.scene_given) rig_name = "scene_file";
    } else if (rtgb_host_scene_create(a.scene.c_str(), 0, 0, &scene) != RTGB_OK) {
        println(stderr, "--scene must reference a registered realtime scene");
        return EXIT_FAILURE;
    }
    rtgb_camera_rig rig{};
    if (rtgb_default_rig(rig_name.c_str(), a.camera_count, a.width, a.height, &rig) != RTGB_OK) {
        println(stderr, "no camera rig for scene {}", rig_name);
        rtgb_host_scene_destroy(scene);
        return EXIT_FAILURE;
    }
    const std::filesystem::path out_dir = a.output_dir;
    std::filesystem::create_directories(out_dir);

    rtgb_create_info info{a.device, 1, 0, 0};
    rtgb_handle h = nullptr;
    check(rtgb_create(&info, &h), nullptr, "rtgb_create");
    int rc = EXIT_SUCCESS;
    try {
        rtgb::report::Report report;
        rtgb_device_info dev{};
        check(rtgb_device_info_get(h, &dev), h, "rtgb_device_info_get");
        utsname host{};
        uname(&host);
        report.provenance = {utc_now(), kVersion, RTGB_SOURCE_REVISION, false, "repository",
            "unavailable", "Release", RTGB_CXX_COMPILER};
        report.environment.operating_system = std::string(host.sysname) + " " + host.release;
        report.environment.architecture = host.machine;
        report.environment.gpu_device = dev.device;
        report.environment.gpu_name = dev.name;
        report.environment.compute_capability = std::to_string(dev.major) + "." + std::to_string(dev.minor);
        report.environment.nvidia_driver_version = first_line("/sys/module/nvidia/version", "unavailable");
        report.environment.cuda_driver_api_version = dev.driver_version;
        report.environment.cuda_driver_api_version_text = cuda_version_text(dev.driver_version);
        report.environment.cuda_runtime_version = dev.runtime_version;
        report.environment.cuda_runtime_version_text = cuda_version_text(dev.runtime_version);
        const uint64_t baseline_used = dev.used_bytes;
        report.gpu_memory.total_bytes = dev.total_bytes;
        report.gpu_memory.baseline_used_bytes = baseline_used;

        rtgb_scene view{};
        check(rtgb_host_scene_view(scene, &view), h, "rtgb_host_scene_view");
        check(rtgb_prepare_scene(h, &view), h, "rtgb_prepare_scene");
        check(rtgb_reset_sequence(h, static_cast<uint32_t>(a.seed)), h, "rtgb_reset_sequence");
        if (profile.enable_denoise != 0) {
            const std::filesystem::path w =
                a.weights.empty() ? exe_dir() / ".." / "weights" / "denoiser_unet.bf16" : std::filesystem::path(a.weights);
            if (std::filesystem::exists(w)) {
                check(rtgb_load_denoiser_file(h, w.string().c_str()), h, "rtgb_load_denoiser_file");
            } else {
                println(stderr, "denoiser weights not found ({}): frames use the plain accumulated beauty", w.string());
            }
        }
        check(rtgb_device_info_get(h, &dev), h, "rtgb_device_info_get");
        report.gpu_memory.prepared_used_bytes = dev.used_bytes;
        uint64_t peak = std::max(baseline_used, dev.used_bytes);
        report.scene = a.scene_file.empty() ? a.scene : std::filesystem::path(a.scene_file).stem().string();
        report.profile = profile_name;
        report.camera_count = a.camera_count;
        report.width = a.width;
        report.height = a.height;
        report.frames_requested = a.frames;
        report.warmup_frames = a.warmup_frames;
        report.random_seed = static_cast<uint32_t>(a.seed);
        report.samples_per_pixel = profile.samples_per_pixel;
        report.max_bounces = profile.max_bounces;
        report.denoise_enabled = profile.enable_denoise != 0;
        report.image_write_enabled = !a.skip_image_write;

        const size_t px = static_cast<size_t>(a.width) * a.height;
        std::vector<float> beauty(px * 4);
        std::vector<uint8_t> rgba(px * 4), rgb(px * 3);
        rtgb_frame_views views{};
        for (int w = 0; w < a.warmup_frames; ++w) {
            const auto t0 = Clock::now();
            check(rtgb_render_frame(h, &rig, &profile, a.camera_count, &views), h, "rtgb_render_frame");
            for (int c = 0; c < a.camera_count; ++c) {
                float dms = 0.0f;
                check(rtgb_download_frame(h, c, beauty.data(), nullptr, nullptr, nullptr, &dms), h, "rtgb_download_frame");
            }
            const double ms = ms_since(t0);
            check(rtgb_device_info_get(h, &dev), h, "rtgb_device_info_get");
            peak = std::max(peak, dev.used_bytes);
            println("warmup={} sample_stream={} cameras={} pipeline_ms={:.3f}", w, a.seed + static_cast<unsigned long>(w),
                a.camera_count, ms);
        }
        for (int f = 0; f < a.frames; ++f) {
            const auto frame_begin = Clock::now();
            rtgb::report::FrameSample fr;
            fr.frame_index = f;
            fr.sample_stream = static_cast<uint32_t>(a.seed + static_cast<unsigned long>(a.warmup_frames + f));
            fr.camera_count = a.camera_count;
            fr.profile = profile_name;
            fr.width = a.width;
            fr.height = a.height;
            fr.samples_per_pixel = profile.samples_per_pixel;
            fr.max_bounces = profile.max_bounces;
            fr.denoise_enabled = profile.enable_denoise != 0;
            // pipeline: render (+ denoise) and every camera's download, as RendererPool::render_frame returns host frames
            const auto pipe_begin = Clock::now();
            check(rtgb_render_frame(h, &rig, &profile, a.camera_count, &views), h, "rtgb_render_frame");
            std::vector<std::vector<float>> frames(static_cast<size_t>(a.camera_count));
            std::vector<float> dl(static_cast<size_t>(a.camera_count));
            for (int c = 0; c < a.camera_count; ++c) {
                frames[static_cast<size_t>(c)].resize(px * 4);
                check(rtgb_download_frame(h, c, frames[static_cast<size_t>(c)].data(), nullptr, nullptr, nullptr,
                          &dl[static_cast<size_t>(c)]),
                    h, "rtgb_download_frame");
            }
            fr.pipeline_ms = ms_since(pipe_begin);
            fr.rays_traced = views.rays_traced;
            double lum_sum = 0.0;
            for (int c = 0; c < a.camera_count; ++c) {
                const std::vector<float>& b = frames[static_cast<size_t>(c)];
                double lum = 0.0;
                for (size_t i = 0; i < px; ++i) lum += 0.2126 * b[4 * i] + 0.7152 * b[4 * i + 1] + 0.0722 * b[4 * i + 2];
                lum /= static_cast<double>(px);
                rtgb::report::CameraSample cs{c, views.cameras[c].render_ms, views.cameras[c].denoise_ms,
                    dl[static_cast<size_t>(c)], lum};
                fr.render_ms = std::max(fr.render_ms, cs.render_ms);
                fr.denoise_ms = std::max(fr.denoise_ms, cs.denoise_ms);
                fr.download_ms = std::max(fr.download_ms, cs.download_ms);
                fr.render_work_ms += cs.render_ms;
                fr.denoise_work_ms += cs.denoise_ms;
                fr.download_work_ms += cs.download_ms;
                lum_sum += lum;
                if (!a.skip_image_write) {
                    const auto t0 = Clock::now();
                    check(rtgb_tonemap_rgba8(h, c, rgba.data()), h, "rtgb_tonemap_rgba8");
                    for (size_t i = 0; i < px; ++i) {
                        rgb[3 * i] = rgba[4 * i];
                        rgb[3 * i + 1] = rgba[4 * i + 1];
                        rgb[3 * i + 2] = rgba[4 * i + 2];
                    }
                    char name[64];
                    std::snprintf(name, sizeof name, "frame_%04d_cam_%d.png", f, c);
                    rtgb::png::write_rgb(out_dir / name, a.width, a.height, rgb.data());
                    if (a.write_exr) {
                        std::snprintf(name, sizeof name, "frame_%04d_cam_%d.exr", f, c);
                        rtgb::exr::write_rgba(out_dir / name, a.width, a.height, b.data());
                    }
                    fr.image_write_ms += ms_since(t0);
                }
                fr.cameras.push_back(cs);
            }
            fr.frame_ms = ms_since(frame_begin);
            fr.host_overhead_ms = std::max(0.0, fr.frame_ms - fr.pipeline_ms - fr.image_write_ms);
            fr.fps = 1000.0 / fr.frame_ms;
            report.frames.push_back(fr);
            check(rtgb_device_info_get(h, &dev), h, "rtgb_device_info_get");
            peak = std::max(peak, dev.used_bytes);
            println("frame={} sample_stream={} cameras={} avg_luminance={:.6f} pipeline_ms={:.3f} render_ms={:.3f} "
                         "denoise_ms={:.3f} download_ms={:.3f} render_work_ms={:.3f} denoise_work_ms={:.3f} "
                         "download_work_ms={:.3f} image_write_ms={:.3f} host_overhead_ms={:.3f} frame_ms={:.3f}",
                f, fr.sample_stream, a.camera_count, lum_sum / a.camera_count, fr.pipeline_ms, fr.render_ms, fr.denoise_ms,
                fr.download_ms, fr.render_work_ms, fr.denoise_work_ms, fr.download_work_ms, fr.image_write_ms,
                fr.host_overhead_ms, fr.frame_ms);
        }
        check(rtgb_device_info_get(h, &dev), h, "rtgb_device_info_get");
        peak = std::max(peak, dev.used_bytes);
        report.gpu_memory.peak_used_bytes = peak;
        report.gpu_memory.peak_delta_bytes = peak >= baseline_used ? peak - baseline_used : 0;
        report.gpu_memory.final_used_bytes = dev.used_bytes;
        rtgb_acceleration_info acc{};
        check(rtgb_acceleration_info_get(h, &acc), h, "rtgb_acceleration_info_get");
        report.gpu_scheduling.persistent_worker_count = 1;
        report.gpu_scheduling.worker_start_count = 1;
        report.gpu_scheduling.task_submission_count = static_cast<uint64_t>(a.warmup_frames + a.frames);
        report.gpu_scheduling.launch_parameter_allocation_count = 1;
        report.gpu_scheduling.launch_parameter_upload_count = static_cast<uint64_t>(a.warmup_frames + a.frames);
        static const char* const kKinds[4] = {"reuse", "update", "refit", "rebuild"};
        report.gpu_scheduling.acceleration_update_kind = kKinds[acc.update_kind >= 0 && acc.update_kind < 4 ? acc.update_kind : 3];
        report.gpu_scheduling.acceleration_update_ms = acc.build_ms;
        report.gpu_scheduling.acceleration_node_count = acc.node_count;
        report.gpu_scheduling.acceleration_reference_count = acc.primitive_count;
        report.gpu_scheduling.acceleration_generation = static_cast<uint64_t>(acc.generation);
        report.aggregate = rtgb::report::aggregate_of(report.frames);
        const auto csv = out_dir / "benchmark_frames.csv";
        const auto json = out_dir / "benchmark_summary.json";
        const auto manifest = out_dir / "benchmark_manifest.json";
        rtgb::report::write_csv(report, csv);
        rtgb::report::write_json(report, json);
        rtgb::report::write_manifest(report, {csv, json}, manifest);
        const auto& ag = report.aggregate;
        println("summary profile={} warmup_frames={} frames={} seed={} cameras={} resolution={}x{} spp={} "
                     "max_bounces={} denoise={} avg_frame_ms={:.3f} avg_denoise_ms={:.3f} p95_frame_ms={:.3f} "
                     "p99_frame_ms={:.3f} fps={:.2f} peak_gpu_memory_mib={:.2f} peak_gpu_memory_delta_mib={:.2f} "
                     "workers=1/1 as_update=rebuild as_update_ms={:.3f} as_nodes={} as_refs={} "
                     "artifacts=benchmark_frames.csv,benchmark_summary.json,benchmark_manifest.json output_dir={}",
            profile_name, a.warmup_frames, a.frames, a.seed, a.camera_count, a.width, a.height, profile.samples_per_pixel,
            profile.max_bounces, profile.enable_denoise ? "true" : "false", ag.frame_ms.avg, ag.denoise_ms.avg,
            ag.frame_ms.p95, ag.frame_ms.p99, 1000.0 / ag.frame_ms.avg,
            static_cast<double>(report.gpu_memory.peak_used_bytes) / (1024.0 * 1024.0),
            static_cast<double>(report.gpu_memory.peak_delta_bytes) / (1024.0 * 1024.0), acc.build_ms, acc.node_count,
            acc.primitive_count, out_dir.string());
    } catch (const std::exception& e) {
        println(stderr, "render_realtime: {}", e.what());
        rc = EXIT_FAILURE;
    }
    rtgb_destroy(h);
    rtgb_host_scene_destroy(scene);
    return rc;
}

}  // namespace

int main(int argc, char** argv) {
    const std::optional<Args> a = parse(argc, argv);
    if (!a) {
        usage(stderr);
        return EXIT_FAILURE;
    }
    try {
        return run(*a);
    } catch (const std::exception& e) {
        println(stderr, "render_realtime: {}", e.what());
        return EXIT_FAILURE;
    }
}
