// render_restir_acceptance: the reference's ReSTIR DI acceptance harness
// (utils/render_restir_acceptance.cpp) over this library's C ABI. It renders
// the acceptance scene (128 x 128 pinhole, 64 point lights, one bounce) as a
// 256-spp plain reference, a 16-spp plain baseline and a 2-frame 1-spp ReSTIR
// DI sequence (temporal + spatial reuse, BASIC bias correction), checks the
// reference's gates and writes reference.png, baseline.png, restir.png and
// report.json (schema restir_di_acceptance_v2) into --output-dir:
//   * quality: ReSTIR's MSE against the reference <= the baseline's (or, with
//     --expect-quality-rejected, the opposite);
//   * performance: over 5 trials ReSTIR's render time beats the baseline's on
//     average and in at least 3 trials;
//   * temporal / spatial / bias correction: no reuse on the first frame, reuse
//     on the second, none again after prepare_scene resets the history;
//   * reference gate: every written PNG within 2 display levels of the same
//     image in --reference-dir (--approve-references copies them there first).
// Exit status 0 when every gate passes, 1 otherwise (the reference throws).
// Extra flag: --device.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "png_reader.h"
#include "png_writer.h"
#include "rtgb.h"

namespace {

constexpr int kReferenceSpp = 256;
constexpr int kBaselineSpp = 16;
constexpr int kRestirFrames = 2;
constexpr int kRestirCandidates = 8;
constexpr int kPerformanceTrials = 5;
constexpr int kLightCount = 64;
constexpr double kQualityRatioLimit = 1.0;

void check(rtgb_status st, rtgb_handle h, const char* what) {
    if (st != RTGB_OK) throw std::runtime_error(std::string(what) + ": " + (h ? rtgb_last_error(h) : "failed"));
}

// make_profile (render_restir_acceptance.cpp:101-118)
rtgb_render_profile make_profile(int spp, bool restir, int spatial) {
    rtgb_render_profile p{};
    check(rtgb_profile_preset("realtime", &p), nullptr, "rtgb_profile_preset");
    p.samples_per_pixel = spp;
    p.max_bounces = 1;
    p.rr_start_bounce = 2;
    p.enable_denoise = 0;
    p.enable_restir_di = restir ? 1 : 0;
    p.restir_initial_candidates = kRestirCandidates;
    p.restir_temporal_reuse = restir ? 1 : 0;
    p.restir_max_history_age = 20;
    p.restir_max_temporal_candidates = 64;
    p.restir_spatial_neighbors = restir ? spatial : 0;
    p.restir_max_spatial_candidates = kRestirCandidates;
    p.restir_bias_correction = 1;
    p.restir_min_analytic_lights = 16;
    return p;
}

struct Frame {
    int width = 0, height = 0;
    std::vector<float> beauty;  // RGBA
    double render_ms = 0.0;
};

struct Handle {
    rtgb_handle h = nullptr;
    explicit Handle(int device) {
        rtgb_create_info ci{};
        ci.device = device;
        ci.use_cuda_graph = 1;
        check(rtgb_create(&ci, &h), nullptr, "rtgb_create");
    }
    ~Handle() { rtgb_destroy(h); }
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;
};

// renders `frames` frames on a prepared handle; the last frame's beauty and the summed render time
Frame render(Handle& r, const rtgb_camera_rig& rig, const rtgb_render_profile& prof, int frames) {
    Frame f;
    for (int i = 0; i < frames; ++i) {
        rtgb_frame_views v{};
        check(rtgb_render_frame(r.h, &rig, &prof, 1, &v), r.h, "rtgb_render_frame");
        f.render_ms += v.frame_render_ms;
        f.width = v.cameras[0].width;
        f.height = v.cameras[0].height;
    }
    f.beauty.resize(static_cast<size_t>(f.width) * f.height * 4);
    check(rtgb_download_frame(r.h, 0, f.beauty.data(), nullptr, nullptr, nullptr, nullptr), r.h, "rtgb_download_frame");
    for (float v : f.beauty) {
        if (!std::isfinite(v) || v < 0.0f) throw std::runtime_error("frame contains non-finite or negative radiance");
    }
    return f;
}

double mse(const Frame& a, const Frame& r) {
    double s = 0.0;
    const size_t px = static_cast<size_t>(a.width) * a.height;
    for (size_t p = 0; p < px; ++p) {
        for (int c = 0; c < 3; ++c) {
            const double d = static_cast<double>(a.beauty[p * 4 + c]) - r.beauty[p * 4 + c];
            s += d * d;
        }
    }
    return s / static_cast<double>(px * 3);
}

// display_channel (render_restir_acceptance.cpp:149-153): Reinhard, sqrt, lround
uint8_t display_channel(float linear) {
    const float mapped = std::max(0.0f, linear) / (1.0f + std::max(0.0f, linear));
    const float encoded = std::sqrt(mapped);
    return static_cast<uint8_t>(std::lround(255.0f * std::min(encoded, 1.0f)));
}

void write_png(const std::filesystem::path& path, const Frame& f) {
    std::vector<uint8_t> rgb(static_cast<size_t>(f.width) * f.height * 3);
    for (size_t p = 0; p < static_cast<size_t>(f.width) * f.height; ++p) {
        for (int c = 0; c < 3; ++c) rgb[p * 3 + c] = display_channel(f.beauty[p * 4 + c]);
    }
    rtgb::png::write_rgb(path, f.width, f.height, rgb.data());
}

double max_display_error(const std::filesystem::path& a, const std::filesystem::path& b) {
    const rtgb::png::Image x = rtgb::png::read_rgb(a), y = rtgb::png::read_rgb(b);
    if (x.width != y.width || x.height != y.height) {
        throw std::runtime_error("invalid ReSTIR reference pair: " + a.string() + " / " + b.string());
    }
    int m = 0;
    for (size_t i = 0; i < x.rgb.size(); ++i) m = std::max(m, std::abs(static_cast<int>(x.rgb[i]) - y.rgb[i]));
    return m;
}

void json_array(std::ostream& o, const std::vector<double>& v) {
    o << '[';
    for (size_t i = 0; i < v.size(); ++i) o << (i ? ", " : "") << v[i];
    o << ']';
}

}  // namespace

int main(int argc, char** argv) try {
    std::filesystem::path output_dir = "restir-acceptance";
    std::filesystem::path reference_dir;
    bool approve = false, expect_rejected = false;
    int spatial = 1, device = 0;
    for (int i = 1; i < argc; ++i) {
        const std::string_view a = argv[i];
        if (a == "--output-dir" && i + 1 < argc) output_dir = argv[++i];
        else if (a == "--reference-dir" && i + 1 < argc) reference_dir = argv[++i];
        else if (a == "--approve-references") approve = true;
        else if (a == "--expect-quality-rejected") expect_rejected = true;
        else if (a == "--spatial-neighbors" && i + 1 < argc) spatial = std::atoi(argv[++i]);
        else if (a == "--device" && i + 1 < argc) device = std::atoi(argv[++i]);
        else throw std::runtime_error("unknown or incomplete argument: " + std::string(a));
    }
    if (reference_dir.empty()) throw std::runtime_error("--reference-dir is required");
    if (spatial < 1 || spatial > 8) throw std::runtime_error("--spatial-neighbors must be in [1, 8]");
    std::filesystem::create_directories(output_dir);

    rtgb_host_scene* hs = nullptr;
    check(rtgb_host_scene_create("restir_acceptance", 0, 0, &hs), nullptr, "rtgb_host_scene_create");
    rtgb_scene scene{};
    check(rtgb_host_scene_view(hs, &scene), nullptr, "rtgb_host_scene_view");
    rtgb_camera_rig rig{};
    check(rtgb_default_rig("restir_acceptance", 1, 0, 0, &rig), nullptr, "rtgb_default_rig");
    const rtgb_render_profile ref_prof = make_profile(kReferenceSpp, false, 0);
    const rtgb_render_profile base_prof = make_profile(kBaselineSpp, false, 0);
    const rtgb_render_profile restir_prof = make_profile(1, true, spatial);

    auto fresh = [&](const rtgb_render_profile& p, int frames) {
        Handle r(device);
        check(rtgb_prepare_scene(r.h, &scene), r.h, "rtgb_prepare_scene");
        return render(r, rig, p, frames);
    };
    const Frame reference = fresh(ref_prof, 1);
    const Frame baseline = fresh(base_prof, 1);

    Handle rr(device);
    check(rtgb_prepare_scene(rr.h, &scene), rr.h, "rtgb_prepare_scene");
    rtgb_restir_stats first{}, final_stats{}, reset{};
    Frame restir;
    double restir_ms = 0.0;
    for (int f = 0; f < kRestirFrames; ++f) {
        restir = render(rr, rig, restir_prof, 1);
        restir_ms += restir.render_ms;
        if (f == 0) check(rtgb_restir_diagnostics(rr.h, 0, &first), rr.h, "rtgb_restir_diagnostics");
    }
    check(rtgb_restir_diagnostics(rr.h, 0, &final_stats), rr.h, "rtgb_restir_diagnostics");
    check(rtgb_prepare_scene(rr.h, &scene), rr.h, "rtgb_prepare_scene");
    render(rr, rig, restir_prof, 1);
    check(rtgb_restir_diagnostics(rr.h, 0, &reset), rr.h, "rtgb_restir_diagnostics");

    std::vector<double> base_trials{baseline.render_ms}, restir_trials{restir_ms};
    for (int t = 1; t < kPerformanceTrials; ++t) {
        base_trials.push_back(fresh(base_prof, 1).render_ms);
        restir_trials.push_back(fresh(restir_prof, kRestirFrames).render_ms);
    }
    rtgb_host_scene_destroy(hs);

    const double base_mse = mse(baseline, reference), restir_mse = mse(restir, reference);
    const double ratio = base_mse > 0.0 ? restir_mse / base_mse : 0.0;
    const bool quality = restir_mse <= base_mse * kQualityRatioLimit + 1e-8;
    const bool quality_expectation = expect_rejected ? !quality : quality;
    double base_mean = 0.0, restir_mean = 0.0;
    int wins = 0;
    for (size_t t = 0; t < base_trials.size(); ++t) {
        base_mean += base_trials[t];
        restir_mean += restir_trials[t];
        wins += restir_trials[t] < base_trials[t] ? 1 : 0;
    }
    base_mean /= static_cast<double>(base_trials.size());
    restir_mean /= static_cast<double>(restir_trials.size());
    const bool performance = restir_mean < base_mean && wins >= (kPerformanceTrials + 1) / 2;
    const bool temporal = first.temporal_reuse_count == 0 && final_stats.temporal_reuse_count > 0 && final_stats.max_age > 0 &&
                          reset.temporal_reuse_count == 0;
    const bool spatial_ok = first.spatial_reuse_count == 0 && final_stats.spatial_reuse_count > 0 && reset.spatial_reuse_count == 0;
    const bool bias_ok = first.bias_corrected_count == 0 && final_stats.bias_corrected_count > 0 && reset.bias_corrected_count == 0;

    write_png(output_dir / "reference.png", reference);
    write_png(output_dir / "baseline.png", baseline);
    write_png(output_dir / "restir.png", restir);
    const char* names[3] = {"reference.png", "baseline.png", "restir.png"};
    if (approve) {
        std::filesystem::create_directories(reference_dir);
        for (const char* n : names) {
            std::filesystem::copy_file(output_dir / n, reference_dir / n, std::filesystem::copy_options::overwrite_existing);
        }
    }
    double max_err = 0.0;
    for (const char* n : names) max_err = std::max(max_err, max_display_error(output_dir / n, reference_dir / n));
    const bool reference_gate = max_err <= 2.0;

    std::ofstream rep(output_dir / "report.json");
    rep << std::fixed << std::setprecision(9) << "{\n"
        << "  \"schema_version\": \"restir_di_acceptance_v2\",\n"
        << "  \"light_count\": " << kLightCount << ",\n"
        << "  \"reference_spp\": " << kReferenceSpp << ",\n"
        << "  \"baseline_spp\": " << kBaselineSpp << ",\n"
        << "  \"restir_frames\": " << kRestirFrames << ",\n"
        << "  \"restir_candidates_per_frame\": " << kRestirCandidates << ",\n"
        << "  \"restir_spatial_neighbors\": " << spatial << ",\n"
        << "  \"restir_bias_correction\": \"basic\",\n"
        << "  \"baseline_mse\": " << base_mse << ",\n"
        << "  \"restir_mse\": " << restir_mse << ",\n"
        << "  \"quality_mse_ratio\": " << ratio << ",\n"
        << "  \"equal_or_better_quality_mse_ratio_limit\": " << kQualityRatioLimit << ",\n"
        << "  \"expected_quality_decision\": \"" << (expect_rejected ? "rejected" : "selected") << "\",\n"
        << "  \"baseline_render_ms\": " << baseline.render_ms << ",\n"
        << "  \"restir_render_ms\": " << restir_ms << ",\n"
        << "  \"performance_trial_count\": " << kPerformanceTrials << ",\n"
        << "  \"performance_win_count\": " << wins << ",\n"
        << "  \"baseline_render_mean_ms\": " << base_mean << ",\n"
        << "  \"restir_render_mean_ms\": " << restir_mean << ",\n"
        << "  \"baseline_render_ms_trials\": ";
    json_array(rep, base_trials);
    rep << ",\n  \"restir_render_ms_trials\": ";
    json_array(rep, restir_trials);
    rep << ",\n"
        << "  \"first_temporal_reuse_pixels\": " << first.temporal_reuse_count << ",\n"
        << "  \"final_temporal_reuse_pixels\": " << final_stats.temporal_reuse_count << ",\n"
        << "  \"reset_temporal_reuse_pixels\": " << reset.temporal_reuse_count << ",\n"
        << "  \"first_spatial_reuse_pixels\": " << first.spatial_reuse_count << ",\n"
        << "  \"final_spatial_reuse_pixels\": " << final_stats.spatial_reuse_count << ",\n"
        << "  \"reset_spatial_reuse_pixels\": " << reset.spatial_reuse_count << ",\n"
        << "  \"first_bias_corrected_pixels\": " << first.bias_corrected_count << ",\n"
        << "  \"final_bias_corrected_pixels\": " << final_stats.bias_corrected_count << ",\n"
        << "  \"reset_bias_corrected_pixels\": " << reset.bias_corrected_count << ",\n"
        << "  \"reference_max_display_error\": " << max_err << ",\n"
        << "  \"reference_gate_passed\": " << (reference_gate ? "true" : "false") << ",\n"
        << "  \"quality_passed\": " << (quality ? "true" : "false") << ",\n"
        << "  \"quality_expectation_passed\": " << (quality_expectation ? "true" : "false") << ",\n"
        << "  \"performance_passed\": " << (performance ? "true" : "false") << ",\n"
        << "  \"temporal_validity_passed\": " << (temporal ? "true" : "false") << ",\n"
        << "  \"spatial_validity_passed\": " << (spatial_ok ? "true" : "false") << ",\n"
        << "  \"bias_correction_passed\": " << (bias_ok ? "true" : "false") << "\n}\n";
    rep.close();
    std::cout << "restir_acceptance baseline_mse=" << base_mse << " restir_mse=" << restir_mse << " quality_ratio=" << ratio
              << " quality_decision=" << (quality ? "selected" : "rejected") << " baseline_mean_ms=" << base_mean
              << " restir_mean_ms=" << restir_mean << " performance_wins=" << wins << '/' << kPerformanceTrials
              << " temporal_pixels=" << final_stats.temporal_reuse_count << " spatial_pixels=" << final_stats.spatial_reuse_count
              << " bias_corrected_pixels=" << final_stats.bias_corrected_count << '\n';
    if (!quality_expectation || !performance || !temporal || !spatial_ok || !bias_ok || !reference_gate) {
        std::cerr << "render_restir_acceptance: ReSTIR DI evaluation failed; inspect " << (output_dir / "report.json").string()
                  << '\n';
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
} catch (const std::exception& e) {
    std::cerr << "render_restir_acceptance: " << e.what() << '\n';
    return EXIT_FAILURE;
}
