// Benchmark report of the render_realtime CLI: the frame CSV, the schema-3
// summary JSON and the artifact manifest the reference writes
// (src/realtime/profiling/benchmark_report.h:10-147, benchmark_report.cpp:
// 203-445), restated field for field so tools reading the reference's reports
// read these. Extensions (ray counts, Mrays/s) live under keys the reference
// does not use ("extensions" in the summary, trailing CSV columns).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace rtgb::report {

struct CameraSample {
    int camera_index = 0;
    double render_ms = 0.0, denoise_ms = 0.0, download_ms = 0.0, average_luminance = 0.0;
};

struct FrameSample {
    int frame_index = 0;
    uint32_t sample_stream = 0;
    int camera_count = 0;
    std::string profile;
    int width = 0, height = 0, samples_per_pixel = 0, max_bounces = 0;
    bool denoise_enabled = false;
    double frame_ms = 0.0, pipeline_ms = 0.0, render_ms = 0.0, denoise_ms = 0.0, download_ms = 0.0;
    double render_work_ms = 0.0, denoise_work_ms = 0.0, download_work_ms = 0.0;
    double image_write_ms = 0.0, host_overhead_ms = 0.0, fps = 0.0;
    uint64_t rays_traced = 0;   // extension
    std::vector<CameraSample> cameras;
};

struct Stats {
    double avg = 0.0, p50 = 0.0, p95 = 0.0, p99 = 0.0, max = 0.0;
};

struct Aggregate {
    Stats frame_ms, pipeline_ms, render_ms, denoise_ms, download_ms, render_work_ms, denoise_work_ms,
        download_work_ms, image_write_ms, host_overhead_ms;
};

struct Provenance {
    std::string captured_at_utc, project_version, source_revision;
    bool source_dirty = false;
    std::string source_scope, source_state_sha256, build_configuration, cxx_compiler;
};

struct Environment {
    std::string operating_system, architecture;
    int gpu_device = 0;
    std::string gpu_name, compute_capability, nvidia_driver_version;
    int cuda_driver_api_version = 0;
    std::string cuda_driver_api_version_text;
    int cuda_runtime_version = 0;
    std::string cuda_runtime_version_text;
    int optix_version = 0;               // no OptiX here: 0 / "unavailable"
    std::string optix_version_text = "unavailable";
};

struct GpuMemory {
    std::string scope = "cuda_device_global";
    uint64_t total_bytes = 0, baseline_used_bytes = 0, prepared_used_bytes = 0, peak_used_bytes = 0,
             peak_delta_bytes = 0, final_used_bytes = 0;
};

struct GpuScheduling {
    int persistent_worker_count = 0;
    uint64_t worker_start_count = 0, task_submission_count = 0, launch_parameter_allocation_count = 0,
             launch_parameter_upload_count = 0;
    std::string acceleration_update_kind;
    double acceleration_update_ms = 0.0;
    int acceleration_node_count = 0, acceleration_reference_count = 0, acceleration_prototype_count = 0,
        acceleration_instance_count = 0, acceleration_instanced_primitive_count = 0;
    uint64_t acceleration_generation = 0;
};

struct Report {
    int schema_version = 3;
    Provenance provenance;
    Environment environment;
    GpuMemory gpu_memory;
    GpuScheduling gpu_scheduling;
    std::string scene, profile;
    int camera_count = 0, width = 0, height = 0, frames_requested = 0, warmup_frames = 0;
    uint32_t random_seed = 0;
    int samples_per_pixel = 0, max_bounces = 0;
    bool denoise_enabled = false, image_write_enabled = true;
    std::vector<FrameSample> frames;
    Aggregate aggregate;
};

// Mean plus nearest-rank percentiles (rank ceil(p * n), 1-based).
inline Stats stats_of(std::vector<double> v) {
    Stats s;
    if (v.empty()) return s;
    std::sort(v.begin(), v.end());
    auto at = [&](double p) {
        const double rank = std::ceil(p * static_cast<double>(v.size()));
        const size_t i = rank <= 1.0 ? 0 : static_cast<size_t>(rank - 1.0);
        return v[std::min(i, v.size() - 1)];
    };
    double sum = 0.0;
    for (double x : v) sum += x;
    s.avg = sum / static_cast<double>(v.size());
    s.p50 = at(0.50);
    s.p95 = at(0.95);
    s.p99 = at(0.99);
    s.max = v.back();
    return s;
}

inline Aggregate aggregate_of(const std::vector<FrameSample>& frames) {
    auto col = [&](double FrameSample::*m) {
        std::vector<double> v;
        v.reserve(frames.size());
        for (const FrameSample& f : frames) v.push_back(f.*m);
        return stats_of(std::move(v));
    };
    return Aggregate{col(&FrameSample::frame_ms), col(&FrameSample::pipeline_ms), col(&FrameSample::render_ms),
        col(&FrameSample::denoise_ms), col(&FrameSample::download_ms), col(&FrameSample::render_work_ms),
        col(&FrameSample::denoise_work_ms), col(&FrameSample::download_work_ms), col(&FrameSample::image_write_ms),
        col(&FrameSample::host_overhead_ms)};
}

inline const char* tf(bool b) { return b ? "true" : "false"; }

inline std::string csv_field(const std::string& v) {
    if (v.find_first_of(",\"\n\r") == std::string::npos) return v;
    std::string out = "\"";
    for (char c : v) out += c == '"' ? std::string("\"\"") : std::string(1, c);
    return out + "\"";
}

inline std::string json_str(const std::string& v) {
    static const char* hex = "0123456789abcdef";
    std::string out;
    for (unsigned char c : v) {
        switch (c) {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\b': out += "\\b"; break;
            case '\f': out += "\\f"; break;
            case '\n': out += "\\n"; break;
            case '\r': out += "\\r"; break;
            case '\t': out += "\\t"; break;
            default:
                if (c < 0x20) {
                    out += "\\u00";
                    out += hex[c >> 4];
                    out += hex[c & 15];
                } else {
                    out += static_cast<char>(c);
                }
        }
    }
    return out;
}

inline std::ofstream open_out(const std::filesystem::path& p, const char* what) {
    std::ofstream out(p);
    if (!out.is_open()) throw std::runtime_error(std::string("failed to open ") + what + " output file: " + p.string());
    return out;
}

inline void check_out(const std::ofstream& out, const std::filesystem::path& p, const char* what) {
    if (!out.good()) throw std::runtime_error(std::string("failed to write ") + what + " output file: " + p.string());
}

inline void write_csv(const Report& r, const std::filesystem::path& path) {
    std::ofstream out = open_out(path, "csv");
    out << "frame_index,sample_stream,camera_count,profile,width,height,samples_per_pixel,max_bounces,"
           "denoise_enabled,frame_ms,pipeline_ms,render_ms,denoise_ms,download_ms,render_work_ms,"
           "denoise_work_ms,download_work_ms,image_write_ms,host_overhead_ms,fps,rays_traced,mrays_per_s\n";
    for (const FrameSample& f : r.frames) {
        const double mrays = f.pipeline_ms > 0.0 ? static_cast<double>(f.rays_traced) / (f.pipeline_ms * 1e3) : 0.0;
        out << f.frame_index << ',' << f.sample_stream << ',' << f.camera_count << ',' << csv_field(f.profile) << ','
            << f.width << ',' << f.height << ',' << f.samples_per_pixel << ',' << f.max_bounces << ','
            << tf(f.denoise_enabled) << ',' << f.frame_ms << ',' << f.pipeline_ms << ',' << f.render_ms << ','
            << f.denoise_ms << ',' << f.download_ms << ',' << f.render_work_ms << ',' << f.denoise_work_ms << ','
            << f.download_work_ms << ',' << f.image_write_ms << ',' << f.host_overhead_ms << ',' << f.fps << ','
            << f.rays_traced << ',' << mrays << '\n';
    }
    out.flush();
    check_out(out, path, "csv");
}

inline void write_stats(std::ostream& out, const char* name, const Stats& s, bool comma) {
    out << "    \"" << name << "\": {\"avg\": " << s.avg << ", \"p50\": " << s.p50 << ", \"p95\": " << s.p95
        << ", \"p99\": " << s.p99 << ", \"max\": " << s.max << "}" << (comma ? "," : "") << "\n";
}

inline void write_json(const Report& r, const std::filesystem::path& path) {
    std::ofstream out = open_out(path, "json");
    const Provenance& p = r.provenance;
    const Environment& e = r.environment;
    const GpuMemory& m = r.gpu_memory;
    const GpuScheduling& g = r.gpu_scheduling;
    out << "{\n  \"schema_version\": " << r.schema_version << ",\n";
    out << "  \"metadata\": {\n"
        << "    \"scene\": \"" << json_str(r.scene) << "\",\n"
        << "    \"profile\": \"" << json_str(r.profile) << "\",\n"
        << "    \"camera_count\": " << r.camera_count << ",\n"
        << "    \"width\": " << r.width << ",\n"
        << "    \"height\": " << r.height << ",\n"
        << "    \"frames_requested\": " << r.frames_requested << ",\n"
        << "    \"warmup_frames\": " << r.warmup_frames << ",\n"
        << "    \"random_seed\": " << r.random_seed << ",\n"
        << "    \"measurement_sample_stream_start\": "
        << static_cast<uint64_t>(r.random_seed) + static_cast<uint64_t>(r.warmup_frames) << ",\n"
        << "    \"rng_algorithm\": \"hashed_pixel_sample_stream_v1\",\n"
        << "    \"samples_per_pixel\": " << r.samples_per_pixel << ",\n"
        << "    \"max_bounces\": " << r.max_bounces << ",\n"
        << "    \"denoise_enabled\": " << tf(r.denoise_enabled) << ",\n"
        << "    \"image_write_enabled\": " << tf(r.image_write_enabled) << "\n  },\n";
    out << "  \"provenance\": {\n"
        << "    \"captured_at_utc\": \"" << json_str(p.captured_at_utc) << "\",\n"
        << "    \"project_version\": \"" << json_str(p.project_version) << "\",\n"
        << "    \"source_revision\": \"" << json_str(p.source_revision) << "\",\n"
        << "    \"source_dirty\": " << tf(p.source_dirty) << ",\n"
        << "    \"source_scope\": \"" << json_str(p.source_scope) << "\",\n"
        << "    \"source_state_sha256\": \"" << json_str(p.source_state_sha256) << "\",\n"
        << "    \"build_configuration\": \"" << json_str(p.build_configuration) << "\",\n"
        << "    \"cxx_compiler\": \"" << json_str(p.cxx_compiler) << "\"\n  },\n";
    out << "  \"environment\": {\n"
        << "    \"operating_system\": \"" << json_str(e.operating_system) << "\",\n"
        << "    \"architecture\": \"" << json_str(e.architecture) << "\",\n"
        << "    \"gpu_device\": " << e.gpu_device << ",\n"
        << "    \"gpu_name\": \"" << json_str(e.gpu_name) << "\",\n"
        << "    \"compute_capability\": \"" << json_str(e.compute_capability) << "\",\n"
        << "    \"nvidia_driver_version\": \"" << json_str(e.nvidia_driver_version) << "\",\n"
        << "    \"cuda_driver_api_version\": " << e.cuda_driver_api_version << ",\n"
        << "    \"cuda_driver_api_version_text\": \"" << json_str(e.cuda_driver_api_version_text) << "\",\n"
        << "    \"cuda_runtime_version\": " << e.cuda_runtime_version << ",\n"
        << "    \"cuda_runtime_version_text\": \"" << json_str(e.cuda_runtime_version_text) << "\",\n"
        << "    \"optix_version\": " << e.optix_version << ",\n"
        << "    \"optix_version_text\": \"" << json_str(e.optix_version_text) << "\"\n  },\n";
    out << "  \"gpu_memory\": {\n"
        << "    \"scope\": \"" << json_str(m.scope) << "\",\n"
        << "    \"total_bytes\": " << m.total_bytes << ",\n"
        << "    \"baseline_used_bytes\": " << m.baseline_used_bytes << ",\n"
        << "    \"prepared_used_bytes\": " << m.prepared_used_bytes << ",\n"
        << "    \"peak_used_bytes\": " << m.peak_used_bytes << ",\n"
        << "    \"peak_delta_bytes\": " << m.peak_delta_bytes << ",\n"
        << "    \"final_used_bytes\": " << m.final_used_bytes << "\n  },\n";
    out << "  \"gpu_scheduling\": {\n"
        << "    \"persistent_worker_count\": " << g.persistent_worker_count << ",\n"
        << "    \"worker_start_count\": " << g.worker_start_count << ",\n"
        << "    \"task_submission_count\": " << g.task_submission_count << ",\n"
        << "    \"launch_parameter_allocation_count\": " << g.launch_parameter_allocation_count << ",\n"
        << "    \"launch_parameter_upload_count\": " << g.launch_parameter_upload_count << ",\n"
        << "    \"acceleration_update_kind\": \"" << json_str(g.acceleration_update_kind) << "\",\n"
        << "    \"acceleration_update_ms\": " << g.acceleration_update_ms << ",\n"
        << "    \"acceleration_node_count\": " << g.acceleration_node_count << ",\n"
        << "    \"acceleration_reference_count\": " << g.acceleration_reference_count << ",\n"
        << "    \"acceleration_prototype_count\": " << g.acceleration_prototype_count << ",\n"
        << "    \"acceleration_instance_count\": " << g.acceleration_instance_count << ",\n"
        << "    \"acceleration_instanced_primitive_count\": " << g.acceleration_instanced_primitive_count << ",\n"
        << "    \"acceleration_generation\": " << g.acceleration_generation << "\n  },\n";
    const Aggregate& a = r.aggregate;
    out << "  \"aggregate\": {\n";
    write_stats(out, "frame_ms", a.frame_ms, true);
    write_stats(out, "pipeline_ms", a.pipeline_ms, true);
    write_stats(out, "render_ms", a.render_ms, true);
    write_stats(out, "denoise_ms", a.denoise_ms, true);
    write_stats(out, "download_ms", a.download_ms, true);
    write_stats(out, "render_work_ms", a.render_work_ms, true);
    write_stats(out, "denoise_work_ms", a.denoise_work_ms, true);
    write_stats(out, "download_work_ms", a.download_work_ms, true);
    write_stats(out, "image_write_ms", a.image_write_ms, true);
    write_stats(out, "host_overhead_ms", a.host_overhead_ms, false);
    out << "  },\n  \"frames\": [\n";
    for (size_t i = 0; i < r.frames.size(); ++i) {
        const FrameSample& f = r.frames[i];
        out << "    {\"frame_index\": " << f.frame_index << ", \"sample_stream\": " << f.sample_stream
            << ", \"camera_count\": " << f.camera_count << ", \"profile\": \"" << json_str(f.profile)
            << "\", \"width\": " << f.width << ", \"height\": " << f.height
            << ", \"samples_per_pixel\": " << f.samples_per_pixel << ", \"max_bounces\": " << f.max_bounces
            << ", \"denoise_enabled\": " << tf(f.denoise_enabled) << ", \"frame_ms\": " << f.frame_ms
            << ", \"pipeline_ms\": " << f.pipeline_ms << ", \"render_ms\": " << f.render_ms
            << ", \"denoise_ms\": " << f.denoise_ms << ", \"download_ms\": " << f.download_ms
            << ", \"render_work_ms\": " << f.render_work_ms << ", \"denoise_work_ms\": " << f.denoise_work_ms
            << ", \"download_work_ms\": " << f.download_work_ms << ", \"image_write_ms\": " << f.image_write_ms
            << ", \"host_overhead_ms\": " << f.host_overhead_ms << ", \"fps\": " << f.fps << "}"
            << (i + 1 != r.frames.size() ? "," : "") << "\n";
    }
    out << "  ],\n  \"per-camera\": [\n";
    bool first = true;
    for (const FrameSample& f : r.frames) {
        for (const CameraSample& c : f.cameras) {
            if (!first) out << ",\n";
            first = false;
            out << "    {\"frame_index\": " << f.frame_index << ", \"camera_index\": " << c.camera_index
                << ", \"render_ms\": " << c.render_ms << ", \"denoise_ms\": " << c.denoise_ms
                << ", \"download_ms\": " << c.download_ms << ", \"average_luminance\": " << c.average_luminance << "}";
        }
    }
    out << "\n  ],\n";
    // extension: traced rays per measured frame and throughput over the pipeline time
    uint64_t rays = 0;
    double pipe = 0.0;
    for (const FrameSample& f : r.frames) {
        rays += f.rays_traced;
        pipe += f.pipeline_ms;
    }
    out << "  \"extensions\": {\"rays_traced\": " << rays
        << ", \"mrays_per_s\": " << (pipe > 0.0 ? static_cast<double>(rays) / (pipe * 1e3) : 0.0) << "}\n}\n";
    out.flush();
    check_out(out, path, "json");
}

inline std::string fnv1a64(const std::filesystem::path& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in.is_open()) throw std::runtime_error("failed to open benchmark artifact: " + path.string());
    uint64_t h = 14695981039346656037ull;
    std::array<char, 8192> buf{};
    while (in) {
        in.read(buf.data(), static_cast<std::streamsize>(buf.size()));
        const std::streamsize n = in.gcount();
        for (std::streamsize i = 0; i < n; ++i) {
            h ^= static_cast<unsigned char>(buf[static_cast<size_t>(i)]);
            h *= 1099511628211ull;
        }
    }
    if (!in.eof()) throw std::runtime_error("failed to read benchmark artifact: " + path.string());
    std::ostringstream d;
    d << std::hex << std::setfill('0') << std::setw(16) << h;
    return d.str();
}

inline void write_manifest(const Report& r, const std::vector<std::filesystem::path>& artifacts,
    const std::filesystem::path& path) {
    if (artifacts.empty()) throw std::invalid_argument("benchmark artifact manifest requires at least one artifact");
    size_t per_camera = 0;
    for (const FrameSample& f : r.frames) per_camera += f.cameras.size();
    std::ofstream out = open_out(path, "artifact manifest");
    out << "{\n  \"schema_version\": 1,\n  \"report_schema_version\": " << r.schema_version << ",\n"
        << "  \"measured_frame_count\": " << r.frames.size() << ",\n"
        << "  \"per_camera_record_count\": " << per_camera << ",\n  \"artifacts\": [\n";
    for (size_t i = 0; i < artifacts.size(); ++i) {
        const std::filesystem::path& a = artifacts[i];
        if (!std::filesystem::is_regular_file(a)) throw std::runtime_error("benchmark artifact is not a regular file: " + a.string());
        out << "    {\"filename\": \"" << json_str(a.filename().string()) << "\", \"kind\": \""
            << (a.extension() == ".csv" ? "raw_frame_samples" : "summary_and_provenance")
            << "\", \"size_bytes\": " << std::filesystem::file_size(a)
            << ", \"digest_algorithm\": \"fnv1a64\", \"digest\": \"" << fnv1a64(a) << "\"}"
            << (i + 1 != artifacts.size() ? "," : "") << "\n";
    }
    out << "  ]\n}\n";
    out.flush();
    check_out(out, path, "artifact manifest");
}

}  // namespace rtgb::report
