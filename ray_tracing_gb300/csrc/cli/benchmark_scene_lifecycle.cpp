// benchmark_scene_lifecycle: the reference's acceleration-lifecycle benchmark
// (utils/benchmark_gpu_scene_lifecycle.cpp) over this library's C ABI.
//
// A grid of spheres (32 per row, 0.3 apart, radius 0.1, one Lambertian
// material) is prepared as: base (rebuild), base again (reuse), a changed
// albedo (update), the grid shifted by 0.01 (refit) and one sphere more
// (rebuild), `iterations` times after one warm-up round; every prepare must
// report the expected kind. Output: the reference's JSON (schema 1) with
// avg / p95 / max of each kind's host wall time around rtgb_prepare_scene,
// plus the device build time of each kind under "device_timings".
//
//   benchmark_scene_lifecycle OUTPUT_JSON [--primitives N] [--iterations K] [--device D]
//
// The reference fixes N = 1024 and K = 20. Its instancing diagnostics
// (prototype / instance counts) have no counterpart here: spheres carry no
// acceleration prototype, so those fields are written as 0.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "rtgb.h"

namespace {

constexpr const char* kKinds[4] = {"reuse", "update", "refit", "rebuild"};

struct GridScene {
    std::vector<rtgb_texture> textures;
    std::vector<rtgb_material> materials;
    std::vector<rtgb_sphere> spheres;
    rtgb_scene view{};
};

// make_instanced_scene of the reference benchmark: sphere i at
// ((i % 32) * 0.3 + offset, (i / 32) * 0.3, -4), radius 0.1.
GridScene make_grid(int count, float offset, float albedo) {
    GridScene g;
    rtgb_texture t{};
    t.type = 0;
    t.even_texture = t.odd_texture = -1;
    t.scale = 1.0f;
    t.color[0] = albedo;
    t.color[1] = 0.3f;
    t.color[2] = 0.2f;
    g.textures.push_back(t);
    rtgb_material m{};
    m.albedo_texture = 0;
    m.emission_texture = -1;
    m.ior = 1.0f;
    m.type = RTGB_MATERIAL_LAMBERTIAN;
    m.openpbr_index = -1;
    g.materials.push_back(m);
    g.spheres.resize(static_cast<size_t>(count));
    for (int i = 0; i < count; ++i) {
        rtgb_sphere& s = g.spheres[static_cast<size_t>(i)];
        s.center[0] = static_cast<float>(i % 32) * 0.3f + offset;
        s.center[1] = static_cast<float>(i / 32) * 0.3f;
        s.center[2] = -4.0f;
        s.radius = 0.1f;
        s.material_index = 0;
    }
    g.view.textures = g.textures.data();
    g.view.texture_count = static_cast<int32_t>(g.textures.size());
    g.view.materials = g.materials.data();
    g.view.material_count = static_cast<int32_t>(g.materials.size());
    g.view.spheres = g.spheres.data();
    g.view.sphere_count = count;
    g.view.background[0] = g.view.background[1] = g.view.background[2] = 0.5f;
    return g;
}

struct Timing {
    double avg = 0.0, p95 = 0.0, max = 0.0;
};

// avg, the ceil(0.95 n)-th smallest value and the maximum, as the reference's summarize()
Timing summarize(std::vector<double> v) {
    if (v.empty()) throw std::runtime_error("lifecycle timing set is empty");
    std::sort(v.begin(), v.end());
    double sum = 0.0;
    for (double x : v) {
        if (!std::isfinite(x) || x < 0.0) throw std::runtime_error("lifecycle timing is invalid");
        sum += x;
    }
    const size_t idx = std::min(v.size() - 1, static_cast<size_t>(std::ceil(static_cast<double>(v.size()) * 0.95) - 1));
    return Timing{sum / static_cast<double>(v.size()), v[idx], v.back()};
}

struct Lifecycle {
    rtgb_handle h = nullptr;
    std::vector<double> host[4], device[4];
    rtgb_acceleration_info last{};

    void prepare(const GridScene& g, int expected, const char* label, bool record) {
        const auto t0 = std::chrono::steady_clock::now();
        const rtgb_status st = rtgb_prepare_scene(h, &g.view);
        const auto t1 = std::chrono::steady_clock::now();
        if (st != RTGB_OK) throw std::runtime_error(std::string(label) + ": " + rtgb_last_error(h));
        rtgb_acceleration_info a{};
        if (rtgb_acceleration_info_get(h, &a) != RTGB_OK) throw std::runtime_error("rtgb_acceleration_info_get");
        if (a.update_kind != expected) {
            throw std::runtime_error(std::string(label) + " expected " + kKinds[expected] + " but observed "
                                     + (a.update_kind >= 0 && a.update_kind < 4 ? kKinds[a.update_kind] : "unknown"));
        }
        if (record) {
            host[expected].push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
            device[expected].push_back(a.build_ms);
        }
        last = a;
    }
};

void write_summary(std::ofstream& out, std::string_view name, const Timing& t, bool comma) {
    out << "    \"" << name << "\": {\"avg_ms\": " << t.avg << ", \"p95_ms\": " << t.p95 << ", \"max_ms\": " << t.max
        << "}" << (comma ? "," : "") << "\n";
}

int parse_int(const char* v, const char* flag, int lo) {
    char* end = nullptr;
    const long x = std::strtol(v, &end, 10);
    if (!end || *end || x < lo || x > (1l << 27)) throw std::invalid_argument(std::string(flag) + " is out of range");
    return static_cast<int>(x);
}

}  // namespace

int main(int argc, const char* argv[]) try {
    if (argc < 2) throw std::invalid_argument("usage: benchmark_scene_lifecycle OUTPUT_JSON [--primitives N] "
                                              "[--iterations K] [--device D]");
    int count = 1024, iterations = 20, device = 0;
    for (int i = 2; i < argc; i += 2) {
        const std::string_view f = argv[i];
        if (i + 1 >= argc) throw std::invalid_argument(std::string(f) + " needs a value");
        if (f == "--primitives") count = parse_int(argv[i + 1], "--primitives", 2);
        else if (f == "--iterations") iterations = parse_int(argv[i + 1], "--iterations", 1);
        else if (f == "--device") device = parse_int(argv[i + 1], "--device", 0);
        else throw std::invalid_argument("unknown argument: " + std::string(f));
    }
    const GridScene base = make_grid(count, 0.0f, 0.7f);
    const GridScene material_update = make_grid(count, 0.0f, 0.9f);
    const GridScene moved = make_grid(count, 0.01f, 0.9f);
    const GridScene topology = make_grid(count + 1, 0.0f, 0.9f);

    rtgb_create_info ci{};
    ci.device = device;
    ci.use_cuda_graph = 1;
    Lifecycle L;
    if (rtgb_create(&ci, &L.h) != RTGB_OK) throw std::runtime_error("rtgb_create failed");
    // warm device allocation, driver state and every lifecycle path
    L.prepare(base, 3, "warmup rebuild", false);
    L.prepare(base, 0, "warmup reuse", false);
    L.prepare(material_update, 1, "warmup update", false);
    L.prepare(moved, 2, "warmup refit", false);
    L.prepare(topology, 3, "warmup topology rebuild", false);
    rtgb_acceleration_info rep{};
    for (int it = 0; it < iterations; ++it) {
        L.prepare(base, 3, "base rebuild", true);
        rep = L.last;
        L.prepare(base, 0, "identical reuse", true);
        L.prepare(material_update, 1, "material update", true);
        L.prepare(moved, 2, "geometry refit", true);
        L.prepare(topology, 3, "topology rebuild", true);
    }
    const int generation = L.last.generation;
    rtgb_destroy(L.h);

    const std::filesystem::path path = argv[1];
    if (path.has_parent_path()) std::filesystem::create_directories(path.parent_path());
    std::ofstream out(path);
    if (!out.is_open()) throw std::runtime_error("failed to open " + path.string());
    out << std::fixed << std::setprecision(6);
    out << "{\n  \"schema_version\": 1,\n  \"iterations\": " << iterations << ",\n  \"primitive_count\": " << count
        << ",\n  \"acceleration\": {\n    \"node_count\": " << rep.node_count
        << ",\n    \"primitive_reference_count\": " << rep.primitive_count
        << ",\n    \"prototype_count\": 0,\n    \"instance_count\": 0,\n    \"instanced_primitive_count\": 0,\n"
        << "    \"generation\": " << generation << "\n  },\n  \"timings\": {\n";
    write_summary(out, "rebuild", summarize(L.host[3]), true);
    write_summary(out, "update", summarize(L.host[1]), true);
    write_summary(out, "refit", summarize(L.host[2]), true);
    write_summary(out, "reuse", summarize(L.host[0]), false);
    out << "  },\n  \"device_timings\": {\n";
    write_summary(out, "rebuild", summarize(L.device[3]), true);
    write_summary(out, "update", summarize(L.device[1]), true);
    write_summary(out, "refit", summarize(L.device[2]), true);
    write_summary(out, "reuse", summarize(L.device[0]), false);
    out << "  }\n}\n";
    if (!out.good()) throw std::runtime_error("failed to write " + path.string());
    std::printf("lifecycle primitives=%d iterations=%d rebuild_ms=%.4f update_ms=%.4f refit_ms=%.4f reuse_ms=%.4f "
                "output=%s\n", count, iterations, summarize(L.host[3]).avg, summarize(L.host[1]).avg,
                summarize(L.host[2]).avg, summarize(L.host[0]).avg, path.string().c_str());
    return EXIT_SUCCESS;
} catch (const std::exception& e) {
    std::fprintf(stderr, "benchmark_scene_lifecycle: %s\n", e.what());
    return EXIT_FAILURE;
}
