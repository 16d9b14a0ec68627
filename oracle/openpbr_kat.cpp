// OpenPBR known-answer driver — TEST INFRASTRUCTURE.
//
// One source, two builds:
//   * into oracle/_bin/liborc.so against the repository's own OpenPBR header
//     (ray_tracing_gb300/csrc/openpbr.h), exporting orc_openpbr_kat;
//   * by oracle/build_ref.py, with -DKAT_REFERENCE, against the reference's
//     src/common/openpbr_core.h into oracle/_ref/libopenpbr_ref.so, exporting
//     ref_openpbr_kat.
// Both run the same battery over the same input records and write the same
// output records, so tests/golden/openpbr holds the reference's answers and
// the test compares the repository header with them word for word.
//
// Input record (kKatIn 32-bit words):
//   [0,51)  OpenPBR parameter block (204 bytes, the reference's OpenPbrCoreMaterial layout)
//   [51,54) frame normal      [54,57) frame tangent
//   [57,60) wo                [60,63) wi
//   [63,66) u_lobe, u1, u2    [66,69) path throughput
//   [69]    boundary distance [70]    segment u
//   [71]    lobe cosine       [72]    sRGB probe value
// Output record (kKatOut words):
//   [0,4)   evaluate: value, pdf
//   [4,18)  sample: wi, value, weight, pdf, discrete_pdf, event, delta, valid
//   [18,24) lobe probabilities, exterior      [24,30) lobe probabilities, interior
//   [30,33) emission
//   [33,41) subsurface medium: extinction, albedo, anisotropy, active
//   [41,46) subsurface segment: weight, distance, scattered
//   [46,49) Henyey-Greenstein direction
//   [49,58) frame: tangent, bitangent, normal
//   [58]    sRGB-to-linear of the probe value
//   [59,62) boundary-material sample: wi   [62] its event  [63] its valid
#include <cstdint>
#include <cstring>

constexpr int kKatIn = 80;
constexpr int kKatOut = 64;

#ifdef KAT_REFERENCE
#include "openpbr_core.h"
namespace kat {
using Mat = rt::OpenPbrCoreMaterial;
using V = rt::OpenPbrVec3;
using Frame = rt::OpenPbrFrame;
using Ctx = rt::OpenPbrTransportContext;
inline Ctx ctx_of(const V& t) {
    Ctx c{};
    c.path_throughput = t;
    return c;
}
inline Frame frame(const V& n, const V& t) { return rt::make_openpbr_frame(n, t); }
inline rt::OpenPbrEvaluation eval(const Mat& m, const Frame& f, const V& wo, const V& wi, const Ctx& c) {
    return rt::evaluate_openpbr_core(m, f, wo, wi, c);
}
inline rt::OpenPbrSample sample(const Mat& m, const Frame& f, const V& wo, float a, float b, float d, const Ctx& c) {
    return rt::sample_openpbr_core(m, f, wo, a, b, d, c);
}
inline rt::OpenPbrSample sample_boundary(const Mat& m, const Frame& f, const V& wo, float a, float b, float d, const Ctx& c) {
    return rt::openpbr_sample_subsurface_boundary(rt::openpbr_subsurface_boundary_material(m), f, wo, a, b, d, c);
}
inline rt::OpenPbrLobeProbabilities lobes(const Mat& m, float co, bool ext, const Ctx& c) {
    return rt::openpbr_lobe_probabilities(m, co, ext, c);
}
inline V emission(const Mat& m) { return rt::emission_openpbr_core(m); }
inline rt::OpenPbrSubsurfaceMedium medium(const Mat& m) { return rt::openpbr_subsurface_medium(m); }
inline rt::OpenPbrSubsurfaceSegment segment(const rt::OpenPbrSubsurfaceMedium& md, float d, float u, const Ctx& c) {
    return rt::openpbr_sample_subsurface_segment(md, d, u, c);
}
inline V hg(const V& in, float g, float a, float b) { return rt::openpbr_sample_henyey_greenstein(in, g, a, b); }
inline float srgb(float v) { return rt::openpbr_srgb_channel_to_linear(v); }
inline int ev(rt::OpenPbrScatterEvent e) { return static_cast<int>(e); }
inline V fr_t(const Frame& f) { return f.tangent; }
inline V fr_b(const Frame& f) { return f.bitangent; }
inline V fr_n(const Frame& f) { return f.normal; }
inline V md_albedo(const rt::OpenPbrSubsurfaceMedium& md) { return md.single_scattering_albedo; }
}  // namespace kat
#define KAT_EXPORT ref_openpbr_kat
#else
#include "openpbr.h"
namespace kat {
namespace p = rtgb::pbr;
using Mat = p::Mat;
using V = p::V3;
using Frame = p::Frame;
using Ctx = p::Context;
inline Ctx ctx_of(const V& t) {
    Ctx c = p::default_context();
    c.throughput = t;
    return c;
}
inline Frame frame(const V& n, const V& t) { return p::make_frame(n, t); }
inline p::Eval eval(const Mat& m, const Frame& f, const V& wo, const V& wi, const Ctx& c) { return p::evaluate(m, f, wo, wi, c); }
inline p::Sample sample(const Mat& m, const Frame& f, const V& wo, float a, float b, float d, const Ctx& c) {
    return p::sample(m, f, wo, a, b, d, c);
}
inline p::Sample sample_boundary(const Mat& m, const Frame& f, const V& wo, float a, float b, float d, const Ctx& c) {
    return p::sample_boundary(p::boundary_material(m), f, wo, a, b, d, c);
}
inline p::Lobes lobes(const Mat& m, float co, bool ext, const Ctx& c) { return p::lobe_probs(m, co, ext, c); }
inline V emission(const Mat& m) { return p::emission(m); }
inline p::Medium medium(const Mat& m) { return p::subsurface_medium(m); }
inline p::Segment segment(const p::Medium& md, float d, float u, const Ctx& c) { return p::subsurface_segment(md, d, u, c); }
inline V hg(const V& in, float g, float a, float b) { return p::sample_hg(in, g, a, b); }
inline float srgb(float v) { return p::srgb_to_linear(v); }
inline int ev(int e) { return e; }
inline V fr_t(const Frame& f) { return f.t; }
inline V fr_b(const Frame& f) { return f.b; }
inline V fr_n(const Frame& f) { return f.n; }
inline V md_albedo(const p::Medium& md) { return md.albedo; }
}  // namespace kat
#define KAT_EXPORT orc_openpbr_kat
#endif

static_assert(sizeof(kat::Mat) == 204, "OpenPBR parameter block must be 204 bytes");

namespace {

kat::V v3(const float* p) {
    kat::V v;
    v.x = p[0];
    v.y = p[1];
    v.z = p[2];
    return v;
}

void put(float* o, const kat::V& v) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
}

float as_word(int v) {
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}

void run_one(const float* in, float* out) {
    kat::Mat m;
    std::memcpy(&m, in, sizeof(kat::Mat));
    const kat::Frame f = kat::frame(v3(in + 51), v3(in + 54));
    const kat::V wo = v3(in + 57);
    const kat::V wi = v3(in + 60);
    const kat::Ctx c = kat::ctx_of(v3(in + 66));
    std::memset(out, 0, sizeof(float) * kKatOut);

    const auto e = kat::eval(m, f, wo, wi, c);
    put(out + 0, e.value);
    out[3] = e.pdf;

    const auto s = kat::sample(m, f, wo, in[63], in[64], in[65], c);
    put(out + 4, s.wi);
    put(out + 7, s.value);
    put(out + 10, s.weight);
    out[13] = s.pdf;
    out[14] = s.discrete_pdf;
    out[15] = as_word(kat::ev(s.event));
    out[16] = as_word(s.delta);
    out[17] = as_word(s.valid);

    for (int side = 0; side < 2; ++side) {
        const auto l = kat::lobes(m, in[71], side == 0, c);
        float* o = out + 18 + 6 * side;
        o[0] = l.diffuse;
        o[1] = l.subsurface;
        o[2] = l.reflection;
        o[3] = l.transmission;
        o[4] = l.coat;
        o[5] = l.fuzz;
    }
    put(out + 30, kat::emission(m));

    const auto md = kat::medium(m);
    put(out + 33, md.extinction);
    put(out + 36, kat::md_albedo(md));
    out[39] = md.anisotropy;
    out[40] = as_word(md.active);

    const auto sg = kat::segment(md, in[69], in[70], c);
    put(out + 41, sg.weight);
    out[44] = sg.distance;
    out[45] = as_word(sg.scattered);

    put(out + 46, kat::hg(wo, m.subsurface_scatter_anisotropy, in[64], in[65]));
    put(out + 49, kat::fr_t(f));
    put(out + 52, kat::fr_b(f));
    put(out + 55, kat::fr_n(f));
    out[58] = kat::srgb(in[72]);

    const auto b = kat::sample_boundary(m, f, wo, in[63], in[64], in[65], c);
    put(out + 59, b.wi);
    out[62] = as_word(kat::ev(b.event));
    out[63] = as_word(b.valid);
}

}  // namespace

// Runs the battery over n input records (kKatIn words each) into n output
// records (kKatOut words each). Returns the record widths packed as
// (kKatIn << 16) | kKatOut so callers can check the layout they assume.
extern "C" int KAT_EXPORT(const float* in, int n, float* out) {
    if (in != nullptr && out != nullptr) {
        for (int i = 0; i < n; ++i) run_one(in + static_cast<int64_t>(i) * kKatIn, out + static_cast<int64_t>(i) * kKatOut);
    }
    return (kKatIn << 16) | kKatOut;
}
