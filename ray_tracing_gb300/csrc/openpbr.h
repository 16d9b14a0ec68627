// OpenPBR surface BSDF (evaluation, sampling, emission, subsurface random walk)
// for host and device.
//
// Restates src/common/openpbr_core.h of the reference: GGX with visible-normal
// sampling and energy compensation, Oren-Nayar diffuse with the Fujii
// multiple-scattering term, coat (darkening, passage tint), fuzz (LTC lobe),
// thin-film Airy interference, Cauchy dispersion, thin-walled transmission and
// the subsurface random walk. The operation order follows the reference so a
// host build (-ffp-contract=off) reproduces its values bit for bit and a device
// build (--fmad=false) differs only by CUDA's transcendental ULPs. Like the
// reference header, one source serves the CPU oracle and the CUDA kernels.
#pragma once

#include <cmath>

// PBR_HD: small helpers, inlined everywhere. PBR_CALL: the large entry points
// (evaluate, sample), kept as real calls on the device so the many call sites
// of the shading kernels share one copy of their code.
#if defined(__CUDACC__)
#define PBR_HD __host__ __device__ __forceinline__
#define PBR_CALL __host__ __device__ inline __noinline__
#else
#define PBR_HD inline
#define PBR_CALL inline
#endif

namespace rtgb {
namespace pbr {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 1.0f / kPi;
constexpr float kLambdaC = 656.3f;  // Fraunhofer C, D, F lines (nm)
constexpr float kLambdaD = 587.6f;
constexpr float kLambdaF = 486.1f;

struct V3 {
    float x, y, z;
};

struct Context {
    V3 wavelengths;  // nm, for dispersion
    V3 throughput;   // path throughput, for channel selection
};

PBR_HD Context default_context() { return Context{{kLambdaC, kLambdaD, kLambdaF}, {1.0f, 1.0f, 1.0f}}; }

// OpenPbrCoreMaterial (openpbr_core.h:33-77) — the first 204 bytes of rtgb_openpbr_material.
struct Mat {
    float base_weight;
    V3 base_color;
    float base_diffuse_roughness;
    float base_metalness;
    float specular_weight;
    V3 specular_color;
    float specular_roughness;
    float specular_ior;
    float specular_roughness_anisotropy;
    float transmission_weight;
    V3 transmission_color;
    float transmission_depth;
    float transmission_dispersion_scale;
    float transmission_dispersion_abbe_number;
    float subsurface_weight;
    V3 subsurface_color;
    float subsurface_radius;
    V3 subsurface_radius_scale;
    float subsurface_scatter_anisotropy;
    float fuzz_weight;
    V3 fuzz_color;
    float fuzz_roughness;
    float coat_weight;
    V3 coat_color;
    float coat_roughness;
    float coat_roughness_anisotropy;
    float coat_ior;
    float coat_darkening;
    float thin_film_weight;
    float thin_film_thickness;
    float thin_film_ior;
    float emission_luminance;
    V3 emission_color;
    float geometry_opacity;
    int geometry_thin_walled;
};
static_assert(sizeof(Mat) == 204, "OpenPBR parameter block layout");

struct Frame {
    V3 t, b, n;
};

enum Event : int {
    kNone = 0,
    kDiffuseReflection = 1,
    kGlossyReflection = 2,
    kGlossyTransmission = 3,
    kThinWalledTransmission = 4,
    kOpacityPassthrough = 5,
    kCoatReflection = 6,
    kFuzzReflection = 7,
    kSubsurfaceEntry = 8,
    kSubsurfaceExit = 9,
};

struct Eval {
    V3 value;
    float pdf;
};

struct Sample {
    V3 wi, value, weight;
    float pdf, discrete_pdf;
    int event, delta, valid;
};

struct Lobes {
    float diffuse, subsurface, reflection, transmission, coat, fuzz;
};

struct Medium {
    V3 extinction, albedo;
    float anisotropy;
    int active;
};

struct Segment {
    V3 weight;
    float distance;
    int scattered;
};

struct Rough {
    float ax, ay;
};

// ---- scalar / vector helpers (openpbr_core.h:181-320) -----------------------------

PBR_HD float mn(float a, float b) { return a < b ? a : b; }
PBR_HD float mx(float a, float b) { return a > b ? a : b; }
PBR_HD float clampf(float v, float lo, float hi) { return mn(mx(v, lo), hi); }
PBR_HD float sat(float v) { return clampf(v, 0.0f, 1.0f); }
PBR_HD float sq(float v) { return v * v; }
PBR_HD float ssqrt(float v) { return sqrtf(mx(0.0f, v)); }
PBR_HD V3 splat(float v) { return V3{v, v, v}; }
PBR_HD V3 zero3() { return V3{0.0f, 0.0f, 0.0f}; }
PBR_HD V3 vadd(const V3& a, const V3& b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
PBR_HD V3 vsub(const V3& a, const V3& b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
PBR_HD V3 vmul(const V3& v, float s) { return V3{v.x * s, v.y * s, v.z * s}; }
PBR_HD V3 vmul(const V3& a, const V3& b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
PBR_HD V3 vdiv(const V3& v, float s) { return vmul(v, 1.0f / s); }
PBR_HD float comp(const V3& v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }
PBR_HD void set_comp(V3& v, int c, float x) {
    if (c == 0) v.x = x;
    else if (c == 1) v.y = x;
    else v.z = x;
}
PBR_HD V3 recip(const V3& v) { return V3{1.0f / mx(v.x, 1e-6f), 1.0f / mx(v.y, 1e-6f), 1.0f / mx(v.z, 1e-6f)}; }
PBR_HD V3 neg(const V3& v) { return V3{-v.x, -v.y, -v.z}; }
PBR_HD float vdot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PBR_HD V3 vcross(const V3& a, const V3& b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
PBR_HD float len2(const V3& v) { return vdot(v, v); }
PBR_HD V3 vnorm(const V3& v) {
    const float l2 = len2(v);
    if (l2 <= 1e-20f) return zero3();
    return vmul(v, 1.0f / sqrtf(l2));
}
PBR_HD V3 lerp3(const V3& a, const V3& b, float t) { return vadd(vmul(a, 1.0f - t), vmul(b, t)); }
PBR_HD V3 nonneg(const V3& v) { return V3{mx(0.0f, v.x), mx(0.0f, v.y), mx(0.0f, v.z)}; }
PBR_HD V3 unit3(const V3& v) { return V3{sat(v.x), sat(v.y), sat(v.z)}; }
PBR_HD V3 vsqrt(const V3& v) { return V3{ssqrt(v.x), ssqrt(v.y), ssqrt(v.z)}; }
PBR_HD V3 vpow(const V3& v, float e) { return V3{powf(mx(v.x, 0.0f), e), powf(mx(v.y, 0.0f), e), powf(mx(v.z, 0.0f), e)}; }

PBR_HD V3 channel_probs(const Context& ctx) {
    const V3 t{mx(0.0f, ctx.throughput.x), mx(0.0f, ctx.throughput.y), mx(0.0f, ctx.throughput.z)};
    const float total = t.x + t.y + t.z;
    return total > 1e-8f ? vdiv(t, total) : splat(1.0f / 3.0f);
}

PBR_HD int pick_channel(const Context& ctx, float u) {
    const V3 p = channel_probs(ctx);
    const float v = clampf(u, 0.0f, 0.99999994f);
    return v < p.x ? 0 : (v < p.x + p.y ? 1 : 2);
}

// ---- texture inputs (openpbr_core.h:322-358) ------------------------------------------

PBR_HD float srgb_to_linear(float v) { return v <= 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f); }

// source color space: 0 raw, 1 linear sRGB, 2 sRGB texture
PBR_HD V3 source_to_linear(const V3& v, int space) {
    if (space != 2) return v;
    return V3{srgb_to_linear(v.x), srgb_to_linear(v.y), srgb_to_linear(v.z)};
}

// input: 0 base color, 1 specular color, 2 transmission color, 3 emission color
PBR_HD void apply_color(Mat& m, int input, const V3& source, int space) {
    const V3 v = source_to_linear(source, space);
    if (input == 0) m.base_color = v;
    else if (input == 1) m.specular_color = v;
    else if (input == 2) m.transmission_color = v;
    else if (input == 3) m.emission_color = v;
}

// input: 0 base metalness, 1 specular roughness
PBR_HD void apply_scalar(Mat& m, int input, float v) {
    if (input == 0) m.base_metalness = v;
    else if (input == 1) m.specular_roughness = v;
}

PBR_HD float luminance(const V3& v) { return 0.2126f * mx(0.0f, v.x) + 0.7152f * mx(0.0f, v.y) + 0.0722f * mx(0.0f, v.z); }

// ---- transmission volume and subsurface (openpbr_core.h:360-519) ------------------------

PBR_HD V3 surface_transmission_color(const Mat& m) {
    if (m.geometry_thin_walled != 0 || m.transmission_depth <= 0.0f) return unit3(m.transmission_color);
    return splat(1.0f);
}

PBR_HD float ss_single_albedo(float observed, float anisotropy) {
    const float c = sat(observed);
    const float g = clampf(anisotropy, -0.999f, 0.999f);
    const float s = mx(0.0f, 4.09712f + 4.20863f * c - sqrtf(mx(0.0f, 9.59217f + 41.6808f * c + 17.7126f * c * c)));
    const float s2 = s * s;
    return sat((1.0f - s2) / mx(1.0f - g * s2, 1e-6f));
}

PBR_HD bool ss_finite_mfp(const Mat& m) {
    const float r = mx(0.0f, m.subsurface_radius);
    const V3 sc = nonneg(m.subsurface_radius_scale);
    return r * mx(sc.x, mx(sc.y, sc.z)) > 1e-6f;
}

PBR_HD bool random_walk(const Mat& m) {
    return m.geometry_thin_walled == 0 && sat(m.subsurface_weight) > 0.0f && sat(m.base_metalness) < 1.0f
           && sat(m.transmission_weight) < 1.0f && ss_finite_mfp(m);
}

PBR_HD bool thin_walled_ss(const Mat& m) { return m.geometry_thin_walled != 0 && sat(m.subsurface_weight) > 0.0f; }

PBR_HD float thin_walled_ss_prob(const Mat& m, bool transmission) {
    const float a = clampf(m.subsurface_scatter_anisotropy, -1.0f, 1.0f);
    return 0.5f * (1.0f + (transmission ? a : -a));
}

PBR_HD Medium subsurface_medium(const Mat& m) {
    Medium med{zero3(), zero3(), 0.0f, 0};
    if (!random_walk(m)) return med;
    const float r = mx(0.0f, m.subsurface_radius);
    const V3 rs = nonneg(m.subsurface_radius_scale);
    const V3 mfp{mx(r * rs.x, 1e-6f), mx(r * rs.y, 1e-6f), mx(r * rs.z, 1e-6f)};
    med.extinction = recip(mfp);
    const V3 c = unit3(m.subsurface_color);
    med.albedo = V3{ss_single_albedo(c.x, m.subsurface_scatter_anisotropy),
        ss_single_albedo(c.y, m.subsurface_scatter_anisotropy), ss_single_albedo(c.z, m.subsurface_scatter_anisotropy)};
    med.anisotropy = clampf(m.subsurface_scatter_anisotropy, -0.999f, 0.999f);
    med.active = 1;
    return med;
}

PBR_HD Segment subsurface_segment(const Medium& med, float boundary_distance, float u, const Context& ctx) {
    Segment seg{splat(1.0f), mx(0.0f, boundary_distance), 0};
    if (med.active == 0 || seg.distance <= 0.0f) return seg;
    const V3 contrib = vmul(nonneg(ctx.throughput), med.albedo);
    const float total = contrib.x + contrib.y + contrib.z;
    const V3 probs = total > 1e-12f ? vdiv(contrib, total) : splat(1.0f / 3.0f);
    const float choice = clampf(u, 0.0f, 0.99999994f);
    int channel = 2;
    float cu = 0.0f;
    float cdf = 0.0f;
    for (int i = 0; i < 3; ++i) {
        const float p = comp(probs, i);
        if (choice < cdf + p || i == 2) {
            channel = i;
            cu = (choice - cdf) / mx(p, 1e-8f);
            break;
        }
        cdf += p;
    }
    const float sigma = comp(med.extinction, channel);
    const float d = -logf(mx(1.0f - sat(cu), 1e-7f)) / mx(sigma, 1e-6f);
    seg.scattered = d < seg.distance ? 1 : 0;
    seg.distance = seg.scattered != 0 ? d : seg.distance;
    const float sd = mx(0.0f, seg.distance);
    const V3 tr{expf(-med.extinction.x * sd), expf(-med.extinction.y * sd), expf(-med.extinction.z * sd)};
    if (seg.scattered != 0) {
        const V3 density = vmul(med.extinction, tr);
        const float mix_pdf = vdot(probs, density);
        seg.weight = vdiv(vmul(density, med.albedo), mx(mix_pdf, 1e-12f));
    } else {
        const float survive = vdot(probs, tr);
        seg.weight = vdiv(tr, mx(survive, 1e-12f));
    }
    return seg;
}

// ---- frames (openpbr_core.h:521-590) --------------------------------------------------

PBR_HD float pow5(float v) {
    const float s = v * v;
    return s * s * v;
}

PBR_HD V3 schlick(const V3& c0, const V3& c90, float cosine) { return lerp3(c0, c90, pow5(1.0f - sat(cosine))); }

PBR_HD Frame make_frame(const V3& normal, const V3& tangent) {
    Frame f{V3{1.0f, 0.0f, 0.0f}, V3{0.0f, 1.0f, 0.0f}, V3{0.0f, 0.0f, 1.0f}};
    f.n = vnorm(normal);
    if (len2(f.n) <= 0.0f) f.n = V3{0.0f, 0.0f, 1.0f};
    const V3 proj = vsub(tangent, vmul(f.n, vdot(f.n, tangent)));
    if (len2(proj) > 1e-12f) {
        f.t = vnorm(proj);
    } else {
        const V3 helper = fabsf(f.n.z) < 0.999f ? V3{0.0f, 0.0f, 1.0f} : V3{0.0f, 1.0f, 0.0f};
        f.t = vnorm(vcross(helper, f.n));
    }
    f.b = vnorm(vcross(f.n, f.t));
    f.t = vnorm(vcross(f.b, f.n));
    return f;
}

PBR_HD Frame face(Frame f, const V3& wo) {
    if (vdot(f.n, wo) < 0.0f) {
        f.n = neg(f.n);
        f.b = neg(f.b);
    }
    return f;
}

PBR_HD V3 to_local(const Frame& f, const V3& v) { return V3{vdot(v, f.t), vdot(v, f.b), vdot(v, f.n)}; }
PBR_HD V3 to_world(const Frame& f, const V3& v) { return vadd(vadd(vmul(f.t, v.x), vmul(f.b, v.y)), vmul(f.n, v.z)); }

PBR_HD V3 sample_hg(const V3& incident, float anisotropy, float u1, float u2) {
    const float g = clampf(anisotropy, -0.999f, 0.999f);
    float c = 1.0f - 2.0f * sat(u1);
    if (fabsf(g) > 1e-3f) {
        const float ratio = (1.0f - g * g) / mx(1.0f - g + 2.0f * g * sat(u1), 1e-6f);
        c = clampf((1.0f + g * g - ratio * ratio) / (2.0f * g), -1.0f, 1.0f);
    }
    const float s = ssqrt(1.0f - c * c);
    const float phi = 2.0f * kPi * sat(u2);
    const V3 local{s * cosf(phi), s * sinf(phi), c};
    return vnorm(to_world(make_frame(vnorm(incident), zero3()), local));
}

// ---- Fresnel (openpbr_core.h:592-659) -------------------------------------------------

PBR_HD float fresnel_dielectric(float cosine, float eta) {
    cosine = clampf(cosine, -1.0f, 1.0f);
    eta = mx(eta, 1e-4f);
    if (cosine < 0.0f) {
        eta = 1.0f / eta;
        cosine = -cosine;
    }
    const float sin2_i = mx(0.0f, 1.0f - cosine * cosine);
    const float sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= 1.0f) return 1.0f;
    const float cos_t = ssqrt(1.0f - sin2_t);
    const float par = (eta * cosine - cos_t) / mx(eta * cosine + cos_t, 1e-8f);
    const float perp = (cosine - eta * cos_t) / mx(cosine + eta * cos_t, 1e-8f);
    return 0.5f * (par * par + perp * perp);
}

struct Polar {
    float p, s;
};

PBR_HD Polar fresnel_polarized(float cosine, float eta) {
    const float c2 = sq(sat(cosine));
    const float s2 = 1.0f - c2;
    const float t0 = mx(eta * eta - s2, 0.0f);
    const float t1 = t0 + c2;
    const float t2 = 2.0f * sqrtf(t0) * sat(cosine);
    const float rs = (t1 - t2) / mx(t1 + t2, 1e-8f);
    const float t3 = c2 * t0 + s2 * s2;
    const float t4 = t2 * s2;
    const float rp = rs * (t3 - t4) / mx(t3 + t4, 1e-8f);
    return Polar{rp, rs};
}

PBR_HD Polar fresnel_real_polarized(float cosine, float ior) {
    const float c2 = sq(sat(cosine));
    const float s2 = 1.0f - c2;
    const float i2 = ior * ior;
    const float t0 = i2 - s2;
    const float mag = fabsf(t0);
    const float t1 = mag + c2;
    const float a = ssqrt(0.5f * (mag + t0));
    const float t2 = 2.0f * a * sat(cosine);
    const float rs = (t1 - t2) / mx(t1 + t2, 1e-8f);
    const float t3 = c2 * mag + s2 * s2;
    const float t4 = t2 * s2;
    const float rp = rs * (t3 - t4) / mx(t3 + t4, 1e-8f);
    return Polar{rp, rs};
}

PBR_HD Polar reflection_phase(float cosine, float ior_i, float ior_t) {
    const float s2 = 1.0f - sq(sat(cosine));
    const float t2 = ior_t * ior_t;
    const float i2 = ior_i * ior_i;
    const float a = t2 - i2 * s2;
    const float u = ssqrt(0.5f * (a + fabsf(a)));
    const float sden = u * u - sq(ior_i * cosine);
    const float pden = sq(t2 * cosine) - i2 * u * u;
    return Polar{pden < 0.0f ? kPi : 0.0f, sden < 0.0f ? kPi : 0.0f};
}

// ---- thin film (openpbr_core.h:661-813): Belcour-Barla Airy summation with the
// published Gaussian fit of the CIE XYZ sensitivity, two orders.
PBR_HD V3 film_sensitivity(float opd, const V3& shift) {
    const float phase = 2.0f * kPi * opd;
    const V3 val{5.4856e-13f, 4.4201e-13f, 5.2481e-13f};
    const V3 pos{1.6810e6f, 1.7953e6f, 2.2084e6f};
    const V3 var{4.3278e9f, 9.3046e9f, 6.6121e9f};
    V3 xyz{val.x * sqrtf(2.0f * kPi * var.x) * cosf(pos.x * phase + shift.x) * expf(-var.x * phase * phase),
        val.y * sqrtf(2.0f * kPi * var.y) * cosf(pos.y * phase + shift.y) * expf(-var.y * phase * phase),
        val.z * sqrtf(2.0f * kPi * var.z) * cosf(pos.z * phase + shift.z) * expf(-var.z * phase * phase)};
    xyz.x += 9.7470e-14f * sqrtf(2.0f * kPi * 4.5282e9f) * cosf(2.2399e6f * phase + shift.x)
             * expf(-4.5282e9f * phase * phase);
    return vdiv(xyz, 1.0685e-7f);
}

PBR_HD V3 xyz_to_rgb(const V3& c) {
    return V3{2.3706743f * c.x - 0.9000405f * c.y - 0.4706338f * c.z, -0.5138850f * c.x + 1.4253036f * c.y + 0.0885814f * c.z,
        0.0052982f * c.x - 0.0146949f * c.y + 1.0093968f * c.z};
}

PBR_HD float f0_to_ior(float f0) {
    const float r = sqrtf(clampf(f0, 0.01f, 0.99f));
    return (1.0f + r) / mx(1.0f - r, 1e-5f);
}

PBR_HD float film_cos_t(float cosine, float ior_i, float ior_f) {
    const float ratio = ior_i / mx(ior_f, 1e-4f);
    const float s2 = (1.0f - sq(sat(cosine))) * ratio * ratio;
    return s2 < 1.0f ? ssqrt(1.0f - s2) : 0.0f;
}

PBR_HD V3 film_airy(float cosine, float thickness_nm, float ior_i, float ior_f, const V3& ior_sub,
    const V3& gen_reflectance, bool gen_schlick) {
    const float eta1 = mx(ior_i, 1e-4f);
    const float eta2 = mx(ior_f, 1e-4f);
    const float ct = sat(fabsf(cosine));
    const float ctt = film_cos_t(ct, eta1, eta2);
    if (ctt <= 0.0f) return splat(1.0f);
    const Polar r12 = fresnel_polarized(ct, eta2 / eta1);
    const Polar t121{1.0f - r12.p, 1.0f - r12.s};
    V3 r23p = zero3(), r23s = zero3(), phi23p = zero3(), phi23s = zero3();
    for (int c = 0; c < 3; ++c) {
        const float eta3 = comp(ior_sub, c);
        if (gen_schlick) {
            const float r = 0.5f * sat(comp(gen_reflectance, c));
            const float phase = eta3 < eta2 ? kPi : 0.0f;
            set_comp(r23p, c, r);
            set_comp(r23s, c, r);
            set_comp(phi23p, c, phase);
            set_comp(phi23s, c, phase);
        } else {
            const Polar r = fresnel_real_polarized(ctt, eta3 / eta2);
            const Polar ph = reflection_phase(ctt, eta2, eta3);
            set_comp(r23p, c, r.p);
            set_comp(r23s, c, r.s);
            set_comp(phi23p, c, ph.p);
            set_comp(phi23s, c, ph.s);
        }
    }
    const float brewster = eta1 / sqrtf(eta1 * eta1 + eta2 * eta2);
    const Polar phi21{ct < brewster ? 0.0f : kPi, kPi};
    const V3 r123p{sqrtf(mx(r12.p * r23p.x, 0.0f)), sqrtf(mx(r12.p * r23p.y, 0.0f)), sqrtf(mx(r12.p * r23p.z, 0.0f))};
    const V3 r123s{sqrtf(mx(r12.s * r23s.x, 0.0f)), sqrtf(mx(r12.s * r23s.y, 0.0f)), sqrtf(mx(r12.s * r23s.z, 0.0f))};
    const float opd = 2.0f * eta2 * ctt * thickness_nm * 1e-9f;
    const V3 rs{t121.p * t121.p * r23p.x / mx(1.0f - r12.p * r23p.x, 1e-6f),
        t121.p * t121.p * r23p.y / mx(1.0f - r12.p * r23p.y, 1e-6f),
        t121.p * t121.p * r23p.z / mx(1.0f - r12.p * r23p.z, 1e-6f)};
    V3 result = vadd(splat(r12.p), rs);
    V3 coef = vsub(rs, splat(t121.p));
    for (int order = 1; order <= 2; ++order) {
        coef = vmul(coef, r123p);
        const V3 shift = vmul(vadd(phi23p, splat(phi21.p)), static_cast<float>(order));
        result = vadd(result, vmul(coef, vmul(film_sensitivity(static_cast<float>(order) * opd, shift), 2.0f)));
    }
    const V3 rp{t121.s * t121.s * r23s.x / mx(1.0f - r12.s * r23s.x, 1e-6f),
        t121.s * t121.s * r23s.y / mx(1.0f - r12.s * r23s.y, 1e-6f),
        t121.s * t121.s * r23s.z / mx(1.0f - r12.s * r23s.z, 1e-6f)};
    result = vadd(result, vadd(splat(r12.s), rp));
    coef = vsub(rp, splat(t121.s));
    for (int order = 1; order <= 2; ++order) {
        coef = vmul(coef, r123s);
        const V3 shift = vmul(vadd(phi23s, splat(phi21.s)), static_cast<float>(order));
        result = vadd(result, vmul(coef, vmul(film_sensitivity(static_cast<float>(order) * opd, shift), 2.0f)));
    }
    return unit3(xyz_to_rgb(vmul(result, 0.5f)));
}

// ---- IOR, dispersion, roughness (openpbr_core.h:815-913) --------------------------------

PBR_HD float modulated_ior(const Mat& m) {
    const float eta = mx(m.specular_ior, 1e-4f);
    const float ratio = (eta - 1.0f) / (eta + 1.0f);
    const float f0 = clampf(mx(0.0f, m.specular_weight) * ratio * ratio, 0.0f, 0.9999f);
    const float sign = eta < 1.0f ? -1.0f : (eta > 1.0f ? 1.0f : 0.0f);
    const float e = sign * sqrtf(f0);
    return mx((1.0f + e) / mx(1.0f - e, 1e-4f), 1e-4f);
}

PBR_HD bool dispersive(const Mat& m) { return m.transmission_dispersion_scale > 0.0f && sat(m.base_metalness) < 1.0f; }

// Cauchy fit through the material's IOR at the D line with the given Abbe number.
PBR_HD float cauchy_ior(float ior0, float scale_in, float abbe, float nm) {
    const float scale = sat(scale_in);
    if (scale <= 0.0f || fabsf(ior0 - 1.0f) <= 1e-8f) return ior0;
    const bool inv = ior0 < 1.0f;
    const float ior = inv ? 1.0f / mx(ior0, 1e-6f) : ior0;
    const float v = mx(abbe, 1e-4f) / scale;
    const float f2 = 1.0f / sq(kLambdaF);
    const float c2 = 1.0f / sq(kLambdaC);
    const float b = (ior - 1.0f) / (v * (f2 - c2));
    const float a = ior - b / sq(kLambdaD);
    const float adj = a + b / sq(mx(nm, 1e-4f));
    return inv ? 1.0f / mx(adj, 1e-6f) : adj;
}

PBR_HD V3 dispersion_iors(const Mat& m, const Context& ctx) {
    const float ior = modulated_ior(m);
    if (!dispersive(m)) return splat(ior);
    return V3{cauchy_ior(ior, m.transmission_dispersion_scale, m.transmission_dispersion_abbe_number, ctx.wavelengths.x),
        cauchy_ior(ior, m.transmission_dispersion_scale, m.transmission_dispersion_abbe_number, ctx.wavelengths.y),
        cauchy_ior(ior, m.transmission_dispersion_scale, m.transmission_dispersion_abbe_number, ctx.wavelengths.z)};
}

PBR_HD Rough roughness(float r_in, float aniso_in) {
    const float r = sat(r_in);
    const float an = sat(aniso_in);
    const float aspect = 1.0f - an;
    const float scale = sqrtf(2.0f / mx(aspect * aspect + 1.0f, 1e-8f));
    const float ax = mx(r * r * scale, 1e-4f);
    return Rough{ax, mx(aspect * ax, 1e-4f)};
}

PBR_HD float effective_specular_roughness(const Mat& m) {
    const float s = sat(m.specular_roughness);
    const float c = sat(m.coat_roughness);
    const float s2 = s * s;
    const float c2 = c * c;
    const float affected = sqrtf(sqrtf(mn(1.0f, s2 * s2 + 2.0f * c2 * c2)));
    const float w = sat(m.coat_weight);
    return s + (affected - s) * w;
}

PBR_HD Rough spec_rough(const Mat& m) { return roughness(effective_specular_roughness(m), m.specular_roughness_anisotropy); }
PBR_HD Rough coat_rough(const Mat& m) { return roughness(m.coat_roughness, m.coat_roughness_anisotropy); }
PBR_HD bool smooth(const Rough& r) { return mx(r.ax, r.ay) < 1e-3f; }
PBR_HD bool smooth(const Mat& m) { return smooth(spec_rough(m)); }
PBR_HD float mean_alpha(const Rough& r) { return sqrtf(r.ax * r.ay); }

// ---- GGX (openpbr_core.h:915-1042) -----------------------------------------------------

// Rational fit of the GGX directional albedo (color0 / color90 split).
PBR_HD float ggx_albedo(float cosine, float alpha, float color0, float color90) {
    const float x = sat(cosine);
    const float y = sat(alpha);
    const float x2 = x * x;
    const float y2 = y * y;
    const float na = 0.1003f - 0.6303f * x + 9.748f * y - 2.038f * x * y + 29.34f * x2 - 8.245f * y2 - 26.44f * x2 * y
                     + 19.99f * x * y2 - 5.448f * x2 * y2;
    const float nb = 0.9345f - 2.323f * x + 2.229f * y - 3.748f * x * y + 1.424f * x2 - 0.7684f * y2 + 1.436f * x2 * y
                     + 0.2913f * x * y2 + 0.6286f * x2 * y2;
    const float da = 1.0f - 1.765f * x + 8.263f * y + 11.53f * x * y + 28.96f * x2 - 7.507f * y2 - 36.11f * x2 * y
                     + 15.86f * x * y2 + 33.37f * x2 * y2;
    const float db = 1.0f + 0.2281f * x + 15.94f * y - 55.83f * x * y + 13.08f * x2 + 41.26f * y2 + 54.9f * x2 * y
                     + 300.2f * x * y2 - 285.1f * x2 * y2;
    const float ca = sat(na / mx(da, 1e-6f));
    const float cb = sat(nb / mx(db, 1e-6f));
    return sat(color0) * ca + sat(color90) * cb;
}

PBR_HD V3 ggx_compensation(float cosine, float alpha, const V3& f_single) {
    if (alpha < 1e-3f) return splat(1.0f);
    const float e = ggx_albedo(cosine, alpha, 1.0f, 1.0f);
    const float missing = (1.0f - e) / mx(e, 1e-4f);
    return vadd(splat(1.0f), vmul(unit3(f_single), missing));
}

PBR_HD float ggx_d(const Rough& r, const V3& m) {
    if (m.z <= 0.0f) return 0.0f;
    const float x = m.x / r.ax;
    const float y = m.y / r.ay;
    const float den = x * x + y * y + m.z * m.z;
    return 1.0f / (kPi * r.ax * r.ay * den * den);
}

PBR_HD float ggx_lambda(const Rough& r, const V3& v) {
    const float az = fabsf(v.z);
    if (az <= 1e-8f) return 1e20f;
    const float proj = r.ax * r.ax * v.x * v.x + r.ay * r.ay * v.y * v.y;
    const float t2 = proj / (az * az);
    return 0.5f * (sqrtf(1.0f + t2) - 1.0f);
}

PBR_HD float ggx_g1(const Rough& r, const V3& v) { return 1.0f / (1.0f + ggx_lambda(r, v)); }
PBR_HD float ggx_g(const Rough& r, const V3& wo, const V3& wi) {
    return 1.0f / (1.0f + ggx_lambda(r, wo) + ggx_lambda(r, wi));
}

PBR_HD float vndf_pdf(const Rough& r, const V3& wo, const V3& m) {
    const float ac = fabsf(wo.z);
    if (ac <= 1e-8f) return 0.0f;
    return ggx_g1(r, wo) * ggx_d(r, m) * fabsf(vdot(wo, m)) / ac;
}

// Heitz's visible-normal sampling (stretch, sample the projected disk, unstretch).
PBR_HD V3 sample_vndf(const Rough& r, const V3& wo, float u1, float u2) {
    V3 wh = vnorm(V3{r.ax * wo.x, r.ay * wo.y, wo.z});
    if (wh.z < 0.0f) wh = neg(wh);
    const V3 t1 = wh.z < 0.99999f ? vnorm(vcross(V3{0.0f, 0.0f, 1.0f}, wh)) : V3{1.0f, 0.0f, 0.0f};
    const V3 t2 = vcross(wh, t1);
    const float rad = sqrtf(sat(u1));
    const float phi = 2.0f * kPi * sat(u2);
    const float dx = rad * cosf(phi);
    float dy = rad * sinf(phi);
    const float horizon = ssqrt(1.0f - dx * dx);
    const float warp = 0.5f * (1.0f + wh.z);
    dy = horizon * (1.0f - warp) + dy * warp;
    const float dz = ssqrt(1.0f - dx * dx - dy * dy);
    const V3 nh = vadd(vadd(vmul(t1, dx), vmul(t2, dy)), vmul(wh, dz));
    return vnorm(V3{r.ax * nh.x, r.ay * nh.y, mx(1e-6f, nh.z)});
}

PBR_HD V3 reflect_about(const V3& wo, const V3& m) { return vsub(vmul(m, 2.0f * vdot(wo, m)), wo); }

PBR_HD bool refract_through(const V3& wo, V3 m, float eta, float& eta_path, V3& wi) {
    float ci = vdot(m, wo);
    eta_path = mx(eta, 1e-4f);
    if (ci < 0.0f) {
        m = neg(m);
        ci = -ci;
        eta_path = 1.0f / eta_path;
    }
    const float s2i = mx(0.0f, 1.0f - ci * ci);
    const float s2t = s2i / (eta_path * eta_path);
    if (s2t >= 1.0f) return false;
    const float ct = ssqrt(1.0f - s2t);
    wi = vadd(vmul(wo, -1.0f / eta_path), vmul(m, ci / eta_path - ct));
    wi = vnorm(wi);
    return true;
}

// ---- coat (openpbr_core.h:1044-1107) ---------------------------------------------------

PBR_HD float coat_fresnel(const Mat& m, float cosine) { return fresnel_dielectric(cosine, mx(m.coat_ior, 1e-4f)); }

PBR_HD float coat_albedo(const Mat& m, float cosine) {
    const Rough r = coat_rough(m);
    if (smooth(r)) return coat_fresnel(m, cosine);
    const float a = mean_alpha(r);
    const float c0 = coat_fresnel(m, 1.0f);
    const float single = ggx_albedo(cosine, a, c0, 1.0f);
    const float white = ggx_albedo(cosine, a, 1.0f, 1.0f);
    const float comp_ = 1.0f + coat_fresnel(m, cosine) * (1.0f - white) / mx(white, 1e-4f);
    return sat(single * comp_);
}

PBR_HD V3 coat_passage(const Mat& m, float cosine) {
    const float presence = sat(m.coat_weight);
    const V3 tint = unit3(m.coat_color);
    if (presence <= 0.0f || cosine <= 0.0f || (tint.x >= 1.0f && tint.y >= 1.0f && tint.z >= 1.0f)) return splat(1.0f);
    const float eta = mx(m.coat_ior, 1e-4f);
    const float s2t = mx(0.0f, 1.0f - cosine * cosine) / (eta * eta);
    const float ct = ssqrt(1.0f - mn(s2t, 1.0f));
    const float scale = 1.0f / mx(ct, 1e-4f);
    return lerp3(splat(1.0f), vpow(vsqrt(tint), scale), presence);
}

PBR_HD V3 coat_darkening(const Mat& m) {
    const float presence = sat(m.coat_weight) * sat(m.coat_darkening);
    if (presence <= 0.0f) return splat(1.0f);
    const float eta = mx(m.coat_ior, 1e-4f);
    const float f0 = coat_fresnel(m, 1.0f);
    const float internal = sat(1.0f - (1.0f - f0) / mx(eta * eta, 1e-6f));
    const V3 dielectric = vmul(unit3(m.base_color), sat(m.base_weight));
    const V3 metal = vmul(dielectric, sat(m.specular_weight));
    const V3 base = lerp3(dielectric, metal, sat(m.base_metalness));
    const float num = 1.0f - internal;
    const V3 dark{num / mx(1.0f - base.x * internal, 1e-5f), num / mx(1.0f - base.y * internal, 1e-5f),
        num / mx(1.0f - base.z * internal, 1e-5f)};
    return lerp3(splat(1.0f), unit3(dark), presence);
}

// ---- fuzz (openpbr_core.h:1109-1209): Zeltner et al. sheen LTC fit ------------------------

PBR_HD float fuzz_albedo(float cosine, float rough_in) {
    const float x = sat(cosine);
    const float y = clampf(rough_in, 0.01f, 1.0f);
    const float s = y * (0.0206607f + 1.58491f * y) / (0.0379424f + y * (1.32227f + y));
    const float y2 = y * y;
    const float m = y * (-0.193854f + y * (-1.14885f + y * (1.7932f - 0.95943f * y2))) / (0.046391f + y);
    const float o = y * (0.000654023f + (-0.0207818f + 0.119681f * y) * y) / (1.26264f + y * (-1.92021f + y));
    const float z = (x - m) / mx(s, 1e-5f);
    const float g = expf(-0.5f * z * z) / (mx(s, 1e-5f) * sqrtf(2.0f * kPi));
    return sat(g + o);
}

PBR_HD Frame fuzz_frame(const V3& wo) {
    const V3 proj{wo.x, wo.y, 0.0f};
    const V3 t = len2(proj) > 1e-12f ? vnorm(proj) : V3{1.0f, 0.0f, 0.0f};
    return Frame{t, V3{-t.y, t.x, 0.0f}, V3{0.0f, 0.0f, 1.0f}};
}

PBR_HD V3 fuzz_ltc(float cosine, float rough_in) {
    const float x = sat(cosine);
    const float y = clampf(rough_in, 0.01f, 1.0f);
    const float ai = (2.58126f * x + 0.813703f * y) * y / (1.0f + 0.310327f * x * x + 2.60994f * x * y);
    const float bi = ssqrt(1.0f - x) * (y - 1.0f) * y * y * y / (0.0000254053f + 1.71228f * x - 1.71506f * x * y + 1.34174f * y * y);
    return V3{mx(ai, 1e-5f), bi, fuzz_albedo(x, y)};
}

PBR_HD float fuzz_pdf(const Mat& m, const V3& wo, const V3& wi) {
    if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    const Frame f = fuzz_frame(wo);
    const V3 al = to_local(f, wi);
    const V3 c = fuzz_ltc(wo.z, m.fuzz_roughness);
    const V3 tr{c.x * al.x + c.y * al.z, c.x * al.y, al.z};
    const float l2 = len2(tr);
    if (l2 <= 1e-16f || tr.z <= 0.0f) return 0.0f;
    const float j = c.x / l2;
    return tr.z * kInvPi * j * j;
}

PBR_HD V3 sample_fuzz(const Mat& m, const V3& wo, float u1, float u2) {
    const float rad = sqrtf(sat(u1));
    const float phi = 2.0f * kPi * sat(u2);
    const V3 cs{rad * cosf(phi), rad * sinf(phi), ssqrt(1.0f - rad * rad)};
    const V3 c = fuzz_ltc(wo.z, m.fuzz_roughness);
    const float ia = 1.0f / c.x;
    const V3 al = vnorm(V3{cs.x * ia - cs.z * c.y * ia, cs.y * ia, cs.z});
    return vnorm(to_world(fuzz_frame(wo), al));
}

PBR_HD V3 fuzz_value(const Mat& m, const V3& wo, const V3& wi) {
    const float presence = sat(m.fuzz_weight);
    if (presence <= 0.0f || wo.z <= 0.0f || wi.z <= 0.0f) return zero3();
    const float refl = fuzz_albedo(wo.z, m.fuzz_roughness);
    const float density = fuzz_pdf(m, wo, wi);
    return vmul(unit3(m.fuzz_color), presence * refl * density / mx(wi.z, 1e-6f));
}

PBR_HD float fuzz_base_scale(const Mat& m, float co, float ci, bool exterior) {
    if (!exterior) return 1.0f;
    const float presence = sat(m.fuzz_weight);
    const float out = 1.0f - presence * fuzz_albedo(co, m.fuzz_roughness);
    const float in = ci > 0.0f ? 1.0f - presence * fuzz_albedo(ci, m.fuzz_roughness) : 1.0f;
    return sat(out) * sat(in);
}

PBR_HD V3 coat_base_scale(const Mat& m, float co, float ci, bool exterior) {
    const float presence = sat(m.coat_weight);
    if (presence <= 0.0f) return splat(1.0f);
    if (!exterior) return ci < 0.0f ? coat_passage(m, -ci) : splat(1.0f);
    const float ro = presence * coat_albedo(m, co);
    const V3 out = vmul(coat_passage(m, co), sat(1.0f - ro));
    V3 in = splat(1.0f);
    if (ci > 0.0f) {
        const float ri = presence * coat_albedo(m, ci);
        in = vmul(coat_passage(m, ci), sat(1.0f - ri));
    }
    return vmul(vmul(out, in), coat_darkening(m));
}

PBR_HD V3 substrate_scale(const Mat& m, float co, float ci, bool exterior) {
    return vmul(coat_base_scale(m, co, ci, exterior), fuzz_base_scale(m, co, ci, exterior));
}

PBR_HD V3 coat_value(const Mat& m, const V3& wo, const V3& wi) {
    const float presence = sat(m.coat_weight);
    if (presence <= 0.0f || wo.z <= 0.0f || wi.z <= 0.0f) return zero3();
    const Rough r = coat_rough(m);
    if (smooth(r)) return zero3();
    const V3 sum = vadd(wi, wo);
    if (len2(sum) <= 1e-16f) return zero3();
    V3 wm = vnorm(sum);
    if (wm.z < 0.0f) wm = neg(wm);
    const float om = vdot(wo, wm);
    if (om <= 0.0f) return zero3();
    const float d = ggx_d(r, wm);
    const float g = ggx_g(r, wo, wi);
    const float f = coat_fresnel(m, om);
    const float c = ggx_compensation(wo.z, mean_alpha(r), splat(f)).x;
    return splat(presence * f * c * d * g / mx(4.0f * wo.z * wi.z, 1e-8f));
}

PBR_HD float coat_pdf(const Mat& m, const V3& wo, const V3& wi) {
    if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    const Rough r = coat_rough(m);
    if (smooth(r)) return 0.0f;
    const V3 sum = vadd(wi, wo);
    if (len2(sum) <= 1e-16f) return 0.0f;
    V3 wm = vnorm(sum);
    if (wm.z < 0.0f) wm = neg(wm);
    const float om = vdot(wo, wm);
    if (om <= 0.0f) return 0.0f;
    return vndf_pdf(r, wo, wm) / mx(4.0f * fabsf(om), 1e-8f);
}

// ---- base reflectances (openpbr_core.h:1475-1677) ---------------------------------------

PBR_HD float dielectric_fresnel(const Mat& m, float cosine, bool entering) {
    float eta = modulated_ior(m);
    if (m.geometry_thin_walled == 0 && !entering) eta = 1.0f / eta;
    float f = fresnel_dielectric(cosine, eta);
    if (m.geometry_thin_walled != 0 && f < 1.0f) {
        const float t = 1.0f - f;
        f += t * t * f / mx(1.0f - f * f, 1e-6f);
    }
    return sat(f);
}

// F82-tint metal Fresnel (Kutz/Hoffman) at the edge cosine 1/7.
PBR_HD V3 metal_fresnel(const Mat& m, float cosine) {
    constexpr float kEdge = 1.0f / 7.0f;
    const float mu = sat(fabsf(cosine));
    const V3 c0 = vmul(unit3(m.base_color), sat(m.base_weight));
    const V3 c90 = splat(1.0f);
    const V3 s = schlick(c0, c90, mu);
    const V3 s_edge = schlick(c0, c90, kEdge);
    const V3 want = vmul(s_edge, unit3(m.specular_color));
    const float omu = 1.0f - mu;
    const float oedge = 1.0f - kEdge;
    const float corr = mu * pow5(omu) * omu / (kEdge * pow5(oedge) * oedge);
    const V3 f82 = vsub(s, vmul(vsub(s_edge, want), corr));
    return vmul(unit3(f82), sat(m.specular_weight));
}

PBR_HD float weighted_coat_ior(const Mat& m) { return 1.0f + sat(m.coat_weight) * (mx(m.coat_ior, 1e-4f) - 1.0f); }

PBR_HD V3 thin_wall_window(const V3& iface) {
    const V3 r = unit3(iface);
    return V3{sat(r.x + sq(1.0f - r.x) * r.x / mx(1.0f - r.x * r.x, 1e-6f)),
        sat(r.y + sq(1.0f - r.y) * r.y / mx(1.0f - r.y * r.y, 1e-6f)), sat(r.z + sq(1.0f - r.z) * r.z / mx(1.0f - r.z * r.z, 1e-6f))};
}

PBR_HD V3 apply_film(const Mat& m, float cosine, const V3& base, float ior_i, const V3& ior_sub, const V3& gen, bool gen_schlick) {
    const float w = sat(m.thin_film_weight);
    const float nm = mx(m.thin_film_thickness, 0.0f) * 1000.0f;
    if (w <= 0.0f || nm <= 0.0f) return base;
    V3 film = film_airy(cosine, nm, ior_i, m.thin_film_ior, ior_sub, gen, gen_schlick);
    if (m.geometry_thin_walled != 0 && !gen_schlick) film = thin_wall_window(film);
    return lerp3(base, film, w);
}

PBR_HD V3 dielectric_reflectance(const Mat& m, float cosine, bool entering, const Context& ctx) {
    if (!dispersive(m)) {
        const float base = dielectric_fresnel(m, cosine, entering);
        const float bior = modulated_ior(m);
        const float cior = weighted_coat_ior(m);
        const float iior = entering ? cior : bior;
        const float sior = entering ? bior : cior;
        return apply_film(m, cosine, splat(base), iior, splat(sior), zero3(), false);
    }
    const V3 iors = dispersion_iors(m, ctx);
    const V3 paths = entering ? iors : recip(iors);
    V3 base{fresnel_dielectric(cosine, paths.x), fresnel_dielectric(cosine, paths.y), fresnel_dielectric(cosine, paths.z)};
    if (m.geometry_thin_walled != 0) base = thin_wall_window(base);
    const float cior = weighted_coat_ior(m);
    if (entering) return apply_film(m, cosine, base, cior, iors, zero3(), false);
    V3 out = zero3();
    for (int c = 0; c < 3; ++c) {
        const V3 film = apply_film(m, cosine, base, comp(iors, c), splat(cior), zero3(), false);
        set_comp(out, c, comp(film, c));
    }
    return out;
}

PBR_HD V3 metal_reflectance(const Mat& m, float cosine) {
    const V3 base = metal_fresnel(m, cosine);
    const float iior = weighted_coat_ior(m);
    const float ctt = film_cos_t(cosine, iior, m.thin_film_ior);
    const V3 at_film = metal_fresnel(m, ctt);
    const V3 normal = metal_fresnel(m, 1.0f);
    const V3 sub{iior * f0_to_ior(normal.x), iior * f0_to_ior(normal.y), iior * f0_to_ior(normal.z)};
    return apply_film(m, cosine, base, iior, sub, at_film, true);
}

PBR_HD Lobes lobe_probs(const Mat& m, float co, bool exterior, const Context& ctx) {
    const float metal = sat(m.base_metalness);
    const float trans = sat(m.transmission_weight);
    const float bw = sat(m.base_weight);
    const float msw = sat(m.specular_weight);
    const float eta = modulated_ior(m);
    const float er = (eta - 1.0f) / (eta + 1.0f);
    const float f0 = er * er;
    float dsr = f0;
    float msr = msw * luminance(vmul(unit3(m.base_color), bw));
    if ((m.thin_film_weight > 0.0f && m.thin_film_thickness > 0.0f) || dispersive(m)) {
        dsr = luminance(dielectric_reflectance(m, co, true, ctx));
        msr = luminance(metal_reflectance(m, co));
    }
    const float opaque = (1.0f - metal) * (1.0f - trans) * sat(1.0f - dsr);
    const float ssw = sat(m.subsurface_weight);
    float diffuse = 0.0f;
    float subsurface = 0.0f;
    if (ssw <= 0.0f) {
        diffuse = opaque * bw * luminance(unit3(m.base_color));
    } else {
        const bool rw = random_walk(m);
        const bool tw = thin_walled_ss(m);
        const float local_ss = rw || tw ? 0.0f : ssw;
        const V3 local_color = vadd(vmul(unit3(m.base_color), bw * (1.0f - ssw)), vmul(unit3(m.subsurface_color), local_ss));
        diffuse = opaque * luminance(local_color);
        if (rw || tw) subsurface = opaque * ssw * luminance(unit3(m.subsurface_color));
    }
    const float dielectric_refl = (1.0f - metal) * dsr * luminance(unit3(m.specular_color));
    const float metal_refl = metal * msr;
    const float transmission = (1.0f - metal) * trans * sat(1.0f - dsr) * luminance(surface_transmission_color(m));
    const float coat = exterior ? sat(m.coat_weight) * coat_albedo(m, co) : 0.0f;
    const float fuzz = exterior ? sat(m.fuzz_weight) * fuzz_albedo(co, m.fuzz_roughness) * luminance(unit3(m.fuzz_color)) : 0.0f;
    const float sub_scale = sat(1.0f - coat) * sat(1.0f - fuzz);
    const float d = diffuse * sub_scale;
    const float s = subsurface * sub_scale;
    const float r = (dielectric_refl + metal_refl) * sub_scale;
    const float t = transmission * sub_scale;
    const float total = d + s + r + t + coat + fuzz;
    if (total <= 1e-10f) return Lobes{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    return Lobes{d / total, s / total, r / total, t / total, coat / total, fuzz / total};
}

// ---- diffuse: energy-preserving Oren-Nayar (Fujii) (openpbr_core.h:1389-1473) -----------

PBR_HD float on_albedo(float cosine, float rough) {
    constexpr float k1 = 0.5f - 2.0f / (3.0f * kPi);
    const float c = clampf(cosine, 1e-6f, 1.0f);
    const float sigma = sat(rough);
    const float a = 1.0f / (1.0f + k1 * sigma);
    const float b = sigma * a;
    const float s = ssqrt(1.0f - c * c);
    const float g = s * (acosf(c) - s * c) + 2.0f * ((s / c) * (1.0f - s * s * s) - s) / 3.0f;
    return sat(a + b * g * kInvPi);
}

PBR_HD float on_average(float rough) {
    constexpr float k1 = 0.5f - 2.0f / (3.0f * kPi);
    constexpr float k2 = 2.0f / 3.0f - 28.0f / (15.0f * kPi);
    const float sigma = sat(rough);
    const float a = 1.0f / (1.0f + k1 * sigma);
    return sat(a * (1.0f + k2 * sigma));
}

PBR_HD V3 diffuse_value(const Mat& m, const V3& wo, const V3& wi) {
    if (wo.z <= 0.0f || wi.z <= 0.0f) return zero3();
    const float metal = sat(m.base_metalness);
    const float trans = sat(m.transmission_weight);
    const float ssw = sat(m.subsurface_weight);
    float mix_ = sat(m.base_weight);
    V3 color = unit3(m.base_color);
    if (ssw > 0.0f) {
        const float bmix = sat(m.base_weight) * (1.0f - ssw);
        const float smix = random_walk(m) || thin_walled_ss(m) ? 0.0f : ssw;
        mix_ = bmix + smix;
        color = unit3(vdiv(vadd(vmul(unit3(m.base_color), bmix), vmul(unit3(m.subsurface_color), smix)), mx(mix_, 1e-8f)));
    }
    const float coef = mix_ * (1.0f - metal) * (1.0f - trans);
    if (coef <= 0.0f) return zero3();
    constexpr float k1 = 0.5f - 2.0f / (3.0f * kPi);
    const float sigma = sat(m.base_diffuse_roughness);
    const float a = 1.0f / (1.0f + k1 * sigma);
    const float s = vdot(wi, wo) - wi.z * wo.z;
    const float s_over_t = s > 0.0f ? s / mx(wi.z, wo.z) : s;
    const V3 single = vmul(color, a * (1.0f + sigma * s_over_t));
    const float ein = on_albedo(wi.z, sigma);
    const float eout = on_albedo(wo.z, sigma);
    const float eavg = on_average(sigma);
    const float missing = mx(1.0f - eavg, 1e-6f);
    const V3 c2 = vmul(color, color);
    const V3 ms_color{c2.x * eavg / mx(1.0f - color.x * (1.0f - eavg), 1e-6f), c2.y * eavg / mx(1.0f - color.y * (1.0f - eavg), 1e-6f),
        c2.z * eavg / mx(1.0f - color.z * (1.0f - eavg), 1e-6f)};
    const float ms_scale = (1.0f - ein) * (1.0f - eout) / missing;
    return vmul(vadd(single, vmul(ms_color, ms_scale)), coef * kInvPi);
}

PBR_HD V3 thin_walled_ss_value(const Mat& m, const V3& wo, const V3& wi, bool transmission) {
    if (!thin_walled_ss(m)) return zero3();
    Mat d = m;
    d.base_weight = sat(m.subsurface_weight) * thin_walled_ss_prob(m, transmission);
    d.base_color = unit3(m.subsurface_color);
    d.subsurface_weight = 0.0f;
    return diffuse_value(d, wo, wi);
}

PBR_HD V3 dielectric_albedo_rgb(const Mat& m, float cosine, bool entering, const Context& ctx) {
    if ((m.thin_film_weight <= 0.0f || m.thin_film_thickness <= 0.0f) && !dispersive(m)) {
        const Rough r = spec_rough(m);
        const float a = mean_alpha(r);
        if (smooth(m)) return splat(dielectric_fresnel(m, cosine, entering));
        const float c0 = dielectric_fresnel(m, 1.0f, entering);
        if (c0 <= 1e-8f) return zero3();
        const float single = ggx_albedo(cosine, a, c0, 1.0f);
        const float white = ggx_albedo(cosine, a, 1.0f, 1.0f);
        const float df = dielectric_fresnel(m, cosine, entering);
        const float comp_ = 1.0f + df * (1.0f - white) / mx(white, 1e-4f);
        return splat(sat(single * comp_));
    }
    const Rough r = spec_rough(m);
    const float a = mean_alpha(r);
    const V3 mirror = dielectric_reflectance(m, cosine, entering, ctx);
    if (smooth(m)) return mirror;
    const V3 c0 = dielectric_reflectance(m, 1.0f, entering, ctx);
    const V3 rough{ggx_albedo(cosine, a, c0.x, 1.0f), ggx_albedo(cosine, a, c0.y, 1.0f), ggx_albedo(cosine, a, c0.z, 1.0f)};
    return lerp3(mirror, rough, sqrtf(sat(a)));
}

PBR_HD V3 reflection_fresnel(const Mat& m, float cm, float co, bool entering, const Context& ctx) {
    const float metal = sat(m.base_metalness);
    const float a = mean_alpha(spec_rough(m));
    const V3 df = dielectric_reflectance(m, cm, entering, ctx);
    const V3 ds = vmul(entering || m.geometry_thin_walled != 0 ? unit3(m.specular_color) : splat(1.0f), df);
    const V3 dielectric = vmul(ds, ggx_compensation(co, a, df));
    const V3 ms = metal_reflectance(m, cm);
    const V3 metal_v = vmul(ms, ggx_compensation(co, a, ms));
    return lerp3(dielectric, metal_v, metal);
}

// ---- evaluate_openpbr_core (openpbr_core.h:1679-1860) ---------------------------------

// The body, inlined where the call is hot (the shade kernel's next-event
// estimation, the BSDF sampler's own evaluation); `evaluate` below is the
// out-of-line copy the ReSTIR kernels' many call sites share.
PBR_HD Eval evaluate_inline(const Mat& m, Frame f, const V3& wo_world, const V3& wi_world, const Context& ctx) {
    Eval res{zero3(), 0.0f};
    const V3 won = vnorm(wo_world);
    const V3 win = vnorm(wi_world);
    if (len2(won) <= 0.0f || len2(win) <= 0.0f) return res;
    const bool entering = m.geometry_thin_walled != 0 || vdot(f.n, won) >= 0.0f;
    f = face(f, won);
    const V3 wo = to_local(f, won);
    const V3 wi = to_local(f, win);
    if (wo.z <= 1e-7f || fabsf(wi.z) <= 1e-7f) return res;
    const float opacity = sat(m.geometry_opacity);
    const bool exterior = entering;
    const Lobes p = lobe_probs(m, wo.z, exterior, ctx);
    const Rough r = spec_rough(m);
    const bool is_smooth = smooth(r);
    if (wi.z * wo.z > 0.0f) {
        const V3 atten = vsub(splat(1.0f), dielectric_albedo_rgb(m, wo.z, entering, ctx));
        res.value = vadd(diffuse_value(m, wo, wi), thin_walled_ss_value(m, wo, wi, false));
        res.value = vmul(res.value, unit3(atten));
        res.pdf = p.diffuse * wi.z * kInvPi;
        if (thin_walled_ss(m)) res.pdf += p.subsurface * thin_walled_ss_prob(m, false) * wi.z * kInvPi;
        const V3 sum = vadd(wi, wo);
        if (!is_smooth && len2(sum) > 1e-16f) {
            V3 wm = vnorm(sum);
            if (wm.z < 0.0f) wm = neg(wm);
            const float om = vdot(wo, wm);
            if (om > 0.0f) {
                const float d = ggx_d(r, wm);
                const float g = ggx_g(r, wo, wi);
                const V3 fr = reflection_fresnel(m, om, wo.z, entering, ctx);
                res.value = vadd(res.value, vmul(fr, d * g / mx(4.0f * wo.z * wi.z, 1e-8f)));
                res.pdf += p.reflection * (vndf_pdf(r, wo, wm) / mx(4.0f * fabsf(om), 1e-8f));
            }
        }
        res.value = vmul(res.value, substrate_scale(m, wo.z, wi.z, exterior));
        if (exterior) {
            const V3 coat = vmul(coat_value(m, wo, wi), fuzz_base_scale(m, wo.z, wi.z, true));
            res.value = vadd(res.value, coat);
            res.value = vadd(res.value, fuzz_value(m, wo, wi));
            res.pdf += p.coat * coat_pdf(m, wo, wi);
            res.pdf += p.fuzz * fuzz_pdf(m, wo, wi);
        }
    } else if (thin_walled_ss(m) && p.subsurface > 0.0f) {
        const V3 wr{wi.x, wi.y, -wi.z};
        const V3 atten = vsub(splat(1.0f), dielectric_albedo_rgb(m, wo.z, true, ctx));
        res.value = thin_walled_ss_value(m, wo, wr, true);
        res.value = vmul(res.value, vmul(unit3(atten), substrate_scale(m, wo.z, wi.z, true)));
        res.pdf = p.subsurface * thin_walled_ss_prob(m, true) * fabsf(wi.z) * kInvPi;
    } else if (!is_smooth && m.geometry_thin_walled == 0 && p.transmission > 0.0f) {
        if (!dispersive(m)) {
            const float eta = modulated_ior(m);
            const float ep = entering ? eta : 1.0f / eta;
            const V3 sum = vadd(vmul(wi, ep), wo);
            if (len2(sum) > 1e-16f) {
                V3 wm = vnorm(sum);
                if (wm.z < 0.0f) wm = neg(wm);
                const float im = vdot(wi, wm);
                const float om = vdot(wo, wm);
                if (im * wi.z > 0.0f && om * wo.z > 0.0f) {
                    const V3 refl = dielectric_reflectance(m, om, entering, default_context());
                    const float hd = im + om / ep;
                    const float d2 = hd * hd;
                    if (d2 > 1e-16f) {
                        const float d = ggx_d(r, wm);
                        const float g = ggx_g(r, wo, wi);
                        float t = d * g * fabsf(im * om / (wi.z * wo.z * d2));
                        t /= ep * ep;
                        t *= (1.0f - sat(m.base_metalness)) * sat(m.transmission_weight);
                        res.value = vmul(vmul(surface_transmission_color(m), unit3(vsub(splat(1.0f), refl))), t);
                        res.pdf = p.transmission * (vndf_pdf(r, wo, wm) * (fabsf(im) / d2));
                    }
                }
            }
        } else {
            const V3 iors = dispersion_iors(m, ctx);
            const V3 eps = entering ? iors : recip(iors);
            const V3 tc = surface_transmission_color(m);
            const float ms = (1.0f - sat(m.base_metalness)) * sat(m.transmission_weight);
            V3 cpdf = zero3();
            for (int c = 0; c < 3; ++c) {
                const float ep = comp(eps, c);
                const V3 sum = vadd(vmul(wi, ep), wo);
                if (len2(sum) <= 1e-16f) continue;
                V3 wm = vnorm(sum);
                if (wm.z < 0.0f) wm = neg(wm);
                const float im = vdot(wi, wm);
                const float om = vdot(wo, wm);
                if (im * wi.z <= 0.0f || om * wo.z <= 0.0f) continue;
                const float hd = im + om / ep;
                const float d2 = hd * hd;
                if (d2 <= 1e-16f) continue;
                const float d = ggx_d(r, wm);
                const float g = ggx_g(r, wo, wi);
                float t = d * g * fabsf(im * om / (wi.z * wo.z * d2));
                t *= ms / (ep * ep);
                const V3 refl = dielectric_reflectance(m, om, entering, ctx);
                set_comp(res.value, c, comp(tc, c) * sat(1.0f - comp(refl, c)) * t);
                set_comp(cpdf, c, vndf_pdf(r, wo, wm) * (fabsf(im) / d2));
            }
            res.pdf = p.transmission * vdot(cpdf, channel_probs(ctx));
        }
        res.value = vmul(res.value, substrate_scale(m, wo.z, wi.z, exterior));
    }
    res.value = vmul(res.value, opacity);
    res.pdf *= opacity;
    return res;
}

PBR_CALL Eval evaluate(const Mat& m, Frame f, const V3& wo_world, const V3& wi_world, const Context& ctx) {
    return evaluate_inline(m, f, wo_world, wi_world, ctx);
}

// emission_openpbr_core (openpbr_core.h:1868-1883)
PBR_HD V3 emission(const Mat& m) {
    V3 e = vmul(nonneg(m.emission_color), mx(0.0f, m.emission_luminance) * sat(m.geometry_opacity));
    const float coat_t = 1.0f - sat(m.coat_weight) * coat_albedo(m, 1.0f);
    e = vmul(e, vmul(coat_passage(m, 1.0f), sat(coat_t)));
    const float fuzz_t = 1.0f - sat(m.fuzz_weight) * fuzz_albedo(1.0f, m.fuzz_roughness);
    return vmul(e, sat(fuzz_t));
}

PBR_HD V3 cosine_hemisphere(float u1, float u2) {
    const float rad = sqrtf(sat(u1));
    const float phi = 2.0f * kPi * sat(u2);
    return V3{rad * cosf(phi), rad * sinf(phi), ssqrt(1.0f - rad * rad)};
}

PBR_HD Mat boundary_material(const Mat& m) {
    Mat b = m;
    b.base_weight = 0.0f;
    b.base_metalness = 0.0f;
    b.transmission_weight = 1.0f;
    b.transmission_color = splat(1.0f);
    b.transmission_depth = 0.0f;
    b.transmission_dispersion_scale = 0.0f;
    b.subsurface_weight = 0.0f;
    b.fuzz_weight = 0.0f;
    b.coat_weight = 0.0f;
    b.geometry_opacity = 1.0f;
    return b;
}

PBR_HD Sample empty_sample() {
    Sample s;
    s.wi = zero3();
    s.value = zero3();
    s.weight = zero3();
    s.pdf = 0.0f;
    s.discrete_pdf = 0.0f;
    s.event = kNone;
    s.delta = 0;
    s.valid = 0;
    return s;
}

PBR_HD Sample finish_from_eval(Sample s, const Mat& m, const Frame& authored, const Frame& f, const V3& won, const V3& wi,
    const Context& ctx) {
    s.wi = vnorm(to_world(f, wi));
    const Eval e = evaluate_inline(m, authored, won, s.wi, ctx);
    if (e.pdf <= 1e-12f) return empty_sample();
    s.value = e.value;
    s.pdf = e.pdf;
    s.weight = vmul(e.value, fabsf(vdot(f.n, s.wi)) / e.pdf);
    s.valid = 1;
    return s;
}

// openpbr_sample_subsurface_boundary (openpbr_core.h:1907-1993)
PBR_HD Sample sample_boundary(const Mat& m, Frame f, const V3& wo_world, float u_lobe, float u1, float u2, const Context& ctx) {
    Sample s = empty_sample();
    const V3 won = vnorm(wo_world);
    if (len2(won) <= 0.0f) return s;
    const Frame authored = f;
    const bool entering = vdot(f.n, won) >= 0.0f;
    f = face(f, won);
    const V3 wo = to_local(f, won);
    if (wo.z <= 1e-7f) return s;
    const Lobes p = lobe_probs(m, wo.z, false, ctx);
    const float choice = clampf(u_lobe, 0.0f, 0.99999994f);
    V3 wi = zero3();
    if (choice < p.reflection) {
        if (smooth(m)) {
            wi = V3{-wo.x, -wo.y, wo.z};
            s.wi = vnorm(to_world(f, wi));
            s.discrete_pdf = p.reflection;
            if (s.discrete_pdf <= 0.0f) return empty_sample();
            s.weight = vdiv(reflection_fresnel(m, wo.z, wo.z, entering, ctx), s.discrete_pdf);
            s.event = kGlossyReflection;
            s.delta = 1;
            s.valid = 1;
            return s;
        }
        const V3 wm = sample_vndf(spec_rough(m), wo, u1, u2);
        wi = reflect_about(wo, wm);
        if (wi.z <= 1e-7f) return s;
        s.event = kGlossyReflection;
    } else {
        const float eta = modulated_ior(m);
        const float mep = entering ? eta : 1.0f / eta;
        float ep = 1.0f;
        V3 wm{0.0f, 0.0f, 1.0f};
        if (!smooth(m)) wm = sample_vndf(spec_rough(m), wo, u1, u2);
        if (!refract_through(wo, wm, mep, ep, wi) || (!smooth(m) && wi.z >= -1e-7f)) return s;
        if (smooth(m)) {
            const V3 t = unit3(vsub(splat(1.0f), dielectric_reflectance(m, wo.z, entering, ctx)));
            s.wi = vnorm(to_world(f, wi));
            s.discrete_pdf = p.transmission;
            if (s.discrete_pdf <= 0.0f) return empty_sample();
            s.weight = vdiv(vmul(t, 1.0f / (ep * ep)), s.discrete_pdf);
            s.event = kGlossyTransmission;
            s.delta = 1;
            s.valid = 1;
            return s;
        }
        s.event = kGlossyTransmission;
    }
    return finish_from_eval(s, m, authored, f, won, wi, ctx);
}

// sample_openpbr_core (openpbr_core.h:1995-2297)
PBR_CALL Sample sample(const Mat& m, Frame f, const V3& wo_world, float u_lobe, float u1, float u2, const Context& ctx) {
    Sample s = empty_sample();
    const V3 won = vnorm(wo_world);
    if (len2(won) <= 0.0f) return s;
    const Frame authored = f;
    const bool entering = m.geometry_thin_walled != 0 || vdot(f.n, won) >= 0.0f;
    f = face(f, won);
    const V3 wo = to_local(f, won);
    if (wo.z <= 1e-7f) return s;
    const float opacity = sat(m.geometry_opacity);
    const float pass = 1.0f - opacity;
    u_lobe = sat(u_lobe);
    if (u_lobe < pass) {
        s.wi = neg(won);
        s.weight = splat(1.0f);
        s.discrete_pdf = pass;
        s.event = kOpacityPassthrough;
        s.delta = 1;
        s.valid = 1;
        return s;
    }
    if (opacity <= 0.0f) return s;
    const float choice = clampf((u_lobe - pass) / opacity, 0.0f, 0.99999994f);
    if (!entering && random_walk(m)) {
        const Mat b = boundary_material(m);
        s = sample_boundary(b, authored, won, choice, u1, u2, ctx);
        if (s.valid == 0) return s;
        const V3 scale = substrate_scale(m, wo.z, vdot(f.n, s.wi), false);
        s.value = vmul(s.value, vmul(scale, opacity));
        s.weight = vmul(s.weight, scale);
        s.pdf *= opacity;
        s.discrete_pdf *= opacity;
        if (s.event == kGlossyTransmission) s.event = kSubsurfaceExit;
        return s;
    }
    const bool exterior = entering;
    const Lobes p = lobe_probs(m, wo.z, exterior, ctx);
    if (p.diffuse + p.subsurface + p.reflection + p.transmission + p.coat + p.fuzz <= 0.0f) return s;
    V3 wi = zero3();
    const float fuzz_end = p.fuzz;
    const float coat_end = fuzz_end + p.coat;
    const float diffuse_end = coat_end + p.diffuse;
    const float ss_end = diffuse_end + p.subsurface;
    const float refl_end = ss_end + p.reflection;
    if (choice < fuzz_end) {
        wi = sample_fuzz(m, wo, u1, u2);
        if (wi.z <= 1e-7f) return s;
        s.event = kFuzzReflection;
    } else if (choice < coat_end) {
        const Rough cr = coat_rough(m);
        if (smooth(cr)) {
            wi = V3{-wo.x, -wo.y, wo.z};
            V3 coef = splat(sat(m.coat_weight) * coat_fresnel(m, wo.z) * opacity);
            coef = vmul(coef, fuzz_base_scale(m, wo.z, wi.z, exterior));
            s.wi = vnorm(to_world(f, wi));
            s.discrete_pdf = opacity * p.coat;
            if (s.discrete_pdf <= 0.0f) return empty_sample();
            s.weight = vdiv(coef, s.discrete_pdf);
            s.event = kCoatReflection;
            s.delta = 1;
            s.valid = 1;
            return s;
        }
        const V3 wm = sample_vndf(cr, wo, u1, u2);
        wi = reflect_about(wo, wm);
        if (wi.z <= 1e-7f) return s;
        s.event = kCoatReflection;
    } else if (choice < diffuse_end) {
        wi = cosine_hemisphere(u1, u2);
        s.event = kDiffuseReflection;
    } else if (choice < ss_end) {
        if (thin_walled_ss(m)) {
            const float cc = clampf((choice - diffuse_end) / mx(p.subsurface, 1e-8f), 0.0f, 0.99999994f);
            const float rp = thin_walled_ss_prob(m, false);
            wi = cosine_hemisphere(u1, u2);
            if (cc < rp) {
                s.event = kDiffuseReflection;
            } else {
                wi.z = -wi.z;
                s.event = kThinWalledTransmission;
            }
        } else {
            const Mat b = boundary_material(m);
            const Lobes bp = lobe_probs(b, wo.z, false, ctx);
            if (bp.transmission <= 0.0f || p.subsurface <= 0.0f) return s;
            const float cc = clampf((choice - diffuse_end) / p.subsurface, 0.0f, 0.99999994f);
            const float bc = bp.reflection + cc * bp.transmission;
            s = sample_boundary(b, authored, won, bc, u1, u2, ctx);
            if (s.valid == 0 || s.event != kGlossyTransmission) return empty_sample();
            const float ms = (1.0f - sat(m.base_metalness)) * (1.0f - sat(m.transmission_weight)) * sat(m.subsurface_weight);
            const V3 layer = substrate_scale(m, wo.z, vdot(f.n, s.wi), true);
            const V3 wscale = vmul(layer, ms * bp.transmission / mx(p.subsurface, 1e-8f));
            s.value = vmul(s.value, vmul(layer, ms * opacity));
            s.weight = vmul(s.weight, wscale);
            s.pdf *= opacity * p.subsurface / bp.transmission;
            s.discrete_pdf *= opacity * p.subsurface / bp.transmission;
            s.event = kSubsurfaceEntry;
            return s;
        }
    } else if (choice < refl_end) {
        if (smooth(m)) {
            wi = V3{-wo.x, -wo.y, wo.z};
            V3 coef = vmul(reflection_fresnel(m, wo.z, wo.z, entering, ctx), opacity);
            coef = vmul(coef, substrate_scale(m, wo.z, wi.z, exterior));
            s.wi = vnorm(to_world(f, wi));
            s.discrete_pdf = opacity * p.reflection;
            if (s.discrete_pdf <= 0.0f) return empty_sample();
            s.weight = vdiv(coef, s.discrete_pdf);
            s.event = kGlossyReflection;
            s.delta = 1;
            s.valid = 1;
            return s;
        }
        const V3 wm = sample_vndf(spec_rough(m), wo, u1, u2);
        wi = reflect_about(wo, wm);
        if (wi.z <= 1e-7f) return s;
        s.event = kGlossyReflection;
    } else if (m.geometry_thin_walled != 0) {
        wi = neg(wo);
        const V3 t = unit3(vsub(splat(1.0f), dielectric_reflectance(m, wo.z, true, ctx)));
        V3 coef = vmul(vmul(surface_transmission_color(m), t),
            opacity * (1.0f - sat(m.base_metalness)) * sat(m.transmission_weight));
        coef = vmul(coef, substrate_scale(m, wo.z, wi.z, exterior));
        s.wi = to_world(f, wi);
        s.discrete_pdf = opacity * p.transmission;
        if (s.discrete_pdf <= 0.0f) return empty_sample();
        s.weight = vdiv(coef, s.discrete_pdf);
        s.event = kThinWalledTransmission;
        s.delta = 1;
        s.valid = 1;
        return s;
    } else if (smooth(m)) {
        if (dispersive(m)) {
            const float cu = clampf((choice - refl_end) / mx(p.transmission, 1e-8f), 0.0f, 0.99999994f);
            const int ch = pick_channel(ctx, cu);
            const V3 iors = dispersion_iors(m, ctx);
            const float mep = entering ? comp(iors, ch) : 1.0f / comp(iors, ch);
            float rep = 1.0f;
            if (!refract_through(wo, V3{0.0f, 0.0f, 1.0f}, mep, rep, wi)) return s;
            const V3 t = unit3(vsub(splat(1.0f), dielectric_reflectance(m, wo.z, entering, ctx)));
            const V3 tc = surface_transmission_color(m);
            V3 coef = zero3();
            set_comp(coef, ch, comp(tc, ch) * comp(t, ch) * opacity * (1.0f - sat(m.base_metalness))
                                   * sat(m.transmission_weight) / (rep * rep));
            coef = vmul(coef, substrate_scale(m, wo.z, wi.z, exterior));
            const float cp = comp(channel_probs(ctx), ch);
            s.wi = vnorm(to_world(f, wi));
            s.discrete_pdf = opacity * p.transmission * cp;
            if (s.discrete_pdf <= 0.0f) return empty_sample();
            s.weight = vdiv(coef, s.discrete_pdf);
            s.event = kGlossyTransmission;
            s.delta = 1;
            s.valid = 1;
            return s;
        }
        const float mep = entering ? modulated_ior(m) : 1.0f / modulated_ior(m);
        float rep = 1.0f;
        if (!refract_through(wo, V3{0.0f, 0.0f, 1.0f}, mep, rep, wi)) return s;
        const V3 t = unit3(vsub(splat(1.0f), dielectric_reflectance(m, wo.z, entering, ctx)));
        V3 coef = vmul(vmul(surface_transmission_color(m), t),
            opacity * (1.0f - sat(m.base_metalness)) * sat(m.transmission_weight) / (rep * rep));
        coef = vmul(coef, substrate_scale(m, wo.z, wi.z, exterior));
        s.wi = vnorm(to_world(f, wi));
        s.discrete_pdf = opacity * p.transmission;
        if (s.discrete_pdf <= 0.0f) return empty_sample();
        s.weight = vdiv(coef, s.discrete_pdf);
        s.event = kGlossyTransmission;
        s.delta = 1;
        s.valid = 1;
        return s;
    } else {
        const Rough r = spec_rough(m);
        const V3 wm = sample_vndf(r, wo, u1, u2);
        float mep = entering ? modulated_ior(m) : 1.0f / modulated_ior(m);
        if (dispersive(m)) {
            const float cu = clampf((choice - refl_end) / mx(p.transmission, 1e-8f), 0.0f, 0.99999994f);
            const int ch = pick_channel(ctx, cu);
            const V3 iors = dispersion_iors(m, ctx);
            mep = entering ? comp(iors, ch) : 1.0f / comp(iors, ch);
        }
        float ep = 1.0f;
        if (!refract_through(wo, wm, mep, ep, wi) || wi.z >= -1e-7f) return s;
        s.event = kGlossyTransmission;
    }
    return finish_from_eval(s, m, authored, f, won, wi, ctx);
}

}  // namespace pbr
}  // namespace rtgb

#undef PBR_HD
#undef PBR_CALL
