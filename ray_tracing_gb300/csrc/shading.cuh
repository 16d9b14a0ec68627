// Surface reconstruction, materials, textures and light sampling used by the
// shade stage. Each function restates the reference device function named in
// its comment (src/realtime/gpu/programs.cu) with the same operation order; the
// reference's O(#lights) scans are replaced by index maps, binary CDF searches
// and a light BVH that return the same results.
#pragma once

#include <cstddef>

#include "device_common.cuh"
#include "noise_sin.h"
#include "openpbr.h"

namespace rtgb {

static_assert(offsetof(rtgb_openpbr_material, color_texture) == sizeof(pbr::Mat),
    "rtgb_openpbr_material starts with the OpenPBR parameter block");

struct Hit {
    float t;
    float3 pos;
    float u, v;
    float3 gn, sn;
    float3 base, emis;
    float fuzz, ior;
    int openpbr, mtype, ptype, pidx;
    bool front;
};

struct AnalyticHit {
    bool hit;
    float t;
    float3 pos;
    float3 normal;
    int light;
};

// Path registers the shade stage needs (PathState, programs.cu:45-61).
struct PathRegs {
    float3 o, d;
    float3 thr, rad;
    float3 prev_pos, prev_nrm;
    float prev_pdf;
    int prev_mtype, prev_ptype, prev_pidx;
    bool prev_valid, prev_delta, alive;
};

struct LightSample {
    float3 position, normal, direction, emission;
    float distance, pdf;
    int material_index, light_index;
    bool infinite, delta, valid;
};

RTGB_D LightSample empty_sample() {
    LightSample s;
    s.position = f3(0.0f, 0.0f, 0.0f);
    s.normal = f3(0.0f, 0.0f, 1.0f);
    s.direction = f3(0.0f, 0.0f, 1.0f);
    s.emission = f3(0.0f, 0.0f, 0.0f);
    s.distance = 0.0f;
    s.pdf = 0.0f;
    s.material_index = -1;
    s.light_index = -1;
    s.infinite = false;
    s.delta = false;
    s.valid = false;
    return s;
}

// ---- textures: programs.cu:184-302 ------------------------------------------------

RTGB_D float fractf(float v) { return v - floorf(v); }
RTGB_D float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

RTGB_D void sphere_uv(const float3& p, float& u, float& v) {
    const float theta = acosf(fminf(fmaxf(-p.y, -1.0f), 1.0f));
    const float phi = atan2f(-p.z, p.x) + kPi;
    u = phi / (2.0f * kPi);
    v = theta / kPi;
}

// The noise texture's sines use rtgb_noise::noise_sinf (noise_sin.h): the
// hash amplifies the last bit of sin by 43758, so the kernels and the CPU
// oracle share one bit-exact single-precision sine there.
RTGB_D float hash_noise(const float3& p) {
    const float n = rtgb_noise::noise_sinf(dot(p, f3(12.9898f, 78.233f, 37.719f))) * 43758.5453f;
    return fractf(n) * 2.0f - 1.0f;
}

RTGB_D float turbulence(float3 p) {
    float acc = 0.0f, w = 1.0f;
    for (int i = 0; i < 7; ++i) {
        acc += w * hash_noise(p);
        p = mul(p, 2.0f);
        w *= 0.5f;
    }
    return fabsf(acc);
}

RTGB_D float address_coord(float c, int mode, bool& valid) {
    if (mode == 0 && (c < 0.0f || c > 1.0f)) {
        valid = false;
        return 0.0f;
    }
    if (mode == 2) return c - floorf(c);
    if (mode == 3) {
        const float period = c - 2.0f * floorf(0.5f * c);
        return period <= 1.0f ? period : 2.0f - period;
    }
    return clamp01(c);
}

RTGB_D float3 image_texel(const DeviceScene& s, const rtgb_texture& t, int x, int y) {
    x = x < 0 ? 0 : (x >= t.image_width ? t.image_width - 1 : x);
    y = y < 0 ? 0 : (y >= t.image_height ? t.image_height - 1 : y);
    const int idx = t.image_offset + y * t.image_width + x;
    return idx >= 0 && idx < s.texel_count ? ld3(s.texels + 3 * static_cast<long long>(idx)) : f3(0.0f, 1.0f, 1.0f);
}

RTGB_D float3 sample_image(const DeviceScene& s, const rtgb_texture& t, float u, float v) {
    if (s.texels == nullptr || t.image_width <= 0 || t.image_height <= 0) return f3(0.0f, 1.0f, 1.0f);
    bool valid = true;
    const float au = address_coord(u, t.u_address_mode, valid);
    const float av = 1.0f - address_coord(v, t.v_address_mode, valid);
    if (!valid) return f3(0.0f, 0.0f, 0.0f);
    if (t.filter_type == 0) {
        int x = static_cast<int>(au * static_cast<float>(t.image_width));
        int y = static_cast<int>(av * static_cast<float>(t.image_height));
        x = x >= t.image_width ? t.image_width - 1 : x;
        y = y >= t.image_height ? t.image_height - 1 : y;
        return image_texel(s, t, x, y);
    }
    const float x = au * static_cast<float>(t.image_width - 1);
    const float y = av * static_cast<float>(t.image_height - 1);
    const int x0 = static_cast<int>(floorf(x));
    const int y0 = static_cast<int>(floorf(y));
    const float tx = x - static_cast<float>(x0);
    const float ty = y - static_cast<float>(y0);
    const float3 top = add(mul(image_texel(s, t, x0, y0), 1.0f - tx), mul(image_texel(s, t, x0 + 1, y0), tx));
    const float3 bot = add(mul(image_texel(s, t, x0, y0 + 1), 1.0f - tx), mul(image_texel(s, t, x0 + 1, y0 + 1), tx));
    return add(mul(top, 1.0f - ty), mul(bot, ty));
}

RTGB_D float3 eval_texture(const DeviceScene& s, int index, float u, float v, const float3& p) {
    for (int depth = 0; depth < 8; ++depth) {
        if (index < 0 || index >= s.texture_count || s.textures == nullptr) return f3(1.0f, 0.0f, 1.0f);
        const rtgb_texture t = s.textures[index];
        if (t.type == 0) return ld3(t.color);
        if (t.type == 1) {
            if (fabsf(t.scale) < 1e-8f) {
                index = t.even_texture;
                continue;
            }
            const int x = static_cast<int>(floorf(p.x / t.scale));
            const int y = static_cast<int>(floorf(p.y / t.scale));
            const int z = static_cast<int>(floorf(p.z / t.scale));
            index = ((x + y + z) % 2) == 0 ? t.even_texture : t.odd_texture;
            continue;
        }
        if (t.type == 2) return sample_image(s, t, u, v);
        if (t.type == 3) {
            const float turb = turbulence(p);
            const float value = 0.5f * (1.0f + rtgb_noise::noise_sinf(t.scale * p.z + 10.0f * turb));
            return f3(value, value, value);
        }
        return f3(1.0f, 0.0f, 1.0f);
    }
    return f3(1.0f, 0.0f, 1.0f);
}

// ---- OpenPBR materials (programs.cu:148-160, :909-960) ----------------------------

RTGB_D pbr::V3 pv(const float3& v) { return pbr::V3{v.x, v.y, v.z}; }
RTGB_D float3 fv(const pbr::V3& v) { return f3(v.x, v.y, v.z); }

// resolve_openpbr_material, programs.cu:909-921
RTGB_D const rtgb_openpbr_material* openpbr_material(const DeviceScene& s, int index) {
    if (index < 0 || index >= s.openpbr_count || s.openpbr == nullptr) return nullptr;
    return s.openpbr + index;
}

RTGB_D void openpbr_load(const rtgb_openpbr_material& c, pbr::Mat& m) {
    const float* src = reinterpret_cast<const float*>(&c);
    float* dst = reinterpret_cast<float*>(&m);
#pragma unroll
    for (int k = 0; k < static_cast<int>(sizeof(pbr::Mat) / 4); ++k) dst[k] = src[k];
}

// evaluate_openpbr_color_binding, programs.cu:923-932 (input 0 base, 1 specular,
// 2 transmission, 3 emission color)
RTGB_D void openpbr_color_binding(const DeviceScene& s, pbr::Mat& m, const rtgb_openpbr_material& c, int input,
    float u, float v, const float3& p);

// evaluate_openpbr_scattering_material, programs.cu:944-960: the parameters the
// BSDF sees at a hit (the base color already evaluated by populate_material).
RTGB_D void openpbr_scattering(const DeviceScene& s, const Hit& h, pbr::Mat& m);

RTGB_D pbr::Context transport_context(const float3& throughput) {
    pbr::Context ctx = pbr::default_context();
    ctx.throughput = pv(throughput);
    return ctx;
}

// populate_material, programs.cu:961-1009. Instances without kPbr resolve no
// OpenPBR material (they run only for scenes that have none).
template <bool kPbr>
RTGB_D void populate_material(const DeviceScene& s, int mi, Hit& h) {
    if (mi < 0 || mi >= s.material_count || s.materials == nullptr) {
        h.base = f3(0.0f, 0.0f, 0.0f);
        h.emis = f3(0.0f, 0.0f, 0.0f);
        h.mtype = 0;
        h.ior = 1.0f;
        h.fuzz = 0.0f;
        h.openpbr = -1;
        return;
    }
    const rtgb_material m = s.materials[mi];
    h.openpbr = m.openpbr_index;
    h.mtype = m.type;
    h.fuzz = m.fuzz;
    h.ior = m.ior;
    h.base = eval_texture(s, m.albedo_texture, h.u, h.v, h.pos);
    h.emis = eval_texture(s, m.emission_texture, h.u, h.v, h.pos);
    if (h.mtype == 2) {
        h.base = f3(0.92f, 0.95f, 1.0f);
        h.emis = f3(0.0f, 0.0f, 0.0f);
    }
    if (h.mtype == 3 && !h.front) h.emis = f3(0.0f, 0.0f, 0.0f);
    if (h.mtype != 3) h.emis = f3(0.0f, 0.0f, 0.0f);
    if (h.mtype == 5) {
        const rtgb_openpbr_material* c = kPbr ? openpbr_material(s, m.openpbr_index) : nullptr;
        if (c == nullptr) {
            h.mtype = -1;
            h.base = f3(0.0f, 0.0f, 0.0f);
            h.emis = f3(0.0f, 0.0f, 0.0f);
            return;
        }
        if constexpr (kPbr) {
            pbr::Mat params;
            openpbr_load(*c, params);
            openpbr_color_binding(s, params, *c, 0, h.u, h.v, h.pos);
            openpbr_color_binding(s, params, *c, 3, h.u, h.v, h.pos);
            h.base = fv(params.base_color);
            h.emis = fv(pbr::emission(params));
        }
    }
}

RTGB_D void set_face(const float3& d, const float3& outward, Hit& h) {
    h.front = dot(d, outward) < 0.0f;
    h.gn = outward;
    h.sn = h.front ? outward : mul(outward, -1.0f);
}

// Rebuilds the full hit record of the winning primitive (try_hit_sphere/quad/
// triangle, programs.cu:1421-1547). Re-running the test over (eps, far) picks
// the same root the traversal accepted, so t, uv and normals are identical.
template <bool kPbr>
RTGB_D bool reconstruct_surface(const DeviceScene& s, int code, const float3& o, const float3& d, Hit& h) {
    const int type = static_cast<unsigned>(code) >> 28;
    const int idx = code & 0x0fffffff;
    h.ptype = type;
    h.pidx = idx;
    h.u = 0.0f;
    h.v = 0.0f;
    int mi = -1;
    if (type == 0) {
        const rtgb_sphere sp = s.spheres[idx];
        const float3 center = ld3(sp.center);
        float t;
        if (!sphere_t(center, sp.radius, o, d, kRayEpsilon, kRayFar, t)) return false;
        h.t = t;
        h.pos = add(o, mul(d, t));
        const float3 outward = divs(sub(h.pos, center), sp.radius);
        sphere_uv(outward, h.u, h.v);
        set_face(d, outward, h);
        mi = sp.material_index;
    } else if (type == 1) {
        const rtgb_quad q = s.quads[idx];
        const float3 origin = ld3(q.origin), eu = ld3(q.edge_u), ev = ld3(q.edge_v);
        const float3 n = cross(eu, ev);
        const float nls = len_sq(n);
        if (nls <= 1e-12f) return false;
        const float3 normal = divs(n, sqrtf(nls));
        const float3 w = divs(n, nls);
        float t, u, v;
        if (!quad_t(origin, normal, w, eu, ev, o, d, kRayEpsilon, kRayFar, t, u, v)) return false;
        h.t = t;
        h.pos = add(o, mul(d, t));
        h.u = u;
        h.v = v;
        set_face(d, normal, h);
        mi = q.material_index;
    } else if (type == 2) {
        const rtgb_triangle tr = s.triangles[idx];
        const float3 p0 = ld3(tr.p0), p1 = ld3(tr.p1), p2 = ld3(tr.p2);
        const float3 e1 = sub(p1, p0), e2 = sub(p2, p0);
        float t, u, v;
        if (!triangle_t(p0, e1, e2, o, d, kRayEpsilon, kRayFar, t, u, v)) return false;
        const float3 normal = normalize(cross(e1, e2));
        const float w = 1.0f - u - v;
        h.t = t;
        h.pos = add(o, mul(d, t));
        if (tr.has_texcoords != 0) {
            h.u = tr.uv0[0] * w + tr.uv1[0] * u + tr.uv2[0] * v;
            h.v = tr.uv0[1] * w + tr.uv1[1] * u + tr.uv2[1] * v;
        } else {
            h.u = u;
            h.v = v;
        }
        set_face(d, normal, h);
        if (tr.has_vertex_normals != 0) {
            float3 sh = add(mul(ld3(tr.n0), w), add(mul(ld3(tr.n1), u), mul(ld3(tr.n2), v)));
            if (!near_zero(sh)) {
                sh = normalize(sh);
                if (dot(sh, normal) < 0.0f) sh = mul(sh, -1.0f);
                h.sn = h.front ? sh : mul(sh, -1.0f);
            }
        }
        mi = tr.material_index;
    } else {
        return false;
    }
    populate_material<kPbr>(s, mi, h);
    return true;
}

// Medium scattering event (programs.cu:1738-1750): no primitive identity.
template <bool kPbr>
RTGB_D void reconstruct_medium(const DeviceScene& s, int medium, float t, const float3& o, const float3& d, Hit& h) {
    h.t = t;
    h.pos = add(o, mul(d, t));
    h.front = true;
    h.gn = mul(normalize(d), -1.0f);
    h.sn = h.gn;
    h.u = 0.0f;
    h.v = 0.0f;
    h.ptype = -1;
    h.pidx = -1;
    populate_material<kPbr>(s, s.media[medium].material_index, h);
}

// hit_medium_boundary, programs.cu:1356-1419
RTGB_D bool medium_boundary(const rtgb_medium& m, const float3& ro, const float3& rd, float tmin, float tmax,
    float& entry, float& exit) {
    const float3 shifted = sub(ro, ld3(m.translation));
    const float3 r0 = ld3(m.rotation_row0), r1 = ld3(m.rotation_row1), r2 = ld3(m.rotation_row2);
    const float3 lo = f3(dot(r0, shifted), dot(r1, shifted), dot(r2, shifted));
    const float3 ld = f3(dot(r0, rd), dot(r1, rd), dot(r2, rd));
    if (m.boundary_type == 0) {
        const float3 center = ld3(m.local_center_or_min);
        const float3 oc = sub(lo, center);
        const float a = len_sq(ld);
        const float hb = dot(oc, ld);
        const float c = len_sq(oc) - m.radius * m.radius;
        const float disc = hb * hb - a * c;
        if (disc <= 0.0f) return false;
        const float sd = sqrtf(disc);
        float t0 = (-hb - sd) / a, t1 = (-hb + sd) / a;
        if (t0 > t1) {
            const float tmp = t0;
            t0 = t1;
            t1 = tmp;
        }
        entry = fmaxf(t0, tmin);
        exit = fminf(t1, tmax);
        return entry < exit;
    }
    if (m.boundary_type == 1) {
        float t0 = tmin, t1 = tmax;
        const float oo[3] = {lo.x, lo.y, lo.z}, dd[3] = {ld.x, ld.y, ld.z};
        for (int a = 0; a < 3; ++a) {
            if (fabsf(dd[a]) < 1e-8f) {
                if (oo[a] < m.local_center_or_min[a] || oo[a] > m.local_max[a]) return false;
                continue;
            }
            float a0 = (m.local_center_or_min[a] - oo[a]) / dd[a];
            float a1 = (m.local_max[a] - oo[a]) / dd[a];
            if (a0 > a1) {
                const float tmp = a0;
                a0 = a1;
                a1 = tmp;
            }
            t0 = fmaxf(t0, a0);
            t1 = fminf(t1, a1);
            if (t0 >= t1) return false;
        }
        entry = t0;
        exit = t1;
        return true;
    }
    return false;
}

// ---- analytic lights: programs.cu:649-891 ------------------------------------------

RTGB_D float3 analytic_normal(const rtgb_analytic_light& l) {
    return normalize(mul(cross(ld3(l.basis_x), ld3(l.basis_y)), -1.0f));
}

RTGB_D bool plane_coords(const float3& bx, const float3& by, const float3& center, const float3& p, float& lx, float& ly) {
    const float3 local = sub(p, center);
    const float xx = dot(bx, bx), xy = dot(bx, by), yy = dot(by, by);
    const float det = xx * yy - xy * xy;
    if (det <= 1e-16f) return false;
    const float px = dot(local, bx), py = dot(local, by);
    lx = (px * yy - py * xy) / det;
    ly = (py * xx - px * xy) / det;
    return true;
}

RTGB_D bool hit_analytic(const rtgb_analytic_light& l, const float3& ro, const float3& rd, float tmin, float tmax,
    AnalyticHit& h) {
    const float3 center = ld3(l.position);
    if (l.type == 0) {
        const float radius = l.radius * len(ld3(l.basis_x));
        const float3 oc = sub(ro, center);
        const float a = len_sq(rd);
        const float hb = dot(oc, rd);
        const float c = len_sq(oc) - radius * radius;
        const float disc = hb * hb - a * c;
        if (a <= 1e-16f || disc < 0.0f) return false;
        const float rt = sqrtf(disc);
        float root = (-hb - rt) / a;
        if (root <= tmin || root >= tmax) root = (-hb + rt) / a;
        if (root <= tmin || root >= tmax) return false;
        const float3 pos = add(ro, mul(rd, root));
        const float3 n = normalize(sub(pos, center));
        if (dot(rd, n) >= 0.0f) return false;
        h.hit = true;
        h.t = root;
        h.pos = pos;
        h.normal = n;
        return true;
    }
    if (l.type == 1 || l.type == 2) {
        const float3 n = analytic_normal(l);
        const float den = dot(rd, n);
        if (den >= -1e-8f) return false;
        const float t = dot(sub(center, ro), n) / den;
        if (t <= tmin || t >= tmax) return false;
        const float3 pos = add(ro, mul(rd, t));
        float lx = 0.0f, ly = 0.0f;
        if (!plane_coords(ld3(l.basis_x), ld3(l.basis_y), center, pos, lx, ly)) return false;
        const bool inside = l.type == 1 ? lx * lx + ly * ly <= l.radius * l.radius
                                        : fabsf(lx) <= 0.5f * l.width && fabsf(ly) <= 0.5f * l.height;
        if (!inside) return false;
        h.hit = true;
        h.t = t;
        h.pos = pos;
        h.normal = n;
        return true;
    }
    if (l.type != 3) return false;
    const float3 bx = ld3(l.basis_x), by = ld3(l.basis_y), bz = ld3(l.basis_z);
    const float scale = len(bx);
    if (scale <= 1e-8f) return false;
    const float3 ax = divs(bx, scale), ay = divs(by, scale), az = normalize(bz);
    const float3 lo = sub(ro, center);
    const float ox = dot(lo, ax), oy = dot(lo, ay), oz = dot(lo, az);
    const float dx = dot(rd, ax), dy = dot(rd, ay), dz = dot(rd, az);
    const float radius = l.radius * scale;
    const float a = dx * dx + dy * dy;
    const float hb = ox * dx + oy * dy;
    const float c = ox * ox + oy * oy - radius * radius;
    const float disc = hb * hb - a * c;
    if (a <= 1e-16f || disc < 0.0f) return false;
    const float rt = sqrtf(disc);
    float root = (-hb - rt) / a;
    float z = oz + root * dz;
    const float half_len = 0.5f * l.length * len(bz);
    if (root <= tmin || root >= tmax || fabsf(z) > half_len) {
        root = (-hb + rt) / a;
        z = oz + root * dz;
    }
    if (root <= tmin || root >= tmax || fabsf(z) > half_len) return false;
    const float x = ox + root * dx, y = oy + root * dy;
    const float3 n = normalize(add(mul(ax, x), mul(ay, y)));
    if (dot(rd, n) >= 0.0f) return false;
    h.hit = true;
    h.t = root;
    h.pos = add(ro, mul(rd, root));
    h.normal = n;
    return true;
}

// hit_analytic of light li; disk and rect lights read only its hot record
// (the normal there is analytic_light_normal, computed once per scene).
RTGB_D bool hit_analytic_at(const DeviceScene& s, int li, const float3& ro, const float3& rd, float tmin, float tmax,
    AnalyticHit& h) {
    const float4* hot = s.analytic_hot + static_cast<long long>(kAnalyticHot) * li;
    const float4 h4 = __ldg(hot + 4);
    const int type = __float_as_int(h4.w);
    if (type != 1 && type != 2) return hit_analytic(s.analytic[li], ro, rd, tmin, tmax, h);
    const float3 n = xyz(h4);
    const float den = dot(rd, n);
    if (den >= -1e-8f) return false;
    const float3 center = xyz(__ldg(hot));
    const float t = dot(sub(center, ro), n) / den;
    if (t <= tmin || t >= tmax) return false;
    const float4 h1 = __ldg(hot + 1), h2 = __ldg(hot + 2);
    const float3 pos = add(ro, mul(rd, t));
    float lx = 0.0f, ly = 0.0f;
    if (!plane_coords(xyz(h1), xyz(h2), center, pos, lx, ly)) return false;
    const bool inside = type == 1 ? lx * lx + ly * ly <= h1.w * h1.w
                                  : fabsf(lx) <= 0.5f * h1.w && fabsf(ly) <= 0.5f * h2.w;
    if (!inside) return false;
    h.hit = true;
    h.t = t;
    h.pos = pos;
    h.normal = n;
    return true;
}

// Closest analytic-light hit below `tmax` (intersect_analytic_lights,
// programs.cu:795-813) over the light BVH; returns the light index or -1.
RTGB_D int traverse_analytic(const DeviceScene& s, const float3& o, const float3& d, float tmin, float tmax, float& t_hit) {
    if (s.analytic_bvh_count <= 0) return -1;
    float closest = tmax;
    int best = -1;
    auto leaf = [&](int slot) {
        const int li = s.analytic_leaf[slot];
        AnalyticHit h;
        h.hit = false;
        if (hit_analytic_at(s, li, o, d, tmin, closest, h)) {
            closest = h.t;
            best = li;
        }
    };
    if (s.analytic_bvh_count == 1) {
        leaf(0);
        t_hit = closest;
        return best;
    }
    const RayInv ri = ray_inv(o, d);
    int stack[kTraversalStack];
    int sp = 0;
    int node = 0;
    int dropped = 0;
    const int limit = s.bounds.traversal;
    int guard = 0;
    for (; guard < limit; ++guard) {
        const float4* np = reinterpret_cast<const float4*>(s.analytic_nodes + node);
        const float4 a = __ldg(np + 0), b = __ldg(np + 1), c = __ldg(np + 2), e = __ldg(np + 3);
        const int c0 = __float_as_int(a.w), c1 = __float_as_int(b.w);
        float t0, t1;
        bool h0 = box_hit(xyz(a), xyz(b), ri.inv, ri.oinv, tmin, closest, t0);
        bool h1 = box_hit(xyz(c), xyz(e), ri.inv, ri.oinv, tmin, closest, t1);
        if (h0 && c0 < 0) {
            leaf(~c0);
            h0 = false;
        }
        if (h1 && c1 < 0) {
            leaf(~c1);
            h1 = false;
        }
        if (h0 && h1) {
            const bool first0 = t0 <= t1;
            if (sp < kTraversalStack) stack[sp++] = first0 ? c1 : c0;
            else ++dropped;  // a dropped subtree is reported below
            node = first0 ? c0 : c1;
            continue;
        }
        if (h0) {
            node = c0;
            continue;
        }
        if (h1) {
            node = c1;
            continue;
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    if ((guard >= limit || dropped != 0) && s.bounds.gave_up) atomicAdd(s.bounds.gave_up, 1);
    t_hit = closest;
    return best;
}

RTGB_D float analytic_pdf_for_hit(const rtgb_analytic_light& l, const float3& origin, const float3& dir,
    const AnalyticHit& h) {
    if (l.delta != 0 || l.treat_as_point != 0 || l.treat_as_line != 0) return 0.0f;
    if (l.type == 0) {
        const float3 center = ld3(l.position);
        const float radius = l.radius * len(ld3(l.basis_x));
        const float d2 = len_sq(sub(center, origin));
        const float r2 = radius * radius;
        if (d2 <= r2) return 0.0f;
        return uniform_cone_pdf(sqrtf(fmaxf(0.0f, 1.0f - r2 / d2)));
    }
    const float d2 = len_sq(sub(h.pos, origin));
    const float ac = fmaxf(dot(h.normal, mul(dir, -1.0f)), 0.0f);
    return area_pdf(l.world_area, d2, ac);
}

RTGB_D float analytic_emission_mis(const DeviceScene& s, const PathRegs& st, const AnalyticHit& h) {
    if (!st.prev_valid || st.prev_delta || h.light < 0) return 1.0f;
    const rtgb_analytic_light& l = s.analytic[h.light];
    const float3 dir = normalize(st.d);
    const float lp = l.selection_pdf * analytic_pdf_for_hit(l, st.prev_pos, dir, h);
    return power_heuristic(st.prev_pdf, lp);
}

RTGB_D float3 analytic_infinite_radiance(const DeviceScene& s, const PathRegs& st) {
    float3 rad = f3(0.0f, 0.0f, 0.0f);
    const float3 dir = normalize(st.d);
    for (int k = 0; k < s.infinite_analytic_count; ++k) {
        const rtgb_analytic_light& l = s.analytic[s.infinite_analytic[k]];
        bool in_dir = false;
        if (l.type == 5) {
            in_dir = true;
        } else {
            const float3 axis = normalize(ld3(l.basis_z));
            const float thr = l.delta != 0 ? 0.999999f : l.cos_theta_max;
            in_dir = dot(axis, dir) >= thr;
        }
        if (!in_dir) continue;
        float w = 1.0f;
        if (st.prev_valid && !st.prev_delta) {
            const float cond = l.delta != 0 ? 0.0f : (l.type == 5 ? uniform_sphere_pdf() : uniform_cone_pdf(l.cos_theta_max));
            if (cond <= 0.0f) continue;
            w = power_heuristic(st.prev_pdf, l.selection_pdf * cond);
        }
        rad = add(rad, mul(ld3(l.radiance), w));
    }
    return rad;
}

// ---- emissive geometry: programs.cu:559-647, 1057-1232 --------------------------

RTGB_D int find_light(const DeviceScene& s, int type, int prim) {
    if (type == 3) return s.environment_light;
    if (prim < 0) return -1;
    if (type == 0) return prim < s.sphere_count ? s.sphere_light[prim] : -1;
    if (type == 1) return prim < s.quad_count ? s.quad_light[prim] : -1;
    if (type == 2) return prim < s.triangle_count ? s.triangle_light[prim] : -1;
    return -1;
}

RTGB_D float effective_selection_pdf(const DeviceScene& s, int light, int ex_type, int ex_index) {
    const int ex = ex_type < 0 ? -1 : find_light(s, ex_type, ex_index);
    if (ex == light) return 0.0f;
    const float eligible = ex < 0 ? 1.0f : 1.0f - s.lights[ex].selection_pdf;
    return eligible > 1e-8f ? s.lights[light].selection_pdf / eligible : 0.0f;
}

RTGB_D float conditional_pdf_for_hit(const DeviceScene& s, const PackedLight& light, const float3& origin,
    const float3& dir, const Hit* h) {
    if (light.type == 3) return uniform_sphere_pdf();
    if (h == nullptr || h->ptype != light.type || h->pidx != light.primitive_index || !h->front) return 0.0f;
    if (light.type == 0) {
        const rtgb_sphere sp = s.spheres[light.primitive_index];
        const float d2 = len_sq(sub(ld3(sp.center), origin));
        const float r2 = sp.radius * sp.radius;
        if (d2 <= r2) return 0.0f;
        return uniform_cone_pdf(sqrtf(fmaxf(0.0f, 1.0f - r2 / d2)));
    }
    const float d2 = len_sq(sub(h->pos, origin));
    const float ac = fmaxf(dot(h->gn, mul(dir, -1.0f)), 0.0f);
    if (light.type == 1) {
        const rtgb_quad q = s.quads[light.primitive_index];
        return area_pdf(len(cross(ld3(q.edge_u), ld3(q.edge_v))), d2, ac);
    }
    const rtgb_triangle t = s.triangles[light.primitive_index];
    const float area = 0.5f * len(cross(sub(ld3(t.p1), ld3(t.p0)), sub(ld3(t.p2), ld3(t.p0))));
    return area_pdf(area, d2, ac);
}

RTGB_D float emission_mis_weight(const DeviceScene& s, const PathRegs& st, const Hit* h, bool env) {
    if (!st.prev_valid || st.prev_delta) return 1.0f;
    if (!env && (h == nullptr || h->ptype < 0)) return 1.0f;
    const int li = env ? s.environment_light : find_light(s, h->ptype, h->pidx);
    if (li < 0) return 1.0f;
    const PackedLight light = s.lights[li];
    const float3 dir = normalize(st.d);
    const float cond = env ? (st.prev_mtype == 4 ? uniform_sphere_pdf() : fmaxf(dot(st.prev_nrm, dir), 0.0f) / kPi)
                           : conditional_pdf_for_hit(s, light, st.prev_pos, dir, h);
    const float sel = effective_selection_pdf(s, li, st.prev_ptype, st.prev_pidx);
    return power_heuristic(st.prev_pdf, sel * cond);
}

RTGB_D float3 cone_direction(const float3& axis, float ctm, float u0, float u1) {
    const float ct = 1.0f - u0 * (1.0f - ctm);
    const float stt = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    const float phi = 2.0f * kPi * u1;
    const float3 helper = fabsf(axis.x) > 0.9f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
    const float3 tangent = normalize(cross(helper, axis));
    const float3 bitangent = cross(axis, tangent);
    return normalize(add(mul(axis, ct), add(mul(tangent, stt * cosf(phi)), mul(bitangent, stt * sinf(phi)))));
}

RTGB_D float3 sphere_direction(float u0, float u1) {
    const float z = 1.0f - 2.0f * u0;
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    const float phi = 2.0f * kPi * u1;
    return f3(r * cosf(phi), r * sinf(phi), z);
}

// evaluate_material_emission, programs.cu:1011-1024
template <bool kPbr>
RTGB_D float3 material_emission(const DeviceScene& s, const rtgb_material& m, float u, float v, const float3& p) {
    if (m.type == 5) {
        if constexpr (kPbr) {
            const rtgb_openpbr_material* c = openpbr_material(s, m.openpbr_index);
            if (c == nullptr) return f3(0.0f, 0.0f, 0.0f);
            pbr::Mat params;
            openpbr_load(*c, params);
            openpbr_color_binding(s, params, *c, 3, u, v, p);
            return fv(pbr::emission(params));
        }
        return f3(0.0f, 0.0f, 0.0f);
    }
    return eval_texture(s, m.emission_texture, u, v, p);
}

template <bool kPbr>
RTGB_D LightSample sample_direct(const DeviceScene& s, const Hit& rcv, uint32_t& rng) {
    LightSample smp = empty_sample();
    const float3 sp = rcv.pos;
    const int ex = rcv.ptype < 0 ? -1 : find_light(s, rcv.ptype, rcv.pidx);
    const float eligible = ex < 0 ? 1.0f : 1.0f - s.lights[ex].selection_pdf;
    if (eligible <= 1e-8f) return smp;
    int li = -1;
    if (ex < 0) {
        li = sample_cdf_guided(s.light_cdf, s.light_guide, s.light_count, rnd(rng));
    } else {
        // Receiver is itself an emitter: sequential renormalised scan, as the
        // reference accumulates it (programs.cu:1073-1093).
        const float target = rnd(rng) * eligible;
        float acc = 0.0f;
        for (int i = 0; i < s.light_count; ++i) {
            if (i == ex) continue;
            acc += s.lights[i].selection_pdf;
            if (target < acc) {
                li = i;
                break;
            }
        }
        if (li < 0) {
            for (int i = s.light_count - 1; i >= 0; --i) {
                if (i != ex) {
                    li = i;
                    break;
                }
            }
        }
    }
    if (li < 0) return smp;
    const PackedLight light = s.lights[li];
    const float sel = light.selection_pdf / eligible;
    if (sel <= 0.0f) return smp;
    if (light.type == 3) {
        if (rcv.mtype == 4) {
            smp.direction = random_unit_vector(rng, s.bounds);
            smp.pdf = sel * uniform_sphere_pdf();
        } else {
            smp.direction = add(rcv.sn, random_unit_vector(rng, s.bounds));
            if (near_zero(smp.direction)) smp.direction = rcv.sn;
            smp.direction = normalize(smp.direction);
            const float c = fmaxf(dot(rcv.sn, smp.direction), 0.0f);
            smp.pdf = sel * c / kPi;
        }
        smp.emission = ld3(s.background);
        smp.distance = kRayFar;
        smp.infinite = true;
        smp.valid = smp.pdf > 0.0f;
        return smp;
    }
    float tu = 0.0f, tv = 0.0f, cond = 0.0f;
    if (light.type == 0) {
        if (light.primitive_index < 0 || light.primitive_index >= s.sphere_count) return smp;
        const rtgb_sphere sph = s.spheres[light.primitive_index];
        const float3 center = ld3(sph.center);
        const float3 tc = sub(center, sp);
        const float d2 = len_sq(tc);
        const float r2 = sph.radius * sph.radius;
        if (d2 <= r2 * (1.0f + 1e-6f)) return smp;
        const float ctm = sqrtf(fmaxf(0.0f, 1.0f - r2 / d2));
        const float3 axis = normalize(tc);
        const float u0 = rnd(rng);
        const float u1 = rnd(rng);
        smp.direction = cone_direction(axis, ctm, u0, u1);
        const float3 oc = sub(sp, center);
        const float hb = dot(oc, smp.direction);
        const float disc = hb * hb - (len_sq(oc) - r2);
        if (disc <= 0.0f) return smp;
        smp.distance = -hb - sqrtf(disc);
        if (smp.distance <= kRayEpsilon) return smp;
        smp.position = add(sp, mul(smp.direction, smp.distance));
        smp.normal = normalize(sub(smp.position, center));
        sphere_uv(smp.normal, tu, tv);
        smp.material_index = sph.material_index;
        cond = uniform_cone_pdf(ctm);
    } else if (light.type == 1) {
        if (light.primitive_index < 0 || light.primitive_index >= s.quad_count) return smp;
        const rtgb_quad q = s.quads[light.primitive_index];
        const float3 o = ld3(q.origin), eu = ld3(q.edge_u), ev = ld3(q.edge_v);
        tu = rnd(rng);
        tv = rnd(rng);
        smp.position = add(o, add(mul(eu, tu), mul(ev, tv)));
        const float3 an = cross(eu, ev);
        const float area = len(an);
        if (area <= 1e-12f) return smp;
        smp.normal = divs(an, area);
        smp.material_index = q.material_index;
        const float3 tl = sub(smp.position, sp);
        const float d2 = len_sq(tl);
        if (d2 <= 1e-12f) return empty_sample();
        smp.distance = sqrtf(d2);
        smp.direction = divs(tl, smp.distance);
        const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
        cond = area_pdf(area, d2, ac);
    } else {
        if (light.primitive_index < 0 || light.primitive_index >= s.triangle_count) return smp;
        const rtgb_triangle t = s.triangles[light.primitive_index];
        const float3 p0 = ld3(t.p0), p1 = ld3(t.p1), p2 = ld3(t.p2);
        float w0 = 0.0f, w1 = 0.0f, w2 = 0.0f;
        const float u0 = rnd(rng);
        const float u1 = rnd(rng);
        sample_uniform_triangle(u0, u1, w0, w1, w2);
        smp.position = add(mul(p0, w0), add(mul(p1, w1), mul(p2, w2)));
        if (t.has_texcoords != 0) {
            tu = t.uv0[0] * w0 + t.uv1[0] * w1 + t.uv2[0] * w2;
            tv = t.uv0[1] * w0 + t.uv1[1] * w1 + t.uv2[1] * w2;
        } else {
            tu = w1;
            tv = w2;
        }
        const float3 an = cross(sub(p1, p0), sub(p2, p0));
        const float da = len(an);
        if (da <= 1e-12f) return smp;
        smp.normal = divs(an, da);
        smp.material_index = t.material_index;
        const float3 tl = sub(smp.position, sp);
        const float d2 = len_sq(tl);
        if (d2 <= 1e-12f) return empty_sample();
        smp.distance = sqrtf(d2);
        smp.direction = divs(tl, smp.distance);
        const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
        cond = area_pdf(0.5f * da, d2, ac);
    }
    if (cond <= 0.0f || smp.material_index < 0 || smp.material_index >= s.material_count) return empty_sample();
    smp.emission = material_emission<kPbr>(s, s.materials[smp.material_index], tu, tv, smp.position);
    smp.pdf = sel * cond;
    smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
    return smp;
}

// A ReSTIR candidate over emissive geometry (no reference counterpart: the
// reference's ReSTIR DI resamples analytic lights only, programs.cu:1915-1924).
// Light `li` of the emissive list sampled with the given (u0, u1) the way
// sample_direct samples it for a receiver that is not itself an emitter, so a
// candidate re-evaluates to the same point at any surface: cone sampling
// toward spheres, uniform area sampling on quads and triangles, and for the
// environment the cosine distribution about the receiver normal built from
// (u0, u1) (normal + a uniform sphere point), whose pdf the BSDF-side MIS
// weight of emission_mis_weight assumes; isotropic receivers take the uniform
// sphere point.
template <bool kPbr>
RTGB_D LightSample emissive_candidate(const DeviceScene& s, const float3& sp, const float3& sn, int rcv_mtype, int li,
    float u0, float u1) {
    LightSample smp = empty_sample();
    if (li < 0 || li >= s.light_count) return smp;
    const PackedLight light = s.lights[li];
    const float sel = light.selection_pdf;
    if (sel <= 0.0f) return smp;
    smp.light_index = li;
    if (light.type == 3) {
        const float3 q = sphere_direction(u0, u1);
        if (rcv_mtype == 4) {
            smp.direction = q;
            smp.pdf = sel * uniform_sphere_pdf();
        } else {
            smp.direction = add(sn, q);
            if (near_zero(smp.direction)) smp.direction = sn;
            smp.direction = normalize(smp.direction);
            smp.pdf = sel * fmaxf(dot(sn, smp.direction), 0.0f) / kPi;
        }
        smp.emission = ld3(s.background);
        smp.distance = kRayFar;
        smp.infinite = true;
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }
    float tu = 0.0f, tv = 0.0f, cond = 0.0f;
    if (light.type == 0) {
        if (light.primitive_index < 0 || light.primitive_index >= s.sphere_count) return empty_sample();
        const rtgb_sphere sph = s.spheres[light.primitive_index];
        const float3 center = ld3(sph.center);
        const float3 tc = sub(center, sp);
        const float d2 = len_sq(tc);
        const float r2 = sph.radius * sph.radius;
        if (d2 <= r2 * (1.0f + 1e-6f)) return empty_sample();
        const float ctm = sqrtf(fmaxf(0.0f, 1.0f - r2 / d2));
        smp.direction = cone_direction(normalize(tc), ctm, u0, u1);
        const float3 oc = sub(sp, center);
        const float hb = dot(oc, smp.direction);
        const float disc = hb * hb - (len_sq(oc) - r2);
        if (disc <= 0.0f) return empty_sample();
        smp.distance = -hb - sqrtf(disc);
        if (smp.distance <= kRayEpsilon) return empty_sample();
        smp.position = add(sp, mul(smp.direction, smp.distance));
        smp.normal = normalize(sub(smp.position, center));
        sphere_uv(smp.normal, tu, tv);
        smp.material_index = sph.material_index;
        cond = uniform_cone_pdf(ctm);
    } else {
        float3 an;
        if (light.type == 1) {
            if (light.primitive_index < 0 || light.primitive_index >= s.quad_count) return empty_sample();
            const rtgb_quad q = s.quads[light.primitive_index];
            const float3 o = ld3(q.origin), eu = ld3(q.edge_u), ev = ld3(q.edge_v);
            tu = u0;
            tv = u1;
            smp.position = add(o, add(mul(eu, tu), mul(ev, tv)));
            an = cross(eu, ev);
            smp.material_index = q.material_index;
        } else {
            if (light.primitive_index < 0 || light.primitive_index >= s.triangle_count) return empty_sample();
            const rtgb_triangle t = s.triangles[light.primitive_index];
            const float3 p0 = ld3(t.p0), p1 = ld3(t.p1), p2 = ld3(t.p2);
            float w0 = 0.0f, w1 = 0.0f, w2 = 0.0f;
            sample_uniform_triangle(u0, u1, w0, w1, w2);
            smp.position = add(mul(p0, w0), add(mul(p1, w1), mul(p2, w2)));
            if (t.has_texcoords != 0) {
                tu = t.uv0[0] * w0 + t.uv1[0] * w1 + t.uv2[0] * w2;
                tv = t.uv0[1] * w0 + t.uv1[1] * w1 + t.uv2[1] * w2;
            } else {
                tu = w1;
                tv = w2;
            }
            an = cross(sub(p1, p0), sub(p2, p0));
            smp.material_index = t.material_index;
        }
        const float alen = len(an);
        if (alen <= 1e-12f) return empty_sample();
        smp.normal = divs(an, alen);
        const float3 tl = sub(smp.position, sp);
        const float d2 = len_sq(tl);
        if (d2 <= 1e-12f) return empty_sample();
        smp.distance = sqrtf(d2);
        smp.direction = divs(tl, smp.distance);
        const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
        cond = area_pdf(light.type == 1 ? alen : 0.5f * alen, d2, ac);
    }
    if (cond <= 0.0f || smp.material_index < 0 || smp.material_index >= s.material_count) return empty_sample();
    smp.emission = material_emission<kPbr>(s, s.materials[smp.material_index], tu, tv, smp.position);
    smp.pdf = sel * cond;
    smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
    return smp;
}

// sample_analytic_direct_light_candidate, programs.cu:1234-1346
// Disk and rect lights (the common case) read only the light's hot record
// (DeviceScene::analytic_hot); the other types read the full light.
RTGB_D LightSample analytic_candidate(const DeviceScene& s, const float3& sp, int li, float u0, float u1) {
    LightSample smp = empty_sample();
    if (li < 0 || li >= s.analytic_count) return smp;
    const float4* hot = s.analytic_hot + static_cast<long long>(kAnalyticHot) * li;
    const float4 h0 = __ldg(hot);
    const float4 h3 = __ldg(hot + 3);
    const float4 h4 = __ldg(hot + 4);
    if (h0.w <= 0.0f) return smp;  // selection_pdf
    const int type = __float_as_int(h4.w);
    if (type == 1 || type == 2) {
        const float4 h1 = __ldg(hot + 1);
        const float4 h2 = __ldg(hot + 2);
        smp.light_index = li;
        smp.emission = xyz(h3);
        const float3 center = xyz(h0);
        if (type == 1) {
            const float radial = h1.w * sqrtf(u0);  // radius
            const float phi = 2.0f * kPi * u1;
            smp.position = add(center, add(mul(xyz(h1), radial * cosf(phi)), mul(xyz(h2), radial * sinf(phi))));
        } else {
            smp.position = add(center, add(mul(xyz(h1), (u0 - 0.5f) * h1.w), mul(xyz(h2), (u1 - 0.5f) * h2.w)));
        }
        smp.normal = xyz(h4);
        const float3 tl = sub(smp.position, sp);
        const float d2 = len_sq(tl);
        if (d2 <= 1e-12f) return empty_sample();
        smp.distance = sqrtf(d2);
        smp.direction = divs(tl, smp.distance);
        const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
        smp.pdf = h0.w * area_pdf(h3.w, d2, ac);
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }
    const rtgb_analytic_light& l = s.analytic[li];
    smp.light_index = li;
    smp.emission = ld3(l.radiance);
    if (l.type == 5) {
        smp.direction = sphere_direction(u0, u1);
        smp.distance = kRayFar;
        smp.pdf = l.selection_pdf * uniform_sphere_pdf();
        smp.infinite = true;
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }
    if (l.type == 4) {
        const float3 axis = normalize(ld3(l.basis_z));
        smp.direction = l.delta != 0 ? axis : cone_direction(axis, l.cos_theta_max, u0, u1);
        smp.distance = kRayFar;
        smp.pdf = l.selection_pdf * (l.delta != 0 ? 1.0f : uniform_cone_pdf(l.cos_theta_max));
        smp.infinite = true;
        smp.delta = l.delta != 0;
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }
    const float3 center = ld3(l.position);
    if (l.type == 0) {
        const float3 tc = sub(center, sp);
        const float d2 = len_sq(tc);
        const float radius = l.radius * len(ld3(l.basis_x));
        const float r2 = radius * radius;
        if (d2 <= r2 * (1.0f + 1e-6f)) return smp;
        if (l.treat_as_point != 0) {
            smp.distance = sqrtf(d2);
            smp.direction = divs(tc, smp.distance);
            const float iscale = l.world_area > 1e-12f ? l.world_area : 1.0f;
            smp.emission = mul(smp.emission, iscale / d2);
            smp.pdf = l.selection_pdf;
            smp.delta = true;
            smp.valid = max_comp(smp.emission) > 0.0f;
            return smp;
        }
        const float ctm = sqrtf(fmaxf(0.0f, 1.0f - r2 / d2));
        smp.direction = cone_direction(normalize(tc), ctm, u0, u1);
        AnalyticHit sh;
        sh.hit = false;
        if (!hit_analytic(l, sp, smp.direction, kRayEpsilon, kRayFar, sh)) return empty_sample();
        smp.position = sh.pos;
        smp.normal = sh.normal;
        smp.distance = sh.t;
        smp.pdf = l.selection_pdf * uniform_cone_pdf(ctm);
        smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
        return smp;
    }
    if (l.type == 3) {
        const float phi = 2.0f * kPi * u0;
        const float rx = l.radius * cosf(phi);
        const float ry = l.radius * sinf(phi);
        smp.position = add(center, add(add(mul(ld3(l.basis_x), rx), mul(ld3(l.basis_y), ry)),
                                       mul(ld3(l.basis_z), (u1 - 0.5f) * l.length)));
        smp.normal = normalize(add(mul(ld3(l.basis_x), rx), mul(ld3(l.basis_y), ry)));
    } else {
        return empty_sample();
    }
    const float3 tl = sub(smp.position, sp);
    const float d2 = len_sq(tl);
    if (d2 <= 1e-12f) return empty_sample();
    smp.distance = sqrtf(d2);
    smp.direction = divs(tl, smp.distance);
    const float ac = dot(smp.normal, mul(smp.direction, -1.0f));
    smp.pdf = l.selection_pdf * area_pdf(l.world_area, d2, ac);
    smp.valid = smp.pdf > 0.0f && max_comp(smp.emission) > 0.0f;
    return smp;
}

// direct_material_response, programs.cu:1026-1055 (legacy materials)
RTGB_D void openpbr_color_binding(const DeviceScene& s, pbr::Mat& m, const rtgb_openpbr_material& c, int input,
    float u, float v, const float3& p) {
    const int tex = c.color_texture[input];
    if (tex < 0) return;
    pbr::apply_color(m, input, pv(eval_texture(s, tex, u, v, p)), c.color_space[input]);
}

RTGB_D void openpbr_scattering(const DeviceScene& s, const Hit& h, pbr::Mat& m) {
    const rtgb_openpbr_material& c = s.openpbr[h.openpbr];
    openpbr_load(c, m);
    if (c.color_texture[0] >= 0) m.base_color = pv(h.base);
    openpbr_color_binding(s, m, c, 1, h.u, h.v, h.pos);
    openpbr_color_binding(s, m, c, 2, h.u, h.v, h.pos);
    for (int k = 0; k < 2; ++k) {
        if (c.scalar_texture[k] >= 0) pbr::apply_scalar(m, k, eval_texture(s, c.scalar_texture[k], h.u, h.v, h.pos).x);
    }
}

// OpenPBR branch of direct_material_response (programs.cu:1038-1054) with the
// hit's scattering parameters already evaluated; `ray_d` is the incoming ray.
// kInline: the BSDF evaluation inlined (the shade kernel) or the shared
// out-of-line copy (the ReSTIR kernels' many call sites); same arithmetic.
template <bool kInline>
RTGB_D float3 openpbr_response(const pbr::Mat& m, const Hit& h, const float3& ray_d, const float3& thr,
    const float3& ldir, float& bsdf_pdf) {
    const pbr::Frame frame = pbr::make_frame(pv(h.gn), pbr::V3{0.0f, 0.0f, 0.0f});
    const pbr::V3 wo = pv(mul(normalize(ray_d), -1.0f));
    pbr::Eval e{};
    if constexpr (kInline) {
        e = pbr::evaluate_inline(m, frame, wo, pv(ldir), transport_context(thr));
    } else {
        e = pbr::evaluate(m, frame, wo, pv(ldir), transport_context(thr));
    }
    const float cosine = fabsf(dot(h.sn, ldir));
    bsdf_pdf = e.pdf;
    return mul(fv(e.value), cosine);
}

// direct_material_response, programs.cu:1026-1055. `pm` holds the OpenPBR
// scattering parameters when h.mtype == 5 (evaluated once per hit).
template <bool kPbr, bool kInline = false>
RTGB_D float3 direct_response(const Hit& h, const pbr::Mat* pm, const float3& ray_d, const float3& thr,
    const float3& ldir, float& bsdf_pdf) {
    bsdf_pdf = 0.0f;
    if constexpr (kPbr) {
        if (h.mtype == 5) return openpbr_response<kInline>(*pm, h, ray_d, thr, ldir, bsdf_pdf);
    }
    if (h.mtype == 0) {
        const float c = fmaxf(dot(h.sn, ldir), 0.0f);
        bsdf_pdf = c / kPi;
        return mul(h.base, bsdf_pdf);
    }
    if (h.mtype == 4) {
        bsdf_pdf = uniform_sphere_pdf();
        return mul(h.base, bsdf_pdf);
    }
    return f3(0.0f, 0.0f, 0.0f);
}

}  // namespace rtgb
