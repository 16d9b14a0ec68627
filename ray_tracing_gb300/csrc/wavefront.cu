// Wavefront kernels of the realtime radiance path on sm_103a.
//
// The reference renders one camera per launch with a megakernel
// (radiance_kernel, src/realtime/gpu/programs.cu:1828-1953): one thread walks
// one pixel through every sample and bounce. Here every active camera's paths
// share one set of SoA streams and each bounce is three grid-stride launches
// over a compacted queue: trace (closest hit), shade (emission, next-event
// estimation, ReSTIR DI at bounce 0, BSDF sampling, Russian roulette) and
// shadow (any-hit visibility). Per path the RNG is consumed in the
// reference's order, and shadow contributions are added after the bounce's
// emission term exactly where the reference adds them, so a path's radiance is
// the reference's.
#include "shading.cuh"
#include "wavefront.cuh"

namespace rtgb {
namespace {

constexpr int kFlagValid = 1;
constexpr int kFlagDelta = 2;

RTGB_D int camera_of_path(const FrameParams& fp, long long path) {
    int c = 0;
    for (int k = 1; k < fp.cam_count; ++k) {
        if (path >= fp.cam[k].path_offset) c = k;
    }
    return c;
}

RTGB_D int camera_of_pixel(const FrameParams& fp, long long pixel) {
    int c = 0;
    for (int k = 1; k < fp.cam_count; ++k) {
        if (pixel >= fp.cam[k].pixel_offset) c = k;
    }
    return c;
}

// Warp-aggregated queue append: one atomic per warp.
RTGB_D void queue_push(int* queue, int* count, int value, bool pred) {
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, pred);
    if (mask == 0) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(active, base, leader);
    if (pred) queue[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

RTGB_D void count_add(unsigned long long* counter, unsigned long long v) {
    // one atomic per thread with work; called once per thread at kernel end
    if (v) atomicAdd(counter, v);
}

__global__ void k_camera_dirs(CameraDev cam, float4* out) {
    const long long n = static_cast<long long>(cam.width) * cam.height;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(i % cam.width), y = static_cast<int>(i / cam.width);
        const float px = static_cast<float>(x) + 0.5f;
        const float py = static_cast<float>(y) + 0.5f;
        const float3 d = cam.model == RTGB_CAMERA_EQUI62_LUT1D
                             ? unproject_equi(cam.eq_fx, cam.eq_fy, cam.eq_cx, cam.eq_cy, cam.eq_tan, cam.lut,
                                   cam.lut_step, px, py)
                             : unproject_pinhole(cam.pin, px, py);
        out[i] = f4(d, 0.0f);
    }
}

// trace_primary_ray (programs.cu:2086-2099) for every path of every camera.
__global__ void __launch_bounds__(256) k_raygen(const FrameParams* __restrict__ fpp, Paths P, Counters* counters) {
    const FrameParams& fp = *fpp;
    const FrameBufs cur = fp.cur;
    const long long n = fp.total_paths;
    for (long long path = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; path < n;
         path += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int c = camera_of_path(fp, path);
        const CameraDev& cam = fp.cam[c];
        const long long local = path - cam.path_offset;
        const int pixel = static_cast<int>(local / fp.spp);
        const int sample = static_cast<int>(local % fp.spp);
        const float3 dc = xyz(__ldg(cam.dirs + pixel));
        P.ray_o[path] = f4(ld3(cam.origin_f), 0.0f);
        P.ray_d[path] = f4(cam_to_world(cam, dc), 0.0f);
        P.thr[path] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        P.rad[path] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        P.prev_pos[path] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(kFlagDelta));
        P.prev_nrm[path] = make_float4(0.0f, 0.0f, 1.0f, __int_as_float(-1));
        P.prev_prim[path] = make_int2(-1, -1);
        P.rng[path] = rng_for(pixel, sample, fp.stream);
        P.aux_n[path] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        P.aux_a[path] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        P.queue[0][path] = static_cast<int>(path);
        if (P.res_written) P.res_written[path] = 0;
        if (sample == 0) cur.reservoirs[cam.pixel_offset + pixel] = zero_reservoir();
        if (fp.record_paths) {
            for (int b = 0; b < fp.max_bounces; ++b) P.codes[path * fp.max_bounces + b] = -2;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters->active[0] = static_cast<int>(n);
        counters->rays[0] = 0;
        counters->rays[1] = 0;
        counters->rays[2] = 0;
        counters->rays[3] = 0;
        counters->restir_pixels = 0;
    }
}

// intersect_scene (programs.cu:1654-1757) + intersect_analytic_lights (:795-813)
__global__ void __launch_bounds__(128) k_trace(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters, int bounce) {
    const int in = bounce & 1;
    const int count = counters->active[in];
    if (blockIdx.x == 0 && threadIdx.x == 0 && bounce < 64) counters->bounce_active[bounce] = count;
    int overflow = 0;
    unsigned long long traced = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.queue[in][i];
        const float3 o = xyz(P.ray_o[path]);
        const float3 d = xyz(P.ray_d[path]);
        float closest = kRayFar;
        int code = traverse_closest(s, o, d, kRayEpsilon, closest, overflow);
        ++traced;
        if (s.medium_count > 0) {
            uint32_t rng = P.rng[path];
            const float ray_len = len(d);
            if (ray_len > 1e-8f) {
                for (int m = 0; m < s.medium_count; ++m) {
                    const rtgb_medium med = s.media[m];
                    if (med.density <= 0.0f) continue;
                    float entry = 0.0f, exit = 0.0f;
                    if (!medium_boundary(med, o, d, kRayEpsilon, closest, entry, exit)) continue;
                    entry = fmaxf(entry, kRayEpsilon);
                    exit = fminf(exit, closest);
                    if (entry >= exit) continue;
                    const float inside = (exit - entry) * ray_len;
                    const float u = fmaxf(rnd(rng), 1e-6f);
                    const float hd = -logf(u) / med.density;
                    if (hd >= inside) continue;
                    closest = entry + hd / ray_len;
                    code = (4 << 28) | m;
                }
            }
            P.rng[path] = rng;
        }
        float at = kRayFar;
        const int light = traverse_analytic(s, o, d, kRayEpsilon, code != -1 ? closest : kRayFar, at);
        P.hit[path] = make_float4(closest, __int_as_float(code), __int_as_float(light), at);
    }
    count_add(&counters->rays[bounce == 0 ? 0 : 1], traced);
    if (overflow) atomicAdd(&counters->overflow, overflow);
}

struct ShadeCtx {
    const FrameParams& fp;
    const DeviceScene& s;
    int overflow;
    unsigned long long vis_rays;
    unsigned long long restir_runs;
    const float* analytic_cdf;  // shared-memory copy when it fits, else global
};

RTGB_D float restir_lum(const float3& v) { return fmaxf(0.0f, 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z); }

RTGB_D float3 unshadowed(const Hit& h, const LightSample& l, bool bsdf_avail, float& target) {
    target = 0.0f;
    if (!l.valid || l.pdf <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
    float bp = 0.0f;
    const float3 resp = direct_response(h, l.direction, bp);
    if (max_comp(resp) <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
    const float mis = l.delta || !bsdf_avail ? 1.0f : power_heuristic(l.pdf, bp);
    const float3 num = mul(mul(l.emission, resp), mis);
    target = restir_lum(num);
    return num;
}

RTGB_D Surface restir_surface(const Hit& h) {
    Surface s;
    s.position[0] = h.pos.x;
    s.position[1] = h.pos.y;
    s.position[2] = h.pos.z;
    s.normal[0] = h.sn.x;
    s.normal[1] = h.sn.y;
    s.normal[2] = h.sn.z;
    s.material_type = h.mtype;
    s.primitive_type = h.ptype;
    s.primitive_index = h.pidx;
    return s;
}

// restir_previous_pixel, programs.cu:2144-2171 (pixel index inside the camera)
RTGB_D bool previous_pixel(const FrameParams& fp, int c, const Hit& h, int& index) {
    index = -1;
    if (fp.history_length[c] <= 0 || fp.prev_valid[c] == 0) return false;
    const CameraDev& pc = fp.prev[c];
    const float3 off = sub(h.pos, ld3(pc.origin_f));
    const float3 cp = f3(dot(off, ld3(pc.bx_f)), dot(off, ld3(pc.by_f)), dot(off, ld3(pc.bz_f)));
    const float2 px = project_camera(pc, cp);
    if (!isfinite(px.x) || !isfinite(px.y)) return false;
    const int x = static_cast<int>(floorf(px.x));
    const int y = static_cast<int>(floorf(px.y));
    const CameraDev& cc = fp.cam[c];
    if (x < 0 || x >= cc.width || y < 0 || y >= cc.height) return false;
    index = y * cc.width + x;
    return true;
}

// restir_target_at_previous_surface, programs.cu:2210-2247: one closest-hit
// visibility ray from the previous camera to the reuse source's surface.
RTGB_D float target_at_previous(ShadeCtx& ctx, int c, const Surface& src, const Candidate& sel, bool bsdf_avail) {
    const FrameParams& fp = ctx.fp;
    if (fp.prev_valid[c] == 0) return 0.0f;
    const float3 spos = ld3(src.position);
    const float3 origin = ld3(fp.prev[c].origin_f);
    const float3 off = sub(spos, origin);
    const float dist = len(off);
    if (!isfinite(dist) || dist <= kRayEpsilon) return 0.0f;
    const float3 dir = mul(off, 1.0f / dist);
    float closest = dist + 0.05f;
    ++ctx.vis_rays;
    const int code = traverse_closest(ctx.s, origin, dir, kRayEpsilon, closest, ctx.overflow);
    if (code == -1) return 0.0f;
    Hit sh;
    if (!reconstruct_surface(ctx.s, code, origin, dir, sh)) return 0.0f;
    if (sh.mtype != src.material_type || sh.ptype != src.primitive_type || sh.pidx != src.primitive_index) {
        return 0.0f;
    }
    const float tol = fmaxf(0.01f, 0.02f * dist);
    if (len_sq(sub(sh.pos, spos)) > tol * tol || dot(sh.sn, ld3(src.normal)) < 0.95f) return 0.0f;
    const LightSample l = analytic_candidate(ctx.s, sh.pos, sel.light_index, sel.u0, sel.u1);
    float t = 0.0f;
    unshadowed(sh, l, bsdf_avail, t);
    return t;
}

RTGB_D Surface load_surface(const Reservoir* r) {
    Surface s;
    const Surface* p = &r->surface;
    for (int k = 0; k < 3; ++k) {
        s.position[k] = p->position[k];
        s.normal[k] = p->normal[k];
    }
    s.material_type = p->material_type;
    s.primitive_type = p->primitive_type;
    s.primitive_index = p->primitive_index;
    return s;
}

// accumulate_restir_analytic_direct_light, programs.cu:2315-2449. Writes the
// reservoir and the shadow query of its selected sample into slot 1.
RTGB_D void restir_direct(ShadeCtx& ctx, const Paths& P, FrameBufs& cur, const FrameBufs& hist, int c, int x, int y,
    long long path, const Hit& h, uint32_t& rng, bool bsdf_avail, const float3& thr, float4& sh_o, float4& sh_d,
    float4& sh_c) {
    const FrameParams& fp = ctx.fp;
    const DeviceScene& s = ctx.s;
    ++ctx.restir_runs;
    const CameraDev& cam = fp.cam[c];
    Reservoir r = empty_reservoir();
    const int req = fp.restir_candidates > 0 ? fp.restir_candidates : 1;
    const int count = req < 32 ? req : 32;
    for (int k = 0; k < count; ++k) {
        Candidate cand;
        cand.light_index = sample_cdf(ctx.analytic_cdf, s.analytic_count, rnd(rng));
        cand.u0 = rnd(rng);
        cand.u1 = rnd(rng);
        const LightSample l = analytic_candidate(s, h.pos, cand.light_index, cand.u0, cand.u1);
        float t = 0.0f;
        unshadowed(h, l, bsdf_avail, t);
        const float w = l.pdf > 0.0f ? t / l.pdf : 0.0f;
        reservoir_update(r, cand, t, w, 1, rnd(rng));
    }
    const int canonical = r.candidate_count;
    // Reuse sources are kept as history pixel indices; their surfaces are
    // re-read for bias correction instead of being held in local memory.
    int src_index[9];
    int mult[9];
    int nsrc = 0;
    int selected_src = -1;
    const Reservoir* hres = hist.reservoirs + cam.pixel_offset;
    const Surface cur_surface = restir_surface(h);
    const int nbrs = fp.restir_spatial < 8 ? fp.restir_spatial : 8;
    int reproj = -1;
    // restir_temporal_candidate and restir_spatial_candidate reproject the
    // same hit into the same previous camera; the projection runs once.
    const bool have_prev = (fp.restir_temporal != 0 || nbrs > 0) && previous_pixel(fp, c, h, reproj);
    if (fp.restir_temporal != 0 && have_prev) {
        const Reservoir prev = hres[reproj];
        const float tol = fmaxf(0.005f, 0.01f * h.t);
        if (surface_valid(cur_surface, prev, tol, 0.95f, fp.restir_max_age)) {
            const LightSample l = analytic_candidate(s, h.pos, prev.selected.light_index, prev.selected.u0,
                prev.selected.u1);
            float t = 0.0f;
            unshadowed(h, l, bsdf_avail, t);
            const MergeResult m = reservoir_merge(r, prev, t, fp.restir_max_temporal, rnd(rng), true);
            if (m.multiplicity > 0) {
                src_index[nsrc] = reproj;
                mult[nsrc] = m.multiplicity;
                if (m.selected != 0) selected_src = nsrc;
                ++nsrc;
            }
        }
    }
    if (nbrs > 0 && have_prev) {
        const int rot = (x * 3 + y * 5 + static_cast<int>(fp.stream)) & 7;
        for (int k = 0; k < nbrs; ++k) {
            const int oi = (rot + k) & 7;
            // kOffsets of programs.cu:2187-2196
            const int dx = (oi == 0 || oi == 4 || oi == 6) ? -1 : ((oi == 1 || oi == 5 || oi == 7) ? 1 : 0);
            const int dy = (oi == 2 || oi == 4 || oi == 5) ? -1 : ((oi == 3 || oi == 6 || oi == 7) ? 1 : 0);
            const int nx = reproj % cam.width + dx, ny = reproj / cam.width + dy;
            if (nx < 0 || nx >= cam.width || ny < 0 || ny >= cam.height) continue;
            const int ni = ny * cam.width + nx;
            const Reservoir prev = hres[ni];
            const float tol = fmaxf(0.01f, 0.02f * h.t);
            if (!surface_valid(cur_surface, prev, tol, 0.95f, fp.restir_max_age)) continue;
            const LightSample l = analytic_candidate(s, h.pos, prev.selected.light_index, prev.selected.u0,
                prev.selected.u1);
            float t = 0.0f;
            unshadowed(h, l, bsdf_avail, t);
            const MergeResult m = reservoir_merge(r, prev, t, fp.restir_max_spatial, rnd(rng), false);
            if (m.multiplicity > 0 && nsrc < 9) {
                src_index[nsrc] = ni;
                mult[nsrc] = m.multiplicity;
                if (m.selected != 0) selected_src = nsrc;
                ++nsrc;
            }
        }
    }
    r.surface = cur_surface;
    if (fp.restir_bias == 1 && nsrc > 0 && r.valid != 0) {
        float sel_t = r.selected_target;
        float sum = r.selected_target * static_cast<float>(canonical);
        for (int k = 0; k < nsrc; ++k) {
            const float t = target_at_previous(ctx, c, load_surface(hres + src_index[k]), r.selected, bsdf_avail);
            sum += t * static_cast<float>(mult[k]);
            if (selected_src == k) sel_t = t;
        }
        reservoir_finalize_basic(r, sel_t, sum, nsrc);
    } else {
        reservoir_finalize(r);
    }
    if (fp.spp == 1) {
        cur.reservoirs[cam.pixel_offset + y * cam.width + x] = r;
    } else {
        P.res_scratch[path] = r;
        P.res_written[path] = 1;
    }
    if (r.valid == 0) return;
    const LightSample l = analytic_candidate(s, h.pos, r.selected.light_index, r.selected.u0, r.selected.u1);
    float t = 0.0f;
    const float3 num = unshadowed(h, l, bsdf_avail, t);
    if (!l.valid || t <= 0.0f) return;
    const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
    if (max_t <= kRayEpsilon) return;
    sh_o = f4(add(h.pos, mul(l.direction, kRayEpsilon * 2.0f)), max_t);
    sh_d = f4(l.direction, 0.0f);
    sh_c = f4(mul(thr, mul(num, r.estimator_weight)), 1.0f);
}

RTGB_D void load_path(const Paths& P, int path, PathRegs& st) {
    st.o = xyz(P.ray_o[path]);
    st.d = xyz(P.ray_d[path]);
    const float4 thr4 = P.thr[path];
    st.thr = xyz(thr4);
    st.prev_pdf = thr4.w;
    st.rad = xyz(P.rad[path]);
    const float4 pp = P.prev_pos[path];
    const float4 pn = P.prev_nrm[path];
    const int2 pprim = P.prev_prim[path];
    st.prev_pos = xyz(pp);
    st.prev_nrm = xyz(pn);
    const int flags = __float_as_int(pp.w);
    st.prev_valid = (flags & kFlagValid) != 0;
    st.prev_delta = (flags & kFlagDelta) != 0;
    st.prev_mtype = __float_as_int(pn.w);
    st.prev_ptype = pprim.x;
    st.prev_pidx = pprim.y;
    st.alive = true;
}

// sample_bsdf (programs.cu:2463-2565) and apply_russian_roulette (:1764-1771):
// returns whether the path continues.
RTGB_D bool scatter(const FrameParams& fp, const Hit& h, int bounce, uint32_t& rng, PathRegs& st) {
    bool scattered = false;
    float pdf = 0.0f;
    bool delta = true;
    if (h.mtype == 0) {
        float3 dir = add(h.sn, random_unit_vector(rng));
        if (near_zero(dir)) dir = h.sn;
        st.o = add(h.pos, mul(h.sn, kRayEpsilon));
        st.d = normalize(dir);
        st.thr = mul(st.thr, h.base);
        pdf = fmaxf(dot(h.sn, st.d), 0.0f) / kPi;
        delta = false;
        scattered = true;
    } else if (h.mtype == 1) {
        const float3 refl = reflect(normalize(st.d), h.sn);
        const float3 fz = mul(random_in_unit_sphere(rng), fminf(fmaxf(h.fuzz, 0.0f), 1.0f));
        const float3 sc = normalize(add(refl, fz));
        if (dot(sc, h.sn) > 0.0f) {
            st.o = add(h.pos, mul(h.sn, kRayEpsilon));
            st.d = sc;
            st.thr = mul(st.thr, h.base);
            scattered = true;
        }
    } else if (h.mtype == 2) {
        const float ratio = h.front ? (1.0f / fmaxf(h.ior, 1e-4f)) : fmaxf(h.ior, 1e-4f);
        const float3 ud = normalize(st.d);
        const float ct = fminf(dot(mul(ud, -1.0f), h.sn), 1.0f);
        const float stt = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        bool refl = ratio * stt > 1.0f;
        if (!refl) {
            float r0 = (1.0f - ratio) / (1.0f + ratio);
            r0 *= r0;
            refl = r0 + (1.0f - r0) * powf(1.0f - ct, 5.0f) > rnd(rng);
        }
        const float3 dir = refl ? reflect(ud, h.sn) : refract(ud, h.sn, ratio);
        st.o = add(h.pos, mul(dir, kRayEpsilon));
        st.d = normalize(dir);
        st.thr = mul(st.thr, h.base);
        scattered = true;
    } else if (h.mtype == 4) {
        const float3 dir = random_unit_vector(rng);
        st.o = add(h.pos, mul(dir, kRayEpsilon));
        st.d = dir;
        st.thr = mul(st.thr, h.base);
        pdf = uniform_sphere_pdf();
        delta = false;
        scattered = true;
    }
    if (!scattered) return false;
    st.prev_pos = h.pos;
    st.prev_nrm = h.sn;
    st.prev_pdf = pdf;
    st.prev_mtype = h.mtype;
    st.prev_ptype = h.ptype;
    st.prev_pidx = h.pidx;
    st.prev_valid = true;
    st.prev_delta = delta;
    if (bounce >= fp.rr_start) {
        const float q = fminf(fmaxf(max_comp(st.thr), 0.05f), 0.95f);
        if (rnd(rng) > q) return false;
        st.thr = divs(st.thr, q);
    }
    return bounce + 1 < fp.max_bounces;
}

RTGB_D void store_path(const Paths& P, int path, const PathRegs& st) {
    P.ray_o[path] = f4(st.o, 0.0f);
    P.ray_d[path] = f4(st.d, 0.0f);
    P.thr[path] = f4(st.thr, st.prev_pdf);
    P.prev_pos[path] = f4(st.prev_pos, __int_as_float((st.prev_valid ? kFlagValid : 0) | (st.prev_delta ? kFlagDelta : 0)));
    P.prev_nrm[path] = f4(st.prev_nrm, __int_as_float(st.prev_mtype));
    P.prev_prim[path] = make_int2(st.prev_ptype, st.prev_pidx);
}

// Surface rebuild for a queued path (the hit record of this bounce).
RTGB_D bool rebuild_hit(const DeviceScene& s, const float4& hr, const PathRegs& st, Hit& h) {
    const int code = __float_as_int(hr.y);
    if ((static_cast<unsigned>(code) >> 28) == 4) {
        reconstruct_medium(s, code & 0x0fffffff, hr.x, st.o, st.d, h);
        return true;
    }
    return reconstruct_surface(s, code, st.o, st.d, h);
}

// One bounce of radiance_kernel's loop body (programs.cu:1855-1932) per path.
// At the ReSTIR bounce, surfaces that run ReSTIR DI stop after the
// emissive-geometry NEE and continue in k_restir, which consumes the RNG
// stream from exactly this point.
__global__ void __launch_bounds__(128) k_shade(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters, int bounce) {
    const FrameParams& fp = *fpp;
    const int in = bounce & 1;
    const int out = in ^ 1;
    const int count = counters->active[in];
    const bool restir_bounce = fp.restir_enabled != 0 && bounce == 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.queue[in][i];
        const float4 hr = P.hit[path];
        const int code = __float_as_int(hr.y);
        const int alight = __float_as_int(hr.z);
        PathRegs st;
        load_path(P, path, st);
        uint32_t rng = P.rng[path];
        if (fp.record_paths) {
            P.codes[static_cast<long long>(path) * fp.max_bounces + bounce] =
                alight >= 0 ? ((5 << 28) | alight) : code;
        }
        float4 sh_o[2], sh_d[2], sh_c[2];
        sh_c[0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        sh_c[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bool keep = false;
        bool deferred = false;
        if (alight >= 0) {
            AnalyticHit ah;
            ah.hit = hit_analytic(s.analytic[alight], st.o, st.d, kRayEpsilon, kRayFar, ah);
            ah.light = alight;
            const float w = analytic_emission_mis(s, st, ah);
            st.rad = add(st.rad, mul(st.thr, mul(ld3(s.analytic[alight].radiance), w)));
        } else if (code == -1) {
            const float w = emission_mis_weight(s, st, nullptr, true);
            st.rad = add(st.rad, mul(st.thr, mul(ld3(s.background), w)));
            st.rad = add(st.rad, mul(st.thr, analytic_infinite_radiance(s, st)));
        } else {
            Hit h;
            if (!rebuild_hit(s, hr, st, h)) {
                atomicAdd(&counters->error, 1);
            } else {
                if (bounce == 0) {
                    P.aux_n[path] = f4(h.sn, h.t);
                    P.aux_a[path] = f4(h.base, 1.0f);
                }
                const float ew = emission_mis_weight(s, st, &h, false);
                st.rad = add(st.rad, mul(st.thr, mul(h.emis, ew)));
                const bool bsdf_avail = bounce + 1 < fp.max_bounces;
                // accumulate_direct_light (programs.cu:2249-2280) -> shadow slot 0
                if (h.mtype != 3 && s.light_count > 0) {
                    const LightSample l = sample_direct(s, h, rng);
                    if (l.valid) {
                        float bp = 0.0f;
                        const float3 resp = direct_response(h, l.direction, bp);
                        if (max_comp(resp) > 0.0f) {
                            const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
                            if (max_t > kRayEpsilon) {
                                const float mis = bsdf_avail ? power_heuristic(l.pdf, bp) : 1.0f;
                                const float3 direct = mul(mul(l.emission, resp), mis / l.pdf);
                                sh_o[0] = f4(add(h.pos, mul(l.direction, kRayEpsilon * 2.0f)), max_t);
                                sh_d[0] = f4(l.direction, 0.0f);
                                sh_c[0] = f4(mul(st.thr, direct), 1.0f);
                            }
                        }
                    }
                }
                if (restir_bounce) {
                    // accumulate_restir_analytic_direct_light returns before any
                    // draw for emitters and light-less scenes (programs.cu:2318-2321)
                    deferred = h.mtype != 3 && s.analytic_count > 0;
                } else if (h.mtype != 3 && s.analytic_count > 0) {
                    // accumulate_analytic_direct_light (programs.cu:2282-2313) -> shadow slot 1
                    const int li = sample_cdf(s.analytic_cdf, s.analytic_count, rnd(rng));
                    const float u0 = rnd(rng);
                    const float u1 = rnd(rng);
                    const LightSample l = analytic_candidate(s, h.pos, li, u0, u1);
                    if (l.valid) {
                        float bp = 0.0f;
                        const float3 resp = direct_response(h, l.direction, bp);
                        if (max_comp(resp) > 0.0f) {
                            const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
                            if (max_t > kRayEpsilon) {
                                const float mis = l.delta || !bsdf_avail ? 1.0f : power_heuristic(l.pdf, bp);
                                const float3 direct = mul(mul(l.emission, resp), mis / l.pdf);
                                sh_o[1] = f4(add(h.pos, mul(l.direction, kRayEpsilon * 2.0f)), max_t);
                                sh_d[1] = f4(l.direction, 0.0f);
                                sh_c[1] = f4(mul(st.thr, direct), 1.0f);
                            }
                        }
                    }
                }
                if (!deferred && bsdf_avail) keep = scatter(fp, h, bounce, rng, st);
            }
        }
        P.rad[path] = f4(st.rad, 0.0f);
        P.rng[path] = rng;
        if (keep) store_path(P, path, st);
        if (deferred) {
            // slot 0 travels to k_restir, which adds slot 1 and queues the shadow rays
            P.sh_c[0][path] = sh_c[0];
            if (sh_c[0].w != 0.0f) {
                P.sh_o[0][path] = sh_o[0];
                P.sh_d[0][path] = sh_d[0];
            }
        } else {
            const bool any_shadow = sh_c[0].w != 0.0f || sh_c[1].w != 0.0f;
            for (int k = 0; k < 2; ++k) {
                if (sh_c[k].w != 0.0f) {
                    P.sh_o[k][path] = sh_o[k];
                    P.sh_d[k][path] = sh_d[k];
                }
                if (any_shadow) P.sh_c[k][path] = sh_c[k];
            }
            queue_push(P.shadow_queue, &counters->shadow, path, any_shadow);
        }
        queue_push(P.queue[out], &counters->active[out], path, keep);
        queue_push(P.restir_queue, &counters->restir, path, deferred);
    }
}

// ReSTIR DI for the deferred bounce-0 surfaces, then their BSDF scatter.
constexpr int kSharedCdf = 4096;

__global__ void __launch_bounds__(128) k_restir(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters) {
    __shared__ float cdf_shared[kSharedCdf];
    const FrameParams& fp = *fpp;
    FrameBufs cur = fp.cur;
    const FrameBufs hist = fp.hist;
    const int count = counters->restir;
    if (count == 0) return;
    const bool shared = s.analytic_count <= kSharedCdf;
    if (shared) {
        for (int k = threadIdx.x; k < s.analytic_count; k += blockDim.x) cdf_shared[k] = s.analytic_cdf[k];
        __syncthreads();
    }
    ShadeCtx ctx{fp, s, 0, 0ull, 0ull, shared ? cdf_shared : s.analytic_cdf};
    constexpr int bounce = 0;
    const int out = 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.restir_queue[i];
        const float4 hr = P.hit[path];
        PathRegs st;
        load_path(P, path, st);
        uint32_t rng = P.rng[path];
        Hit h;
        rebuild_hit(s, hr, st, h);
        const bool bsdf_avail = bounce + 1 < fp.max_bounces;
        const int c = camera_of_path(fp, path);
        const CameraDev& cam = fp.cam[c];
        const int pixel = static_cast<int>((path - cam.path_offset) / fp.spp);
        float4 sh_o1, sh_d1, sh_c1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        restir_direct(ctx, P, cur, hist, c, pixel % cam.width, pixel / cam.width, path, h, rng, bsdf_avail, st.thr,
            sh_o1, sh_d1, sh_c1);
        const bool keep = bsdf_avail && scatter(fp, h, bounce, rng, st);
        P.rng[path] = rng;
        if (keep) store_path(P, path, st);
        const bool slot0 = P.sh_c[0][path].w != 0.0f;
        const bool any_shadow = slot0 || sh_c1.w != 0.0f;
        if (sh_c1.w != 0.0f) {
            P.sh_o[1][path] = sh_o1;
            P.sh_d[1][path] = sh_d1;
        }
        if (any_shadow) P.sh_c[1][path] = sh_c1;
        queue_push(P.shadow_queue, &counters->shadow, path, any_shadow);
        queue_push(P.queue[out], &counters->active[out], path, keep);
    }
    count_add(&counters->rays[3], ctx.vis_rays);
    count_add(&counters->restir_pixels, ctx.restir_runs);
    if (ctx.overflow) atomicAdd(&counters->overflow, ctx.overflow);
}

// is_occluded (programs.cu:1759-1762) for the bounce's NEE samples; visible
// contributions are added in slot order (emissive geometry, then analytic).
__global__ void __launch_bounds__(128) k_shadow(DeviceScene s, Paths P, Counters* counters, int bounce) {
    const int count = counters->shadow;
    int overflow = 0;
    unsigned long long traced = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.shadow_queue[i];
        float3 rad = xyz(P.rad[path]);
        for (int k = 0; k < 2; ++k) {
            const float4 c = P.sh_c[k][path];
            if (c.w == 0.0f) continue;
            const float4 o = P.sh_o[k][path];
            const float4 d = P.sh_d[k][path];
            ++traced;
            if (!traverse_any(s, xyz(o), xyz(d), kRayEpsilon, o.w, overflow)) rad = add(rad, xyz(c));
        }
        P.rad[path] = f4(rad, 0.0f);
    }
    count_add(&counters->rays[2], traced);
    if (bounce < 64) count_add(&counters->shadow_bounce[bounce], traced);
    if (overflow) atomicAdd(&counters->overflow, overflow);
}

// Sample averaging and store_output (programs.cu:1935-1952, :1773-1805).
__global__ void __launch_bounds__(256) k_finalize(const FrameParams* __restrict__ fpp, Paths P, Counters* counters) {
    const FrameParams& fp = *fpp;
    const FrameBufs cur = fp.cur;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) counters->cum_rays[k] += counters->rays[k];
    }
    for (long long pix = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; pix < fp.total_pixels;
         pix += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int c = camera_of_pixel(fp, pix);
        const CameraDev& cam = fp.cam[c];
        const long long local = pix - cam.pixel_offset;
        const long long base = cam.path_offset + local * fp.spp;
        float3 beauty = f3(0.0f, 0.0f, 0.0f), nsum = f3(0.0f, 0.0f, 0.0f), asum = f3(0.0f, 0.0f, 0.0f);
        float dsum = 0.0f;
        int aux = 0;
        int last_res = -1;
        for (int smp = 0; smp < fp.spp; ++smp) {
            beauty = add(beauty, xyz(P.rad[base + smp]));
            const float4 aa = P.aux_a[base + smp];
            if (aa.w != 0.0f) {
                const float4 an = P.aux_n[base + smp];
                nsum = add(nsum, xyz(an));
                asum = add(asum, xyz(aa));
                dsum += an.w;
                ++aux;
            }
            if (P.res_written && P.res_written[base + smp]) last_res = smp;
        }
        if (last_res >= 0) cur.reservoirs[pix] = P.res_scratch[base + last_res];
        const float inv_spp = 1.0f / static_cast<float>(fp.spp);
        const float3 bavg = mul(beauty, inv_spp);
        const float inv_aux = aux > 0 ? (1.0f / static_cast<float>(aux)) : 0.0f;
        const float3 navg = aux > 0 ? normalize(mul(nsum, inv_aux)) : f3(0.0f, 0.0f, 1.0f);
        const float3 aavg = aux > 0 ? mul(asum, inv_aux) : f3(0.0f, 0.0f, 0.0f);
        const float davg = aux > 0 ? dsum * inv_aux : 0.0f;
        cur.beauty[pix] = f4(bavg, 1.0f);
        cur.normal[pix] = f4(clamp3(add(mul(navg, 0.5f), f3(0.5f, 0.5f, 0.5f)), 0.0f, 1.0f), 1.0f);
        cur.dnormal[pix] = f4(normalize(f3(dot(navg, ld3(cam.bx_f)), dot(navg, ld3(cam.by_f)), dot(navg, ld3(cam.bz_f)))), 1.0f);
        cur.albedo[pix] = f4(clamp3(aavg, 0.0f, 1.0f), 1.0f);
        cur.depth[pix] = davg;
    }
}

// resolve_reprojection_kernel, programs.cu:1955-2067
__global__ void __launch_bounds__(256) k_resolve(const FrameParams* __restrict__ fpp) {
    const FrameParams& fp = *fpp;
    const FrameBufs cur = fp.cur;
    const FrameBufs hist = fp.hist;
    for (long long pix = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; pix < fp.total_pixels;
         pix += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int c = camera_of_pixel(fp, pix);
        const CameraDev& cam = fp.cam[c];
        const int local = static_cast<int>(pix - cam.pixel_offset);
        const int x = local % cam.width, y = local / cam.width;
        cur.flow[pix] = make_float2(0.0f, 0.0f);
        cur.trust[pix] = 0.0f;
        const int hl = fp.history_length[c];
        if (hl <= 0) continue;
        const float4 cb = cur.beauty[pix];
        const float4 cn = cur.normal[pix];
        const float cd = cur.depth[pix];
        const float pxf = static_cast<float>(x) + 0.5f;
        const float pyf = static_cast<float>(y) + 0.5f;
        const float3 dw = cam_to_world(cam, xyz(__ldg(cam.dirs + local)));
        const float3 wp = add(ld3(cam.origin_f), mul(dw, cd));
        const CameraDev& pc = fp.prev[c];
        const float3 off = f3(static_cast<float>(wp.x - pc.origin[0]), static_cast<float>(wp.y - pc.origin[1]),
            static_cast<float>(wp.z - pc.origin[2]));
        const float3 pcs = f3(dot(off, ld3(pc.bx_f)), dot(off, ld3(pc.by_f)), dot(off, ld3(pc.bz_f)));
        const CameraDev& proj = fp.prev_valid[c] != 0 ? pc : cam;
        const float2 pp = project_camera(proj, pcs);
        const bool finite = isfinite(pp.x) && isfinite(pp.y);
        if (finite) cur.flow[pix] = make_float2(pxf - pp.x, pyf - pp.y);
        const int px = finite ? static_cast<int>(floorf(pp.x)) : -1;
        const int py = finite ? static_cast<int>(floorf(pp.y)) : -1;
        bool valid = false;
        long long pj = 0;
        if (finite && px >= 0 && px < cam.width && py >= 0 && py < cam.height) {
            pj = cam.pixel_offset + py * cam.width + px;
            const float4 hn4 = hist.normal[pj];
            const float3 hn = f3(hn4.x * 2.0f - 1.0f, hn4.y * 2.0f - 1.0f, hn4.z * 2.0f - 1.0f);
            const float3 curn = f3(cn.x * 2.0f - 1.0f, cn.y * 2.0f - 1.0f, cn.z * 2.0f - 1.0f);
            const float nd = dot(curn, hn);
            const float hd = hist.depth[pj];
            const float ed = len(pcs);
            const float tol = fmaxf(0.02f, 0.05f * fmaxf(ed, hd));
            if (nd > 0.95f && fabsf(ed - hd) < tol) valid = true;
        }
        if (!valid) continue;
        cur.trust[pix] = 1.0f;
        const float4 hb = hist.beauty[pj];
        const float4 hn = hist.normal[pj];
        const float hd = hist.depth[pj];
        const float blend = 1.0f / static_cast<float>(hl + 1);
        const float ccx = fminf(fmaxf(cb.x, 0.0f), 10.0f), ccy = fminf(fmaxf(cb.y, 0.0f), 10.0f),
                    ccz = fminf(fmaxf(cb.z, 0.0f), 10.0f);
        if (fp.restir_enabled == 0) {
            cur.beauty[pix] = make_float4(hb.x + (ccx - hb.x) * blend, hb.y + (ccy - hb.y) * blend,
                hb.z + (ccz - hb.z) * blend, 1.0f);
        }
        cur.normal[pix] = make_float4(hn.x + (cn.x - hn.x) * blend, hn.y + (cn.y - hn.y) * blend,
            hn.z + (cn.z - hn.z) * blend, hn.w + (cn.w - hn.w) * blend);
        cur.depth[pix] = hd + (cd - hd) * blend;
    }
}

// Clears the next bounce's queue length and the shadow / ReSTIR queue lengths.
__global__ void k_reset_counters(Counters* counters, int bounce) {
    if (threadIdx.x == 0) {
        counters->active[(bounce & 1) ^ 1] = 0;
        counters->shadow = 0;
        counters->restir = 0;
        if (bounce == 0) {
            for (int b = 0; b < 64; ++b) counters->shadow_bounce[b] = 0;
        }
    }
}

// direction_debug_kernel, programs.cu:1807-1826
__global__ void k_direction_debug(CameraDev cam, uint8_t* rgba) {
    const long long n = static_cast<long long>(cam.width) * cam.height;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float3 d = cam_to_world(cam, xyz(cam.dirs[i]));
        auto enc = [](float v) { return static_cast<uint8_t>(255.0f * clamp01(0.5f * (v + 1.0f))); };
        reinterpret_cast<uchar4*>(rgba)[i] = make_uchar4(enc(d.x), enc(d.y), enc(d.z), 255);
    }
}

// tone_map_to_rgba8, src/realtime/viewer/cuda_gl_presenter.cu:23-38: sqrt gamma,
// clamp to 0.999, round to 8 bits; into a plain device buffer.
__global__ void k_tonemap(const float4* __restrict__ beauty, uint8_t* rgba, long long n) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float4 b = beauty[i];
        auto ch = [](float v) {
            const float c = fminf(fmaxf(sqrtf(fmaxf(v, 0.0f)), 0.0f), 0.999f);
            return static_cast<uint8_t>(lroundf(c * 255.0f));
        };
        reinterpret_cast<uchar4*>(rgba)[i] = make_uchar4(ch(b.x), ch(b.y), ch(b.z), 255);
    }
}

}  // namespace

void launch_camera_dirs(const CameraDev& cam, float4* out, cudaStream_t stream) {
    const long long n = static_cast<long long>(cam.width) * cam.height;
    const int grid = static_cast<int>((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
    k_camera_dirs<<<grid > 0 ? grid : 1, 256, 0, stream>>>(cam, out);
}

void launch_raygen(const FrameParams* fp, Paths paths, Counters* counters, LaunchShape shape, cudaStream_t stream) {
    k_raygen<<<shape.grid, 256, 0, stream>>>(fp, paths, counters);
}

void launch_trace(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, cudaStream_t stream) {
    k_trace<<<shape.grid, 128, 0, stream>>>(fp, scene, paths, counters, bounce);
}

void launch_shade(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, cudaStream_t stream) {
    k_shade<<<shape.grid, 128, 0, stream>>>(fp, scene, paths, counters, bounce);
}

void launch_shadow(DeviceScene scene, Paths paths, Counters* counters, int bounce, LaunchShape shape,
    cudaStream_t stream) {
    k_shadow<<<shape.grid, 128, 0, stream>>>(scene, paths, counters, bounce);
}

void launch_restir(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, LaunchShape shape,
    cudaStream_t stream) {
    k_restir<<<shape.grid, 128, 0, stream>>>(fp, scene, paths, counters);
}

void launch_finalize(const FrameParams* fp, Paths paths, Counters* counters, LaunchShape shape, cudaStream_t stream) {
    k_finalize<<<shape.grid, 256, 0, stream>>>(fp, paths, counters);
}

void launch_resolve(const FrameParams* fp, LaunchShape shape, cudaStream_t stream) {
    k_resolve<<<shape.grid, 256, 0, stream>>>(fp);
}

void query_launch_shapes(int sm_count, LaunchShape* shapes) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_raygen, 256, 0);
    shapes[0] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 256};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_trace, 128, 0);
    shapes[1] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shade, 128, 0);
    shapes[2] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shadow, 128, 0);
    shapes[3] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_finalize, 256, 0);
    shapes[4] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 256};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_resolve, 256, 0);
    shapes[5] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 256};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir, 128, 0);
    shapes[6] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
}

void launch_reset_counters(Counters* counters, int bounce, cudaStream_t stream) {
    k_reset_counters<<<1, 32, 0, stream>>>(counters, bounce);
}

void launch_direction_debug(const CameraDev& cam, uint8_t* rgba, cudaStream_t stream) {
    k_direction_debug<<<1024, 256, 0, stream>>>(cam, rgba);
}

void launch_tonemap(const float4* beauty, uint8_t* rgba, long long pixels, cudaStream_t stream) {
    k_tonemap<<<1024, 256, 0, stream>>>(beauty, rgba, pixels);
}

}  // namespace rtgb
