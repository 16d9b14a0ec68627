// Shade stage of the wavefront path tracer: emission, next-event estimation,
// ReSTIR DI, BSDF sampling and Russian roulette (k_shade, k_restir) plus the
// queue helpers every stage uses.
//
// k_shade and k_restir are templates on kPbr. The kPbr = true instances carry
// the OpenPBR BSDF (src/common/openpbr_core.h) and the random-walk subsurface
// state and are compiled in shade_pbr.cu and restir_pbr.cu; the kPbr = false instances keep
// only the legacy materials (programs.cu:2463-2565) and are what scenes without
// OpenPBR materials run, so their register budget is not paid for the OpenPBR
// code. The two give identical results on scenes without OpenPBR materials.
#pragma once

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

// Parity record of one bounce: (k << 28) | (decisions << 22) | index, the
// decisions being bit 0 emissive NEE visible, bit 1 analytic (or ReSTIR) NEE
// visible, bits 2-5 the scatter event (OpenPBR sample event 1-9, 10 a
// random-walk scattering inside the medium, 0 otherwise).
constexpr int kDecisionShift = 22;
constexpr int kDecisionWalk = 10;

RTGB_D void record_decision(const Paths& P, const FrameParams& fp, long long path, int bounce, int bits) {
    P.codes[path * fp.max_bounces + bounce] |= bits << kDecisionShift;
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

struct ShadeCtx {
    const FrameParams& fp;
    const DeviceScene& s;
    int overflow;
    unsigned long long vis_rays;
    unsigned long long restir_runs;
    const float* cdf;    // the ReSTIR candidates' light CDF: shared-memory copy when it fits, else global
    int cdf_count;       // its length: analytic lights, or the emissive list (FrameParams::restir_emissive)
};

// The ReSTIR candidate of light `li` with (u0, u1) at a surface: an analytic
// light (the reference's ReSTIR DI), or with FrameParams::restir_emissive a
// light of the emissive-geometry list (emissive_candidate).
template <bool kPbr>
RTGB_D LightSample restir_candidate(const ShadeCtx& ctx, const float3& pos, const float3& sn, int mtype, int li,
    float u0, float u1) {
    if (ctx.fp.restir_emissive != 0) return emissive_candidate<kPbr>(ctx.s, pos, sn, mtype, li, u0, u1);
    return analytic_candidate(ctx.s, pos, li, u0, u1);
}

RTGB_D float restir_lum(const float3& v) { return fmaxf(0.0f, 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z); }

// restir_unshadowed_numerator, programs.cu:2122-2142
template <bool kPbr>
RTGB_D float3 unshadowed(const Hit& h, const pbr::Mat* pm, const float3& ray_d, const float3& thr, const LightSample& l,
    bool bsdf_avail, float& target) {
    target = 0.0f;
    if (!l.valid || l.pdf <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
    float bp = 0.0f;
    const float3 resp = direct_response<kPbr>(h, pm, ray_d, thr, l.direction, bp);
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
template <bool kPbr>
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
    if (!reconstruct_surface<kPbr>(ctx.s, code, origin, dir, sh)) return 0.0f;
    if (sh.mtype != src.material_type || sh.ptype != src.primitive_type || sh.pidx != src.primitive_index) {
        return 0.0f;
    }
    const float tol = fmaxf(0.01f, 0.02f * dist);
    if (len_sq(sub(sh.pos, spos)) > tol * tol || dot(sh.sn, ld3(src.normal)) < 0.95f) return 0.0f;
    const LightSample l = restir_candidate<kPbr>(ctx, sh.pos, sh.sn, sh.mtype, sel.light_index, sel.u0, sel.u1);
    // the source path state is fresh: unit throughput, ray from the previous camera
    pbr::Mat spm;
    if constexpr (kPbr) {
        if (sh.mtype == 5) openpbr_scattering(ctx.s, sh, spm);
    }
    float t = 0.0f;
    unshadowed<kPbr>(sh, &spm, dir, f3(1.0f, 1.0f, 1.0f), l, bsdf_avail, t);
    return t;
}

// The surface of a stored reservoir (its first sector).
RTGB_D Surface load_surface(const ReservoirRec* r) { return unpack_surface(r->q[0], r->q[1]); }

// Where a bounce-0 path's reservoir lives during the frame: in its pixel's
// frame record when there is one sample per pixel (written by k_restir_ris,
// finalised in place by k_restir), else in the path's scratch record, which
// k_finalize copies into the frame for the pixel's last ReSTIR sample.
RTGB_D ReservoirRec* reservoir_slot(const FrameParams& fp, const Paths& P, const FrameBufs& cur, int c,
    long long path) {
    const CameraDev& cam = fp.cam[c];
    if (fp.spp == 1) return cur.reservoirs + cam.pixel_offset + (path - cam.path_offset);
    return P.res_scratch + path;
}

// ---- ReSTIR DI (accumulate_restir_analytic_direct_light, programs.cu:2315-2449) ----
//
// Three wavefront passes at the ReSTIR bounce, in the reference's order of
// RNG draws and floating-point sums:
//   k_restir_ris  initial RIS over the candidates, then the temporal and
//                 spatial merges (every RNG draw of the reuse); the reservoir
//                 and its reuse sources are parked per path;
//   k_restir_vis  the BASIC bias-correction target of every reuse source: one
//                 closest-hit ray from the previous camera to the source surface
//                 (restir_target_at_previous_surface, :2210-2247);
//   k_restir      bias-corrected finalisation, the reservoir store, the
//                 selected sample's shadow query and the BSDF scatter.
// Splitting the visibility rays out of the RIS loop lets each pass run with its
// own register budget and occupancy; no value or draw order changes.

constexpr int kMaxSources = kMaxReuseSources;
// Builds guide[0..kGuide] over cdf (all threads of the block; ends with a barrier).
RTGB_D void build_guide(const float* cdf, int count, int* guide) {
    for (int j = threadIdx.x; j <= kGuide; j += blockDim.x) {
        const float t = static_cast<float>(j) * (1.0f / static_cast<float>(kGuide));
        int lo = 0, hi = count;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (t < cdf[mid]) hi = mid;
            else lo = mid + 1;
        }
        guide[j] = j == kGuide ? count : lo;
    }
    __syncthreads();
}

// meta word of a parked reservoir: source count, selected source + 1, canonical M
RTGB_D int pack_meta(int nsrc, int selected_src, int canonical) {
    return nsrc | ((selected_src + 1) << 8) | (canonical << 16);
}

// Initial RIS and reuse merges (programs.cu:2322-2399). Leaves the reservoir
// with its surface set and the merge sources in src_index/mult.
template <bool kPbr>
RTGB_D void restir_gather(ShadeCtx& ctx, const FrameBufs& hist, const int* guide, int c, int x, int y, const Hit& h,
    const pbr::Mat* pm, const float3& ray_d, uint32_t& rng, bool bsdf_avail, const float3& thr, Reservoir& r,
    int* src_index, int* mult, int& nsrc, int& selected_src, int& canonical) {
    const FrameParams& fp = ctx.fp;
    const DeviceScene& s = ctx.s;
    const CameraDev& cam = fp.cam[c];
    r = empty_reservoir();
    const int req = fp.restir_candidates > 0 ? fp.restir_candidates : 1;
    const int count = req < 32 ? req : 32;
    // Two candidates per step: the four draws of each (light, u0, u1, then the
    // reservoir's) keep their order, and the two light evaluations overlap.
    int k = 0;
    for (; k + 1 < count; k += 2) {
        Candidate ca, cb;
        ca.light_index = sample_cdf_guided(ctx.cdf, guide, ctx.cdf_count, rnd(rng));
        ca.u0 = rnd(rng);
        ca.u1 = rnd(rng);
        const float ua = rnd(rng);
        cb.light_index = sample_cdf_guided(ctx.cdf, guide, ctx.cdf_count, rnd(rng));
        cb.u0 = rnd(rng);
        cb.u1 = rnd(rng);
        const float ub = rnd(rng);
        const LightSample la = restir_candidate<kPbr>(ctx, h.pos, h.sn, h.mtype, ca.light_index, ca.u0, ca.u1);
        const LightSample lb = restir_candidate<kPbr>(ctx, h.pos, h.sn, h.mtype, cb.light_index, cb.u0, cb.u1);
        float ta = 0.0f, tb = 0.0f;
        unshadowed<kPbr>(h, pm, ray_d, thr, la, bsdf_avail, ta);
        unshadowed<kPbr>(h, pm, ray_d, thr, lb, bsdf_avail, tb);
        reservoir_update(r, ca, ta, la.pdf > 0.0f ? ta / la.pdf : 0.0f, 1, ua);
        reservoir_update(r, cb, tb, lb.pdf > 0.0f ? tb / lb.pdf : 0.0f, 1, ub);
    }
    if (k < count) {
        Candidate cand;
        cand.light_index = sample_cdf_guided(ctx.cdf, guide, ctx.cdf_count, rnd(rng));
        cand.u0 = rnd(rng);
        cand.u1 = rnd(rng);
        const LightSample l = restir_candidate<kPbr>(ctx, h.pos, h.sn, h.mtype, cand.light_index, cand.u0, cand.u1);
        float t = 0.0f;
        unshadowed<kPbr>(h, pm, ray_d, thr, l, bsdf_avail, t);
        const float w = l.pdf > 0.0f ? t / l.pdf : 0.0f;
        reservoir_update(r, cand, t, w, 1, rnd(rng));
    }
    canonical = r.candidate_count;
    nsrc = 0;
    selected_src = -1;
    const ReservoirRec* hres = hist.reservoirs + cam.pixel_offset;
    const Surface cur_surface = restir_surface(h);
    const int nbrs = fp.restir_spatial < 8 ? fp.restir_spatial : 8;
    int reproj = -1;
    // restir_temporal_candidate and restir_spatial_candidate reproject the
    // same hit into the same previous camera; the projection runs once.
    const bool have_prev = (fp.restir_temporal != 0 || nbrs > 0) && previous_pixel(fp, c, h, reproj);
    if (fp.restir_temporal != 0 && have_prev) {
        const Reservoir prev = load_reuse(hres + reproj);
        const float tol = fmaxf(0.005f, 0.01f * h.t);
        if (surface_valid(cur_surface, prev, tol, 0.95f, fp.restir_max_age)) {
            const LightSample l = restir_candidate<kPbr>(ctx, h.pos, h.sn, h.mtype, prev.selected.light_index, prev.selected.u0,
                prev.selected.u1);
            float t = 0.0f;
            unshadowed<kPbr>(h, pm, ray_d, thr, l, bsdf_avail, t);
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
        for (int n = 0; n < nbrs; ++n) {
            const int oi = (rot + n) & 7;
            // kOffsets of programs.cu:2187-2196
            const int dx = (oi == 0 || oi == 4 || oi == 6) ? -1 : ((oi == 1 || oi == 5 || oi == 7) ? 1 : 0);
            const int dy = (oi == 2 || oi == 4 || oi == 5) ? -1 : ((oi == 3 || oi == 6 || oi == 7) ? 1 : 0);
            const int nx = reproj % cam.width + dx, ny = reproj / cam.width + dy;
            if (nx < 0 || nx >= cam.width || ny < 0 || ny >= cam.height) continue;
            const int ni = ny * cam.width + nx;
            const Reservoir prev = load_reuse(hres + ni);
            const float tol = fmaxf(0.01f, 0.02f * h.t);
            if (!surface_valid(cur_surface, prev, tol, 0.95f, fp.restir_max_age)) continue;
            const LightSample l = restir_candidate<kPbr>(ctx, h.pos, h.sn, h.mtype, prev.selected.light_index, prev.selected.u0,
                prev.selected.u1);
            float t = 0.0f;
            unshadowed<kPbr>(h, pm, ray_d, thr, l, bsdf_avail, t);
            const MergeResult m = reservoir_merge(r, prev, t, fp.restir_max_spatial, rnd(rng), false);
            if (m.multiplicity > 0 && nsrc < kMaxSources) {
                src_index[nsrc] = ni;
                mult[nsrc] = m.multiplicity;
                if (m.selected != 0) selected_src = nsrc;
                ++nsrc;
            }
        }
    }
    r.surface = cur_surface;
}

// Bias correction, reservoir store and the selected sample's shadow query
// (programs.cu:2400-2449) from the parked reservoir and the source targets.
template <bool kPbr>
RTGB_D void restir_finish(ShadeCtx& ctx, const Paths& P, ReservoirRec* slot, long long path, const Hit& h,
    const pbr::Mat* pm, const float3& ray_d, bool bsdf_avail, const float3& thr, int meta, float4& sh_o, float4& sh_d,
    float4& sh_c) {
    const FrameParams& fp = ctx.fp;
    const DeviceScene& s = ctx.s;
    const int nsrc = meta & 0xff;
    const int selected_src = ((meta >> 8) & 0xff) - 1;
    const int canonical = meta >> 16;
    // the parked reservoir's sample and sums (its surface sector stays as written)
    Reservoir r = zero_reservoir();
    unpack_sample(slot->q[2], slot->q[3], r);
    unpack_sums(slot->q[4], slot->q[5], r);
    if (fp.restir_bias == 1 && nsrc > 0 && r.valid != 0) {
        float sel_t = r.selected_target;
        float sum = r.selected_target * static_cast<float>(canonical);
        for (int k = 0; k < nsrc; ++k) {
            const float t = P.res_src_t[k * P.src_stride + path];
            sum += t * static_cast<float>(P.res_src[k * P.src_stride + path].y);
            if (selected_src == k) sel_t = t;
        }
        reservoir_finalize_basic(r, sel_t, sum, nsrc);
    } else {
        reservoir_finalize(r);
    }
    float4 q[4];
    pack_sample(r, q[0], q[1]);
    pack_sums(r, q[2], q[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) slot->q[2 + k] = q[k];
    if (fp.spp != 1) P.res_written[path] = 1;
    if (r.valid == 0) return;
    const LightSample l = restir_candidate<kPbr>(ctx, h.pos, h.sn, h.mtype, r.selected.light_index, r.selected.u0,
        r.selected.u1);
    float t = 0.0f;
    const float3 num = unshadowed<kPbr>(h, pm, ray_d, thr, l, bsdf_avail, t);
    if (!l.valid || t <= 0.0f) return;
    const float max_t = l.infinite ? kRayFar : l.distance - kRayEpsilon * 3.0f;
    if (max_t <= kRayEpsilon) return;
    sh_o = f4(add(h.pos, mul(l.direction, kRayEpsilon * 2.0f)), max_t);
    sh_d = f4(l.direction, 0.0f);
    sh_c = f4(mul(thr, mul(num, r.estimator_weight)), 1.0f);
}

// The ray and throughput of a queued path, without the previous-scatter
// record and radiance: for the ReSTIR passes, which rebuild the hit and (in
// k_restir) scatter, and scatter rewrites every previous-scatter field before
// store_path writes them.
RTGB_D void load_ray(const Paths& P, int path, PathRegs& st) {
    st.o = xyz(P.ray_o[path]);
    st.d = xyz(P.ray_d[path]);
    const float4 thr4 = P.thr[path];
    st.thr = xyz(thr4);
    st.prev_pdf = thr4.w;
    st.rad = f3(0.0f, 0.0f, 0.0f);
    st.prev_pos = f3(0.0f, 0.0f, 0.0f);
    st.prev_nrm = f3(0.0f, 0.0f, 0.0f);
    st.prev_valid = false;
    st.prev_delta = false;
    st.prev_mtype = -1;
    st.prev_ptype = -1;
    st.prev_pidx = -1;
    st.alive = true;
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
// returns whether the path continues. `pm` holds the OpenPBR scattering
// parameters when h.mtype == 5; `sss_event` reports an OpenPBR subsurface
// entry (1) or exit (2).
template <bool kPbr>
RTGB_D bool scatter(const FrameParams& fp, const LoopBounds& lb, const Hit& h, const pbr::Mat* pm, int bounce,
    uint32_t& rng, PathRegs& st, int& sss_event, int& event) {
    sss_event = 0;
    event = 0;
    bool scattered = false;
    float pdf = 0.0f;
    bool delta = true;
    if (h.mtype == 0) {
        float3 dir = add(h.sn, random_unit_vector(rng, lb));
        if (near_zero(dir)) dir = h.sn;
        st.o = add(h.pos, mul(h.sn, kRayEpsilon));
        st.d = normalize(dir);
        st.thr = mul(st.thr, h.base);
        pdf = fmaxf(dot(h.sn, st.d), 0.0f) / kPi;
        delta = false;
        scattered = true;
    } else if (h.mtype == 1) {
        const float3 refl = reflect(normalize(st.d), h.sn);
        const float3 fz = mul(random_in_unit_sphere(rng, lb), fminf(fmaxf(h.fuzz, 0.0f), 1.0f));
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
    } else if (kPbr && h.mtype == 5) {
        const pbr::Frame frame = pbr::make_frame(pv(h.gn), pbr::V3{0.0f, 0.0f, 0.0f});
        const float u_lobe = rnd(rng);
        const float u1 = rnd(rng);
        const float u2 = rnd(rng);
        const pbr::Sample smp =
            pbr::sample(*pm, frame, pv(mul(normalize(st.d), -1.0f)), u_lobe, u1, u2, transport_context(st.thr));
        if (smp.valid != 0) {
            const float3 dir = fv(smp.wi);
            st.o = add(h.pos, mul(dir, kRayEpsilon));
            st.d = normalize(dir);
            st.thr = mul(st.thr, fv(smp.weight));
            pdf = smp.pdf;
            delta = smp.delta != 0;
            scattered = true;
            sss_event = smp.event == pbr::kSubsurfaceEntry ? 1 : (smp.event == pbr::kSubsurfaceExit ? 2 : 0);
            event = smp.event;
        }
    } else if (h.mtype == 4) {
        const float3 dir = random_unit_vector(rng, lb);
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
template <bool kPbr>
RTGB_D bool rebuild_hit(const DeviceScene& s, const float4& hr, const PathRegs& st, Hit& h) {
    const int code = __float_as_int(hr.y);
    if ((static_cast<unsigned>(code) >> 28) == 4) {
        reconstruct_medium<kPbr>(s, code & 0x0fffffff, hr.x, st.o, st.d, h);
        return true;
    }
    return reconstruct_surface<kPbr>(s, code, st.o, st.d, h);
}

// The path enters or leaves an OpenPBR random-walk medium (sample_bsdf,
// programs.cu:2545-2551). A medium is kept only while active, so "inside" is
// sss_mat >= 0.
RTGB_D void update_subsurface(const Paths& P, int path, const Hit& h, const pbr::Mat& m, int sss_event) {
    if (sss_event == 1) {
        const pbr::Medium med = pbr::subsurface_medium(m);
        P.sss_ext[path] = make_float4(med.extinction.x, med.extinction.y, med.extinction.z, med.anisotropy);
        P.sss_alb[path] = make_float4(med.albedo.x, med.albedo.y, med.albedo.z, 0.0f);
        P.sss_mat[path] = med.active != 0 ? h.openpbr : -1;
    } else if (sss_event == 2) {
        P.sss_mat[path] = -1;
    }
}

// Random-walk segment of a path inside an OpenPBR medium (programs.cu:1878-1902).
// Returns 0 to shade the hit, 1 when the path ends, 2 when it scattered inside
// the medium (st then holds the new ray).
RTGB_D int subsurface_step(const Paths& P, int path, int sss, const Hit& h, uint32_t& rng, PathRegs& st) {
    if (h.mtype != 5 || h.openpbr != sss || h.front) return 1;
    const float4 ext = P.sss_ext[path];
    const float4 alb = P.sss_alb[path];
    pbr::Medium med;
    med.extinction = pbr::V3{ext.x, ext.y, ext.z};
    med.albedo = pbr::V3{alb.x, alb.y, alb.z};
    med.anisotropy = ext.w;
    med.active = 1;
    const float ray_len = sqrtf(len_sq(st.d));
    const pbr::Segment seg = pbr::subsurface_segment(med, h.t * ray_len, rnd(rng), transport_context(st.thr));
    st.thr = mul(st.thr, fv(seg.weight));
    if (seg.scattered == 0) return 0;
    const float3 incident = normalize(st.d);
    const float g1 = rnd(rng);
    const float g2 = rnd(rng);
    const float3 dir = fv(pbr::sample_hg(pv(incident), med.anisotropy, g1, g2));
    st.o = add(st.o, mul(st.d, seg.distance / fmaxf(ray_len, 1e-8f)));
    st.d = dir;
    st.o = add(st.o, mul(st.d, kRayEpsilon));
    st.prev_valid = false;
    return 2;
}

// One bounce of radiance_kernel's loop body (programs.cu:1855-1932) per path.
// At the ReSTIR bounce, surfaces that run ReSTIR DI stop after the
// emissive-geometry NEE and continue in k_restir, which consumes the RNG
// stream from exactly this point. With kSplit (the OpenPBR instance) every
// path stops there: the ones that scatter are queued for k_scatter, which
// samples the BSDF from the same RNG state, so each kernel carries only half
// of the OpenPBR code (evaluation here, sampling there) and fewer registers.
template <bool kPbr, bool kSplit = false>
__global__ void __launch_bounds__(128, kSplit ? 6 : 1) k_shade(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters, int bounce) {
    const FrameParams& fp = *fpp;
    const int in = bounce & 1;
    const int out = in ^ 1;
    const int count = counters->active[in];
    const bool restir_bounce = fp.restir_enabled != 0 && bounce == 0;
    const int* __restrict__ order = bounce >= fp.sort_from_bounce ? P.sorted : P.queue[in];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = order[i];
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
        bool to_scatter = false;
        bool thr_changed = false;
        if (alight >= 0) {
            AnalyticHit ah;
            ah.hit = hit_analytic_at(s, alight, st.o, st.d, kRayEpsilon, kRayFar, ah);
            ah.light = alight;
            const float w = analytic_emission_mis(s, st, ah);
            st.rad = add(st.rad, mul(st.thr, mul(ld3(s.analytic[alight].radiance), w)));
        } else if (code == -1) {
            const float w = emission_mis_weight(s, st, nullptr, true);
            st.rad = add(st.rad, mul(st.thr, mul(ld3(s.background), w)));
            st.rad = add(st.rad, mul(st.thr, analytic_infinite_radiance(s, st)));
        } else {
            Hit h;
            if (!rebuild_hit<kPbr>(s, hr, st, h)) {
                atomicAdd(&counters->error, 1);
            } else {
                int walk = 0;
                if constexpr (kPbr) {
                    const int sss = P.sss_mat[path];
                    if (sss >= 0) {
                        walk = subsurface_step(P, path, sss, h, rng, st);
                        thr_changed = true;
                    }
                }
                if (walk == 2) {
                    keep = bounce + 1 < fp.max_bounces;
                    if (fp.record_paths) record_decision(P, fp, path, bounce, kDecisionWalk << 2);
                } else if (walk == 0) {
                    // shared, not stack: as in k_scatter (one slot for the
                    // legacy instances, which never touch it)
                    __shared__ pbr::Mat shade_mats[kPbr ? 128 : 1];
                    pbr::Mat& pm = shade_mats[kPbr ? threadIdx.x : 0];
                    if constexpr (kPbr) {
                        if (h.mtype == 5) openpbr_scattering(s, h, pm);
                    }
                    if (bounce == 0) {
                        P.aux_n[path] = f4(h.sn, h.t);
                        P.aux_a[path] = f4(h.base, 1.0f);
                    }
                    const float ew = emission_mis_weight(s, st, &h, false);
                    st.rad = add(st.rad, mul(st.thr, mul(h.emis, ew)));
                    const bool bsdf_avail = bounce + 1 < fp.max_bounces;
                    // ReSTIR over emissive geometry (opt-in, FrameParams::restir_emissive)
                    // takes the place of the emissive NEE for receivers that are not
                    // emitters themselves; its sample fills shadow slot 0 in k_restir
                    const bool emissive_restir = restir_bounce && fp.restir_emissive != 0 && h.mtype != 3
                                                 && s.light_count > 0 && find_light(s, h.ptype, h.pidx) < 0;
                    // accumulate_direct_light (programs.cu:2249-2280) -> shadow slot 0
                    if (h.mtype != 3 && s.light_count > 0 && !emissive_restir) {
                        const LightSample l = sample_direct<kPbr>(s, h, rng);
                        if (l.valid) {
                            float bp = 0.0f;
                            const float3 resp = direct_response<kPbr, true>(h, &pm, st.d, st.thr, l.direction, bp);
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
                    if (restir_bounce && fp.restir_emissive == 0) {
                        // accumulate_restir_analytic_direct_light returns before any
                        // draw for emitters and light-less scenes (programs.cu:2318-2321)
                        deferred = h.mtype != 3 && s.analytic_count > 0;
                    } else if (h.mtype != 3 && s.analytic_count > 0) {
                        // accumulate_analytic_direct_light (programs.cu:2282-2313) -> shadow slot 1
                        const int li = sample_cdf_guided(s.analytic_cdf, s.analytic_guide, s.analytic_count, rnd(rng));
                        const float u0 = rnd(rng);
                        const float u1 = rnd(rng);
                        const LightSample l = analytic_candidate(s, h.pos, li, u0, u1);
                        if (l.valid) {
                            float bp = 0.0f;
                            const float3 resp = direct_response<kPbr, true>(h, &pm, st.d, st.thr, l.direction, bp);
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
                    deferred = deferred || emissive_restir;
                    if (!deferred && bsdf_avail) {
                        if constexpr (kSplit) {
                            to_scatter = true;
                        } else {
                            int sss_event = 0, event = 0;
                            keep = scatter<kPbr>(fp, s.bounds, h, &pm, bounce, rng, st, sss_event, event);
                            if constexpr (kPbr) {
                                if (keep && sss_event != 0) update_subsurface(P, path, h, pm, sss_event);
                                if (fp.record_paths && event != 0) record_decision(P, fp, path, bounce, event << 2);
                            }
                        }
                    }
                }
            }
        }
        P.rad[path] = f4(st.rad, 0.0f);
        P.rng[path] = rng;
        if (keep) store_path(P, path, st);
        // the random walk scaled the throughput k_scatter starts from
        if (kSplit && to_scatter && thr_changed) P.thr[path] = f4(st.thr, st.prev_pdf);
        if (deferred) {
            // the NEE slot travels to k_restir, which adds the ReSTIR slot (1 for
            // analytic lights, 0 for emissive geometry) and queues the shadow rays
            const bool em = fp.restir_emissive != 0;
            const float4 kc = em ? sh_c[1] : sh_c[0];
            (em ? P.sh_c[1] : P.sh_c[0])[path] = kc;
            if (kc.w != 0.0f) {
                (em ? P.sh_o[1] : P.sh_o[0])[path] = em ? sh_o[1] : sh_o[0];
                (em ? P.sh_d[1] : P.sh_d[0])[path] = em ? sh_d[1] : sh_d[0];
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
        if constexpr (kSplit) queue_push(P.scatter_queue, &counters->scatter, path, to_scatter);
    }
}

// BSDF sampling and Russian roulette (sample_bsdf, programs.cu:2463-2565;
// apply_russian_roulette, :1764-1771) of the paths k_shade<kPbr, true> queued,
// continuing their RNG stream where the next-event estimation left it.
template <bool kPbr>
__global__ void __launch_bounds__(128, 6) k_scatter(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters, int bounce) {
    const FrameParams& fp = *fpp;
    const int out = (bounce & 1) ^ 1;
    const int count = counters->scatter;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.scatter_queue[i];
        const float4 hr = P.hit[path];
        PathRegs st;
        load_ray(P, path, st);
        uint32_t rng = P.rng[path];
        Hit h;
        rebuild_hit<kPbr>(s, hr, st, h);  // rebuilt in k_shade from the same record
        // The thread's OpenPBR parameters live in shared memory: the BSDF
        // sampler is an out-of-line call that reads them by reference, and on
        // the stack they would travel through L1 / L2 with every other
        // thread's stack (204 B a thread, an odd word stride: no bank conflicts).
        __shared__ pbr::Mat mats[128];
        pbr::Mat& pm = mats[threadIdx.x];
        if constexpr (kPbr) {
            if (h.mtype == 5) openpbr_scattering(s, h, pm);
        }
        int sss_event = 0, event = 0;
        const bool keep = scatter<kPbr>(fp, s.bounds, h, &pm, bounce, rng, st, sss_event, event);
        if constexpr (kPbr) {
            if (keep && sss_event != 0) update_subsurface(P, path, h, pm, sss_event);
            if (fp.record_paths && event != 0) record_decision(P, fp, path, bounce, event << 2);
        }
        P.rng[path] = rng;
        if (keep) store_path(P, path, st);
        queue_push(P.queue[out], &counters->active[out], path, keep);
    }
}

// ReSTIR DI for the deferred bounce-0 surfaces: the three passes described at
// restir_gather, then the BSDF scatter.
constexpr int kSharedCdf = 4096;

// Shared-memory copy of the analytic-light CDF (when it fits) and its guide table.
struct RestirShared {
    float cdf[kSharedCdf];
    int guide[kGuide + 1];
};

RTGB_D const float* stage_cdf(const FrameParams& fp, const DeviceScene& s, RestirShared& sh, int& count) {
    const float* src = fp.restir_emissive != 0 ? s.light_cdf : s.analytic_cdf;
    count = fp.restir_emissive != 0 ? s.light_count : s.analytic_count;
    const bool shared = count <= kSharedCdf;
    if (shared) {
        for (int k = threadIdx.x; k < count; k += blockDim.x) sh.cdf[k] = src[k];
        __syncthreads();
    }
    const float* cdf = shared ? sh.cdf : src;
    build_guide(cdf, count, sh.guide);
    return cdf;
}

// Six resident blocks (80 registers) measured fastest among 1, 6, 8 and 10.
template <bool kPbr>
__global__ void __launch_bounds__(128, 6) k_restir_ris(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters) {
    __shared__ RestirShared sh;
    const FrameParams& fp = *fpp;
    const FrameBufs hist = fp.hist;
    const int count = counters->restir;
    if (count == 0) return;
    int cdf_count = 0;
    const float* cdf = stage_cdf(fp, s, sh, cdf_count);
    ShadeCtx ctx{fp, s, 0, 0ull, 0ull, cdf, cdf_count};
    constexpr int bounce = 0;
    const bool bsdf_avail = bounce + 1 < fp.max_bounces;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.restir_queue[i];
        const float4 hr = P.hit[path];
        PathRegs st;
        load_ray(P, path, st);
        uint32_t rng = P.rng[path];
        Hit h;
        rebuild_hit<kPbr>(s, hr, st, h);
        pbr::Mat pm;
        if constexpr (kPbr) {
            if (h.mtype == 5) openpbr_scattering(s, h, pm);
        }
        const int c = camera_of_path(fp, path);
        const CameraDev& cam = fp.cam[c];
        const int pixel = static_cast<int>((path - cam.path_offset) / fp.spp);
        Reservoir r;
        int src_index[kMaxSources], mult[kMaxSources];
        int nsrc = 0, selected_src = -1, canonical = 0;
        restir_gather<kPbr>(ctx, hist, sh.guide, c, pixel % cam.width, pixel / cam.width, h, &pm, st.d, rng,
            bsdf_avail, st.thr, r, src_index, mult, nsrc, selected_src, canonical);
        store_reservoir(reservoir_slot(fp, P, fp.cur, c, path), r);
        P.rng[path] = rng;
        P.res_meta[path] = pack_meta(nsrc, selected_src, canonical);
        for (int k = 0; k < nsrc; ++k) P.res_src[k * P.src_stride + path] = make_int2(src_index[k], mult[k]);
        const bool bias = fp.restir_bias == 1 && r.valid != 0;
        for (int k = 0; k < kMaxSources; ++k) {
            queue_push(P.vis_queue, &counters->vis, (path << 4) | k, bias && k < nsrc);
        }
    }
}

template <bool kPbr>
__global__ void __launch_bounds__(128) k_restir_vis(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters) {
    const FrameParams& fp = *fpp;
    const FrameBufs hist = fp.hist;
    const int count = counters->vis;
    ShadeCtx ctx{fp, s, 0, 0ull, 0ull, nullptr, 0};
    constexpr int bounce = 0;
    const bool bsdf_avail = bounce + 1 < fp.max_bounces;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int item = P.vis_queue[i];
        const int path = item >> 4;
        const int k = item & 15;
        const int c = camera_of_path(fp, path);
        const long long slot = k * P.src_stride + path;
        const ReservoirRec* hres = hist.reservoirs + fp.cam[c].pixel_offset;
        const float4 sq = reservoir_slot(fp, P, fp.cur, c, path)->q[2];
        const Candidate sel{__float_as_int(sq.x), sq.y, sq.z};
        P.res_src_t[slot] = target_at_previous<kPbr>(ctx, c, load_surface(hres + P.res_src[slot].x), sel, bsdf_avail);
    }
    count_add(&counters->rays[3], ctx.vis_rays);
    if (ctx.overflow) atomicAdd(&counters->overflow, ctx.overflow);
}

template <bool kPbr>
__global__ void __launch_bounds__(128) k_restir(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters) {
    const FrameParams& fp = *fpp;
    FrameBufs cur = fp.cur;
    const int count = counters->restir;
    ShadeCtx ctx{fp, s, 0, 0ull, 0ull, nullptr, 0};
    constexpr int bounce = 0;
    const int out = 1;
    unsigned long long runs = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.restir_queue[i];
        const float4 hr = P.hit[path];
        PathRegs st;
        load_ray(P, path, st);
        uint32_t rng = P.rng[path];
        Hit h;
        rebuild_hit<kPbr>(s, hr, st, h);
        pbr::Mat pm;
        if constexpr (kPbr) {
            if (h.mtype == 5) openpbr_scattering(s, h, pm);
        }
        const bool bsdf_avail = bounce + 1 < fp.max_bounces;
        const int c = camera_of_path(fp, path);
        float4 sh_o1, sh_d1, sh_c1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ++runs;
        restir_finish<kPbr>(ctx, P, reservoir_slot(fp, P, cur, c, path), path, h, &pm, st.d, bsdf_avail, st.thr,
            P.res_meta[path], sh_o1, sh_d1, sh_c1);
        int sss_event = 0, event = 0;
        const bool keep = bsdf_avail && scatter<kPbr>(fp, s.bounds, h, &pm, bounce, rng, st, sss_event, event);
        if constexpr (kPbr) {
            if (keep && sss_event != 0) update_subsurface(P, path, h, pm, sss_event);
            if (fp.record_paths && event != 0) record_decision(P, fp, path, bounce, event << 2);
        }
        P.rng[path] = rng;
        if (keep) store_path(P, path, st);
        // the ReSTIR sample's slot: 1 beside the emissive NEE in slot 0 (the
        // reference), or 0 when ReSTIR resamples the emissive geometry itself
        const int rs = fp.restir_emissive != 0 ? 0 : 1;
        const bool nee = P.sh_c[rs ^ 1][path].w != 0.0f;
        const bool any_shadow = nee || sh_c1.w != 0.0f;
        if (sh_c1.w != 0.0f) {
            P.sh_o[rs][path] = sh_o1;
            P.sh_d[rs][path] = sh_d1;
        }
        if (any_shadow) P.sh_c[rs][path] = sh_c1;
        queue_push(P.shadow_queue, &counters->shadow, path, any_shadow);
        queue_push(P.queue[out], &counters->active[out], path, keep);
    }
    count_add(&counters->restir_pixels, runs);
    (void)ctx;
}

}  // namespace
}  // namespace rtgb
