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
#include "shade_stage.cuh"

namespace rtgb {
namespace {

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
        P.sss_mat[path] = -1;
        if (P.res_written) P.res_written[path] = 0;
        if (fp.record_paths) {
            for (int b = 0; b < fp.max_bounces; ++b) P.codes[path * fp.max_bounces + b] = -2;
        }
    }
    // The per-launch memset of the reservoir buffer (optix_renderer.cpp:253-254)
    // as flat 16-byte stores over every active pixel's 96-byte record (all-zero
    // bits decode to the zeroed reservoir).
    {
        const long long n16 = fp.total_pixels * static_cast<long long>(sizeof(ReservoirRec) / 16);
        float4* base = reinterpret_cast<float4*>(cur.reservoirs);
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n16;
             i += static_cast<long long>(gridDim.x) * blockDim.x) {
            base[i] = z;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters->active[0] = static_cast<int>(n);
        counters->rays[0] = 0;
        counters->rays[1] = 0;
        counters->rays[2] = 0;
        counters->rays[3] = 0;
        counters->restir_pixels = 0;
        counters->gave_up = 0;
    }
}

// The first kStagedNodes4 wide-BVH nodes (the top levels: nodes are numbered
// breadth-first) into this block's shared memory; returns how many.
RTGB_D int stage_nodes4(const DeviceScene& s, float4* smem4) {
    const int staged = s.node4_count < kStagedNodes4 ? s.node4_count : kStagedNodes4;
    for (int k = threadIdx.x; k < staged * kNode4; k += blockDim.x) smem4[k] = __ldg(s.nodes4 + k);
    __syncthreads();
    return staged;
}

constexpr int kStagedBytes = kStagedNodes4 * kNode4 * static_cast<int>(sizeof(float4));

// intersect_scene (programs.cu:1654-1757) + intersect_analytic_lights (:795-813).
// kDeep: the instance for deep hierarchies (deep_bvh), held to 80 registers so
// six blocks share an SM.
template <bool kDeep>
__global__ void __launch_bounds__(128, kDeep ? 6 : 1) k_trace(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters, int bounce) {
    extern __shared__ float4 smem4[];
    const int staged = stage_nodes4(s, smem4);
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
        int code = traverse_closest(s, o, d, kRayEpsilon, closest, overflow, smem4, staged);
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

// is_occluded (programs.cu:1759-1762) for the bounce's NEE samples; visible
// contributions are added in slot order (emissive geometry, then analytic).
template <bool kDeep>
__global__ void __launch_bounds__(128, kDeep ? 6 : 1) k_shadow(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    Counters* counters, int bounce) {
    extern __shared__ float4 smem4[];
    const int staged = stage_nodes4(s, smem4);
    const FrameParams& fp = *fpp;
    const int count = counters->shadow;
    int overflow = 0;
    unsigned long long traced = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int path = P.shadow_queue[i];
        float3 rad = xyz(P.rad[path]);
        int visible = 0;
        for (int k = 0; k < 2; ++k) {
            const float4 c = P.sh_c[k][path];
            if (c.w == 0.0f) continue;
            const float4 o = P.sh_o[k][path];
            const float4 d = P.sh_d[k][path];
            ++traced;
            if (!traverse_any(s, xyz(o), xyz(d), kRayEpsilon, o.w, overflow, smem4, staged)) {
                rad = add(rad, xyz(c));
                visible |= 1 << k;  // kDecisionNeeEmissive, kDecisionNeeAnalytic
            }
        }
        P.rad[path] = f4(rad, 0.0f);
        if (fp.record_paths && visible != 0) record_decision(P, fp, path, bounce, visible);
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
        // the reference accumulates beauty only without its (analytic) ReSTIR;
        // the emissive-geometry ReSTIR extension keeps the accumulation, so it
        // changes the direct-light estimator and nothing else
        if (fp.restir_enabled == 0 || fp.restir_emissive != 0) {
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
        counters->vis = 0;
        counters->scatter = 0;
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

// The light sampler's per-light records (DeviceScene::analytic_hot), once per
// scene. The normal is analytic_light_normal (programs.cu:661-666), the same
// device function the candidates would run, so the table holds exactly the
// values they would compute; the other fields are copies.
__global__ void k_analytic_hot(DeviceScene s, float4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.analytic_count) return;
    const rtgb_analytic_light& l = s.analytic[i];
    const bool rect = l.type == 2;
    float4* o = out + static_cast<long long>(kAnalyticHot) * i;
    o[0] = make_float4(l.position[0], l.position[1], l.position[2], l.selection_pdf);
    o[1] = make_float4(l.basis_x[0], l.basis_x[1], l.basis_x[2], rect ? l.width : l.radius);
    o[2] = make_float4(l.basis_y[0], l.basis_y[1], l.basis_y[2], rect ? l.height : l.length);
    o[3] = make_float4(l.radiance[0], l.radiance[1], l.radiance[2], l.world_area);
    o[4] = f4(analytic_normal(l), __int_as_float(l.type));
}

void launch_analytic_hot(DeviceScene scene, float4* out, cudaStream_t stream) {
    if (scene.analytic_count <= 0) return;
    k_analytic_hot<<<(scene.analytic_count + 255) / 256, 256, 0, stream>>>(scene, out);
}

void launch_camera_dirs(const CameraDev& cam, float4* out, cudaStream_t stream) {
    const long long n = static_cast<long long>(cam.width) * cam.height;
    const int grid = static_cast<int>((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
    k_camera_dirs<<<grid > 0 ? grid : 1, 256, 0, stream>>>(cam, out);
}

void launch_raygen(const FrameParams* fp, Paths paths, Counters* counters, LaunchShape shape, cudaStream_t stream) {
    k_raygen<<<shape.grid, shape.block, 0, stream>>>(fp, paths, counters);
}

void launch_trace(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, cudaStream_t stream) {
    if (deep_bvh(scene)) {
        k_trace<true><<<shape.grid, shape.block, kStagedBytes, stream>>>(fp, scene, paths, counters, bounce);
    } else {
        k_trace<false><<<shape.grid, shape.block, kStagedBytes, stream>>>(fp, scene, paths, counters, bounce);
    }
}

void launch_shade(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, LaunchShape scatter_shape, cudaStream_t stream) {
    if (scene.openpbr_count > 0) {
        launch_shade_pbr(fp, scene, paths, counters, bounce, shape, scatter_shape, stream);
        return;
    }
    k_shade<false><<<shape.grid, shape.block, 0, stream>>>(fp, scene, paths, counters, bounce);
}

void launch_shadow(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce, LaunchShape shape,
    cudaStream_t stream) {
    if (deep_bvh(scene)) {
        k_shadow<true><<<shape.grid, shape.block, kStagedBytes, stream>>>(fp, scene, paths, counters, bounce);
    } else {
        k_shadow<false><<<shape.grid, shape.block, kStagedBytes, stream>>>(fp, scene, paths, counters, bounce);
    }
}

void launch_restir(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters,
    const LaunchShape* shapes, cudaStream_t stream) {
    if (scene.openpbr_count > 0) {
        launch_restir_pbr(fp, scene, paths, counters, shapes, stream);
        return;
    }
    k_restir_ris<false><<<shapes[9].grid, shapes[9].block, 0, stream>>>(fp, scene, paths, counters);
    k_restir_vis<false><<<shapes[10].grid, shapes[10].block, 0, stream>>>(fp, scene, paths, counters);
    k_restir<false><<<shapes[6].grid, shapes[6].block, 0, stream>>>(fp, scene, paths, counters);
}

void launch_finalize(const FrameParams* fp, Paths paths, Counters* counters, LaunchShape shape, cudaStream_t stream) {
    k_finalize<<<shape.grid, shape.block, 0, stream>>>(fp, paths, counters);
}

void launch_resolve(const FrameParams* fp, LaunchShape shape, cudaStream_t stream) {
    k_resolve<<<shape.grid, shape.block, 0, stream>>>(fp);
}

void query_launch_shapes(int sm_count, LaunchShape* shapes) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_raygen, 256, 0);
    shapes[0] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 256};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_trace<false>, 128, kStagedBytes);
    shapes[1] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_trace<true>, 128, kStagedBytes);
    shapes[14] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shade<false>, 128, 0);
    shapes[2] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shadow<false>, 128, kStagedBytes);
    shapes[3] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shadow<true>, 128, kStagedBytes);
    shapes[15] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_finalize, 256, 0);
    shapes[4] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 256};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_resolve, 256, 0);
    shapes[5] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 256};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir<false>, 128, 0);
    shapes[6] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir_ris<false>, 128, 0);
    shapes[9] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir_vis<false>, 128, 0);
    shapes[10] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    shapes[7] = query_shade_pbr_shape(sm_count);
    shapes[13] = query_scatter_pbr_shape(sm_count);
    query_restir_pbr_shapes(sm_count, shapes);
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
