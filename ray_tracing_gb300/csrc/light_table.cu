// The emissive light table on the device: build_light_distribution
// (packed_scene_preparation.cpp:265-302) and the guide table of its CDF.
//
// The reference walks the primitives on the host, appends every one whose
// weight (area x emission luminance) is finite and above 1e-12, appends the
// environment, then normalises by the sequential float sum of the weights and
// accumulates the CDF in the same order. Here:
//   k_light_count    per 2048-primitive chunk, how many primitives are lights;
//   k_light_offsets  one block: exclusive scan of the chunk counts;
//   k_light_place    each chunk places its lights in primitive order (a block
//                    scan of per-thread runs) and writes the primitive -> light
//                    maps (-1 for the others);
//   k_light_finish   one warp: the environment entry, the total and the CDF as
//                    the reference's two sequential single-precision loops
//                    (warp-wide loads, one running sum carried through the
//                    shuffled values in order), so every pdf and cdf is
//                    bit-identical to the host construction;
//   k_light_guide    the sample_cdf_guided bucket starts by bisection.
#include "light_table.cuh"

namespace rtgb {
namespace {

constexpr int kLtThreads = 256;
constexpr int kLtItems = 8;
constexpr int kLtChunk = kLtThreads * kLtItems;
constexpr int kLtScanThreads = 1024;

__device__ __forceinline__ float material_lum(const LightSources& s, int mi) {
    return mi < 0 || mi >= s.material_count ? 0.0f : s.material_lum[mi];
}

// Primitive e of the scene order (spheres, quads, triangles): its type and
// index within its array.
__device__ __forceinline__ void classify(const LightSources& s, int e, int& type, int& index) {
    if (e < s.sphere_count) {
        type = 0;
        index = e;
    } else if (e < s.sphere_count + s.quad_count) {
        type = 1;
        index = e - s.sphere_count;
    } else {
        type = 2;
        index = e - s.sphere_count - s.quad_count;
    }
}

// The light weight of primitive e, in the reference's order of operations.
__device__ float light_weight(const LightSources& s, int e) {
    constexpr float kPiF = 3.14159265358979323846f;
    int type, index;
    classify(s, e, type, index);
    if (type == 0) {
        const rtgb_sphere& sp = s.spheres[index];
        return 4.0f * kPiF * sp.radius * sp.radius * material_lum(s, sp.material_index);
    }
    if (type == 1) {
        const rtgb_quad& q = s.quads[index];
        const float cx = q.edge_u[1] * q.edge_v[2] - q.edge_u[2] * q.edge_v[1];
        const float cy = q.edge_u[2] * q.edge_v[0] - q.edge_u[0] * q.edge_v[2];
        const float cz = q.edge_u[0] * q.edge_v[1] - q.edge_u[1] * q.edge_v[0];
        return sqrtf(cx * cx + cy * cy + cz * cz) * material_lum(s, q.material_index);
    }
    const rtgb_triangle& t = s.triangles[index];
    const float ax = t.p1[0] - t.p0[0], ay = t.p1[1] - t.p0[1], az = t.p1[2] - t.p0[2];
    const float bx = t.p2[0] - t.p0[0], by = t.p2[1] - t.p0[1], bz = t.p2[2] - t.p0[2];
    const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    return 0.5f * sqrtf(cx * cx + cy * cy + cz * cz) * material_lum(s, t.material_index);
}

__device__ __forceinline__ bool is_light(float w) { return isfinite(w) && w > 1e-12f; }

// Exclusive prefix over the block of each thread's value; *total = the sum.
template <int kThreads>
__device__ int block_exclusive_scan(int v, int* total) {
    __shared__ int warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kThreads / 32 ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
    *total = warp_sums[kThreads / 32 - 1];
    __syncthreads();  // warp_sums is reused by the next call
    return before;
}

__global__ void __launch_bounds__(kLtThreads) k_light_count(LightSources s, int primitives, int* chunk_counts) {
    const int base = blockIdx.x * kLtChunk;
    int c = 0;
    for (int k = 0; k < kLtItems; ++k) {
        const int e = base + k * kLtThreads + static_cast<int>(threadIdx.x);
        if (e < primitives && is_light(light_weight(s, e))) ++c;
    }
    int total;
    block_exclusive_scan<kLtThreads>(c, &total);
    if (threadIdx.x == 0) chunk_counts[blockIdx.x] = total;
}

// chunk_counts -> exclusive chunk offsets (in place); counts[0] = their sum
__global__ void __launch_bounds__(kLtScanThreads) k_light_offsets(int* chunk_counts, int chunks, int* counts) {
    int carry = 0;
    for (int base = 0; base < chunks; base += kLtScanThreads) {
        const int i = base + static_cast<int>(threadIdx.x);
        const int v = i < chunks ? chunk_counts[i] : 0;
        int sum;
        const int before = block_exclusive_scan<kLtScanThreads>(v, &sum);
        if (i < chunks) chunk_counts[i] = carry + before;
        carry += sum;
    }
    if (threadIdx.x == 0) counts[0] = carry;
}

__global__ void __launch_bounds__(kLtThreads) k_light_place(LightSources s, int primitives, const int* chunk_offsets,
    LightTable out) {
    // each thread owns a run of kLtItems consecutive primitives, so the block
    // scan of the runs' counts keeps the lights in primitive order
    const int first = blockIdx.x * kLtChunk + static_cast<int>(threadIdx.x) * kLtItems;
    float w[kLtItems];
    int c = 0;
#pragma unroll
    for (int k = 0; k < kLtItems; ++k) {
        w[k] = first + k < primitives ? light_weight(s, first + k) : 0.0f;
        if (first + k < primitives && is_light(w[k])) ++c;
    }
    int total;
    int pos = chunk_offsets[blockIdx.x] + block_exclusive_scan<kLtThreads>(c, &total);
#pragma unroll
    for (int k = 0; k < kLtItems; ++k) {
        const int e = first + k;
        if (e >= primitives) break;
        int type, index;
        classify(s, e, type, index);
        int* map = type == 0 ? out.sphere_light : (type == 1 ? out.quad_light : out.triangle_light);
        if (is_light(w[k])) {
            out.lights[pos] = PackedLight{type, index, w[k], 0.0f};
            map[index] = pos++;
        } else {
            map[index] = -1;
        }
    }
}

// One warp: the environment entry, then the reference's normalisation loops.
__global__ void __launch_bounds__(32) k_light_finish(LightSources s, LightTable out) {
    const int lane = static_cast<int>(threadIdx.x);
    int n = out.counts[0];
    int env = -1;
    if (is_light(s.environment_weight)) {
        env = n;
        if (lane == 0) out.lights[n] = PackedLight{3, -1, s.environment_weight, 0.0f};
        ++n;
    }
    __syncwarp();
    float total = 0.0f;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const float w = i < n ? out.lights[i].selection_pdf : 0.0f;
        const int m = min(32, n - base);
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            const float v = __shfl_sync(0xffffffffu, w, k);
            if (k < m) total += v;
        }
    }
    float cdf = 0.0f;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const float p = i < n ? out.lights[i].selection_pdf / total : 0.0f;
        const int m = min(32, n - base);
        float mine = 0.0f;
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            const float v = __shfl_sync(0xffffffffu, p, k);
            if (k < m) {
                cdf += v;
                if (lane == k) mine = cdf;
            }
        }
        if (i < n) {
            const float c = i == n - 1 ? 1.0f : mine;
            out.lights[i].selection_pdf = p;
            out.lights[i].cdf = c;
            out.cdf[i] = c;
        }
    }
    if (lane == 0) {
        out.counts[0] = n;
        out.counts[1] = env;
    }
}

// guide[j] = first i with j / kGuide < cdf[i]; guide[kGuide] = the count
__global__ void k_light_guide(LightTable out) {
    const int j = blockIdx.x * blockDim.x + static_cast<int>(threadIdx.x);
    if (j > kGuide) return;
    const int n = out.counts[0];
    if (j == kGuide) {
        out.guide[j] = n;
        return;
    }
    const float t = static_cast<float>(j) * (1.0f / static_cast<float>(kGuide));
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (t < out.cdf[mid]) hi = mid;
        else lo = mid + 1;
    }
    out.guide[j] = lo;
}

int chunks_of(long long primitives) { return static_cast<int>((primitives + kLtChunk - 1) / kLtChunk); }

}  // namespace

size_t light_table_scratch_bytes(long long primitives) {
    return static_cast<size_t>(chunks_of(primitives) + 1) * sizeof(int);
}

cudaError_t launch_light_table(const LightSources& src, const LightTable& out, void* scratch, cudaStream_t stream) {
    const long long prims = static_cast<long long>(src.sphere_count) + src.quad_count + src.triangle_count;
    if (prims >= (1ll << 30)) return cudaErrorInvalidValue;
    const int n = static_cast<int>(prims);
    const int chunks = chunks_of(n);
    int* chunk_counts = static_cast<int*>(scratch);
    if (chunks > 0) {
        k_light_count<<<chunks, kLtThreads, 0, stream>>>(src, n, chunk_counts);
        k_light_offsets<<<1, kLtScanThreads, 0, stream>>>(chunk_counts, chunks, out.counts);
        k_light_place<<<chunks, kLtThreads, 0, stream>>>(src, n, chunk_counts, out);
    } else {
        const cudaError_t e = cudaMemsetAsync(out.counts, 0, sizeof(int), stream);
        if (e != cudaSuccess) return e;
    }
    k_light_finish<<<1, 32, 0, stream>>>(src, out);
    k_light_guide<<<(kGuide + 1 + 255) / 256, 256, 0, stream>>>(out);
    return cudaGetLastError();
}

}  // namespace rtgb
