// Material-coherent shading order: the bounce's shade queue bucketed by the
// material of each path's hit before k_shade runs, so the 32 paths of a warp
// share material parameters and take the same OpenPBR branches (texture
// bindings, metal / dielectric / coat / fuzz / transmission lobes) instead of
// serialising over up to 32 different ones.
//
// A counting sort over kSortBins material buckets in three launches:
//   k_bucket_count    each block counts the keys of its contiguous chunk of
//                     the queue in shared memory (keys kept per slot) and adds
//                     its nonzero bins to the global histogram;
//   k_bucket_scan     one block turns the histogram into bucket starts and
//                     clears it for the next bounce;
//   k_bucket_scatter  each block reserves one range per nonzero bin with a
//                     single global atomic, then places its paths with shared
//                     atomics.
// Only the order in which paths are shaded changes; every path's arithmetic
// (and so every result) is the same as without the sort. Keys: 0 miss, 1
// analytic-light hit or medium event, 2 + material (mod kSortBins - 2).
#include "wavefront.cuh"

namespace rtgb {
namespace {

constexpr int kSortBlock = 256;

__device__ __forceinline__ int shade_key(const DeviceScene& s, const float4& hr) {
    const int code = __float_as_int(hr.y);
    if (__float_as_int(hr.z) >= 0) return 1;
    if (code == -1) return 0;
    const int type = static_cast<int>(static_cast<unsigned>(code) >> 28);
    const int idx = code & 0x0fffffff;
    int mi;
    if (type == 0) {
        mi = __ldg(&s.spheres[idx].material_index);
    } else if (type == 1) {
        mi = __ldg(&s.quads[idx].material_index);
    } else if (type == 2) {
        mi = __ldg(&s.triangles[idx].material_index);
    } else {
        return 1;
    }
    return 2 + (mi < 0 ? 0 : mi % (kSortBins - 2));
}

// the contiguous slice of [0, count) a block owns (same split in both passes)
__device__ __forceinline__ void chunk_of(int count, int& begin, int& end) {
    const int per = (count + static_cast<int>(gridDim.x) - 1) / static_cast<int>(gridDim.x);
    begin = min(count, static_cast<int>(blockIdx.x) * per);
    end = min(count, begin + per);
}

__global__ void __launch_bounds__(kSortBlock) k_bucket_count(const FrameParams* __restrict__ fpp, DeviceScene s, Paths P,
    const Counters* __restrict__ counters, int bounce) {
    if (bounce < fpp->sort_from_bounce) return;
    __shared__ int bins[kSortBins];
    for (int b = threadIdx.x; b < kSortBins; b += blockDim.x) bins[b] = 0;
    __syncthreads();
    const int in = bounce & 1;
    int begin, end;
    chunk_of(counters->active[in], begin, end);
    const int lane = static_cast<int>(threadIdx.x) & 31;
    for (int i = begin + static_cast<int>(threadIdx.x); i < end; i += blockDim.x) {
        const int key = shade_key(s, P.hit[P.queue[in][i]]);
        P.sort_key[i] = key;
        // one shared atomic per distinct key in the warp (few materials would
        // otherwise serialise 32 lanes on one address)
        const unsigned peers = __match_any_sync(__activemask(), key);
        if (lane == __ffs(peers) - 1) atomicAdd(&bins[key], __popc(peers));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kSortBins; b += blockDim.x) {
        if (bins[b] != 0) atomicAdd(&P.sort_hist[b], bins[b]);
    }
}

// one block of kSortBins threads: exclusive scan of the histogram into the
// bucket cursors; the histogram is zeroed for the next bounce
__global__ void __launch_bounds__(kSortBins) k_bucket_scan(const FrameParams* __restrict__ fpp, Paths P, int bounce) {
    if (bounce < fpp->sort_from_bounce) return;
    __shared__ int warp_sums[kSortBins / 32];
    const int b = threadIdx.x;
    const int v = P.sort_hist[b];
    const int lane = b & 31, warp = b >> 5;
    int x = v;  // inclusive scan within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    P.sort_cursor[b] = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
    P.sort_hist[b] = 0;
}

__global__ void __launch_bounds__(kSortBlock) k_bucket_scatter(const FrameParams* __restrict__ fpp, Paths P,
    const Counters* __restrict__ counters, int bounce) {
    if (bounce < fpp->sort_from_bounce) return;
    __shared__ int bins[kSortBins];
    __shared__ int base[kSortBins];
    for (int b = threadIdx.x; b < kSortBins; b += blockDim.x) bins[b] = 0;
    __syncthreads();
    const int in = bounce & 1;
    int begin, end;
    chunk_of(counters->active[in], begin, end);
    const int lane = static_cast<int>(threadIdx.x) & 31;
    for (int i = begin + static_cast<int>(threadIdx.x); i < end; i += blockDim.x) {
        const int key = P.sort_key[i];
        const unsigned peers = __match_any_sync(__activemask(), key);
        if (lane == __ffs(peers) - 1) atomicAdd(&bins[key], __popc(peers));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kSortBins; b += blockDim.x) {
        base[b] = bins[b] != 0 ? atomicAdd(&P.sort_cursor[b], bins[b]) : 0;
        bins[b] = 0;
    }
    __syncthreads();
    for (int i = begin + static_cast<int>(threadIdx.x); i < end; i += blockDim.x) {
        const int key = P.sort_key[i];
        const unsigned act = __activemask();
        const unsigned peers = __match_any_sync(act, key);
        const int leader = __ffs(peers) - 1;
        int start = 0;
        if (lane == leader) start = atomicAdd(&bins[key], __popc(peers));
        start = __shfl_sync(act, start, leader);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        P.sorted[base[key] + start + rank] = P.queue[in][i];
    }
}

}  // namespace

void launch_shade_sort(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce, int grid,
    cudaStream_t stream) {
    k_bucket_count<<<grid, kSortBlock, 0, stream>>>(fp, scene, paths, counters, bounce);
    k_bucket_scan<<<1, kSortBins, 0, stream>>>(fp, paths, bounce);
    k_bucket_scatter<<<grid, kSortBlock, 0, stream>>>(fp, paths, counters, bounce);
}

}  // namespace rtgb
