// Device LBVH build (Karras 2012, "Maximizing parallelism in the construction
// of BVHs, octrees, and k-d trees"): Morton codes of primitive centroids,
// a stable LSD radix sort (4-bit digits, warp-match ranking), one thread per
// internal node for the hierarchy, and an atomic bottom-up pass for bounds.
//
// Ties between equal Morton codes break by primitive index (the sort is
// stable over index-ordered input, and the Karras prefix length falls back to
// the index when keys are equal), so the leaf order is a pure function of the
// input and oracle/lbvh.py reproduces it bit for bit.
#include "lbvh.cuh"

#include <algorithm>

namespace rtgb {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kDigits = 16;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int sort_blocks(int n) { return (n + kSortTile - 1) / kSortTile; }

RTGB_D unsigned int float_to_ordered(float f) {
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
RTGB_D float ordered_to_float(unsigned int u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_init_bounds(unsigned int* bits) {
    if (threadIdx.x < 3) bits[threadIdx.x] = 0xffffffffu;          // min: ordered max
    else if (threadIdx.x < 6) bits[threadIdx.x] = 0u;             // max: ordered min
}

// Centroid bounds via ordered-int atomics (one warp-reduced update per warp).
__global__ void k_centroid_bounds(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
    unsigned int* bits) {
    unsigned int mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = lo[i], b = hi[i];
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        for (int k = 0; k < 3; ++k) {
            const unsigned int o = float_to_ordered(c[k]);
            mn[k] = min(mn[k], o);
            mx[k] = max(mx[k], o);
        }
    }
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicMin(bits + k, mn[k]);
            atomicMax(bits + 3 + k, mx[k]);
        }
    }
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
    const unsigned int* __restrict__ bits, uint32_t* keys, int* vals) {
    float blo[3], bhi[3];
    for (int k = 0; k < 3; ++k) {
        blo[k] = ordered_to_float(bits[k]);
        bhi[k] = ordered_to_float(bits[3 + k]);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = lo[i], b = hi[i];
        keys[i] = morton30((a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f, blo, bhi);
        vals[i] = i;
    }
}

// Per-tile digit histogram (digit-major layout: hist[d * blocks + b]).
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint32_t* __restrict__ keys, int n, int shift,
    uint32_t* hist) {
    __shared__ uint32_t counts[kDigits];
    if (threadIdx.x < kDigits) counts[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&counts[(keys[i] >> shift) & (kDigits - 1)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < kDigits) hist[threadIdx.x * gridDim.x + blockIdx.x] = counts[threadIdx.x];
}

// Exclusive scan of the digit-major histogram (one block, any length).
__global__ void __launch_bounds__(1024) k_sort_scan(uint32_t* hist, int len) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < len; base += 1024) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < len ? hist[i] : 0u;
        uint32_t x = v;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if ((threadIdx.x & 31) >= off) x += y;
        }
        if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            uint32_t w = warp_sums[threadIdx.x];
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
                if (threadIdx.x >= off) w += y;
            }
            warp_sums[threadIdx.x] = w;
        }
        __syncthreads();
        const uint32_t warp_prefix = (threadIdx.x >= 32) ? warp_sums[(threadIdx.x >> 5) - 1] : 0u;
        if (i < len) hist[i] = carry + warp_prefix + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += warp_prefix + x;
        __syncthreads();
    }
}

// Stable scatter: items of a tile are ranked in input order (round by round,
// warp by warp, lane by lane) with __match_any_sync.
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const uint32_t* __restrict__ keys_in,
    const int* __restrict__ vals_in, int n, int shift, const uint32_t* __restrict__ hist, uint32_t* keys_out,
    int* vals_out) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ uint32_t running[kDigits];
    __shared__ uint32_t warp_counts[kWarps][kDigits];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < kDigits) running[threadIdx.x] = hist[threadIdx.x * gridDim.x + blockIdx.x];
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        for (int k = threadIdx.x; k < kWarps * kDigits; k += kSortThreads) (&warp_counts[0][0])[k] = 0;
        __syncthreads();
        const int i = base + r * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys_in[i] : 0u;
        const int digit = valid ? static_cast<int>((key >> shift) & (kDigits - 1)) : kDigits;  // invalid: own group
        const unsigned int peers = __match_any_sync(0xffffffffu, digit);
        const int rank_in_warp = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank_in_warp == 0) warp_counts[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t offset = running[digit];
            for (int w = 0; w < warp; ++w) offset += warp_counts[w][digit];
            const uint32_t dst = offset + static_cast<uint32_t>(rank_in_warp);
            keys_out[dst] = key;
            vals_out[dst] = vals_in[i];
        }
        __syncthreads();
        if (threadIdx.x < kDigits) {
            uint32_t total = 0;
            for (int w = 0; w < kWarps; ++w) total += warp_counts[w][threadIdx.x];
            running[threadIdx.x] += total;
        }
        __syncthreads();
    }
}

// Karras prefix length with index tie-break for equal keys.
RTGB_D int delta(const uint32_t* __restrict__ keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + __clz(static_cast<uint32_t>(i ^ j));
    return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ keys, int n, int* children, int* parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1) {
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    }
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = (lo == gamma) ? ~gamma : gamma;            // leaf slot gamma or internal node gamma
    const int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    children[2 * i] = left;
    children[2 * i + 1] = right;
    // parent[] holds internal parents for internal nodes [0, n-1) and leaves [n-1, 2n-1)
    parent[left >= 0 ? left : (n - 1 + ~left)] = i;
    parent[right >= 0 ? right : (n - 1 + ~right)] = i;
    if (i == 0) parent[0] = -1;
}

// Bottom-up bounds: each leaf walks to the root; the second arrival at a node
// unions both children and writes the node record.
__global__ void k_bounds(const float4* __restrict__ aabb_lo, const float4* __restrict__ aabb_hi,
    const int* __restrict__ sorted_vals, int n, const int* __restrict__ children, const int* __restrict__ parent,
    int* flags, float4* node_lo, float4* node_hi, BvhNode* nodes) {
    const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    int node = parent[n - 1 + leaf];
    for (int guard = 0; guard < 2 * n && node >= 0; ++guard) {
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;  // first arrival: sibling finishes this node
        __threadfence();
        float4 lo[2], hi[2];
        for (int k = 0; k < 2; ++k) {
            const int c = children[2 * node + k];
            if (c < 0) {
                const int src = sorted_vals[~c];
                lo[k] = aabb_lo[src];
                hi[k] = aabb_hi[src];
            } else {
                lo[k] = __ldcg(node_lo + c);
                hi[k] = __ldcg(node_hi + c);
            }
        }
        const int c0 = children[2 * node], c1 = children[2 * node + 1];
        BvhNode out;
        out.a = make_float4(lo[0].x, lo[0].y, lo[0].z, __int_as_float(c0));
        out.b = make_float4(hi[0].x, hi[0].y, hi[0].z, __int_as_float(c1));
        out.c = make_float4(lo[1].x, lo[1].y, lo[1].z, 0.0f);
        out.d = make_float4(hi[1].x, hi[1].y, hi[1].z, 0.0f);
        nodes[node] = out;
        __stcg(node_lo + node, make_float4(fminf(lo[0].x, lo[1].x), fminf(lo[0].y, lo[1].y), fminf(lo[0].z, lo[1].z), 0.0f));
        __stcg(node_hi + node, make_float4(fmaxf(hi[0].x, hi[1].x), fmaxf(hi[0].y, hi[1].y), fmaxf(hi[0].z, hi[1].z), 0.0f));
        node = parent[node];
    }
}

}  // namespace

size_t lbvh_scratch_bytes(int n) {
    const size_t nn = static_cast<size_t>(std::max(n, 2));
    const size_t blocks = static_cast<size_t>(sort_blocks(static_cast<int>(nn)));
    size_t b = 0;
    b += 2 * align256(nn * sizeof(float4));          // aabb lo/hi
    b += 2 * align256(nn * sizeof(uint32_t));        // keys
    b += 2 * align256(nn * sizeof(int));             // vals
    b += align256(kDigits * blocks * sizeof(uint32_t));
    b += align256(2 * nn * sizeof(int));             // parent
    b += align256(nn * sizeof(int));                 // flags
    b += 2 * align256(nn * sizeof(float4));          // node bounds
    b += align256(2 * nn * sizeof(int));             // children
    b += align256(8 * sizeof(unsigned int));
    return b;
}

LbvhScratch lbvh_carve(void* base, int n) {
    const size_t nn = static_cast<size_t>(std::max(n, 2));
    const size_t blocks = static_cast<size_t>(sort_blocks(static_cast<int>(nn)));
    char* p = static_cast<char*>(base);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += align256(bytes);
        return r;
    };
    LbvhScratch s;
    s.aabb_lo = reinterpret_cast<float4*>(take(nn * sizeof(float4)));
    s.aabb_hi = reinterpret_cast<float4*>(take(nn * sizeof(float4)));
    s.keys[0] = reinterpret_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    s.keys[1] = reinterpret_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    s.vals[0] = reinterpret_cast<int*>(take(nn * sizeof(int)));
    s.vals[1] = reinterpret_cast<int*>(take(nn * sizeof(int)));
    s.block_hist = reinterpret_cast<uint32_t*>(take(kDigits * blocks * sizeof(uint32_t)));
    s.parent = reinterpret_cast<int*>(take(2 * nn * sizeof(int)));
    s.flags = reinterpret_cast<int*>(take(nn * sizeof(int)));
    s.node_lo = reinterpret_cast<float4*>(take(nn * sizeof(float4)));
    s.node_hi = reinterpret_cast<float4*>(take(nn * sizeof(float4)));
    s.children = reinterpret_cast<int*>(take(2 * nn * sizeof(int)));
    s.bounds_bits = reinterpret_cast<unsigned int*>(take(8 * sizeof(unsigned int)));
    return s;
}

cudaError_t lbvh_build(LbvhScratch& s, int n, BvhNode* nodes, int** sorted_vals, uint32_t** sorted_keys,
    cudaStream_t stream) {
    if (n < 2) return cudaErrorInvalidValue;
    // An error left on this thread by earlier work is returned unchanged (and
    // not cleared) before anything is launched, so the launch check at the end
    // sees this build's launches only.
    if (const cudaError_t pending = cudaPeekAtLastError(); pending != cudaSuccess) return pending;
    const int threads = 256;
    const int grid = std::min((n + threads - 1) / threads, 4096);
    k_init_bounds<<<1, 32, 0, stream>>>(s.bounds_bits);
    k_centroid_bounds<<<grid, threads, 0, stream>>>(s.aabb_lo, s.aabb_hi, n, s.bounds_bits);
    k_morton<<<grid, threads, 0, stream>>>(s.aabb_lo, s.aabb_hi, n, s.bounds_bits, s.keys[0], s.vals[0]);
    const int blocks = sort_blocks(n);
    int cur = 0;
    for (int shift = 0; shift < 30; shift += 4) {
        k_sort_hist<<<blocks, kSortThreads, 0, stream>>>(s.keys[cur], n, shift, s.block_hist);
        k_sort_scan<<<1, 1024, 0, stream>>>(s.block_hist, kDigits * blocks);
        k_sort_scatter<<<blocks, kSortThreads, 0, stream>>>(s.keys[cur], s.vals[cur], n, shift, s.block_hist,
            s.keys[cur ^ 1], s.vals[cur ^ 1]);
        cur ^= 1;
    }
    k_karras<<<(n - 1 + threads - 1) / threads, threads, 0, stream>>>(s.keys[cur], n, s.children, s.parent);
    if (const cudaError_t e = cudaMemsetAsync(s.flags, 0, static_cast<size_t>(n) * sizeof(int), stream); e != cudaSuccess) {
        return e;
    }
    k_bounds<<<(n + threads - 1) / threads, threads, 0, stream>>>(s.aabb_lo, s.aabb_hi, s.vals[cur], n, s.children,
        s.parent, s.flags, s.node_lo, s.node_hi, nodes);
    *sorted_vals = s.vals[cur];
    *sorted_keys = s.keys[cur];
    return cudaGetLastError();
}

int collapse_bvh4(const int* children, int n, std::vector<int>& child4, std::vector<int>& ref4) {
    child4.clear();
    ref4.clear();
    if (n < 2) return 0;
    std::vector<int> source(1, 0);  // binary node behind each BVH4 node, breadth-first
    source.reserve(static_cast<size_t>(n));
    for (size_t i = 0; i < source.size(); ++i) {
        const int p = source[i];
        int slot = 0;
        int c4[4] = {kEmptyChild, kEmptyChild, kEmptyChild, kEmptyChild};
        int r4[4] = {-1, -1, -1, -1};
        for (int k = 0; k < 2; ++k) {
            const int ck = children[2 * p + k];
            if (ck >= 0) {  // internal: its two children become this node's
                for (int kk = 0; kk < 2; ++kk) {
                    const int g = children[2 * ck + kk];
                    r4[slot] = 2 * ck + kk;
                    if (g >= 0) {
                        c4[slot] = static_cast<int>(source.size());
                        source.push_back(g);
                    } else {
                        c4[slot] = g;
                    }
                    ++slot;
                }
            } else {
                r4[slot] = 2 * p + k;
                c4[slot] = ck;
                ++slot;
            }
        }
        child4.insert(child4.end(), c4, c4 + 4);
        ref4.insert(ref4.end(), r4, r4 + 4);
    }
    return static_cast<int>(source.size());
}

namespace {

__global__ void k_fill_bvh4(const BvhNode* __restrict__ nodes2, const int* __restrict__ child4,
    const int* __restrict__ ref4, int n4, float4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n4) return;
    float lo[3][4], hi[3][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int r = ref4[4 * i + k];
        float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
        if (r >= 0) {
            const BvhNode& nd = nodes2[r >> 1];
            a = (r & 1) ? nd.c : nd.a;
            b = (r & 1) ? nd.d : nd.b;
        }
        lo[0][k] = a.x; lo[1][k] = a.y; lo[2][k] = a.z;
        hi[0][k] = b.x; hi[1][k] = b.y; hi[2][k] = b.z;
    }
    float4* o = out + static_cast<long long>(kNode4) * i;
    for (int ax = 0; ax < 3; ++ax) {
        o[ax] = make_float4(lo[ax][0], lo[ax][1], lo[ax][2], lo[ax][3]);
        o[3 + ax] = make_float4(hi[ax][0], hi[ax][1], hi[ax][2], hi[ax][3]);
    }
    o[6] = make_float4(__int_as_float(child4[4 * i]), __int_as_float(child4[4 * i + 1]), __int_as_float(child4[4 * i + 2]),
        __int_as_float(child4[4 * i + 3]));
    o[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

}  // namespace

cudaError_t fill_bvh4(const BvhNode* nodes2, const int* child4, const int* ref4, int n4, float4* nodes4,
    cudaStream_t stream) {
    if (n4 <= 0) return cudaSuccess;
    k_fill_bvh4<<<(n4 + 127) / 128, 128, 0, stream>>>(nodes2, child4, ref4, n4, nodes4);
    return cudaGetLastError();
}

cudaError_t lbvh_refit(LbvhScratch& s, int n, const int* sorted_vals, const int* children, const int* parent,
    BvhNode* nodes, cudaStream_t stream) {
    if (n < 2) return cudaErrorInvalidValue;
    const int threads = 256;
    if (const cudaError_t e = cudaMemsetAsync(s.flags, 0, static_cast<size_t>(n) * sizeof(int), stream); e != cudaSuccess) {
        return e;
    }
    k_bounds<<<(n + threads - 1) / threads, threads, 0, stream>>>(s.aabb_lo, s.aabb_hi, sorted_vals, n, children,
        parent, s.flags, s.node_lo, s.node_hi, nodes);
    return cudaGetLastError();
}

}  // namespace rtgb
