// Device LBVH builder: Morton codes -> stable radix sort -> Karras hierarchy ->
// bottom-up bounds written as BVH2 nodes (see BvhNode in device_common.cuh).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "device_common.cuh"

namespace rtgb {

// Scratch owned by the caller (device pointers), sized for `n` primitives.
struct LbvhScratch {
    float4* aabb_lo;        // per input primitive (padded)
    float4* aabb_hi;
    uint32_t* keys[2];      // Morton codes (ping-pong)
    int* vals[2];           // primitive indices (ping-pong)
    uint32_t* block_hist;   // 16 * blocks
    int* parent;            // per node / leaf: parent internal node
    int* flags;             // per internal node arrival counter
    float4* node_lo;        // per internal node union box
    float4* node_hi;
    int* children;          // per internal node: 2 children (Karras encoding)
    unsigned int* bounds_bits;  // 6 ordered-int words: centroid min.xyz, max.xyz
};

size_t lbvh_scratch_bytes(int n);
LbvhScratch lbvh_carve(void* base, int n);

// Builds the hierarchy over `n` primitive boxes already in scratch.aabb_lo/hi
// and writes `n - 1` nodes (n >= 2). The sorted order (slot -> input index) is
// left in *sorted_vals, the sorted Morton codes in *sorted_keys.
cudaError_t lbvh_build(LbvhScratch& s, int n, BvhNode* nodes, int** sorted_vals, uint32_t** sorted_keys,
    cudaStream_t stream);

// Refits the node boxes of an existing hierarchy (children/parent of an
// earlier lbvh_build over the same primitive count, leaf order `sorted_vals`)
// to the boxes now in s.aabb_lo/hi: the bottom-up bounds pass of the build
// without Morton codes, sort or hierarchy (GpuSceneAcceleration::refit,
// src/realtime/gpu/gpu_scene_acceleration.cpp:347-365).
cudaError_t lbvh_refit(LbvhScratch& s, int n, const int* sorted_vals, const int* children, const int* parent,
    BvhNode* nodes, cudaStream_t stream);

// Collapses the binary hierarchy into the wide BVH of DeviceScene::nodes4 (host
// side, breadth-first): `children` holds the binary children (2 per internal
// node, a negative child c the leaf of sorted slot ~c); per BVH4 node it
// writes 4 child indices (BVH4 node, ~slot or kEmptyChild) and 4 box
// references (2 * binary node + which child, whose inline box is the child's
// box; -1 unused). Returns the BVH4 node count.
int collapse_bvh4(const int* children, int n, std::vector<int>& child4, std::vector<int>& ref4);

// Writes the wide BVH's nodes from the binary nodes' inline child boxes (after
// every build and refit).
cudaError_t fill_bvh4(const BvhNode* nodes2, const int* child4, const int* ref4, int n4, float4* nodes4,
    cudaStream_t stream);

// Morton code of a centroid inside the centroid bounds, 10 bits per axis.
// The CPU restatement in oracle/lbvh.py (numpy) follows it operation for operation.
RTGB_HD uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

RTGB_HD uint32_t quantize10(float c, float lo, float hi) {
    const float extent = hi - lo;
    const float scale = extent > 0.0f ? 1024.0f / extent : 0.0f;
    float q = (c - lo) * scale;
    q = q < 0.0f ? 0.0f : (q > 1023.0f ? 1023.0f : q);
    return static_cast<uint32_t>(q);
}

RTGB_HD uint32_t morton30(float cx, float cy, float cz, const float* lo, const float* hi) {
    return (expand_bits10(quantize10(cx, lo[0], hi[0])) << 2) | (expand_bits10(quantize10(cy, lo[1], hi[1])) << 1)
           | expand_bits10(quantize10(cz, lo[2], hi[2]));
}

}  // namespace rtgb
