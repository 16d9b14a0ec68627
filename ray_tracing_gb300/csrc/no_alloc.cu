// rtgb_build_lbvh_static: the device LBVH build over caller-owned boxes that
// allocates nothing.
//
// Who needs it: callers that may not allocate device memory at the moment they
// build — an engine that rebuilds a small dynamic BVH every frame from inside a
// fixed-memory frame loop, a process under a hard device-memory budget, or code
// running where cudaMalloc would synchronise the device and stall the other
// streams. The regular path (rtgb_prepare_scene) sizes its scratch per scene
// with cudaMalloc; this entry point instead carves the same scratch out of one
// file-scope device array whose size is fixed at load time, so it works for up
// to RTGB_STATIC_LBVH_MAX_PRIMITIVES primitives and rejects anything larger.
//
// Set-up: the first call for a device looks up the array's address on that
// device (cudaGetSymbolAddress, with that device current) and caches it; later
// calls only launch. That first call may load the module and create the primary
// context, so make it once before any stream capture or latency-critical loop.
// The cached address belongs to the device's primary context: after
// cudaDeviceReset on that device it is stale, so a process that resets a
// device must not call this entry point for that device again.
// The one array is shared by every call on a device: calls that overlap in time
// (two host threads, or two streams without an ordering between them) race on
// it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "lbvh.cuh"
#include "rtgb.h"

namespace rtgb {
namespace {

// 100 bytes per primitive covers every scratch array of the build (boxes,
// ping-pong keys and indices, parents, arrival flags, node bounds, children)
// at 256-byte alignment; the slack covers the per-block radix histograms.
constexpr size_t kStaticScratchBytes = size_t(100) * RTGB_STATIC_LBVH_MAX_PRIMITIVES + (size_t(1) << 16);

static __device__ __align__(256) unsigned char g_lbvh_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_address[kMaxDevices] = {};

void set_message(char* msg, size_t cap, const char* text) {
    if (msg == nullptr || cap == 0) return;
    std::snprintf(msg, cap, "%s", text);
}

rtgb_status fail(char* msg, size_t cap, rtgb_status st, const char* what, cudaError_t err = cudaSuccess) {
    if (msg != nullptr && cap != 0) {
        if (err != cudaSuccess) std::snprintf(msg, cap, "%s: %s", what, cudaGetErrorString(err));
        else std::snprintf(msg, cap, "%s", what);
    }
    return st;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Restores the caller's current device when the call returns.
struct DeviceGuard {
    int previous = -1;
    bool switched = false;
    cudaError_t enter(int device) {
        cudaError_t e = cudaGetDevice(&previous);
        if (e != cudaSuccess) return e;
        if (previous == device) return cudaSuccess;
        e = cudaSetDevice(device);
        switched = e == cudaSuccess;
        return e;
    }
    ~DeviceGuard() {
        if (switched) cudaSetDevice(previous);
    }
};

}  // namespace
}  // namespace rtgb

extern "C" rtgb_status rtgb_build_lbvh_static(int32_t device, const float* aabb_lo, const float* aabb_hi,
    int32_t primitive_count, uint32_t* sorted_morton, int32_t* sorted_primitive, int32_t* node_children,
    float* nodes, void* stream, char* message, size_t message_size) {
    using namespace rtgb;
    set_message(message, message_size, "");
    if (device < 0 || device >= kMaxDevices) return fail(message, message_size, RTGB_INVALID_ARGUMENT, "device index out of range");
    if (primitive_count < 2)
        return fail(message, message_size, RTGB_INVALID_ARGUMENT, "primitive_count must be at least 2");
    if (primitive_count > RTGB_STATIC_LBVH_MAX_PRIMITIVES) {
        char text[160];
        std::snprintf(text, sizeof text, "primitive_count %d exceeds the static scratch limit of %d primitives",
            primitive_count, RTGB_STATIC_LBVH_MAX_PRIMITIVES);
        return fail(message, message_size, RTGB_INVALID_ARGUMENT, text);
    }
    if (aabb_lo == nullptr || aabb_hi == nullptr || sorted_morton == nullptr || sorted_primitive == nullptr
        || node_children == nullptr || nodes == nullptr)
        return fail(message, message_size, RTGB_INVALID_ARGUMENT, "null device pointer");
    if (!aligned16(aabb_lo) || !aligned16(aabb_hi) || !aligned16(nodes))
        return fail(message, message_size, RTGB_INVALID_ARGUMENT, "boxes and nodes must be 16-byte aligned");
    const size_t need = lbvh_scratch_bytes(primitive_count);
    if (need > kStaticScratchBytes)
        return fail(message, message_size, RTGB_RUNTIME_ERROR, "static scratch smaller than the build needs");

    std::lock_guard<std::mutex> lock(g_mutex);
    DeviceGuard guard;
    cudaError_t e = guard.enter(device);
    if (e != cudaSuccess) return fail(message, message_size, RTGB_RUNTIME_ERROR, "cudaSetDevice", e);
    // an error from earlier work on this thread is reported as such and left
    // in place for its owner
    if ((e = cudaPeekAtLastError()) != cudaSuccess)
        return fail(message, message_size, RTGB_RUNTIME_ERROR, "a CUDA error was pending before the call", e);
    if (g_scratch_address[device] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(message, message_size, RTGB_RUNTIME_ERROR, "cudaGetSymbolAddress(static LBVH scratch)", e);
        g_scratch_address[device] = p;
    }
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int n = primitive_count;
    // Same carve as the regular path; the box slots point at the caller's
    // arrays instead (the build only reads them). Arrival flags are cleared
    // and centroid bounds re-initialised inside lbvh_build on every call;
    // every other scratch word is written before it is read.
    LbvhScratch ls = lbvh_carve(g_scratch_address[device], n);
    ls.aabb_lo = reinterpret_cast<float4*>(const_cast<float*>(aabb_lo));
    ls.aabb_hi = reinterpret_cast<float4*>(const_cast<float*>(aabb_hi));
    int* svals = nullptr;
    uint32_t* skeys = nullptr;
    e = lbvh_build(ls, n, reinterpret_cast<BvhNode*>(nodes), &svals, &skeys, s);
    if (e != cudaSuccess) return fail(message, message_size, RTGB_RUNTIME_ERROR, "LBVH build launch", e);
    const size_t n4 = static_cast<size_t>(n) * 4;
    if ((e = cudaMemcpyAsync(sorted_morton, skeys, n4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess
        || (e = cudaMemcpyAsync(sorted_primitive, svals, n4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess
        || (e = cudaMemcpyAsync(node_children, ls.children, static_cast<size_t>(n - 1) * 8, cudaMemcpyDeviceToDevice, s))
               != cudaSuccess)
        return fail(message, message_size, RTGB_RUNTIME_ERROR, "copy of the build outputs", e);
    return RTGB_OK;
}
