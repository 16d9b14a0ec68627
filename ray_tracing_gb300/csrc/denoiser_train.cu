// Training kernels of the denoiser's 3x3 convolution on the sm_103a tensor
// cores (the backward pass of k_conv3x3; the input gradient is k_conv3x3 itself
// with flipped, transposed weights).
//
// k_conv3x3_wgrad: dW[o][i][dy][dx] = sum over pixels p of
// dY[p][o] * X[p + (dy - 1, dx - 1)][i], an implicit GEMM per tap with the
// pixels as the reduction dimension:
//   * a CTA owns every 8 x 16-pixel tile j with j % gridDim.x == blockIdx.x and
//     the taps of blockIdx.y's group; the tile's 10 x 18 input halo (one TMA
//     box per 8-channel block, as k_conv3x3 loads it) and its dY tile (one
//     8 x 16 box per block) stream through two shared-memory stages;
//   * per tap and per 16 pixels (two tile rows) one tcgen05.mma with
//     M = 128 input channels (blocks past c_in stay zero), N = c_out,
//     K = 16 pixels. Both operands are MN-major straight from the blocked
//     layout: a core matrix is 8 pixels x 8 channels = 128 contiguous bytes;
//     the next 8 pixels along K are one row on (the descriptor's leading byte
//     offset: 160 bytes in the halo, 128 in dY) and the next 8 channels along
//     M or N one box on (its stride byte offset) -- for MN-major no-swizzle
//     operands, as for K-major ones, the leading offset steps along K (checked
//     against all four assignments on this GPU; only this one is exact);
//   * the per-tap FP32 accumulators live in TMEM for the CTA's whole run; at
//     the end four warps write them to a per-CTA partial buffer, which
//     k_wgrad_reduce sums into dW (no atomics).
// k_bias_grad sums dY over pixels per channel.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "denoiser.cuh"
#include "rtgb.h"
#include "tc_primitives.cuh"

namespace rtgb {
namespace {

constexpr int kTileW = 8;
constexpr int kTileH = 16;
constexpr int kHaloW = kTileW + 2;
constexpr int kHaloH = kTileH + 2;
constexpr int kXBoxBytes = kHaloW * kHaloH * 16;     // 2880
constexpr int kXBoxStride = 2944;                    // 128-byte aligned
constexpr int kYBoxBytes = kTileW * kTileH * 16;     // 2048
constexpr int kHaloRow = kHaloW * 16;                // 160: next pixel row of a halo box
constexpr int kTileRow = kTileW * 16;                // 128: next pixel row of a dY box
constexpr int kMBlocks = 16;                         // M = 128 input channels
constexpr int kStageBytes = kMBlocks * kXBoxStride + 8 * kYBoxBytes;  // 63488
constexpr int kWgradSmem = 256 + 2 * kStageBytes;
constexpr int kWgradThreads = 192;                   // producer, issuer, four epilogue warps
constexpr int kSpin = 1 << 22;

struct WgradArgs {
    int n, h, w, cin, cout;
    int tap0, taps;        // this launch's tap group: taps [tap0 + blockIdx.y * taps, ...)
    uint32_t tmem_cols;    // power of two >= taps * cout
    float* partial;        // [gridDim.x][9][128][cout]
    int* err;
    // descriptor byte offsets of the halo (A) and dY (B) operands: leading
    // (along K) and stride (along M or N)
    uint32_t a_lbo, a_sbo, b_lbo, b_sbo;
};

// Instruction descriptor of kind::f16 with both operands MN-major.
__host__ __device__ constexpr uint32_t idesc_bf16_f32_mn(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__global__ void __launch_bounds__(kWgradThreads, 1) k_conv3x3_wgrad(const __grid_constant__ CUtensorMap xmap,
    const __grid_constant__ CUtensorMap ymap, WgradArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* full_bar = reinterpret_cast<uint64_t*>(smem);  // [2] stage landed
    uint64_t* empty_bar = full_bar + 2;                       // [2] stage consumed (UMMA commit)
    uint64_t* done_bar = full_bar + 4;                        // every UMMA of the CTA completed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 64);
    volatile int* stop = reinterpret_cast<volatile int*>(smem + 72);
    uint8_t* stage0 = smem + 256;
    const int xboxes = a.cin >> 3, yboxes = a.cout >> 3;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // channel blocks past c_in stay zero in both stages (TMA never writes them)
    for (int s = 0; s < 2; ++s) {
        uint4* pad = reinterpret_cast<uint4*>(stage0 + s * kStageBytes + xboxes * kXBoxStride);
        const int words = (kMBlocks - xboxes) * kXBoxStride / 16;
        for (int i = threadIdx.x; i < words; i += blockDim.x) pad[i] = make_uint4(0, 0, 0, 0);
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < 5; ++i) tc::mbar_init(full_bar + i, 1);
        *stop = 0;
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, a.tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const int tiles_x = (a.w + kTileW - 1) / kTileW;
    const int tiles_y = (a.h + kTileH - 1) / kTileH;
    const int per_image = tiles_x * tiles_y;
    const int total = per_image * a.n;
    const int count = static_cast<int>(blockIdx.x) < total ? (total - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1 : 0;
    const int tap_first = a.tap0 + static_cast<int>(blockIdx.y) * a.taps;
    const int tap_count = 9 - tap_first < a.taps ? 9 - tap_first : a.taps;
    auto fail = [&](int code) {
        *stop = 1;
        if (a.err != nullptr) atomicExch(a.err, code);
    };

    if (warp == 0) {
        // ---- producer
        if (lane == 0) {
            int issued = 0;
            for (int j = 0; j < count; ++j) {
                const int s = j & 1;
                if (j >= 2 && !tc::mbar_wait_or_abort(empty_bar + s, static_cast<uint32_t>(j / 2 - 1) & 1u, kSpin, stop)) {
                    fail(11);
                    break;
                }
                const int tile = static_cast<int>(blockIdx.x) + j * static_cast<int>(gridDim.x);
                const int img = tile / per_image;
                const int t = tile - img * per_image;
                const int ty = t / tiles_x;
                const int x0 = (t - ty * tiles_x) * kTileW;
                const int y0 = ty * kTileH;
                uint8_t* st = stage0 + s * kStageBytes;
                tc::mbar_arrive_expect_tx(full_bar + s, static_cast<uint32_t>(xboxes * kXBoxBytes + yboxes * kYBoxBytes));
                for (int b = 0; b < xboxes; ++b) {
                    tc::tma_load_3d(st + b * kXBoxStride, &xmap, full_bar + s, 8 * (x0 - 1), y0 - 1, img * xboxes + b);
                }
                for (int b = 0; b < yboxes; ++b) {
                    tc::tma_load_3d(st + kMBlocks * kXBoxStride + b * kYBoxBytes, &ymap, full_bar + s, 8 * x0, y0,
                        img * yboxes + b);
                }
                issued = j + 1;
            }
            for (int j = issued > 2 ? issued - 2 : 0; j < issued; ++j) {
                tc::mbar_wait(full_bar + (j & 1), static_cast<uint32_t>(j / 2) & 1u, kSpin);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---- issuer: per tile, per tap of the group, 8 UMMAs of 16 pixels
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_f32_mn(128, a.cout);
            bool committed = false;
            for (int j = 0; j < count; ++j) {
                const int s = j & 1;
                if (!tc::mbar_wait_or_abort(full_bar + s, static_cast<uint32_t>(j / 2) & 1u, kSpin, stop)) {
                    fail(12);
                    break;
                }
                tc::tc_fence_after();
                const uint32_t xs = tc::smem_u32(stage0 + s * kStageBytes);
                const uint32_t ys = xs + kMBlocks * kXBoxStride;
                for (int q = 0; q < tap_count; ++q) {
                    const int tap = tap_first + q;
                    const int dy = tap / 3, dx = tap - 3 * (tap / 3);
                    const uint32_t acc = tmem + static_cast<uint32_t>(q * a.cout);
                    for (int k = 0; k < kTileH / 2; ++k) {
                        // pixels of tile rows 2k, 2k + 1: halo rows 2k + dy.., columns dx..dx + 7
                        const uint64_t ad = tc::smem_desc(
                            xs + static_cast<uint32_t>(((2 * k + dy) * kHaloW + dx) * 16), a.a_lbo, a.a_sbo);
                        const uint64_t bd = tc::smem_desc(ys + static_cast<uint32_t>(2 * k * kTileRow), a.b_lbo, a.b_sbo);
                        tc::umma_bf16(acc, ad, bd, idesc, (j > 0 || k > 0) ? 1u : 0u);
                    }
                }
                tc::umma_commit(empty_bar + s);
                committed = true;
            }
            if (committed) tc::umma_commit(done_bar);
            else tc::mbar_arrive(done_bar);  // nothing issued: the epilogue writes zeros
        }
        __syncwarp();
    } else {
        // ---- epilogue: TMEM lane = input channel, columns = (tap, output channel)
        const int quarter = warp & 3;
        const bool done = tc::mbar_wait_or_abort(done_bar, 0u, kSpin, stop);
        if (__all_sync(0xffffffffu, done)) {
            tc::tc_fence_after();
            const int ci = quarter * 32 + lane;
            for (int q = 0; q < tap_count; ++q) {
                float* dst = a.partial + ((static_cast<long long>(blockIdx.x) * 9 + tap_first + q) * 128 + ci) * a.cout;
                for (int g = 0; g < (a.cout >> 4); ++g) {
                    uint32_t v[16];
                    tc::tmem_ld16(tmem + (static_cast<uint32_t>(quarter * 32) << 16) + static_cast<uint32_t>(q * a.cout + g * 16), v);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int e = 0; e < 16; ++e) dst[g * 16 + e] = count > 0 ? __uint_as_float(v[e]) : 0.0f;
                }
            }
        } else if (lane == 0) {
            fail(13);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, a.tmem_cols);
}

// dW[o][i][tap] (PyTorch's out x in x 3 x 3 order) = sum over CTAs of the partials.
__global__ void k_wgrad_reduce(const float* __restrict__ partial, int ctas, int cin, int cout, float* __restrict__ dw) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cout * cin * 9) return;
    const int tap = e % 9;
    const int i = (e / 9) % cin;
    const int o = e / (9 * cin);
    float sum = 0.0f;
    for (int c = 0; c < ctas; ++c) sum += partial[((static_cast<long long>(c) * 9 + tap) * 128 + i) * cout + o];
    dw[e] = sum;
}

// db[o] += sum over pixels of dY (blocked layout, `hw` pixels per image); a
// block sums a run of pixels of one 8-channel block: each thread a strided
// slice of 16-byte loads, then warp shuffles and a shared-memory pass across
// the block's warps, so each block adds one value per channel (atomics on the
// few bias words used to come from every warp and serialised in L2).
constexpr int kBiasThreads = 256;
constexpr int kBiasLoadsPerThread = 16;

__global__ void __launch_bounds__(kBiasThreads) k_bias_grad(const __nv_bfloat16* __restrict__ dy, int n, long long hw,
    int cout, float* __restrict__ db) {
    __shared__ float part[kBiasThreads / 32][8];
    const int blocks = cout >> 3;
    const int cb = blockIdx.y % blocks, img = blockIdx.y / blocks;
    const __nv_bfloat16* base = dy + (static_cast<long long>(img) * blocks + cb) * hw * 8;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < hw;
         p += static_cast<long long>(gridDim.x) * blockDim.x) {
        const uint4 q = *reinterpret_cast<const uint4*>(base + p * 8);
        const __nv_bfloat16* v = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] += __bfloat162float(v[k]);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float v = acc[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) part[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        float v = 0.0f;
        for (int w = 0; w < kBiasThreads / 32; ++w) v += part[w][threadIdx.x];
        atomicAdd(db + cb * 8 + threadIdx.x, v);
    }
    (void)n;
}

struct Scratch {
    void* p = nullptr;
    size_t bytes = 0;
    std::mutex m;
};

Scratch& wgrad_scratch() {
    static Scratch s;
    return s;
}

void set_message(char* msg, size_t cap, const char* text) {
    if (msg != nullptr && cap > 0) std::snprintf(msg, cap, "%s", text);
}

}  // namespace

// Tap groups of a layer: as many taps as fit 512 TMEM columns of c_out each.
int wgrad_taps_per_group(int cout) {
    const int t = 512 / cout;
    return t < 9 ? t : 9;
}

cudaError_t launch_conv3x3_wgrad(const void* x, int n, int h, int w, int cin, const void* dy, int cout, float* dweight,
    float* dbias, int* err, int sms, cudaStream_t stream, float* partial, size_t partial_bytes) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_conv3x3_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgradSmem);
    });
    if (attr != cudaSuccess) return attr;
    CUtensorMap xmap, ymap;
    if (!blocked_tensor_map(&xmap, x, n, h, w, cin, kHaloW, kHaloH) ||
        !blocked_tensor_map(&ymap, dy, n, h, w, cout, kTileW, kTileH)) {
        return cudaErrorInvalidValue;
    }
    const long long tiles = static_cast<long long>((w + kTileW - 1) / kTileW) * ((h + kTileH - 1) / kTileH) * n;
    const int gx = static_cast<int>(tiles < sms ? tiles : sms);
    const int taps = wgrad_taps_per_group(cout);
    const int gy = (9 + taps - 1) / taps;
    if (static_cast<size_t>(gx) * 9 * 128 * cout * sizeof(float) > partial_bytes) return cudaErrorInvalidValue;
    uint32_t cols = 32;
    while (cols < static_cast<uint32_t>(taps * cout)) cols <<= 1;
    WgradArgs a{n, h, w, cin, cout, 0, taps, cols, partial, err, kHaloRow, kXBoxStride, kTileRow, kYBoxBytes};
    k_conv3x3_wgrad<<<dim3(gx, gy), kWgradThreads, kWgradSmem, stream>>>(xmap, ymap, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int elems = cout * cin * 9;
    k_wgrad_reduce<<<(elems + 255) / 256, 256, 0, stream>>>(partial, gx, cin, cout, dweight);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (dbias != nullptr) {
        if ((e = cudaMemsetAsync(dbias, 0, static_cast<size_t>(cout) * sizeof(float), stream)) != cudaSuccess) return e;
        const long long hw = static_cast<long long>(h) * w;
        constexpr long long kPerBlock = static_cast<long long>(kBiasThreads) * kBiasLoadsPerThread;
        long long bx = (hw + kPerBlock - 1) / kPerBlock;
        bx = bx < 64 ? bx : 64;
        k_bias_grad<<<dim3(static_cast<unsigned>(bx), static_cast<unsigned>(n * (cout >> 3))), kBiasThreads, 0, stream>>>(
            static_cast<const __nv_bfloat16*>(dy), n, hw, cout, dbias);
        e = cudaGetLastError();
    }
    return e;
}

size_t wgrad_partial_bytes(int sms, int cout) { return static_cast<size_t>(sms) * 9 * 128 * cout * sizeof(float); }

}  // namespace rtgb

extern "C" rtgb_status rtgb_conv3x3_wgrad_bf16(const void* x, int32_t n, int32_t h, int32_t w, int32_t c_in,
    const void* dy, int32_t c_out, float* dweight, float* dbias, int32_t* device_error, void* stream, char* message,
    size_t message_size) {
    using namespace rtgb;
    set_message(message, message_size, "");
    if (x == nullptr || dy == nullptr || dweight == nullptr || n <= 0 || h <= 0 || w <= 0) {
        set_message(message, message_size, "null pointer or empty extent");
        return RTGB_INVALID_ARGUMENT;
    }
    if (c_in < 16 || c_in > 128 || c_in % 16 != 0 || c_out < 16 || c_out > 64 || c_out % 16 != 0) {
        set_message(message, message_size, "c_in must be a multiple of 16 in [16, 128], c_out a multiple of 16 in [16, 64]");
        return RTGB_INVALID_ARGUMENT;
    }
    if ((reinterpret_cast<uintptr_t>(x) & 15u) != 0 || (reinterpret_cast<uintptr_t>(dy) & 15u) != 0) {
        set_message(message, message_size, "tensors must be 16-byte aligned");
        return RTGB_INVALID_ARGUMENT;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    sms = sms > 0 ? sms : 1;
    Scratch& sc = wgrad_scratch();
    std::lock_guard<std::mutex> lock(sc.m);
    const size_t need = wgrad_partial_bytes(sms, c_out);
    if (sc.bytes < need) {
        // the previous user of the scratch may still be running on its stream
        if (sc.p != nullptr) {
            cudaDeviceSynchronize();
            cudaFree(sc.p);
        }
        sc.p = nullptr;
        sc.bytes = 0;
        if (cudaMalloc(&sc.p, need) != cudaSuccess) {
            set_message(message, message_size, "out of device memory for the weight-gradient partials");
            return RTGB_RUNTIME_ERROR;
        }
        sc.bytes = need;
    }
    const cudaError_t e = launch_conv3x3_wgrad(x, n, h, w, c_in, dy, c_out, dweight, dbias, device_error, sms,
        static_cast<cudaStream_t>(stream), static_cast<float*>(sc.p), sc.bytes);
    if (e != cudaSuccess) {
        set_message(message, message_size, cudaGetErrorString(e));
        return RTGB_RUNTIME_ERROR;
    }
    return RTGB_OK;
}
