// Denoiser convolutions on the sm_103a tensor cores.
//
// k_conv3x3 is an implicit-GEMM 3x3 convolution (stride 1, zero padding 1) over
// channel-blocked BF16 tensors, [n][c/8][h][w][8] (8 channels innermost, then
// x, y, the channel block and the image), with FP32 accumulation in TMEM:
//   * a CTA owns a tile of 8 x 16 output pixels (the GEMM's M = 128 rows) and
//     every output channel (N = C_out <= 64);
//   * the 10 x 18 input halo of the tile arrives by TMA, one box per 8-channel
//     block: in the blocked layout a halo row of one block (10 pixels x 8
//     channels) is 160 contiguous bytes, so the tensor map's innermost
//     dimension is a whole image row of that block and a box is 18 rows of 160
//     bytes, landing as a dense [18][10][8] block; the image border is the
//     TMA's zero fill, which is exactly the convolution's zero padding;
//   * the packed weights of all nine taps stay resident in shared memory;
//   * one thread issues, per tap and per 16 input channels, a
//     tcgen05.mma.kind::f16 (BF16 x BF16 -> FP32) whose A operand is the halo
//     shifted by the tap: with the [row][col][8 channels] box layout an 8-pixel
//     row of the window is one 8 x 16-byte core matrix, core matrices of the
//     next row are 160 bytes apart and those of the next 8 channels one box
//     apart, so no im2col copy exists;
//   * the epilogue reads the accumulators with tcgen05.ld (warp w owns TMEM
//     lanes 32w..32w+31, i.e. tile rows 4w..4w+3), adds the bias, applies ReLU
//     and stores BF16 into a blocked tensor at a channel offset (the eight
//     lanes of a tile row write 128 contiguous bytes per block), so encoder
//     outputs land directly in the decoder's concatenation buffers;
//   * two fused epilogues serve the U-Net: `pool` also writes the 2 x 2
//     average of the (BF16-rounded) output at half resolution, the four pixels
//     of a pooling window being lanes l, l+1, l+8, l+9 of one warp (tiles start
//     at even coordinates), and `up` writes every output pixel to the 2 x 2
//     block of a twice-as-large tensor (nearest upsampling into the decoder's
//     concatenation buffer).
// The grid is persistent and each CTA is warp-specialised: a producer warp
// streams halos through up to four shared-memory stages (as many as fit
// beside the weights), two issuer warps alternate tiles (a single issuing
// thread reaches about half the tensor core's rate on these small-N UMMAs),
// and four epilogue warps drain four TMEM accumulators, all linked by
// mbarriers. Layers small enough keep several such CTAs on one SM. Every
// mbarrier wait is bounded and a failed role stops the others.
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
constexpr int kBoxBytes = kHaloW * kHaloH * 16;   // one 8-channel box: 2880 bytes
constexpr int kBoxStride = 2944;                  // boxes 128-byte aligned in shared memory
constexpr int kRowBytes = kHaloW * 16;            // next tile row of a box
constexpr int kMaxCout = 64;
constexpr int kMaxCin = 128;
constexpr int kSpin = 1 << 22;
// Opt-in shared-memory ceiling; a launch asks for what its layer needs
// (conv_smem_bytes), so small layers run several CTAs per SM.
constexpr int kConvSmem = 227 * 1024;

constexpr int kMaxStages = 4;

// Halo stages of a layer, even so that two issuer warps can share the CTA:
// 4 or 2, whichever still lets two CTAs share an SM (two sets of issuers keep
// the tensor core busier than a deeper ring), else the larger that fits
// beside the weights, else 1 (one issuer).
int conv_stages(int cin, int cout) {
    const int stage = (cin / 8) * kBoxStride;
    const int fixed = 256 + 9 * cin * cout * 2;
    for (int s = kMaxStages; s >= 2; s -= 2) {
        const int bytes = (fixed + s * stage + 1023) & ~1023;
        if (2 * (bytes + 1024) <= 228 * 1024) return s;
    }
    const int room = (kConvSmem - fixed) / stage;
    return room >= 4 ? 4 : (room >= 2 ? 2 : 1);
}

// Shared memory of a CTA with `stages` halo stages (0: conv_stages).
int conv_smem_bytes(int cin, int cout, int stages = 0) {
    const int need = 256 + (stages > 0 ? stages : conv_stages(cin, cout)) * (cin / 8) * kBoxStride + 9 * cin * cout * 2;
    return (need + 1023) & ~1023;
}

// TMEM columns of a CTA: four FP32 accumulators of at least cout (and at
// least 32) columns each, a power of two as tcgen05.alloc takes.
uint32_t conv_tmem_cols(int cout) {
    uint32_t cols = 128;
    while (cols < static_cast<uint32_t>(4 * cout)) cols <<= 1;
    return cols;
}

struct ConvArgs {
    int n, h, w, cin, cout;
    int y_channels, y_offset, relu;
    const uint4* weight;   // packed [tap][cin/8][cout][8] BF16
    const float* bias;     // cout
    __nv_bfloat16* y;
    int* err;
    // fused epilogue variants (k_conv3x3's comment)
    __nv_bfloat16* pool;   // non-null: also write the 2x2 average of the output (dense cout channels)
    int up;                // non-zero: y is twice the input size, each output pixel written 2 x 2
    int stages;            // halo stages in shared memory (conv_stages)
    uint32_t tmem_cols;    // conv_tmem_cols(cout)
};

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// Epilogue of one tile: the accumulators at TMEM column `acc` (this warp's 32
// lanes = 4 tile rows) plus bias, ReLU, BF16 store, and the fused pooling or
// upsampling variant.
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, uint32_t acc, int tile, int tiles_x, int per_image,
    int warp, int lane) {
    const int img = tile / per_image;
    const int t = tile - img * per_image;
    const int ty = t / tiles_x;
    const int x0 = (t - ty * tiles_x) * kTileW;
    const int y0 = ty * kTileH;
    const int m = warp * 32 + lane;
    const int yy = y0 + (m >> 3);
    const int xx = x0 + (m & 7);
    const bool inside = yy < a.h && xx < a.w;
    const int oh = a.up ? 2 * a.h : a.h, ow = a.up ? 2 * a.w : a.w;
    const int oy = a.up ? 2 * yy : yy, ox = a.up ? 2 * xx : xx;
    const int ycb = a.y_channels >> 3;
    const long long oplane = static_cast<long long>(oh) * ow * 8;  // elements of one channel block
    // block (y_offset / 8) of this output pixel; the next block is oplane further
    __nv_bfloat16* out = a.y + ((static_cast<long long>(img) * ycb + (a.y_offset >> 3)) * oh + oy) * ow * 8 + ox * 8;
    const int ph = (a.h + 1) >> 1, pw = (a.w + 1) >> 1;
    const long long pplane = static_cast<long long>(ph) * pw * 8;
    // every 16-column group of this lane's accumulator row in flight at once, one wait
    const int groups = a.cout >> 4;
    uint32_t v[kMaxCout / 16][16];
#pragma unroll
    for (int g = 0; g < kMaxCout / 16; ++g) {
        if (g < groups) tc::tmem_ld16(acc + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(g * 16), v[g]);
    }
    tc::tmem_wait_ld();
#pragma unroll
    for (int g = 0; g < kMaxCout / 16; ++g) {
        if (g >= groups) break;
        uint32_t packed[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float lo = __uint_as_float(v[g][2 * k]) + __ldg(a.bias + g * 16 + 2 * k);
            float hi = __uint_as_float(v[g][2 * k + 1]) + __ldg(a.bias + g * 16 + 2 * k + 1);
            if (a.relu) {
                lo = fmaxf(lo, 0.0f);
                hi = fmaxf(hi, 0.0f);
            }
            packed[k] = pack_bf16x2(lo, hi);
        }
        const uint4 q0 = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        const uint4 q1 = make_uint4(packed[4], packed[5], packed[6], packed[7]);
        if (inside) {
            __nv_bfloat16* blk = out + 2 * g * oplane;  // channels 16g..16g+7 here, 16g+8.. one plane on
            if (a.up) {
                for (int dy = 0; dy < 2; ++dy) {
                    for (int dx = 0; dx < 2; ++dx) {
                        if (oy + dy >= oh || ox + dx >= ow) continue;
                        const long long o = (static_cast<long long>(dy) * ow + dx) * 8;
                        *reinterpret_cast<uint4*>(blk + o) = q0;
                        *reinterpret_cast<uint4*>(blk + oplane + o) = q1;
                    }
                }
            } else {
                *reinterpret_cast<uint4*>(blk) = q0;
                *reinterpret_cast<uint4*>(blk + oplane) = q1;
            }
        }
        if (a.pool != nullptr) {
            // 2x2 window: this lane, lane+1 (next column), lane+8 (next row), lane+9
            const float cnt0 = inside ? 1.0f : 0.0f;
            const float cnt1 = cnt0 + __shfl_down_sync(0xffffffffu, cnt0, 1);
            const float cnt = cnt1 + __shfl_down_sync(0xffffffffu, cnt1, 8);
            uint32_t pooled[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const __nv_bfloat162 b2 = *reinterpret_cast<const __nv_bfloat162*>(&packed[k]);
                float lo = inside ? __low2float(b2) : 0.0f;
                float hi = inside ? __high2float(b2) : 0.0f;
                lo += __shfl_down_sync(0xffffffffu, lo, 1);
                hi += __shfl_down_sync(0xffffffffu, hi, 1);
                lo += __shfl_down_sync(0xffffffffu, lo, 8);
                hi += __shfl_down_sync(0xffffffffu, hi, 8);
                const float inv = cnt > 0.0f ? 1.0f / cnt : 0.0f;
                pooled[k] = pack_bf16x2(lo * inv, hi * inv);
            }
            if (inside && ((m >> 3) & 1) == 0 && (m & 1) == 0) {
                // dense cout-channel blocked tensor at half resolution
                __nv_bfloat16* pblk = a.pool + ((static_cast<long long>(img) * (a.cout >> 3) + 2 * g) * ph + (yy >> 1)) * pw * 8 +
                                      (xx >> 1) * 8;
                *reinterpret_cast<uint4*>(pblk) = make_uint4(pooled[0], pooled[1], pooled[2], pooled[3]);
                *reinterpret_cast<uint4*>(pblk + pplane) = make_uint4(pooled[4], pooled[5], pooled[6], pooled[7]);
            }
        }
    }
}

// Warp roles of k_conv3x3 (kConvThreads = 224): warp 0 is the TMA producer,
// warps 1 and 2 issue the UMMAs of alternating tiles (one issuing thread
// cannot keep the tensor core busy: two reach its rate), warps 3..6 run the
// epilogue, warp w reading TMEM lanes 32 (w % 4) .. + 31. (A second group of
// epilogue warps measured slower: it takes issue slots from the issuers.)
constexpr int kConvThreads = 224;
constexpr int kIssuers = 2;
constexpr int kEpilogueGroups = 1;
constexpr int kAccs = 4;          // accumulators in TMEM: tile j uses j % kAccs, issued by warp 1 + j % kIssuers

__global__ void __launch_bounds__(kConvThreads, 2) k_conv3x3(const __grid_constant__ CUtensorMap xmap, ConvArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* full_bar = reinterpret_cast<uint64_t*>(smem);   // [kMaxStages] halo stage landed (TMA bytes)
    uint64_t* empty_bar = full_bar + kMaxStages;               // [kMaxStages] halo stage consumed (UMMA commit)
    uint64_t* acc_full = empty_bar + kMaxStages;               // [kAccs] accumulator written (UMMA commit)
    uint64_t* acc_empty = acc_full + kAccs;                    // [kAccs] accumulator read (4 epilogue warps)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 128);
    volatile int* stop = reinterpret_cast<volatile int*>(smem + 136);
    const int boxes = a.cin >> 3;
    const int stages = a.stages;
    const int stage_bytes = boxes * kBoxStride;
    uint8_t* sa = smem + 256;
    uint8_t* sb = sa + stages * stage_bytes;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2 * kMaxStages + kAccs; ++i) tc::mbar_init(full_bar + i, 1);
        for (int i = 0; i < kAccs; ++i) tc::mbar_init(acc_empty + i, 4);
        *stop = 0;
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, a.tmem_cols);
        tc::tmem_relinquish();
    }
    const int wvec = 9 * a.cin * a.cout * 2 / 16;
    for (int i = threadIdx.x; i < wvec; i += blockDim.x) reinterpret_cast<uint4*>(sb)[i] = a.weight[i];
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t acc_cols = a.tmem_cols / kAccs;

    const int tiles_x = (a.w + kTileW - 1) / kTileW;
    const int tiles_y = (a.h + kTileH - 1) / kTileH;
    const int per_image = tiles_x * tiles_y;
    const int total = per_image * a.n;
    // this CTA's tiles: blockIdx.x + j * gridDim.x for j < count
    const int count = static_cast<int>(blockIdx.x) < total ? (total - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1 : 0;
    auto tile_of = [&](int j) { return static_cast<int>(blockIdx.x) + j * static_cast<int>(gridDim.x); };
    auto fail = [&](int code) {
        *stop = 1;
        if (a.err != nullptr) atomicExch(a.err, code);
    };

    if (warp == 0) {
        // ---- producer: halo of tile j into stage j % stages once tile j - stages has left it
        int issued = 0;
        if (lane == 0) {
            for (int j = 0; j < count; ++j) {
                const int s = j % stages;
                if (j >= stages &&
                    !tc::mbar_wait_or_abort(empty_bar + s, static_cast<uint32_t>(j / stages - 1) & 1u, kSpin, stop)) {
                    fail(1);
                    break;
                }
                const int tile = tile_of(j);
                const int img = tile / per_image;
                const int t = tile - img * per_image;
                const int ty = t / tiles_x;
                const int x0 = (t - ty * tiles_x) * kTileW;
                const int y0 = ty * kTileH;
                uint8_t* dst = sa + s * stage_bytes;
                tc::mbar_arrive_expect_tx(full_bar + s, static_cast<uint32_t>(boxes * kBoxBytes));
                for (int b = 0; b < boxes; ++b) {
                    tc::tma_load_3d(dst + b * kBoxStride, &xmap, full_bar + s, 8 * (x0 - 1), y0 - 1, img * boxes + b);
                }
                issued = j + 1;
            }
            // the last load of every stage has landed before shared memory is released
            for (int j = issued - stages > 0 ? issued - stages : 0; j < issued; ++j) {
                tc::mbar_wait(full_bar + j % stages, static_cast<uint32_t>(j / stages) & 1u, kSpin);
            }
        }
        __syncwarp();
    } else if (warp <= kIssuers) {
        // ---- issuers: tile j (j % issuers == warp - 1) from stage j % stages into accumulator j % kAccs.
        // A parity wait on an mbarrier only tells two consecutive phases apart, so each barrier's
        // rounds must be waited for in order by one thread: with an even stage count every tile of
        // a stage (and of an accumulator) has the same parity of j, so two issuers can alternate;
        // with an odd count one issuer takes every tile.
        // Descriptors are built once and advanced by constant deltas (their address field is the
        // shared-memory address / 16 and every address stays inside this CTA's window, so the adds
        // never carry out of it).
        const int issuers = (stages & 1) == 0 ? kIssuers : 1;
        if (lane == 0 && warp - 1 < issuers) {
            const uint32_t idesc = tc::idesc_bf16_f32(128, a.cout);
            const uint32_t bstep = static_cast<uint32_t>(a.cout) * 16u;
            const uint64_t b_first = tc::smem_desc(tc::smem_u32(sb), bstep, 128);
            const uint64_t b_step = static_cast<uint64_t>((2u * bstep) >> 4);      // next 16 input channels of a tap
            const uint64_t a_step = static_cast<uint64_t>((2 * kBoxStride) >> 4);  // next two channel boxes
            const int ksteps = boxes >> 1;
            int last = -1;
            for (int j = warp - 1; j < count; j += issuers) {
                const int s = j % stages;
                const int b = j % kAccs;
                if (!tc::mbar_wait_or_abort(full_bar + s, static_cast<uint32_t>(j / stages) & 1u, kSpin, stop)) {
                    fail(2);
                    break;
                }
                if (j >= kAccs &&
                    !tc::mbar_wait_or_abort(acc_empty + b, static_cast<uint32_t>(j / kAccs - 1) & 1u, kSpin, stop)) {
                    fail(3);
                    break;
                }
                tc::tc_fence_after();
                const uint64_t a_first = tc::smem_desc(tc::smem_u32(sa + s * stage_bytes), kBoxStride, kRowBytes);
                const uint32_t acc = tmem + static_cast<uint32_t>(b) * acc_cols;
                uint64_t bd = b_first;
                uint32_t accumulate = 0;
#pragma unroll
                for (int tap = 0; tap < 9; ++tap) {
                    // the tap's window: dy rows (kRowBytes each) and dx pixels (16 bytes each) into the halo
                    uint64_t ad = a_first + static_cast<uint64_t>(((tap / 3) * kRowBytes + (tap % 3) * 16) >> 4);
                    for (int p = 0; p < ksteps; ++p) {
                        tc::umma_bf16(acc, ad, bd, idesc, accumulate);
                        accumulate = 1;
                        ad += a_step;
                        bd += b_step;
                    }
                }
                tc::umma_commit(empty_bar + s);   // the halo stage is free once these UMMAs complete
                tc::umma_commit(acc_full + b);    // and the accumulator is ready for the epilogue
                last = j;
            }
            // every UMMA this thread issued has completed before TMEM is released
            if (last >= 0) tc::mbar_wait(acc_full + last % kAccs, static_cast<uint32_t>(last / kAccs) & 1u, kSpin);
        }
        __syncwarp();
    } else {
        // ---- epilogue: group (warp - 3) / 4 takes every kEpilogueGroups-th tile, this warp the
        // quarter of the accumulator's lanes its warp index selects
        const int quarter = warp & 3;
        for (int j = (warp - 1 - kIssuers) / 4; j < count; j += kEpilogueGroups) {
            const int b = j % kAccs;
            const bool ready = tc::mbar_wait_or_abort(acc_full + b, static_cast<uint32_t>(j / kAccs) & 1u, kSpin, stop);
            if (!__all_sync(0xffffffffu, ready)) {
                if (lane == 0) fail(4);
                break;
            }
            tc::tc_fence_after();
            conv_epilogue(a, tmem + static_cast<uint32_t>(b) * acc_cols, tile_of(j), tiles_x, per_image, quarter, lane);
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(acc_empty + b);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, a.tmem_cols);
}

// ---- host ----------------------------------------------------------------------------------

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled() {
    static std::once_flag once;
    static EncodeTiled fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<EncodeTiled>(p);
        }
    });
    return fn;
}

void set_message(char* msg, size_t cap, const char* text) {
    if (msg != nullptr && cap > 0) std::snprintf(msg, cap, "%s", text);
}

uint16_t to_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return static_cast<uint16_t>((u >> 16) | 0x40u);  // quiet NaN
    u += 0x7fffu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}

}  // namespace

// Encodes the TMA map of a channel-blocked BF16 tensor ([n][c/8][h][w][8]) for
// k_conv3x3's halo boxes: dimension 0 is one image row of a channel block
// (w x 8 elements), then rows, then (image, block) planes; a box is 10 pixels
// x 8 channels by 18 rows. Pixels left of 0 or right of w - 1 fall outside
// dimension 0 and read as zero, like rows outside [0, h).
bool conv_input_map(CUtensorMap* map, const void* x, int n, int h, int w, int c) {
    return blocked_tensor_map(map, x, n, h, w, c, kHaloW, kHaloH);
}

bool blocked_tensor_map(CUtensorMap* map, const void* x, int n, int h, int w, int c, int box_pixels, int box_rows) {
    EncodeTiled enc = encode_tiled();
    if (enc == nullptr) return false;
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(w) * 8, static_cast<cuuint64_t>(h),
        static_cast<cuuint64_t>(n) * static_cast<cuuint64_t>(c / 8)};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(w) * 16, static_cast<cuuint64_t>(h) * w * 16};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(8 * box_pixels), static_cast<cuuint32_t>(box_rows), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(x), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Opts k_conv3x3 into its shared-memory size (once per process; call it
// outside stream capture).
int g_conv_regs = 0;  // registers per thread of k_conv3x3 (set by conv_init)

cudaError_t conv_init() {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
        if (attr == cudaSuccess) {
            attr = cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributePreferredSharedMemoryCarveout,
                cudaSharedmemCarveoutMaxShared);
        }
        cudaFuncAttributes fa{};
        if (attr == cudaSuccess) attr = cudaFuncGetAttributes(&fa, k_conv3x3);
        if (attr == cudaSuccess) g_conv_regs = fa.numRegs;
    });
    return attr;
}

// Launches k_conv3x3; `map` must describe x (conv_input_map).
cudaError_t launch_conv3x3(const CUtensorMap& map, int n, int h, int w, int cin, const void* weight, const float* bias,
    int cout, int relu, void* y, int y_channels, int y_offset, int* err, int grid_limit, cudaStream_t stream,
    void* pool, int up, int stages) {
    const cudaError_t attr = conv_init();
    if (attr != cudaSuccess) return attr;
    if (stages <= 0 || stages > kMaxStages || conv_smem_bytes(cin, cout, stages) > kConvSmem) stages = conv_stages(cin, cout);
    ConvArgs a{n, h, w, cin, cout, y_channels, y_offset, relu, static_cast<const uint4*>(weight), bias,
        static_cast<__nv_bfloat16*>(y), err, static_cast<__nv_bfloat16*>(pool), up, stages, conv_tmem_cols(cout)};
    const int smem = conv_smem_bytes(cin, cout, stages);
    // resident CTAs per SM: 228 KB of shared memory (1 KB reserved per CTA),
    // 512 TMEM columns (conv_tmem_cols each, so no allocation ever waits),
    // 2048 threads and 64 K registers
    int per_sm = (228 * 1024) / (smem + 1024);
    const int tmem_fit = static_cast<int>(512u / a.tmem_cols);
    const int reg_fit = 65536 / ((g_conv_regs > 0 ? g_conv_regs : 255) * kConvThreads);
    per_sm = per_sm < tmem_fit ? per_sm : tmem_fit;
    per_sm = per_sm < reg_fit ? per_sm : reg_fit;
    per_sm = per_sm < 2048 / kConvThreads ? per_sm : 2048 / kConvThreads;
    per_sm = per_sm > 1 ? per_sm : 1;
    const long long tiles = static_cast<long long>((w + kTileW - 1) / kTileW) * ((h + kTileH - 1) / kTileH) * n;
    const long long cap = static_cast<long long>(grid_limit) * per_sm;
    const int grid = static_cast<int>(tiles < cap ? tiles : cap);
    k_conv3x3<<<grid > 0 ? grid : 1, kConvThreads, smem, stream>>>(map, a);
    return cudaGetLastError();
}

bool conv_shape_ok(int cin, int cout, int y_channels, int y_offset) {
    return cin >= 16 && cin <= kMaxCin && cin % 16 == 0 && cout >= 16 && cout <= kMaxCout && cout % 16 == 0 &&
           y_offset >= 0 && y_offset % 8 == 0 && y_channels % 8 == 0 && y_offset + cout <= y_channels;
}

}  // namespace rtgb

extern "C" rtgb_status rtgb_conv3x3_pack_weights(const float* weight_oihw, int32_t c_out, int32_t c_in_used,
    int32_t c_in, uint16_t* packed) {
    if (weight_oihw == nullptr || packed == nullptr || c_in_used > c_in || c_in % 8 != 0 || c_out <= 0 ||
        c_in_used <= 0) {
        return RTGB_INVALID_ARGUMENT;
    }
    // packed[tap][c_in/8][c_out][8], tap = dy * 3 + dx; cross-correlation as conv2d
    const int boxes = c_in / 8;
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
        for (int b = 0; b < boxes; ++b) {
            for (int o = 0; o < c_out; ++o) {
                for (int j = 0; j < 8; ++j) {
                    const int ci = b * 8 + j;
                    const float v = ci < c_in_used ? weight_oihw[((static_cast<size_t>(o) * c_in_used + ci) * 3 + dy) * 3 + dx]
                                                   : 0.0f;
                    packed[((static_cast<size_t>(tap) * boxes + b) * c_out + o) * 8 + j] = rtgb::to_bf16(v);
                }
            }
        }
    }
    return RTGB_OK;
}

extern "C" rtgb_status rtgb_conv3x3_bf16(const void* x, int32_t n, int32_t h, int32_t w, int32_t c_in,
    const void* packed_weight, const float* bias, int32_t c_out, int32_t relu, void* y, int32_t y_channels,
    int32_t y_channel_offset, int32_t* device_error, void* stream, char* message, size_t message_size) {
    using namespace rtgb;
    set_message(message, message_size, "");
    if (x == nullptr || packed_weight == nullptr || bias == nullptr || y == nullptr || n <= 0 || h <= 0 || w <= 0) {
        set_message(message, message_size, "null pointer or empty extent");
        return RTGB_INVALID_ARGUMENT;
    }
    if (!conv_shape_ok(c_in, c_out, y_channels, y_channel_offset)) {
        set_message(message, message_size,
            "c_in must be a multiple of 16 in [16, 128], c_out a multiple of 16 in [16, 64], the output channel "
            "offset and count multiples of 8 with offset + c_out <= count");
        return RTGB_INVALID_ARGUMENT;
    }
    if ((reinterpret_cast<uintptr_t>(x) & 15u) != 0 || (reinterpret_cast<uintptr_t>(y) & 15u) != 0 ||
        (reinterpret_cast<uintptr_t>(packed_weight) & 15u) != 0) {
        set_message(message, message_size, "tensors must be 16-byte aligned");
        return RTGB_INVALID_ARGUMENT;
    }
    CUtensorMap map;
    if (!conv_input_map(&map, x, n, h, w, c_in)) {
        set_message(message, message_size, "cuTensorMapEncodeTiled failed");
        return RTGB_RUNTIME_ERROR;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const cudaError_t e = launch_conv3x3(map, n, h, w, c_in, packed_weight, bias, c_out, relu, y, y_channels,
        y_channel_offset, device_error, sms > 0 ? sms : 1, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        set_message(message, message_size, cudaGetErrorString(e));
        return RTGB_RUNTIME_ERROR;
    }
    return RTGB_OK;
}

// ---- the U-Net -------------------------------------------------------------------------------

#include <string>
#include <vector>


namespace rtgb {
namespace {

constexpr int kInChannels = 16;

__device__ __forceinline__ __nv_bfloat16 bf(float v) { return __float2bfloat16_rn(v); }

// Network input: log1p(radiance), albedo, camera-space normal, log1p(depth), 6
// zeros, as two channel blocks of the blocked layout (`hw` pixels per image).
__global__ void k_dn_pack(const FrameParams* __restrict__ fpp, long long offset, long long count, long long hw,
    __nv_bfloat16* __restrict__ out) {
    const FrameBufs f = fpp->cur;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long p = offset + i;
        const float4 b = f.beauty[p];
        const float4 a = f.albedo[p];
        const float4 nn = f.dnormal[p];
        const float d = f.depth[p];
        __align__(16) __nv_bfloat16 v[16];
        v[0] = bf(log1pf(fmaxf(b.x, 0.0f)));
        v[1] = bf(log1pf(fmaxf(b.y, 0.0f)));
        v[2] = bf(log1pf(fmaxf(b.z, 0.0f)));
        v[3] = bf(a.x);
        v[4] = bf(a.y);
        v[5] = bf(a.z);
        v[6] = bf(nn.x);
        v[7] = bf(nn.y);
        v[8] = bf(nn.z);
        v[9] = bf(log1pf(fmaxf(d, 0.0f)));
#pragma unroll
        for (int k = 10; k < 16; ++k) v[k] = bf(0.0f);
        const long long img = i / hw, px = i - img * hw;
        __nv_bfloat16* blk = out + (img * (kInChannels / 8) * hw + px) * 8;
        *reinterpret_cast<uint4*>(blk) = reinterpret_cast<const uint4*>(v)[0];
        *reinterpret_cast<uint4*>(blk + hw * 8) = reinterpret_cast<const uint4*>(v)[1];
    }
}

// Nearest 2x upsampling of a dense c-channel blocked tensor (h2 x w2) into
// channels [off, off + c) of a cs-channel blocked tensor of size h x w (the
// fallback for sizes that do not double exactly).
__global__ void k_dn_upsample(const __nv_bfloat16* __restrict__ in, int n, int h, int w, int c,
    __nv_bfloat16* __restrict__ out, int cs, int off) {
    const int h2 = (h + 1) >> 1, w2 = (w + 1) >> 1;
    const int groups = c >> 3;
    const long long total = static_cast<long long>(n) * groups * h * w;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(i % w);
        long long r = i / w;
        const int y = static_cast<int>(r % h);
        r /= h;
        const int g = static_cast<int>(r % groups);
        const int img = static_cast<int>(r / groups);
        const uint4 q = *reinterpret_cast<const uint4*>(
            in + ((static_cast<long long>(img) * groups + g) * h2 + (y >> 1)) * w2 * 8 + (x >> 1) * 8);
        *reinterpret_cast<uint4*>(out + ((static_cast<long long>(img) * (cs >> 3) + (off >> 3) + g) * h + y) * w * 8 + x * 8) = q;
    }
}

// Network output (channels 0..2 of a 16-channel blocked tensor, log1p
// radiance; `hw` pixels per image) to float4, into the current frame's
// denoised buffer from pixel `offset` on.
__global__ void k_dn_unpack(const FrameParams* __restrict__ fpp, const __nv_bfloat16* __restrict__ in, long long offset,
    long long count, long long hw) {
    float4* __restrict__ out = fpp->cur.denoised + offset;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long img = i / hw, px = i - img * hw;
        const uint2 q = *reinterpret_cast<const uint2*>(in + (img * 2 * hw + px) * 8);
        const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&q);
        out[i] = make_float4(expm1f(fmaxf(__bfloat162float(e[0]), 0.0f)), expm1f(fmaxf(__bfloat162float(e[1]), 0.0f)),
            expm1f(fmaxf(__bfloat162float(e[2]), 0.0f)), 1.0f);
    }
}

struct DevMem {
    void* p = nullptr;
    size_t bytes = 0;
    void* ensure(size_t b) {
        if (b <= bytes && p) return p;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (cudaMalloc(&p, b) != cudaSuccess) {
            p = nullptr;
            return nullptr;
        }
        bytes = b;
        return p;
    }
    ~DevMem() {
        if (p) cudaFree(p);
    }
};

int grid_for(long long work, int sms) {
    const long long g = (work + 255) / 256;
    const long long cap = static_cast<long long>(sms) * 8;
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

// Activations of one batch shape (n cameras of h x w) and the TMA maps of
// every layer's input. A frame with cameras of several sizes keeps one set per
// size, so launches captured in a CUDA graph keep valid addresses.
struct Acts {
    DevMem mem;
    int n = 0, h = 0, w = 0;
    __nv_bfloat16 *in16 = nullptr, *t1 = nullptr, *cat1 = nullptr, *t5 = nullptr, *t6 = nullptr, *out16 = nullptr;
    __nv_bfloat16 *p1 = nullptr, *t2 = nullptr, *cat2 = nullptr, *t4 = nullptr, *t4b = nullptr;
    __nv_bfloat16 *p2 = nullptr, *t3 = nullptr, *t3b = nullptr;
    CUtensorMap maps[kLayerCount];
    int stages[kLayerCount] = {};  // halo stages per layer chosen by unet_tune (0: the conv_stages rule)
    bool tuned = false;
    DevMem scratch_err;            // error flag of the tuning launches
};

struct UNet {
    DevMem weights[kLayerCount];
    DevMem biases[kLayerCount];
    bool ready = false;
    std::vector<Acts*> sets;
    ~UNet() {
        for (Acts* a : sets) delete a;
    }
};

long long unet_param_count() {
    long long n = 0;
    for (const LayerSpec& l : kLayers) n += static_cast<long long>(l.cout_used) * l.cin_used * 9 + l.cout_used;
    return n;
}

UNet* unet_create() { return new UNet(); }
void unet_destroy(UNet* net) { delete net; }
bool unet_ready(const UNet* net) { return net != nullptr && net->ready; }

bool unet_set_params(UNet* net, const float* params, long long count, std::string& error) {
    net->ready = false;
    if (params == nullptr) return true;
    if (count != unet_param_count()) {
        error = "denoiser parameters: expected " + std::to_string(unet_param_count()) + " values, got " +
                std::to_string(count);
        return false;
    }
    const float* p = params;
    for (int li = 0; li < kLayerCount; ++li) {
        const LayerSpec& l = kLayers[li];
        std::vector<float> w(static_cast<size_t>(l.cout) * l.cin_used * 9, 0.0f);
        std::memcpy(w.data(), p, sizeof(float) * l.cout_used * l.cin_used * 9);  // rows past cout_used stay zero
        p += static_cast<long long>(l.cout_used) * l.cin_used * 9;
        std::vector<float> b(static_cast<size_t>(l.cout), 0.0f);
        std::memcpy(b.data(), p, sizeof(float) * l.cout_used);
        p += l.cout_used;
        std::vector<uint16_t> packed(static_cast<size_t>(9) * l.cin * l.cout);
        if (rtgb_conv3x3_pack_weights(w.data(), l.cout, l.cin_used, l.cin, packed.data()) != RTGB_OK) {
            error = "denoiser parameters: packing failed";
            return false;
        }
        void* dw = net->weights[li].ensure(packed.size() * 2);
        void* db = net->biases[li].ensure(b.size() * 4);
        if (dw == nullptr || db == nullptr || cudaMemcpy(dw, packed.data(), packed.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(db, b.data(), b.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
            error = "denoiser parameters: device upload failed";
            return false;
        }
    }
    net->ready = true;
    return true;
}

namespace {

Acts* unet_buffers(UNet* unet, int n, int h, int w) {
    for (Acts* a : unet->sets) {
        if (a->n == n && a->h == h && a->w == w) return a;
    }
    Acts* net = new Acts();
    const long long full = static_cast<long long>(n) * h * w;
    const long long half = static_cast<long long>(n) * ((h + 1) / 2) * ((w + 1) / 2);
    const long long quarter = static_cast<long long>(n) * ((h + 3) / 4) * ((w + 3) / 4);
    // channels per resolution: full 16 + 32 + 80 + 32 + 32 + 16, half 32 + 48 + 112 + 48 + 48, quarter 48 + 64 + 64
    const long long elems = full * 208 + half * 288 + quarter * 176;
    char* base = static_cast<char*>(net->mem.ensure(static_cast<size_t>(elems) * 2 + 64 * 256));
    if (base == nullptr) {
        delete net;
        return nullptr;
    }
    auto take = [&](long long count, int ch) {
        char* r = base;
        base += ((count * ch * 2) + 255) & ~255ll;
        return reinterpret_cast<__nv_bfloat16*>(r);
    };
    net->in16 = take(full, 16);
    net->t1 = take(full, 32);
    net->cat1 = take(full, 80);
    net->t5 = take(full, 32);
    net->t6 = take(full, 32);
    net->out16 = take(full, 16);
    net->p1 = take(half, 32);
    net->t2 = take(half, 48);
    net->cat2 = take(half, 112);
    net->t4 = take(half, 48);
    net->t4b = take(half, 48);
    net->p2 = take(quarter, 48);
    net->t3 = take(quarter, 64);
    net->t3b = take(quarter, 64);
    const int h2 = (h + 1) / 2, w2 = (w + 1) / 2, h4 = (h2 + 1) / 2, w4 = (w2 + 1) / 2;
    const struct {
        const void* x;
        int h, w, c;
    } inputs[kLayerCount] = {{net->in16, h, w, 16}, {net->t1, h, w, 32}, {net->p1, h2, w2, 32}, {net->t2, h2, w2, 48},
        {net->p2, h4, w4, 48}, {net->t3, h4, w4, 64}, {net->cat2, h2, w2, 112}, {net->t4, h2, w2, 48},
        {net->cat1, h, w, 80}, {net->t5, h, w, 32}, {net->t6, h, w, 32}};
    for (int li = 0; li < kLayerCount; ++li) {
        if (!conv_input_map(&net->maps[li], inputs[li].x, n, inputs[li].h, inputs[li].w, inputs[li].c)) {
            delete net;
            return nullptr;
        }
    }
    net->n = n;
    net->h = h;
    net->w = w;
    unet->sets.push_back(net);
    return net;
}

}  // namespace

namespace {

// Output side of layer li in the U-Net pass over an (n, h, w) batch: its
// input size, output tensor, channel count and offset, fused pooling and
// upsampling (as unet_run issues it).
struct LayerCall {
    int hh, ww;
    void* y;
    int ych, yoff;
    void* pool;
    int up;
};

LayerCall layer_call(const Acts* a, int li, int h, int w) {
    const int h2 = (h + 1) / 2, w2 = (w + 1) / 2, h4 = (h2 + 1) / 2, w4 = (w2 + 1) / 2;
    const bool up2 = 2 * h4 == h2 && 2 * w4 == w2, up1 = 2 * h2 == h && 2 * w2 == w;
    switch (li) {
        case 0: return {h, w, a->t1, 32, 0, nullptr, 0};
        case 1: return {h, w, a->cat1, 80, 0, a->p1, 0};
        case 2: return {h2, w2, a->t2, 48, 0, nullptr, 0};
        case 3: return {h2, w2, a->cat2, 112, 0, a->p2, 0};
        case 4: return {h4, w4, a->t3, 64, 0, nullptr, 0};
        case 5: return up2 ? LayerCall{h4, w4, a->cat2, 112, 48, nullptr, 1} : LayerCall{h4, w4, a->t3b, 64, 0, nullptr, 0};
        case 6: return {h2, w2, a->t4, 48, 0, nullptr, 0};
        case 7: return up1 ? LayerCall{h2, w2, a->cat1, 80, 32, nullptr, 1} : LayerCall{h2, w2, a->t4b, 48, 0, nullptr, 0};
        case 8: return {h, w, a->t5, 32, 0, nullptr, 0};
        case 9: return {h, w, a->t6, 32, 0, nullptr, 0};
        default: return {h, w, a->out16, 16, 0, nullptr, 0};
    }
}

// Picks each layer's halo-stage count for this batch shape by timing the
// layer with every even count that fits shared memory (best of three
// launches, on the set's own buffers; the outputs are overwritten by the
// next pass). A layer where none fits keeps the rule (0).
bool unet_tune(UNet* unet, Acts* a) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int* err = static_cast<int*>(a->scratch_err.ensure(sizeof(int)));
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (err == nullptr || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return false;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    bool ok = true;
    for (int li = 0; li < kLayerCount && ok; ++li) {
        const LayerSpec& l = kLayers[li];
        const LayerCall c = layer_call(a, li, a->h, a->w);
        float best = 1e30f;
        int best_s = 0;
        for (int s = 2; s <= kMaxStages; s += 2) {  // even counts: two issuers per CTA
            if (conv_smem_bytes(l.cin, l.cout, s) > kConvSmem) continue;
            float t_min = 1e30f;
            for (int rep = 0; rep < 3 && ok; ++rep) {
                cudaEventRecord(e0, st);
                ok = launch_conv3x3(a->maps[li], a->n, c.hh, c.ww, l.cin, unet->weights[li].p,
                         static_cast<const float*>(unet->biases[li].p), l.cout, l.relu, c.y, c.ych, c.yoff, err, sms, st,
                         c.pool, c.up, s) == cudaSuccess;
                cudaEventRecord(e1, st);
                ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                t_min = ms < t_min ? ms : t_min;
            }
            if (t_min < best) {
                best = t_min;
                best_s = s;
            }
        }
        a->stages[li] = best_s;
    }
    int h_err = 0;
    ok = ok && cudaMemcpy(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && h_err == 0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (!ok) {
        for (int& s : a->stages) s = 0;  // fall back to the rule
    }
    return ok;
}

}  // namespace

bool unet_prepare(UNet* unet, int n, int h, int w) {
    if (conv_init() != cudaSuccess) return false;
    Acts* a = unet_buffers(unet, n, h, w);
    if (a == nullptr) return false;
    if (unet->ready && !a->tuned) {
        unet_tune(unet, a);
        a->tuned = true;
    }
    return true;
}

cudaError_t unet_run(UNet* unet, const FrameParams* fp, long long pixel_offset, int n, int h, int w, int* err, int sms,
    cudaStream_t stream) {
    if (!unet->ready) return cudaErrorInvalidValue;
    Acts* net = unet_buffers(unet, n, h, w);
    if (net == nullptr) return cudaErrorMemoryAllocation;
    const long long full = static_cast<long long>(n) * h * w;
    const int h2 = (h + 1) / 2, w2 = (w + 1) / 2, h4 = (h2 + 1) / 2, w4 = (w2 + 1) / 2;
    auto conv = [&](int li, int hh, int ww, void* y, int ych, int yoff, void* pool = nullptr, int up = 0) {
        const LayerSpec& l = kLayers[li];
        return launch_conv3x3(net->maps[li], n, hh, ww, l.cin, unet->weights[li].p, static_cast<const float*>(unet->biases[li].p),
            l.cout, l.relu, y, ych, yoff, err, sms, stream, pool, up, net->stages[li]);
    };
    cudaError_t e;
    const long long hw = static_cast<long long>(h) * w;
    k_dn_pack<<<grid_for(full, sms), 256, 0, stream>>>(fp, pixel_offset, full, hw, net->in16);
    if ((e = conv(0, h, w, net->t1, 32, 0)) != cudaSuccess) return e;
    // the encoder's second convolutions also write the pooled tensor; the
    // decoder inputs' upsampled halves are written by the layer below them
    if ((e = conv(1, h, w, net->cat1, 80, 0, net->p1)) != cudaSuccess) return e;
    if ((e = conv(2, h2, w2, net->t2, 48, 0)) != cudaSuccess) return e;
    if ((e = conv(3, h2, w2, net->cat2, 112, 0, net->p2)) != cudaSuccess) return e;
    if ((e = conv(4, h4, w4, net->t3, 64, 0)) != cudaSuccess) return e;
    if (2 * h4 == h2 && 2 * w4 == w2) {
        if ((e = conv(5, h4, w4, net->cat2, 112, 48, nullptr, 1)) != cudaSuccess) return e;
    } else {
        if ((e = conv(5, h4, w4, net->t3b, 64, 0)) != cudaSuccess) return e;
        k_dn_upsample<<<grid_for(static_cast<long long>(n) * h2 * w2 * 8, sms), 256, 0, stream>>>(net->t3b, n, h2, w2, 64, net->cat2, 112, 48);
    }
    if ((e = conv(6, h2, w2, net->t4, 48, 0)) != cudaSuccess) return e;
    if (2 * h2 == h && 2 * w2 == w) {
        if ((e = conv(7, h2, w2, net->cat1, 80, 32, nullptr, 1)) != cudaSuccess) return e;
    } else {
        if ((e = conv(7, h2, w2, net->t4b, 48, 0)) != cudaSuccess) return e;
        k_dn_upsample<<<grid_for(full * 6, sms), 256, 0, stream>>>(net->t4b, n, h, w, 48, net->cat1, 80, 32);
    }
    if ((e = conv(8, h, w, net->t5, 32, 0)) != cudaSuccess) return e;
    if ((e = conv(9, h, w, net->t6, 32, 0)) != cudaSuccess) return e;
    if ((e = conv(10, h, w, net->out16, 16, 0)) != cudaSuccess) return e;
    k_dn_unpack<<<grid_for(full, sms), 256, 0, stream>>>(fp, net->out16, pixel_offset, full, hw);
    return cudaGetLastError();
}

}  // namespace rtgb
