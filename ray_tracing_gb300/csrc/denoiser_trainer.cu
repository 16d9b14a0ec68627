// Native training of the denoiser U-Net: forward, log-space L1 loss,
// backward and Adam, all on this library's kernels (no framework):
//   * forward: k_conv3x3 per layer with the fused pooling / upsampling, every
//     activation kept (BF16, channel-blocked);
//   * input gradients: k_conv3x3 itself with flipped, transposed weights
//     (dX = conv(dZ, W^T flipped)), split into launches of <= 64 output
//     channels;
//   * weight and bias gradients: k_conv3x3_wgrad (denoiser_train.cu);
//   * ReLU masks, the backward of 2 x 2 average pooling and of nearest
//     upsampling, the loss gradient, weight packing and Adam: elementwise
//     kernels below.
// Gradients flow in BF16 between layers and accumulate in FP32 inside each
// GEMM; the master parameters and Adam moments are FP32. Batches are n crops
// of h x w with h and w multiples of 4 (the pooled sizes then halve exactly).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "denoiser.cuh"
#include "rtgb.h"

#include <initializer_list>

namespace rtgb {
namespace {

__device__ __forceinline__ float bf2f(__nv_bfloat16 v) { return __bfloat162float(v); }

// Offset of channel c of pixel (img, y, x) in a blocked tensor of `cs` channels.
__device__ __forceinline__ long long blk(int img, int c, int cs, int h, int w, int y, int x) {
    return ((((static_cast<long long>(img) * (cs >> 3) + (c >> 3)) * h + y) * w + x) << 3) + (c & 7);
}

// Loss gradient of mean |out - target| over n x h x w x 3 (log1p radiance):
// sign / count into channels 0..2 of a 16-channel gradient, 0 elsewhere; the
// loss sum goes to *loss.
__global__ void k_loss_grad(const __nv_bfloat16* __restrict__ out16, const float* __restrict__ target, int n, int h,
    int w, __nv_bfloat16* __restrict__ g16, double* loss) {
    const long long px = static_cast<long long>(n) * h * w;
    const float inv = 1.0f / static_cast<float>(px * 3);
    double local = 0.0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < px;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(i % w);
        const int y = static_cast<int>((i / w) % h);
        const int img = static_cast<int>(i / (static_cast<long long>(w) * h));
        for (int c = 0; c < 16; ++c) {
            float g = 0.0f;
            if (c < 3) {
                const float d = bf2f(out16[blk(img, c, 16, h, w, y, x)]) - target[i * 3 + c];
                local += fabsf(d);
                g = d > 0.0f ? inv : (d < 0.0f ? -inv : 0.0f);
            }
            g16[blk(img, c, 16, h, w, y, x)] = __float2bfloat16_rn(g);
        }
    }
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, local);
}

// out[c] = g[c] * (y[c] > 0) for c < channels; g, y and out are channel ranges
// (offset, channel count of the whole tensor) of blocked tensors of n x h x w.
__global__ void k_relu_mask(const __nv_bfloat16* __restrict__ g, int g_cs, int g_off, const __nv_bfloat16* __restrict__ y,
    int y_cs, int y_off, __nv_bfloat16* __restrict__ out, int o_cs, int o_off, int channels, int n, int h, int w) {
    const long long total = static_cast<long long>(n) * h * w * channels;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int c = static_cast<int>(i % channels);
        long long r = i / channels;
        const int x = static_cast<int>(r % w);
        r /= w;
        const int yy = static_cast<int>(r % h);
        const int img = static_cast<int>(r / h);
        const float gv = bf2f(g[blk(img, g_off + c, g_cs, h, w, yy, x)]);
        const float yv = bf2f(y[blk(img, y_off + c, y_cs, h, w, yy, x)]);
        out[blk(img, o_off + c, o_cs, h, w, yy, x)] = __float2bfloat16_rn(yv > 0.0f ? gv : 0.0f);
    }
}

// Backward passes on whole 8-channel blocks (every channel count and offset of
// the U-Net is a multiple of 8): a thread moves one pixel's 8 channels as one
// 16-byte load per operand, and the index arithmetic is 32-bit on (image,
// channel block, pixel). k_relu_mask8 computes each element as k_relu_mask.
__device__ __forceinline__ void unpack8(const uint4& q, float f[8]) {
    const __nv_bfloat16* v = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
    for (int k = 0; k < 8; ++k) f[k] = bf2f(v[k]);
}
__device__ __forceinline__ uint4 pack8(const float f[8]) {
    uint4 q;
    __nv_bfloat16* v = reinterpret_cast<__nv_bfloat16*>(&q);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __float2bfloat16_rn(f[k]);
    return q;
}
// 16-byte unit of channel block `cb` (of `cbs`) at pixel p of image img, hw pixels
__device__ __forceinline__ long long unit(int img, int cbs, int cb, int hw, int p) {
    return (static_cast<long long>(img) * cbs + cb) * hw + p;
}

__global__ void k_relu_mask8(const uint4* __restrict__ g, int g_cbs, int g_cb0, const uint4* __restrict__ y, int y_cbs,
    int y_cb0, uint4* __restrict__ out, int o_cbs, int o_cb0, int blocks, int n, int hw) {
    const long long total = static_cast<long long>(n) * blocks * hw;
    for (long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; j < total;
         j += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int p = static_cast<int>(j % hw);
        const int t = static_cast<int>(j / hw);
        const int cb = t % blocks, img = t / blocks;
        float gv[8], yv[8], o[8];
        unpack8(g[unit(img, g_cbs, g_cb0 + cb, hw, p)], gv);
        unpack8(y[unit(img, y_cbs, y_cb0 + cb, hw, p)], yv);
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = yv[k] > 0.0f ? gv[k] : 0.0f;
        out[unit(img, o_cbs, o_cb0 + cb, hw, p)] = pack8(o);
    }
}

// Backward of nearest 2x upsampling followed by the ReLU of the layer that
// produced it: out (h x w, dense channel blocks) = (sum of the 2 x 2 gradient
// block of g) * (y > 0), y being the upsampled output itself (any pixel of
// its 2 x 2 block holds the value).
__global__ void k_up_backward_mask8(const uint4* __restrict__ g, int g_cbs, int g_cb0, const uint4* __restrict__ y,
    int y_cbs, int y_cb0, uint4* __restrict__ out, int blocks, int n, int h, int w) {
    const int hw = h * w, w2 = 2 * w, hw2 = 4 * hw;
    const long long total = static_cast<long long>(n) * blocks * hw;
    for (long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; j < total;
         j += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int p = static_cast<int>(j % hw);
        const int t = static_cast<int>(j / hw);
        const int cb = t % blocks, img = t / blocks;
        const int yy = p / w, x = p - yy * w;
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; ++dy) {
            for (int dx = 0; dx < 2; ++dx) {
                float v[8];
                unpack8(g[unit(img, g_cbs, g_cb0 + cb, hw2, (2 * yy + dy) * w2 + 2 * x + dx)], v);
#pragma unroll
                for (int k = 0; k < 8; ++k) s[k] += v[k];
            }
        }
        float yv[8], o[8];
        unpack8(y[unit(img, y_cbs, y_cb0 + cb, hw2, 2 * yy * w2 + 2 * x)], yv);
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = yv[k] > 0.0f ? s[k] : 0.0f;
        out[unit(img, blocks, cb, hw, p)] = pack8(o);
    }
}

// Gradient of a layer whose output feeds both a skip connection (gradient g)
// and a 2 x 2 average pooling (gradient gp at half size): out = (g + gp / 4) *
// (y > 0) into a dense tensor (h, w even).
__global__ void k_pool_backward_mask8(const uint4* __restrict__ g, int g_cbs, int g_cb0, const uint4* __restrict__ gp,
    const uint4* __restrict__ y, int y_cbs, int y_cb0, uint4* __restrict__ out, int blocks, int n, int h, int w) {
    const int hw = h * w, wh = w / 2, hwh = (h / 2) * wh;
    const long long total = static_cast<long long>(n) * blocks * hw;
    for (long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; j < total;
         j += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int p = static_cast<int>(j % hw);
        const int t = static_cast<int>(j / hw);
        const int cb = t % blocks, img = t / blocks;
        const int yy = p / w, x = p - yy * w;
        float gv[8], pv[8], yv[8], o[8];
        unpack8(g[unit(img, g_cbs, g_cb0 + cb, hw, p)], gv);
        unpack8(gp[unit(img, blocks, cb, hwh, (yy / 2) * wh + x / 2)], pv);
        unpack8(y[unit(img, y_cbs, y_cb0 + cb, hw, p)], yv);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float sv = gv[k] + 0.25f * pv[k];
            o[k] = yv[k] > 0.0f ? sv : 0.0f;
        }
        out[unit(img, blocks, cb, hw, p)] = pack8(o);
    }
}

// Packs FP32 weights (cout_used x cin_used x 3 x 3 at `wsrc`) as
// rtgb_conv3x3_pack_weights does, [tap][cin/8][cout][8] BF16 with zero
// padding; with `transposed` the packed kernel is the input-gradient one,
// W'[i][o][2 - dy][2 - dx], for output channels [o0, o0 + cout) of it
// (i.e. layer input channels) and input channels = the layer's cout.
__global__ void k_pack_weights(const float* __restrict__ wsrc, int cout_used, int cin_used, int transposed, int o0,
    int cout, int cin, __nv_bfloat16* __restrict__ packed) {
    const int total = 9 * cin * cout;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int j = e & 7;
        const int o = (e >> 3) % cout;
        const int b = (e >> 3) / cout % (cin >> 3);
        const int tap = (e >> 3) / cout / (cin >> 3);
        const int i = b * 8 + j;
        float v = 0.0f;
        if (!transposed) {
            if (o < cout_used && i < cin_used) v = wsrc[(static_cast<long long>(o) * cin_used + i) * 9 + tap];
        } else {
            // packed output channel o = layer input channel o0 + o, packed input i = layer output channel
            const int li = o0 + o, lo = i;
            if (li < cin_used && lo < cout_used) v = wsrc[(static_cast<long long>(lo) * cin_used + li) * 9 + (8 - tap)];
        }
        packed[e] = __float2bfloat16_rn(v);
    }
}

// The used block of a layer's padded weight gradient (cout x cin x 9) and its
// bias gradient into the flat parameter-gradient vector.
__global__ void k_gather_grad(const float* __restrict__ dw, const float* __restrict__ db, int cout_used, int cin_used,
    int cin, float* __restrict__ flat) {
    const int nw = cout_used * cin_used * 9;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nw + cout_used; e += gridDim.x * blockDim.x) {
        if (e < nw) {
            const int tap = e % 9, i = (e / 9) % cin_used, o = e / (9 * cin_used);
            flat[e] = dw[(static_cast<long long>(o) * cin + i) * 9 + tap];
        } else {
            flat[e] = db[e - nw];
        }
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters, bias-corrected.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
    long long count, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

int grid_of(long long work) {
    long long g = (work + 255) / 256;
    return static_cast<int>(g < 1 ? 1 : (g < 4096 ? g : 4096));
}

}  // namespace

struct Trainer {
    int n = 0, h = 0, w = 0, sms = 1;
    long long count = 0;                 // parameters
    cudaStream_t stream = nullptr;
    std::vector<void*> allocations;
    // FP32 master parameters (flat, layer order: weight out x in x 3 x 3, then bias), gradients, Adam moments
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    long long offset[kLayerCount] = {};  // of each layer's weight in the flat vector
    // packed BF16 weights: forward per layer, input-gradient per layer and 64-channel chunk
    __nv_bfloat16* wf[kLayerCount] = {};
    __nv_bfloat16* wb[kLayerCount][2] = {};
    float* bias[kLayerCount] = {};       // FP32 bias (forward), padded to cout
    float* zero_bias = nullptr;          // 128 zeros for the input-gradient convolutions
    float *dw = nullptr, *db = nullptr, *partial = nullptr;
    size_t partial_bytes = 0;
    // activations (channel-blocked BF16)
    __nv_bfloat16 *t1, *cat1, *p1, *t2, *cat2, *p2, *t3, *t4, *t5, *t6, *out16;
    // gradients
    __nv_bfloat16 *g_out16, *g_t6, *g_t5, *g_cat1, *g_u7, *g_t4, *g_cat2, *g_u5, *g_t3, *g_p2, *g3, *g_t2, *g_p1, *g1,
        *g_t1;
    double* loss = nullptr;
    int* err = nullptr;
    int steps = 0;
    std::string error;

    template <typename T>
    T* alloc(size_t count_elems) {
        void* p = nullptr;
        if (cudaMalloc(&p, count_elems * sizeof(T)) != cudaSuccess) throw std::string("out of device memory");
        allocations.push_back(p);
        cudaMemset(p, 0, count_elems * sizeof(T));
        return static_cast<T*>(p);
    }

    ~Trainer() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : allocations) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    void init(int n_, int h_, int w_, const float* host_params, long long count_) {
        n = n_;
        h = h_;
        w = w_;
        if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) throw std::string("stream");
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long off = 0;
        for (int l = 0; l < kLayerCount; ++l) {
            offset[l] = off;
            off += static_cast<long long>(kLayers[l].cout_used) * kLayers[l].cin_used * 9 + kLayers[l].cout_used;
        }
        if (count_ != off) throw std::string("parameter count mismatch");
        count = off;
        params = alloc<float>(count);
        grads = alloc<float>(count);
        m = alloc<float>(count);
        v = alloc<float>(count);
        cudaMemcpy(params, host_params, count * sizeof(float), cudaMemcpyHostToDevice);
        for (int l = 0; l < kLayerCount; ++l) {
            const LayerSpec& L = kLayers[l];
            wf[l] = alloc<__nv_bfloat16>(9 * static_cast<size_t>(L.cin) * L.cout);
            for (int k = 0; k < 2; ++k) wb[l][k] = alloc<__nv_bfloat16>(9 * static_cast<size_t>(L.cout) * 64);
            bias[l] = alloc<float>(L.cout);
        }
        zero_bias = alloc<float>(128);
        dw = alloc<float>(64 * 128 * 9);
        db = alloc<float>(64);
        partial_bytes = wgrad_partial_bytes(sms, 64);
        partial = alloc<float>(partial_bytes / sizeof(float));
        const size_t full = static_cast<size_t>(n) * h * w, half = full / 4, quarter = full / 16;
        t1 = alloc<__nv_bfloat16>(full * 32);
        cat1 = alloc<__nv_bfloat16>(full * 80);
        p1 = alloc<__nv_bfloat16>(half * 32);
        t2 = alloc<__nv_bfloat16>(half * 48);
        cat2 = alloc<__nv_bfloat16>(half * 112);
        p2 = alloc<__nv_bfloat16>(quarter * 48);
        t3 = alloc<__nv_bfloat16>(quarter * 64);
        t4 = alloc<__nv_bfloat16>(half * 48);
        t5 = alloc<__nv_bfloat16>(full * 32);
        t6 = alloc<__nv_bfloat16>(full * 32);
        out16 = alloc<__nv_bfloat16>(full * 16);
        g_out16 = alloc<__nv_bfloat16>(full * 16);
        g_t6 = alloc<__nv_bfloat16>(full * 32);
        g_t5 = alloc<__nv_bfloat16>(full * 32);
        g_cat1 = alloc<__nv_bfloat16>(full * 80);
        g_u7 = alloc<__nv_bfloat16>(half * 48);
        g_t4 = alloc<__nv_bfloat16>(half * 48);
        g_cat2 = alloc<__nv_bfloat16>(half * 112);
        g_u5 = alloc<__nv_bfloat16>(quarter * 64);
        g_t3 = alloc<__nv_bfloat16>(quarter * 64);
        g_p2 = alloc<__nv_bfloat16>(quarter * 48);
        g3 = alloc<__nv_bfloat16>(half * 48);
        g_t2 = alloc<__nv_bfloat16>(half * 48);
        g_p1 = alloc<__nv_bfloat16>(half * 32);
        g1 = alloc<__nv_bfloat16>(full * 32);
        g_t1 = alloc<__nv_bfloat16>(full * 32);
        loss = alloc<double>(1);
        err = alloc<int>(1);
        if (conv_init() != cudaSuccess) throw std::string("conv_init");
        cudaDeviceSynchronize();
    }

    void check(cudaError_t e, const char* what) {
        if (e != cudaSuccess) throw std::string(what) + ": " + cudaGetErrorString(e);
    }

    // packs every layer's forward and input-gradient weights and copies the biases
    void pack() {
        for (int l = 0; l < kLayerCount; ++l) {
            const LayerSpec& L = kLayers[l];
            const float* W = params + offset[l];
            k_pack_weights<<<grid_of(9LL * L.cin * L.cout), 256, 0, stream>>>(W, L.cout_used, L.cin_used, 0, 0, L.cout,
                L.cin, wf[l]);
            for (int k = 0; k * 64 < L.cin; ++k) {
                const int oc = L.cin - 64 * k < 64 ? L.cin - 64 * k : 64;
                k_pack_weights<<<grid_of(9LL * L.cout * oc), 256, 0, stream>>>(W, L.cout_used, L.cin_used, 1, 64 * k, oc,
                    L.cout, wb[l][k]);
            }
            check(cudaMemsetAsync(bias[l], 0, L.cout * sizeof(float), stream), "bias");
            check(cudaMemcpyAsync(bias[l], W + static_cast<long long>(L.cout_used) * L.cin_used * 9,
                      L.cout_used * sizeof(float), cudaMemcpyDeviceToDevice, stream), "bias");
        }
        check(cudaGetLastError(), "pack");
    }

    // one convolution: input x (cin channels) at hh x ww
    void conv(int l, const void* x, int cin, int hh, int ww, const void* wts, const float* b, int cout, int relu, void* y,
        int ych, int yoff, void* pool = nullptr, int up = 0) {
        CUtensorMap map;
        if (!conv_input_map(&map, x, n, hh, ww, cin)) throw std::string("tensor map");
        check(launch_conv3x3(map, n, hh, ww, cin, wts, b, cout, relu, y, ych, yoff, err, sms, stream, pool, up), "conv");
        (void)l;
    }

    void forward(const void* in16) {
        const int h2 = h / 2, w2 = w / 2, h4 = h / 4, w4 = w / 4;
        conv(0, in16, 16, h, w, wf[0], bias[0], 32, 1, t1, 32, 0);
        conv(1, t1, 32, h, w, wf[1], bias[1], 32, 1, cat1, 80, 0, p1);
        conv(2, p1, 32, h2, w2, wf[2], bias[2], 48, 1, t2, 48, 0);
        conv(3, t2, 48, h2, w2, wf[3], bias[3], 48, 1, cat2, 112, 0, p2);
        conv(4, p2, 48, h4, w4, wf[4], bias[4], 64, 1, t3, 64, 0);
        conv(5, t3, 64, h4, w4, wf[5], bias[5], 64, 1, cat2, 112, 48, nullptr, 1);
        conv(6, cat2, 112, h2, w2, wf[6], bias[6], 48, 1, t4, 48, 0);
        conv(7, t4, 48, h2, w2, wf[7], bias[7], 48, 1, cat1, 80, 32, nullptr, 1);
        conv(8, cat1, 80, h, w, wf[8], bias[8], 32, 1, t5, 32, 0);
        conv(9, t5, 32, h, w, wf[9], bias[9], 32, 1, t6, 32, 0);
        conv(10, t6, 32, h, w, wf[10], bias[10], 16, 0, out16, 16, 0);
    }

    // weight/bias gradients of layer l (x: its input, dz: its masked output gradient) into the flat vector
    void wgrad(int l, const void* x, int hh, int ww, const void* dz) {
        const LayerSpec& L = kLayers[l];
        check(launch_conv3x3_wgrad(x, n, hh, ww, L.cin, dz, L.cout, dw, db, err, sms, stream, partial, partial_bytes),
            "wgrad");
        k_gather_grad<<<grid_of(static_cast<long long>(L.cout_used) * L.cin_used * 9 + L.cout_used), 256, 0, stream>>>(
            dw, db, L.cout_used, L.cin_used, L.cin, grads + offset[l]);
        check(cudaGetLastError(), "gather");
    }

    // input gradient of layer l: dX (cin channels, written at channel xoff of an xcs tensor) from dz (cout channels)
    void dgrad(int l, const void* dz, int hh, int ww, void* dx, int xcs, int xoff) {
        const LayerSpec& L = kLayers[l];
        for (int k = 0; k * 64 < L.cin; ++k) {
            const int oc = L.cin - 64 * k < 64 ? L.cin - 64 * k : 64;
            conv(l, dz, L.cout, hh, ww, wb[l][k], zero_bias, oc, 0, dx, xcs, xoff + 64 * k);
        }
    }

    static bool by8(std::initializer_list<int> v) {
        for (int x : v) {
            if (x % 8 != 0) return false;
        }
        return true;
    }

    void mask(const void* g, int gcs, int goff, const void* y, int ycs, int yoff, void* out, int ocs, int ooff, int ch,
        int hh, int ww) {
        if (by8({gcs, goff, ycs, yoff, ocs, ooff, ch})) {
            k_relu_mask8<<<grid_of(static_cast<long long>(n) * hh * ww * (ch / 8)), 256, 0, stream>>>(
                static_cast<const uint4*>(g), gcs / 8, goff / 8, static_cast<const uint4*>(y), ycs / 8, yoff / 8,
                static_cast<uint4*>(out), ocs / 8, ooff / 8, ch / 8, n, hh * ww);
            check(cudaGetLastError(), "mask");
            return;
        }
        k_relu_mask<<<grid_of(static_cast<long long>(n) * hh * ww * ch), 256, 0, stream>>>(
            static_cast<const __nv_bfloat16*>(g), gcs, goff, static_cast<const __nv_bfloat16*>(y), ycs, yoff,
            static_cast<__nv_bfloat16*>(out), ocs, ooff, ch, n, hh, ww);
        check(cudaGetLastError(), "mask");
    }

    void backward(const void* in16) {
        const int h2 = h / 2, w2 = w / 2, h4 = h / 4, w4 = w / 4;
        const long long full = static_cast<long long>(n) * h * w, half = full / 4, quarter = full / 16;
        // head (no ReLU): dZ = loss gradient
        wgrad(10, t6, h, w, g_out16);
        dgrad(10, g_out16, h, w, g_t6, 32, 0);
        // d1b, d1a
        mask(g_t6, 32, 0, t6, 32, 0, g_t6, 32, 0, 32, h, w);
        wgrad(9, t5, h, w, g_t6);
        dgrad(9, g_t6, h, w, g_t5, 32, 0);
        mask(g_t5, 32, 0, t5, 32, 0, g_t5, 32, 0, 32, h, w);
        wgrad(8, cat1, h, w, g_t5);
        dgrad(8, g_t5, h, w, g_cat1, 80, 0);
        // d2b: its output was upsampled into cat1[32:80]
        k_up_backward_mask8<<<grid_of(half * 6), 256, 0, stream>>>(reinterpret_cast<const uint4*>(g_cat1), 10, 4,
            reinterpret_cast<const uint4*>(cat1), 10, 4, reinterpret_cast<uint4*>(g_u7), 6, n, h2, w2);
        check(cudaGetLastError(), "up backward");
        wgrad(7, t4, h2, w2, g_u7);
        dgrad(7, g_u7, h2, w2, g_t4, 48, 0);
        // d2a
        mask(g_t4, 48, 0, t4, 48, 0, g_t4, 48, 0, 48, h2, w2);
        wgrad(6, cat2, h2, w2, g_t4);
        dgrad(6, g_t4, h2, w2, g_cat2, 112, 0);
        // e3b: its output was upsampled into cat2[48:112]
        k_up_backward_mask8<<<grid_of(quarter * 8), 256, 0, stream>>>(reinterpret_cast<const uint4*>(g_cat2), 14, 6,
            reinterpret_cast<const uint4*>(cat2), 14, 6, reinterpret_cast<uint4*>(g_u5), 8, n, h4, w4);
        check(cudaGetLastError(), "up backward");
        wgrad(5, t3, h4, w4, g_u5);
        dgrad(5, g_u5, h4, w4, g_t3, 64, 0);
        // e3a
        mask(g_t3, 64, 0, t3, 64, 0, g_t3, 64, 0, 64, h4, w4);
        wgrad(4, p2, h4, w4, g_t3);
        dgrad(4, g_t3, h4, w4, g_p2, 48, 0);
        // e2b: output in cat2[0:48] (skip) and pooled into p2
        k_pool_backward_mask8<<<grid_of(half * 6), 256, 0, stream>>>(reinterpret_cast<const uint4*>(g_cat2), 14, 0,
            reinterpret_cast<const uint4*>(g_p2), reinterpret_cast<const uint4*>(cat2), 14, 0, reinterpret_cast<uint4*>(g3), 6, n, h2,
            w2);
        check(cudaGetLastError(), "pool backward");
        wgrad(3, t2, h2, w2, g3);
        dgrad(3, g3, h2, w2, g_t2, 48, 0);
        // e2a
        mask(g_t2, 48, 0, t2, 48, 0, g_t2, 48, 0, 48, h2, w2);
        wgrad(2, p1, h2, w2, g_t2);
        dgrad(2, g_t2, h2, w2, g_p1, 32, 0);
        // e1b: output in cat1[0:32] (skip) and pooled into p1
        k_pool_backward_mask8<<<grid_of(full * 4), 256, 0, stream>>>(reinterpret_cast<const uint4*>(g_cat1), 10, 0,
            reinterpret_cast<const uint4*>(g_p1), reinterpret_cast<const uint4*>(cat1), 10, 0, reinterpret_cast<uint4*>(g1), 4, n, h,
            w);
        check(cudaGetLastError(), "pool backward");
        wgrad(1, t1, h, w, g1);
        dgrad(1, g1, h, w, g_t1, 32, 0);
        // e1a (its input needs no gradient)
        mask(g_t1, 32, 0, t1, 32, 0, g_t1, 32, 0, 32, h, w);
        wgrad(0, in16, h, w, g_t1);
    }

    // forward, loss, backward; then Adam when lr > 0. Returns the mean loss.
    float step(const void* in16, const float* target, float lr) {
        check(cudaMemsetAsync(err, 0, sizeof(int), stream), "err");
        check(cudaMemsetAsync(loss, 0, sizeof(double), stream), "loss");
        pack();
        forward(in16);
        const long long full = static_cast<long long>(n) * h * w;
        k_loss_grad<<<grid_of(full), 256, 0, stream>>>(out16, target, n, h, w, g_out16, loss);
        check(cudaGetLastError(), "loss");
        backward(in16);
        if (lr > 0.0f) {
            ++steps;
            const float c1 = 1.0f - std::pow(0.9f, static_cast<float>(steps));
            const float c2 = 1.0f - std::pow(0.999f, static_cast<float>(steps));
            k_adam<<<grid_of(count), 256, 0, stream>>>(params, grads, m, v, count, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
            check(cudaGetLastError(), "adam");
        }
        double h_loss = 0.0;
        int h_err = 0;
        check(cudaMemcpyAsync(&h_loss, loss, sizeof(double), cudaMemcpyDeviceToHost, stream), "loss");
        check(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, stream), "err");
        check(cudaStreamSynchronize(stream), "step");
        if (h_err != 0) throw std::string("a bounded wait inside a training kernel ran out (code ") + std::to_string(h_err) + ")";
        return static_cast<float>(h_loss / static_cast<double>(full * 3));
    }
};

}  // namespace rtgb

struct rtgb_trainer_s {
    rtgb::Trainer t;
};

extern "C" {

rtgb_status rtgb_trainer_create(int32_t n, int32_t h, int32_t w, const float* params, int64_t count, rtgb_trainer* out) {
    if (out == nullptr || params == nullptr || n <= 0 || h <= 0 || w <= 0 || h % 4 != 0 || w % 4 != 0) {
        return RTGB_INVALID_ARGUMENT;
    }
    *out = nullptr;
    auto* tr = new rtgb_trainer_s();
    try {
        tr->t.init(n, h, w, params, count);
    } catch (const std::string&) {
        delete tr;
        return RTGB_RUNTIME_ERROR;
    }
    *out = tr;
    return RTGB_OK;
}

void rtgb_trainer_destroy(rtgb_trainer t) { delete t; }

rtgb_status rtgb_trainer_step(rtgb_trainer t, const void* input, const float* target, float learning_rate, float* loss) {
    if (t == nullptr || input == nullptr || target == nullptr || !(learning_rate >= 0.0f)) return RTGB_INVALID_ARGUMENT;
    try {
        const float l = t->t.step(input, target, learning_rate);
        if (loss != nullptr) *loss = l;
    } catch (const std::string& e) {
        t->t.error = e;
        return RTGB_RUNTIME_ERROR;
    }
    return RTGB_OK;
}

rtgb_status rtgb_trainer_gradients(rtgb_trainer t, float* grads) {
    if (t == nullptr || grads == nullptr) return RTGB_INVALID_ARGUMENT;
    return cudaMemcpy(grads, t->t.grads, t->t.count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
               ? RTGB_OK
               : RTGB_RUNTIME_ERROR;
}

rtgb_status rtgb_trainer_params(rtgb_trainer t, float* params) {
    if (t == nullptr || params == nullptr) return RTGB_INVALID_ARGUMENT;
    return cudaMemcpy(params, t->t.params, t->t.count * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
               ? RTGB_OK
               : RTGB_RUNTIME_ERROR;
}

const char* rtgb_trainer_last_error(rtgb_trainer t) { return t != nullptr ? t->t.error.c_str() : ""; }

}  // extern "C"
