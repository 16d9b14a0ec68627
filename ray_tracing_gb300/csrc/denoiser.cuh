// The learned denoiser that replaces the OptiX AOV denoiser of the reference
// (src/realtime/gpu/denoiser.cpp:111-185): a small BF16 U-Net over the frame's
// radiance, albedo, camera-space normal and depth, run on the tensor cores by
// k_conv3x3 (denoiser.cu).
//
// Network (3x3 convolutions, ReLU except the last, 2x2 average pooling,
// nearest upsampling, skip connections by channel concatenation):
//   full res   in(10) -> 32 -> 32 ------------------------------ cat(32 + 48) -> 32 -> 32 -> 3
//   1/2 res              pool -> 48 -> 48 -------- cat(48 + 64) -> 48 -> 48 -> up
//   1/4 res                      pool -> 64 -> 64 -> up
// Inputs per pixel: log1p(radiance) (3), albedo (3), camera-space normal (3),
// log1p(depth) (1); output log1p(radiance), expm1 back to linear.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "wavefront.cuh"

#include <cuda.h>

namespace rtgb {

// TMA map of a channel-blocked BF16 tensor ([n][c/8][h][w][8]) whose box is
// `box_pixels` pixels x 8 channels by `box_rows` rows of one channel block
// (the innermost dimension is an image row of a block; pixels outside the
// image read as zero).
bool blocked_tensor_map(CUtensorMap* map, const void* x, int n, int h, int w, int c, int box_pixels, int box_rows);

// Layers of the U-Net in order (e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b head):
// input channels used / padded to a multiple of 16, output channels used /
// padded, ReLU.
struct LayerSpec {
    int cin_used, cin, cout_used, cout, relu;
};
inline constexpr LayerSpec kLayers[] = {
    {10, 16, 32, 32, 1}, {32, 32, 32, 32, 1}, {32, 32, 48, 48, 1}, {48, 48, 48, 48, 1}, {48, 48, 64, 64, 1},
    {64, 64, 64, 64, 1}, {112, 112, 48, 48, 1}, {48, 48, 48, 48, 1}, {80, 80, 32, 32, 1}, {32, 32, 32, 32, 1},
    {32, 32, 3, 16, 0},
};
inline constexpr int kLayerCount = sizeof(kLayers) / sizeof(kLayers[0]);

// TMA map of a k_conv3x3 input (halo boxes of 10 x 18 pixels).
bool conv_input_map(CUtensorMap* map, const void* x, int n, int h, int w, int c);
// Opts k_conv3x3 into its shared memory (once; call outside stream capture).
cudaError_t conv_init();
// k_conv3x3 over an (n, h, w) batch of the blocked tensor `map` describes:
// weights packed as rtgb_conv3x3_pack_weights, output written at channel
// y_offset of a y_channels tensor (twice the size when `up`), and the 2 x 2
// average of the output into `pool` when it is non-null.
// `stages`: halo stages in shared memory, 0 for the built-in rule.
cudaError_t launch_conv3x3(const CUtensorMap& map, int n, int h, int w, int cin, const void* weight, const float* bias,
    int cout, int relu, void* y, int y_channels, int y_offset, int* err, int grid_limit, cudaStream_t stream,
    void* pool = nullptr, int up = 0, int stages = 0);
// Weight (cout x cin x 3 x 3, FP32) and bias gradients of a k_conv3x3 layer
// (denoiser_train.cu); `partial` holds wgrad_partial_bytes(sms, cout).
cudaError_t launch_conv3x3_wgrad(const void* x, int n, int h, int w, int cin, const void* dy, int cout, float* dweight,
    float* dbias, int* err, int sms, cudaStream_t stream, float* partial, size_t partial_bytes);
size_t wgrad_partial_bytes(int sms, int cout);

struct UNet;

UNet* unet_create();
void unet_destroy(UNet* net);
// Parameters in layer order, each layer's weight (out x in x 3 x 3, as PyTorch's
// conv2d) then bias; count must equal unet_param_count(). nullptr clears them.
bool unet_set_params(UNet* net, const float* params, long long count, std::string& error);
bool unet_ready(const UNet* net);
long long unet_param_count();
// Allocates the activations and TMA maps of an (n, h, w) batch; call before
// stream capture so captured launches find them in place.
bool unet_prepare(UNet* net, int n, int h, int w);
// Denoises n cameras of equal size w x h whose pixels start at `pixel_offset`
// in the frame-wide buffers of *fp (fp->cur); writes float4 radiance into
// fp->cur.denoised[pixel_offset ...]. `err` (device int) receives a kernel's
// bounded-wait failure code.
cudaError_t unet_run(UNet* net, const FrameParams* fp, long long pixel_offset, int n, int h, int w, int* err,
    int sm_count, cudaStream_t stream);

}  // namespace rtgb
