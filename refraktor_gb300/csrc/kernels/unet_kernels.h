// Launchers of the denoiser kernels (unet_tc.cu: tensor-core convolutions,
// unet_ops.cu: the memory-bound layers around them). Activations are bf16
// NHWC tensors addressed as (pointer, channels per pixel = cstride, channel
// offset = coff), so a layer can read or write a channel slice of a wider
// tensor (the U-Net's concatenations are written in place).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#define RFK_UNET_RELU 1    // conv epilogue: ReLU after the bias
#define RFK_UNET_F32OUT 2  // conv epilogue: store f32 instead of bf16
#define RFK_UNET_UP2 4     // conv epilogue: store each output pixel at its 2x2 pixels of a (2h, 2w) output
                           // (nearest upsampling into the next level's concatenation; bf16, no accumulate)

#ifdef __cplusplus
extern "C" {
#endif

// 3x3 convolution, stride 1, zero padding 1, on tcgen05: out[:, :, :, coff:coff+cout] (=|+=) epilogue(
// conv(in[..., in_coff:in_coff+cin], weights[cout][9][cin]) + bias) with optional ReLU (flags) and
// multiplication by (mask > 0). Channel counts and offsets are multiples of 32; tensors 64-byte
// aligned. *err is set to 1 if a pipeline wait of the kernel ran out of time.
cudaError_t rfk_unet_conv3x3(const void* in, int n_img, int h, int w, int in_cstride, int in_coff, int cin,
                             const void* weights, int cout, const float* bias, int flags, void* out, int out_cstride,
                             int out_coff, const void* mask, int mask_cstride, int mask_coff, int accumulate, int* err,
                             cudaStream_t s);

// dW[cout][9][cin] (f32) += sum over pixels of dY[p][n] * X[p + tap][c], on tcgen05. dy: dY as
// dense NHWC bf16 (cout channels); x: X as NHWC bf16, channels x_coff .. x_coff + cin of
// x_cstride. w must be a multiple of 64, cin and cout of 32.
cudaError_t rfk_unet_wgrad3x3(const void* dy, const void* x, int x_cstride, int x_coff, int n_img, int h, int w, int cout,
                              int cin, float* dw, int* err, cudaStream_t s);


// Network input (32 bf16 channels per pixel) of a float4 histogram rendered at `spp` and its
// tonemapped image `base` (float4).
cudaError_t rfk_unet_features(const float4* bins, const float4* base, size_t npx, float spp, void* out, cudaStream_t s);
// 2x2 average pool of a channel slice into a dense [n][h/2][w/2][c] tensor.
cudaError_t rfk_unet_avgpool(const void* in, int n_img, int h, int w, int cstride, int coff, int c, void* out,
                             cudaStream_t s);
// Nearest 2x upsample of a dense [n][h][w][c] tensor into a channel slice.
cudaError_t rfk_unet_upsample(const void* in, int n_img, int h, int w, int c, void* out, int cstride, int coff,
                              cudaStream_t s);
// Gradient through the upsample (2x2 sums of a slice of g) times (act > 0); act and out [n][h][w][c].
cudaError_t rfk_unet_up_backward(const void* g, int gcstride, int gcoff, const void* act, int n_img, int h, int w, int c,
                                 void* out, cudaStream_t s);
// Gradient of a skip slice feeding a concatenation and an average pool, times its ReLU derivative.
cudaError_t rfk_unet_skip_backward(const void* gcat, int cstride, int coff, const void* gpool, const void* cat, int n_img,
                                   int h, int w, int c, void* out, cudaStream_t s);
// Mean squared error of base + channels 0..2 (f32 output, 32 per pixel) against f32 RGBA targets;
// bf16 gradient.
cudaError_t rfk_unet_mse(const float* out, const float4* base, const float4* target, size_t npx, void* grad, double* loss,
                         cudaStream_t s);
// db[c] += sum over pixels of g[p][c].
cudaError_t rfk_unet_bias_grad(const void* g, size_t npx, int c, float* db, cudaStream_t s);
// Adam step of one layer (f32 master weights and bias) writing the bf16 forward and input-gradient copies.
cudaError_t rfk_unet_adam(float* w, float* m, float* v, const float* g, int cout, int cin, int live_out, int live_in,
                          float lr, float b1, float b2, float eps, int step, void* wf, void* wb, float* bias, float* bm,
                          float* bv, const float* bg, cudaStream_t s);
// base + network output to an image (RFK_HALF3 .. RFK_FLOAT4; alpha as the tonemapper's).
cudaError_t rfk_unet_to_image(const float* net, const float4* base, const float4* bins, size_t npx, void* out, int format,
                              cudaStream_t s);

#ifdef __cplusplus
}
#endif
