// Launchers of the denoiser kernels (unet_tc.cu: tensor-core convolutions,
// unet_ops.cu: the memory-bound layers around them). Activations are bf16
// NHWC tensors addressed as (pointer, channels per pixel = cstride, channel
// offset = coff), so a layer can read or write a channel slice of a wider
// tensor (the U-Net's concatenations are written in place).
#pragma once

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

// 3x3 convolution, stride 1, zero padding 1, on tcgen05: out[:, :, :, coff:coff+cout] (=|+=) epilogue(
// conv(in[..., in_coff:in_coff+cin], weights[cout][9][cin]) + bias) with optional ReLU and
// multiplication by (mask > 0). Channel counts and offsets are multiples of 32; tensors 64-byte
// aligned. *err is set to 1 if a pipeline wait of the kernel ran out of time.
cudaError_t rfk_unet_conv3x3(const void* in, int n_img, int h, int w, int in_cstride, int in_coff, int cin,
                             const void* weights, int cout, const float* bias, int relu, void* out, int out_cstride,
                             int out_coff, const void* mask, int mask_cstride, int mask_coff, int accumulate, int* err,
                             cudaStream_t s);

// dW[cout][9][cin] (f32) += sum over pixels of dY[p][n] * X[p + tap][c], on tcgen05. dyT: dY as
// [cout][n_img * h * w] bf16; xT[d]: X as [n_img][cin][h][w] bf16 shifted by dx = d - 1 columns
// (rfk_unet_to_chw). w must be a multiple of 64.
cudaError_t rfk_unet_wgrad3x3(const void* dyT, const void* const* xT, int n_img, int h, int w, int cout, int cin,
                              float* dw, int* err, cudaStream_t s);

// Channel-major copy of a channel slice: out[n][c][y][x] = in[n][y][x + dx][coff + c] (0 outside).
cudaError_t rfk_unet_to_chw(const void* in, int n_img, int h, int w, int cstride, int coff, int c, int dx, void* out,
                            cudaStream_t s);

#ifdef __cplusplus
}
#endif
