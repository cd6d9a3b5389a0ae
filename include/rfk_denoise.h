/*
 * rfk_denoise.h - C ABI of the learned denoiser (librfk.so).
 *
 * Stands in for the reference's denoiser plug-in interface
 * (src/librefrakt/include/librefrakt/interface/denoiser.h:21-39:
 * denoiser::make(name, dims, flags, stream) and denoise(in, out, event) ->
 * future<double ms>), whose implementations wrap closed libraries. This one is
 * a 4-level BF16 U-Net (32 / 64 / 128 / 256 channels, 3x3 convolutions, ReLU)
 * on hand-written tcgen05 kernels; it reads the float4 histogram of a
 * low-spp render (density, colour, alpha, spp as input channels) and writes
 * the tonemapped image of a converged render. Training (forward, backward,
 * Adam) runs on the device through the same kernels. Conventions as rfk.h:
 * rfk_status results, rfk_last_error(), device pointers, void* streams.
 */
#ifndef RFK_DENOISE_H
#define RFK_DENOISE_H

#include <stddef.h>
#include <stdint.h>

#include "rfk.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rfk_denoiser rfk_denoiser;

/* denoiser::make(name, dims, flags, stream) by registered name
 * (interface/denoiser.h:21-39, factory.h:71-98). Registered:
 * "rfkt::gb300_unet_denoiser", the U-Net below, with the weights of the .npz
 * file `weights_path` (rfk_denoiser_read_params) or, when it is NULL, seeded
 * initial weights. An unknown name returns RFK_E_INVALID with *out = NULL
 * (the reference's factory returns a null pointer). */
rfk_status rfk_denoiser_make(const char* name, const char* weights_path, rfk_denoiser** out);
/* Registered name number `index` (0-based) into buf; RFK_E_INVALID past the end. */
rfk_status rfk_denoiser_name(int index, char* buf, size_t cap);
/* A network with seeded He-initialised weights. */
rfk_status rfk_denoiser_create(uint64_t seed, rfk_denoiser** out);
void rfk_denoiser_destroy(rfk_denoiser* d);
/* Reads the parameters of a weight file written by the Python side
 * (refraktor_gb300.denoise.denoiser.save: NumPy .npz with a 1-D float16 or
 * float32 `params` array, e.g. refraktor_gb300/workloads/denoiser_weights.npz)
 * into host floats in the rfk_denoiser_set_params layout. *count = the number
 * of parameters; with out == NULL only the count is returned. */
rfk_status rfk_denoiser_read_params(const char* path, float* out, size_t cap, size_t* count);
/* Parameters: per layer the f32 weights [cout][9][cin] then the biases [cout] (host arrays). */
size_t rfk_denoiser_param_count(const rfk_denoiser* d);
rfk_status rfk_denoiser_get_params(const rfk_denoiser* d, float* out, size_t n);
rfk_status rfk_denoiser_set_params(rfk_denoiser* d, const float* in, size_t n);

/* Network input of one w x h float4 histogram rendered at spp and its tonemapped image (float4):
 * 32 bf16 channels per pixel (device). */
rfk_status rfk_denoiser_features(const float* bins, const float* base, uint32_t w, uint32_t h, double spp, void* out,
                                 void* stream);

/* One Adam step (learning rate lr) on n histograms (n x h x w float4, device) rendered at spp, with
 * their tonemapped images (base, n x h x w float4), against n x h x w RGBA f32 targets (device);
 * *loss = mean squared error of RGB before the step. w must be a multiple of 512 and h of 8. */
rfk_status rfk_denoiser_train_step(rfk_denoiser* d, const float* bins, const float* base, uint32_t n, uint32_t w,
                                   uint32_t h, double spp, const float* targets, float lr, double* loss, void* stream);
/* The loss without a step (validation); w and h multiples of 8. */
rfk_status rfk_denoiser_loss(rfk_denoiser* d, const float* bins, const float* base, uint32_t n, uint32_t w, uint32_t h,
                             double spp, const float* targets, double* loss, void* stream);
/* Parameter gradients of the loss (host array in the parameter layout), without a step. */
rfk_status rfk_denoiser_gradients(rfk_denoiser* d, const float* bins, const float* base, uint32_t n, uint32_t w,
                                  uint32_t h, double spp, const float* targets, float* grads, size_t count, void* stream);

/* denoiser::denoise: the w x h histogram of a render at spp and its tonemapped image (base,
 * float4) in, the denoised image out in one of RFK_HALF3 / RFK_HALF4 / RFK_FLOAT3 / RFK_FLOAT4
 * (alpha as the tonemapper's). w and h multiples of 8. */
rfk_status rfk_denoise(rfk_denoiser* d, const float* bins, const float* base, uint32_t w, uint32_t h, double spp,
                       void* out, int format, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RFK_DENOISE_H */
