// Launchers of the flame-independent kernels (image.cu).
#pragma once

#include <cuda_runtime.h>

#define RFK_HISTOGRAM_BINS 97  // granularity 4: 24 * 4 + 1 log2 bins (constants.h:4-6 of the reference)
#define RFK_DE_STEPS 4         // blur radius quantisation: 1/4 px
#define RFK_DE_MAX_RADIUS_CAP 9
#define RFK_DE_LEVELS (RFK_DE_MAX_RADIUS_CAP * RFK_DE_STEPS + 1)
#define RFK_NOALLOC_SCRATCH_BYTES (4u << 20)  // fixed scratch of rfk_prepare_samples_noalloc

#ifdef __cplusplus
extern "C" {
#endif

cudaError_t rfk_launch_catmull(const double* samples, unsigned sample_size, unsigned nseg, float4* coeff, cudaStream_t s);
// q_hits non-null: the quality is *q_hits * q_per_hit, read on the device,
// and scale_constant is ignored.
cudaError_t rfk_launch_tonemap(const float4* bins, unsigned size, void* out, int format, int precise, float gamma,
                               float scale_constant, float brightness, float vibrancy, float highlight_power,
                               unsigned long long* hist, unsigned long long* max_density, const unsigned long long* q_hits,
                               double q_per_hit, cudaStream_t s);
cudaError_t rfk_launch_density_histogram(const float4* bins, unsigned size, unsigned long long* hist,
                                         unsigned long long* max_density, cudaStream_t s);
cudaError_t rfk_launch_de_blur(const float4* in, float4* out, unsigned w, unsigned h, float max_radius, float min_radius,
                               float curve, cudaStream_t s);
cudaError_t rfk_launch_red_v4_probe(float4* buf, unsigned long long n, unsigned iters, unsigned blocks, unsigned threads,
                                    cudaStream_t s);
// out: blocks * threads floats.
cudaError_t rfk_launch_pipe_probe(float* out, unsigned iters, int pipe, unsigned blocks, unsigned threads,
                                  cudaStream_t s);
cudaError_t rfk_launch_clear_counters(unsigned long long* c, cudaStream_t s);
// half3 / half4 image -> float3 (2) / float4 (3) / uchar3 (4) / uchar4 (5).
cudaError_t rfk_launch_convert(const void* in, int in_channels, void* out, int out_format, unsigned w, unsigned h,
                               int flip_y, int swap, cudaStream_t s);
// noalloc.cu: device address and size of the fixed scratch array on the
// current device (taken once per device), and the device fix_rotation.
cudaError_t rfk_noalloc_scratch_address(void** addr, size_t* bytes);
cudaError_t rfk_launch_fix_rotation(double* samples, unsigned n, unsigned sample_size, unsigned flame_size,
                                    const unsigned* aff, unsigned naff, cudaStream_t s);

#ifdef __cplusplus
}
#endif
