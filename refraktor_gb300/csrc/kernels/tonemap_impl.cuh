// Tonemap kernel body shared by two translation units: image.cu compiles it
// with full-precision math (PRECISE) and tonemap_fast.cu with -use_fast_math,
// the way the reference builds assets/kernels/tonemap.cu
// (src/librefrakt/src/image/tonemapper.cpp:10-22), so that the fast variant
// matches the reference kernel.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "image_kernels.h"

namespace rfk_tm {
// ----------------------------------------------------------------- tonemap --
template <int C, bool HALF>
struct pixel_out;
template <>
struct pixel_out<3, true> {
    static __device__ void store(void* out, size_t i, float r, float g, float b, float) {
        __half* o = reinterpret_cast<__half*>(out) + 3 * i;
        o[0] = __float2half_rn(r);
        o[1] = __float2half_rn(g);
        o[2] = __float2half_rn(b);
    }
};
template <>
struct pixel_out<4, true> {
    static __device__ void store(void* out, size_t i, float r, float g, float b, float a) {
        __half2 lo = __floats2half2_rn(r, g), hi = __floats2half2_rn(b, a);
        uint2 v;
        v.x = *reinterpret_cast<unsigned*>(&lo);
        v.y = *reinterpret_cast<unsigned*>(&hi);
        reinterpret_cast<uint2*>(out)[i] = v;
    }
};
template <>
struct pixel_out<3, false> {
    static __device__ void store(void* out, size_t i, float r, float g, float b, float) {
        float* o = reinterpret_cast<float*>(out) + 3 * i;
        o[0] = r;
        o[1] = g;
        o[2] = b;
    }
};
template <>
struct pixel_out<4, false> {
    static __device__ void store(void* out, size_t i, float r, float g, float b, float a) {
        reinterpret_cast<float4*>(out)[i] = make_float4(r, g, b, a);
    }
};

__device__ __forceinline__ float sat(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }

// flam3-style highlight handling (an extension; the reference parses
// highlight_power but never applies it): when the brightest channel of the
// density-scaled colour exceeds 1, scale it to 1 and reduce saturation by
// (1/max)^highlight_power so that hot pixels go white instead of shifting hue.
__device__ void highlight(float& r, float& g, float& b, float hp) {
    const float m = fmaxf(r, fmaxf(g, b));
    if (!(m > 1.0f)) return;
    const float s = 1.0f / m;
    const float ratio = powf(s, hp);
    // at HSV value 1 a channel is 1 - sat * k(hue); scaling sat by `ratio`
    // maps each channel c to 1 - ratio * (1 - c)
    r = 1.0f - ratio * (1.0f - r * s);
    g = 1.0f - ratio * (1.0f - g * s);
    b = 1.0f - ratio * (1.0f - b * s);
}

// Per pixel (assets/kernels/tonemap.cu:67-104 with the host constant of
// src/librefrakt/src/image/tonemapper.cpp:52):
//   w = density, k2 = 10^(-log10(q) - 0.5)
//   f = 0.5 * brightness * log10(1 + w k2) / w;  (r, g, b, w) *= f
//   z = w^(1/gamma) (FP64), gf = z / w
//   c = sat(lerp(c^(1/gamma), c gf, vibrancy))
//   alpha = sat(ln(w_in) * (4 / ln 2) / 96)
// The precise build uses log1pf / powf / logf at full precision; the fast
// build is the same text under -use_fast_math, as the reference kernel. The
// density histogram of density_histo.cu:1-42
// (granularity 4: 97 log2 bins, max density) is accumulated in the same pass
// when `hist` is non-null.
template <int C, bool HALF>
__global__ void __launch_bounds__(256) tonemap_kernel(const float4* __restrict__ bins, void* __restrict__ out, unsigned size,
                                                      float gamma, float scale_constant, float brightness, float vibrancy,
                                                      float highlight_power, unsigned long long* __restrict__ hist,
                                                      unsigned long long* __restrict__ max_density,
                                                      const unsigned long long* __restrict__ q_hits, double q_per_hit) {
    __shared__ unsigned long long sh[RFK_HISTOGRAM_BINS];
    __shared__ unsigned long long smax;
    if (hist) {
        for (int i = threadIdx.x; i < RFK_HISTOGRAM_BINS; i += blockDim.x) sh[i] = 0;
        if (threadIdx.x == 0) smax = 0;
        __syncthreads();
    }
    if (q_hits) {
        // quality from a device counter (batched renders): the host constant
        // of the single-image path, computed here in single precision
        const float q = (float)((double)*q_hits * q_per_hit);
        scale_constant = powf(10.0f, -log10f(q) - 0.5f);
    }
    const float log_div = 4.0f / logf(2.0f);
    const double inv_gamma = 1.0 / (double)gamma;
    const float inv_gamma_f = (float)inv_gamma;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += (size_t)gridDim.x * blockDim.x) {
        float4 col = bins[i];
        if (hist) {
            const float v = col.w;
            if (v >= 1.0f) {
                unsigned long long b = (unsigned long long)(logf(v) * log_div) + 1;
                if (b >= RFK_HISTOGRAM_BINS) b = RFK_HISTOGRAM_BINS - 1;
                atomicAdd(&sh[b], 1ull);
                atomicMax(&smax, (unsigned long long)v);
            } else {
                atomicAdd(&sh[0], 1ull);
            }
        }
        if (col.w == 0.0f) {
            pixel_out<C, HALF>::store(out, i, 0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        const float input_density = col.w;
#ifdef RFK_TONEMAP_FAST
        float lg = logf(1.0f + col.w * scale_constant);
#else
        float lg = log1pf(col.w * scale_constant);
#endif
        const float factor = 0.5f * brightness * lg * 0.434294481903251827651128918916f / col.w;
        col.x *= factor;
        col.y *= factor;
        col.z *= factor;
        col.w *= factor;
#ifdef RFK_TONEMAP_FAST
        // the reference's FP64 w^(1/gamma) / w, for bitwise agreement with it
        const double z = pow((double)col.w, inv_gamma);
        const double gamma_factor = z / col.w;
        float lr = (float)(col.x * gamma_factor), lgc = (float)(col.y * gamma_factor), lb = (float)(col.z * gamma_factor);
#else
        // w^(1/gamma) / w = w^(1/gamma - 1) in one FP32 powf (2 ulp): FP64 pow
        // is slow on this part and the result is already within 1e-6 relative
        const float gamma_factor = powf(col.w, inv_gamma_f - 1.0f);
        float lr = col.x * gamma_factor, lgc = col.y * gamma_factor, lb = col.z * gamma_factor;
#endif
        if (highlight_power >= 0.0f) highlight(lr, lgc, lb, highlight_power);
        const float r = __saturatef(lerpf(powf(col.x, inv_gamma_f), lr, vibrancy));
        const float g = __saturatef(lerpf(powf(col.y, inv_gamma_f), lgc, vibrancy));
        const float b = __saturatef(lerpf(powf(col.z, inv_gamma_f), lb, vibrancy));
        float a = 0.0f;
        if (C == 4) a = __saturatef(logf(input_density) * log_div / 96.0f);
        pixel_out<C, HALF>::store(out, i, r, g, b, a);
    }
    if (hist) {
        __syncthreads();
        for (int i = threadIdx.x; i < RFK_HISTOGRAM_BINS; i += blockDim.x)
            if (sh[i]) atomicAdd(&hist[i], sh[i]);
        if (threadIdx.x == 0) atomicMax(max_density, smax);
    }
}


template <bool HALF, int C>
void launch(unsigned blocks, cudaStream_t s, const float4* bins, void* out, unsigned size, float gamma, float scale_constant,
            float brightness, float vibrancy, float highlight_power, unsigned long long* hist,
            unsigned long long* max_density, const unsigned long long* q_hits, double q_per_hit) {
    tonemap_kernel<C, HALF><<<blocks, 256, 0, s>>>(bins, out, size, gamma, scale_constant, brightness, vibrancy,
                                                    highlight_power, hist, max_density, q_hits, q_per_hit);
}

}  // namespace rfk_tm
