// Memory-bound layers of the denoiser around the tensor-core convolutions.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "unet_kernels.h"

namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ float bf(const bf16 v) { return __bfloat162float(v); }

// Denoiser input of one histogram: 32 bf16 channels per pixel,
//   0: log1p(density) / 8            1-3: mean colour (rgb / density)
//   4: alpha, sat(ln(density) * 4 / ln 2 / 96) as the tonemapper's
//   5: ln(spp) / 8                   6-8: the tonemapped image of the histogram
//   9-31: 0
__global__ void features_kernel(const float4* __restrict__ bins, const float4* __restrict__ base, size_t npx, float spp,
                                bf16* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx) return;
    const float4 b = bins[i];
    const float4 t = base[i];
    float f[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const float d = b.w;
    f[0] = log1pf(fmaxf(d, 0.0f)) * 0.125f;
    if (d > 0.0f) {
        f[1] = b.x / d;
        f[2] = b.y / d;
        f[3] = b.z / d;
    }
    f[4] = d >= 1.0f ? fminf(fmaxf(logf(d) * (4.0f / 0.69314718f) / 96.0f, 0.0f), 1.0f) : 0.0f;
    f[5] = logf(fmaxf(spp, 1.0f)) * 0.125f;
    f[6] = t.x;
    f[7] = t.y;
    f[8] = t.z;
    __nv_bfloat162 h[16];
#pragma unroll
    for (int j = 0; j < 5; j++) h[j] = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
#pragma unroll
    for (int j = 5; j < 16; j++) h[j] = __floats2bfloat162_rn(0.0f, 0.0f);
    uint4* o = reinterpret_cast<uint4*>(out + i * 32);
#pragma unroll
    for (int q = 0; q < 4; q++) o[q] = reinterpret_cast<uint4*>(h)[q];
}

// The layers below move 8 channels (16 bytes) per thread; channel counts,
// strides and offsets are multiples of 8 (32 in this network).
__device__ __forceinline__ void ld8(const bf16* p, float (&v)[8]) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float2 f = __bfloat1622float2(h[j]);
        v[2 * j] = f.x;
        v[2 * j + 1] = f.y;
    }
}

__device__ __forceinline__ void st8(bf16* p, const float (&v)[8]) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int j = 0; j < 4; j++) h[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
    *reinterpret_cast<uint4*>(p) = *reinterpret_cast<uint4*>(h);
}

// 2x2 average pool of a channel slice: out[n][y][x][c] = mean of in[n][2y..2y+1][2x..2x+1][coff + c].
__global__ void avgpool_kernel(const bf16* __restrict__ in, int h, int w, int cstride, int coff, int c,
                               bf16* __restrict__ out, unsigned total) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c8 = c / 8, ho = h / 2, wo = w / 2;
    const int q = (int)(i % c8);
    unsigned r = i / c8;
    const int x = (int)(r % wo);
    r /= wo;
    const int y = (int)(r % ho);
    const unsigned n = r / ho;
    const size_t b = (((size_t)n * h + 2 * y) * w + 2 * x) * cstride + coff + q * 8;
    float a[8], v[8];
    ld8(in + b, a);
    ld8(in + b + cstride, v);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += v[j];
    ld8(in + b + (size_t)w * cstride, v);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += v[j];
    ld8(in + b + (size_t)w * cstride + cstride, v);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = 0.25f * (a[j] + v[j]);
    st8(out + (size_t)i * 8, a);
}

// Nearest 2x upsample into a channel slice: out[n][y][x][coff + c] = in[n][y / 2][x / 2][c].
__global__ void upsample_kernel(const bf16* __restrict__ in, int h, int w, int c, bf16* __restrict__ out, int cstride,
                                int coff, unsigned total) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c8 = c / 8, W = 2 * w, H = 2 * h;
    const int q = (int)(i % c8);
    unsigned r = i / c8;
    const int x = (int)(r % W);
    r /= W;
    const int y = (int)(r % H);
    const unsigned n = r / H;
    const uint4 v = *reinterpret_cast<const uint4*>(in + (((size_t)n * h + y / 2) * w + x / 2) * c + q * 8);
    *reinterpret_cast<uint4*>(out + (((size_t)n * H + y) * W + x) * cstride + coff + q * 8) = v;
}

// Gradient through a nearest 2x upsample (sum of the 2x2 block of a channel
// slice of g), times the ReLU derivative of the upsampled activation:
// out[n][y][x][c] = (act > 0) * sum g[n][2y..][2x..][gcoff + c].
__global__ void up_backward_kernel(const bf16* __restrict__ g, int gcstride, int gcoff, const bf16* __restrict__ act,
                                   int h, int w, int c, bf16* __restrict__ out, unsigned total) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c8 = c / 8;
    const int q = (int)(i % c8);
    unsigned r = i / c8;
    const int x = (int)(r % w);
    r /= w;
    const int y = (int)(r % h);
    const unsigned n = r / h;
    const int W = 2 * w;
    const size_t b = (((size_t)n * 2 * h + 2 * y) * W + 2 * x) * gcstride + gcoff + q * 8;
    float a[8], v[8], m[8];
    ld8(g + b, a);
    ld8(g + b + gcstride, v);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += v[j];
    ld8(g + b + (size_t)W * gcstride, v);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] += v[j];
    ld8(g + b + (size_t)W * gcstride + gcstride, v);
    ld8(act + (size_t)i * 8, m);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = m[j] > 0.0f ? a[j] + v[j] : 0.0f;
    st8(out + (size_t)i * 8, a);
}

// Gradient of a skip activation s (a channel slice of a concatenation) that
// feeds both the concatenation and a 2x2 average pool, times its ReLU
// derivative: out = (s > 0) * (gcat[slice] + gpool[y / 2][x / 2] / 4).
__global__ void skip_backward_kernel(const bf16* __restrict__ gcat, int cstride, int coff, const bf16* __restrict__ gpool,
                                     const bf16* __restrict__ cat, int h, int w, int c, bf16* __restrict__ out,
                                     unsigned total) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c8 = c / 8;
    const int q = (int)(i % c8);
    unsigned r = i / c8;
    const int x = (int)(r % w);
    r /= w;
    const int y = (int)(r % h);
    const unsigned n = r / h;
    const size_t px = ((size_t)n * h + y) * w + x;
    float sv[8], gc[8], gp[8];
    ld8(cat + px * cstride + coff + q * 8, sv);
    ld8(gcat + px * cstride + coff + q * 8, gc);
    ld8(gpool + (((size_t)n * (h / 2) + y / 2) * (w / 2) + x / 2) * c + q * 8, gp);
#pragma unroll
    for (int j = 0; j < 8; j++) gc[j] = sv[j] > 0.0f ? gc[j] + 0.25f * gp[j] : 0.0f;
    st8(out + (size_t)i * 8, gc);
}

// Mean squared error of the prediction base + out[0..2] (out f32, cstride 32;
// the network predicts a correction of the tonemapped low-spp image) against
// target (f32, 4 per pixel), and its gradient as bf16 (channels 3..31 zero).
__global__ void mse_kernel(const float* __restrict__ out, const float4* __restrict__ base, const float4* __restrict__ target,
                           size_t npx, float inv_n, bf16* __restrict__ grad, double* __restrict__ loss) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < npx) {
        const float4 t = target[i];
        const float4 b = base[i];
        const float* o = out + i * 32;
        const float d0 = b.x + o[0] - t.x, d1 = b.y + o[1] - t.y, d2 = b.z + o[2] - t.z;
        l = d0 * d0 + d1 * d1 + d2 * d2;
        __nv_bfloat162 hh[16];
        hh[0] = __floats2bfloat162_rn(2.0f * d0 * inv_n, 2.0f * d1 * inv_n);
        hh[1] = __floats2bfloat162_rn(2.0f * d2 * inv_n, 0.0f);
#pragma unroll
        for (int j = 2; j < 16; j++) hh[j] = __floats2bfloat162_rn(0.0f, 0.0f);
        uint4* g = reinterpret_cast<uint4*>(grad + i * 32);
#pragma unroll
        for (int q = 0; q < 4; q++) g[q] = reinterpret_cast<uint4*>(hh)[q];
    }
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0f) atomicAdd(loss, (double)l);
}

// Per-channel sum over pixels (bias gradient): db[c] += sum_p g[p][c]. A
// thread sums one 8-channel chunk over a strided run of pixels; the block
// reduces in shared memory and adds once per channel.
__global__ void bias_grad_kernel(const bf16* __restrict__ g, unsigned npx, int c, float* __restrict__ db) {
    extern __shared__ float red[];  // [c]
    const int c8 = c / 8;
    for (int j = threadIdx.x; j < c; j += blockDim.x) red[j] = 0.0f;
    __syncthreads();
    const int q = threadIdx.x % c8;
    const int lanes = blockDim.x / c8;
    const int lane = threadIdx.x / c8;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (lane < lanes) {
        for (unsigned p = blockIdx.x * lanes + lane; p < npx; p += gridDim.x * lanes) {
            float v[8];
            ld8(g + (size_t)p * c + q * 8, v);
#pragma unroll
            for (int j = 0; j < 8; j++) acc[j] += v[j];
        }
#pragma unroll
        for (int j = 0; j < 8; j++) atomicAdd(&red[q * 8 + j], acc[j]);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < c; j += blockDim.x) atomicAdd(db + j, red[j]);
}

// Adam (Kingma & Ba 2015) on one conv layer's f32 master weights [cout][9][cin]
// and bias; writes the bf16 copies used by the forward ([cout][9][cin]) and
// input-gradient ([cin][8 - t][cout]) convolutions. Rows / columns outside
// (live_out, live_in) stay zero (padded channels of the first and last layer).
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, int cout, int cin, int live_out, int live_in, float lr, float b1,
                            float b2, float eps, float c1, float c2, bf16* __restrict__ wf, bf16* __restrict__ wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = cout * 9 * cin;
    if (i >= n) return;
    const int ci = i % cin, t = (i / cin) % 9, co = i / (9 * cin);
    float wi = w[i];
    if (co < live_out && ci < live_in) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
    } else {
        wi = 0.0f;
    }
    const bf16 h = __float2bfloat16(wi);
    wf[i] = h;
    wb[((size_t)ci * 9 + (8 - t)) * cout + co] = h;
}

__global__ void adam_bias_kernel(float* __restrict__ b, float* __restrict__ m, float* __restrict__ v,
                                 const float* __restrict__ g, int n, int live, float lr, float b1, float b2, float eps,
                                 float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i >= live) {
        b[i] = 0.0f;
        return;
    }
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    b[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Prediction (base + network output) to an image in the tonemapper's formats,
// clamped to [0, 1]; alpha from the histogram as the tonemapper's.
template <int CH, bool HALF>
__global__ void to_image_kernel(const float* __restrict__ net, const float4* __restrict__ base,
                                const float4* __restrict__ bins, size_t npx, void* out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx) return;
    const float* o = net + i * 32;
    const float4 b = base[i];
    float v[4] = {fminf(fmaxf(b.x + o[0], 0.0f), 1.0f), fminf(fmaxf(b.y + o[1], 0.0f), 1.0f),
                  fminf(fmaxf(b.z + o[2], 0.0f), 1.0f), 0.0f};
    if (CH == 4) {
        const float d = bins[i].w;
        v[3] = d > 0.0f ? fminf(fmaxf(logf(d) * (4.0f / 0.69314718f) / 96.0f, 0.0f), 1.0f) : 0.0f;
    }
    if (HALF) {
        __half* h = static_cast<__half*>(out) + i * CH;
        for (int j = 0; j < CH; j++) h[j] = __float2half_rn(v[j]);
    } else {
        float* f = static_cast<float*>(out) + i * CH;
        for (int j = 0; j < CH; j++) f[j] = v[j];
    }
}

inline unsigned blocks_for(size_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" cudaError_t rfk_unet_features(const float4* bins, const float4* base, size_t npx, float spp, void* out,
                                         cudaStream_t s) {
    if (npx == 0) return cudaSuccess;
    features_kernel<<<blocks_for(npx), 256, 0, s>>>(bins, base, npx, spp, static_cast<bf16*>(out));
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_avgpool(const void* in, int n_img, int h, int w, int cstride, int coff, int c, void* out,
                                        cudaStream_t s) {
    const size_t total = (size_t)n_img * (h / 2) * (w / 2) * (c / 8);
    if (h % 2 || w % 2 || total == 0 || c % 8 || cstride % 8 || coff % 8 || total > 0xFFFFFFFFull) return cudaErrorInvalidValue;
    avgpool_kernel<<<blocks_for(total), 256, 0, s>>>(static_cast<const bf16*>(in), h, w, cstride, coff, c,
                                                      static_cast<bf16*>(out), (unsigned)total);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_upsample(const void* in, int n_img, int h, int w, int c, void* out, int cstride, int coff,
                                         cudaStream_t s) {
    const size_t total = (size_t)n_img * 4 * h * w * (c / 8);
    if (total == 0 || c % 8 || cstride % 8 || coff % 8 || total > 0xFFFFFFFFull) return cudaErrorInvalidValue;
    upsample_kernel<<<blocks_for(total), 256, 0, s>>>(static_cast<const bf16*>(in), h, w, c, static_cast<bf16*>(out),
                                                       cstride, coff, (unsigned)total);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_up_backward(const void* g, int gcstride, int gcoff, const void* act, int n_img, int h, int w,
                                            int c, void* out, cudaStream_t s) {
    const size_t total = (size_t)n_img * h * w * (c / 8);
    if (total == 0 || c % 8 || gcstride % 8 || gcoff % 8 || total > 0xFFFFFFFFull) return cudaErrorInvalidValue;
    up_backward_kernel<<<blocks_for(total), 256, 0, s>>>(static_cast<const bf16*>(g), gcstride, gcoff,
                                                          static_cast<const bf16*>(act), h, w, c, static_cast<bf16*>(out),
                                                          (unsigned)total);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_skip_backward(const void* gcat, int cstride, int coff, const void* gpool, const void* cat,
                                              int n_img, int h, int w, int c, void* out, cudaStream_t s) {
    const size_t total = (size_t)n_img * h * w * (c / 8);
    if (total == 0 || h % 2 || w % 2 || c % 8 || cstride % 8 || coff % 8 || total > 0xFFFFFFFFull)
        return cudaErrorInvalidValue;
    skip_backward_kernel<<<blocks_for(total), 256, 0, s>>>(static_cast<const bf16*>(gcat), cstride, coff,
                                                            static_cast<const bf16*>(gpool), static_cast<const bf16*>(cat),
                                                            h, w, c, static_cast<bf16*>(out), (unsigned)total);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_mse(const float* out, const float4* base, const float4* target, size_t npx, void* grad,
                                    double* loss, cudaStream_t s) {
    if (npx == 0) return cudaSuccess;
    mse_kernel<<<blocks_for(npx), 256, 0, s>>>(out, base, target, npx, 1.0f / (3.0f * (float)npx), static_cast<bf16*>(grad),
                                                loss);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_bias_grad(const void* g, size_t npx, int c, float* db, cudaStream_t s) {
    if (c % 8 || c > 2048 || npx == 0 || npx > 0xFFFFFFFFull) return cudaErrorInvalidValue;
    const unsigned lanes = 256 / (c / 8) > 0 ? 256 / (c / 8) : 1;
    unsigned bx = (unsigned)((npx + lanes * 64 - 1) / (lanes * 64));
    if (bx > 152 * 4) bx = 152 * 4;
    const unsigned threads = (c / 8) > 256 ? (unsigned)(c / 8) : 256;
    bias_grad_kernel<<<bx, threads, (size_t)c * sizeof(float), s>>>(static_cast<const bf16*>(g), (unsigned)npx, c, db);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_adam(float* w, float* m, float* v, const float* g, int cout, int cin, int live_out,
                                     int live_in, float lr, float b1, float b2, float eps, int step, void* wf, void* wb,
                                     float* bias, float* bm, float* bv, const float* bg, cudaStream_t s) {
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    const int n = cout * 9 * cin;
    adam_kernel<<<blocks_for((size_t)n), 256, 0, s>>>(w, m, v, g, cout, cin, live_out, live_in, lr, b1, b2, eps, c1, c2,
                                                       static_cast<bf16*>(wf), static_cast<bf16*>(wb));
    adam_bias_kernel<<<blocks_for((size_t)cout), 256, 0, s>>>(bias, bm, bv, bg, cout, live_out, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

extern "C" cudaError_t rfk_unet_to_image(const float* net, const float4* base, const float4* bins, size_t npx, void* out,
                                         int format, cudaStream_t s) {
    if (npx == 0) return cudaSuccess;
    switch (format) {
    case 0: to_image_kernel<3, true><<<blocks_for(npx), 256, 0, s>>>(net, base, bins, npx, out); break;
    case 1: to_image_kernel<4, true><<<blocks_for(npx), 256, 0, s>>>(net, base, bins, npx, out); break;
    case 2: to_image_kernel<3, false><<<blocks_for(npx), 256, 0, s>>>(net, base, bins, npx, out); break;
    case 3: to_image_kernel<4, false><<<blocks_for(npx), 256, 0, s>>>(net, base, bins, npx, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
