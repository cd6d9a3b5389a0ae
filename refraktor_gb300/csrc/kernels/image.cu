// Flame-independent kernels of the render path, compiled by nvcc for sm_103a:
// Catmull-Rom segment coefficients, log-density tonemap (with the density
// histogram of the reference fused into the same pass), the stand-alone
// density histogram, the density-estimation blur, and two roofline probes.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "image_kernels.h"

namespace {

// ------------------------------------------------------------ Catmull-Rom --
// Centripetal Catmull-Rom (alpha = 0.5, tension 0) segment p1 -> p2 with knot
// distance sqrt(hypot(dp, 1)), as assets/kernels/catmull.cu:11-28, evaluated
// in FP32 from the FP64 packed samples and stored in Hermite form
// (p1, p2, m1, m2). One thread per (segment, real).
__global__ void __launch_bounds__(256) catmull_kernel(const double* __restrict__ samples, unsigned sample_size,
                                                      unsigned nseg, float4* __restrict__ coeff) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (unsigned long long)sample_size * nseg) return;
    const unsigned seg = (unsigned)(i / sample_size), r = (unsigned)(i % sample_size);
    const size_t base = (size_t)seg * sample_size + r;
    const float p0 = (float)samples[base], p1 = (float)samples[base + sample_size];
    const float p2 = (float)samples[base + 2 * (size_t)sample_size], p3 = (float)samples[base + 3 * (size_t)sample_size];
    const float t01 = sqrtf(hypotf(p1 - p0, 1.0f));
    const float t12 = sqrtf(hypotf(p2 - p1, 1.0f));
    const float t23 = sqrtf(hypotf(p3 - p2, 1.0f));
    const float m1 = p2 - p1 + t12 * ((p1 - p0) / t01 - (p2 - p0) / (t01 + t12));
    const float m2 = p2 - p1 + t12 * ((p3 - p2) / t23 - (p3 - p1) / (t12 + t23));
    // Hermite form: a = 2(p1-p2)+m1+m2, b = -3(p1-p2)-2m1-m2, c = m1, d = p1
    // of the reference describe the same cubic
    coeff[i] = make_float4(p1, p2, m1, m2);
}

// ----------------------------------------------------------------- tonemap --
// (kernel text in tonemap_impl.cuh; the fast variant lives in tonemap_fast.cu)
#include "tonemap_impl.cuh"

// ------------------------------------------------------- density histogram --
__global__ void __launch_bounds__(256) density_histogram_kernel(const float4* __restrict__ bins, unsigned size,
                                                                unsigned long long* __restrict__ hist,
                                                                unsigned long long* __restrict__ max_density) {
    __shared__ unsigned long long sh[RFK_HISTOGRAM_BINS];
    __shared__ unsigned long long smax;
    for (int i = threadIdx.x; i < RFK_HISTOGRAM_BINS; i += blockDim.x) sh[i] = 0;
    if (threadIdx.x == 0) smax = 0;
    __syncthreads();
    const float log_div = 4.0f / logf(2.0f);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += (size_t)gridDim.x * blockDim.x) {
        const float v = bins[i].w;
        if (v >= 1.0f) {
            unsigned long long b = (unsigned long long)(logf(v) * log_div) + 1;
            if (b >= RFK_HISTOGRAM_BINS) b = RFK_HISTOGRAM_BINS - 1;
            atomicAdd(&sh[b], 1ull);
            atomicMax(&smax, (unsigned long long)v);
        } else {
            atomicAdd(&sh[0], 1ull);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < RFK_HISTOGRAM_BINS; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
    if (threadIdx.x == 0) atomicMax(max_density, smax);
}

// -------------------------------------------------- density-estimation blur --
// Each source pixel q with density d > 0 spreads its RGBA over a disc of radius
//   r(q) = clamp(max_radius * d^(-curve), min_radius, max_radius)
// quantised to 1/RFK_DE_STEPS px; the weight of integer offset o is
//   k(o) = max(0, 1 - |o|^2 / (r + 1)^2) / Z(r),  Z(r) = sum over |ox|,|oy| <= ceil(r) of the same,
// so a pixel of radius 0 keeps its value and every source conserves its total
// (inside the image). The output gathers, for each pixel, the contributions of
// all sources within max_radius.
#define DE_TILE_X 32
#define DE_TILE_Y 16
#define DE_HALO 9  // RFK_DE_MAX_RADIUS_CAP
#define DE_SW (DE_TILE_X + 2 * DE_HALO)
#define DE_SH (DE_TILE_Y + 2 * DE_HALO)

// Radius level (r * RFK_DE_STEPS, 255 = empty) of a source pixel.
__device__ __forceinline__ unsigned char de_level(float d, float max_radius, float min_radius, float curve) {
    if (!(d > 0.0f)) return 255;
    float r = max_radius * powf(d, -curve);
    r = fminf(fmaxf(r, min_radius), max_radius);
    return (unsigned char)lrintf(r * RFK_DE_STEPS);
}

__global__ void __launch_bounds__(DE_TILE_X * DE_TILE_Y / 2) de_blur_kernel(const float4* __restrict__ in, float4* __restrict__ out,
                                                                            unsigned w, unsigned h, float max_radius,
                                                                            float min_radius, float curve, int reach) {
    __shared__ float4 tile[DE_SH][DE_SW];
    __shared__ unsigned char lv[DE_SH][DE_SW];
    __shared__ float2 tab[RFK_DE_LEVELS];  // (1 / (r + 1)^2, 1 / Z(r)) per level
    __shared__ int max_rc;                  // largest support radius of a source in the tile
    const int tx0 = blockIdx.x * DE_TILE_X - DE_HALO, ty0 = blockIdx.y * DE_TILE_Y - DE_HALO;
    const int nthreads = blockDim.x;
    if (threadIdx.x == 0) max_rc = 0;
    for (int l = threadIdx.x; l < RFK_DE_LEVELS; l += nthreads) {
        const float r = (float)l / RFK_DE_STEPS;
        const float a = 1.0f / ((r + 1.0f) * (r + 1.0f));
        const int rc = (l + RFK_DE_STEPS - 1) / RFK_DE_STEPS;
        float z = 0.0f;
        for (int oy = -rc; oy <= rc; oy++)
            for (int ox = -rc; ox <= rc; ox++) z += fmaxf(0.0f, 1.0f - (float)(ox * ox + oy * oy) * a);
        tab[l] = make_float2(a, 1.0f / z);
    }
    __syncthreads();  // max_rc cleared
    int my_rc = 0;
    for (int i = threadIdx.x; i < DE_SW * DE_SH; i += nthreads) {
        const int sy = i / DE_SW, sx = i % DE_SW;
        const int gx = tx0 + sx, gy = ty0 + sy;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        unsigned char l = 255;
        if (gx >= 0 && gy >= 0 && gx < (int)w && gy < (int)h) {
            v = in[(size_t)gy * w + gx];
            l = de_level(v.w, max_radius, min_radius, curve);
        }
        tile[sy][sx] = v;
        lv[sy][sx] = l;
        if (l != 255) my_rc = max(my_rc, ((int)l + RFK_DE_STEPS - 1) / RFK_DE_STEPS);
    }
    if (my_rc > 0) atomicMax(&max_rc, my_rc);
    __syncthreads();
    // no source of the tile (halo included) reaches further than max_rc, so
    // the offsets beyond it would all be skipped below: the loop stops there
    // (an empty tile writes zeros at once); the sum is unchanged bit for bit
    reach = min(reach, max_rc);
    // two output pixels per thread, rows y and y + DE_TILE_Y/2
    const int ox = threadIdx.x % DE_TILE_X, oy = threadIdx.x / DE_TILE_X;
    for (int half = 0; half < 2; half++) {
        const int py = oy + half * (DE_TILE_Y / 2);
        const int gx = blockIdx.x * DE_TILE_X + ox, gy = blockIdx.y * DE_TILE_Y + py;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int dy = -reach; dy <= reach; dy++) {
            const int sy = py + DE_HALO + dy;
            for (int dx = -reach; dx <= reach; dx++) {
                const int sx = ox + DE_HALO + dx;
                const unsigned char l = lv[sy][sx];
                if (l == 255) continue;
                // the source's support is |ox|,|oy| <= ceil(r)
                const int rc = (l + RFK_DE_STEPS - 1) / RFK_DE_STEPS;
                if (abs(dx) > rc || abs(dy) > rc) continue;
                const float2 t = tab[l];
                const float k = fmaxf(0.0f, 1.0f - (float)(dx * dx + dy * dy) * t.x);
                if (k == 0.0f) continue;
                const float wgt = k * t.y;
                const float4 v = tile[sy][sx];
                acc.x = fmaf(v.x, wgt, acc.x);
                acc.y = fmaf(v.y, wgt, acc.y);
                acc.z = fmaf(v.z, wgt, acc.z);
                acc.w = fmaf(v.w, wgt, acc.w);
            }
        }
        if (gx < (int)w && gy < (int)h) out[(size_t)gy * w + gx] = acc;
    }
}

// ------------------------------------------------------------------ probes --
// Throughput of red.global.add.v4.f32 to pseudo-random float4 slots of a
// buffer: the L2-atomic roofline of the histogram update.
__global__ void red_v4_probe_kernel(float4* __restrict__ buf, unsigned long long n, unsigned iters, unsigned seed) {
    unsigned x = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u + seed;
    for (unsigned i = 0; i < iters; i++) {
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        const unsigned long long idx = ((unsigned long long)x * n) >> 32;
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(buf + idx), "f"(1.0f), "f"(0.5f), "f"(0.25f),
                     "f"(1.0f)
                     : "memory");
    }
}

// Issue-rate probes of the two arithmetic pipes the chain step leans on:
// pipe 0 = FP32 FMA (8 independent fmaf chains per thread), pipe 1 = the
// special-function unit (sin.approx and rsqrt.approx, 8 independent chains:
// sin(x) stays in [-1, 1] and rsqrt of a positive value converges to 1, so no
// chain reaches inf or NaN). Each thread stores its sum so that nothing is
// dead code.
__global__ void pipe_probe_kernel(float* __restrict__ out, unsigned iters, int pipe) {
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = 0.5f + 0.001f * (float)((gid + j) & 255);
    if (pipe == 0) {
        for (unsigned i = 0; i < iters; i++) {
#pragma unroll
            for (int j = 0; j < 8; j++) a[j] = fmaf(a[j], 0.9999f, 0.0001f);
        }
    } else {
        for (unsigned i = 0; i < iters; i++) {
#pragma unroll
            for (int j = 0; j < 4; j++) asm volatile("sin.approx.ftz.f32 %0, %0;" : "+f"(a[j]));
#pragma unroll
            for (int j = 4; j < 8; j++) asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[j]));
        }
    }
    float sum = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++) sum += a[j];
    out[gid] = sum;
}

// ---------------------------------------------------------------- convert --
// convert_to<In, Out> of assets/kernels/convert.cu:70-99: half3 / half4 in,
// uchar3 / uchar4 / float3 / float4 out; a byte is min(v * 255, 255)
// truncated (the reference multiplies in double); flip_y writes row h-1-y,
// swap_channels exchanges R and B; a 4-channel output of a 3-channel input
// gets alpha 1.
template <int CIN, int COUT, bool BYTES>
__global__ void convert_kernel(const __half* __restrict__ in, void* __restrict__ out, unsigned w, unsigned h, int flip_y,
                               int swap) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const __half* p = in + (size_t)i * CIN;
    float v[4] = {__half2float(p[0]), __half2float(p[1]), __half2float(p[2]), CIN == 4 ? __half2float(p[3]) : 1.0f};
    if (swap) {
        const float t = v[0];
        v[0] = v[2];
        v[2] = t;
    }
    unsigned o = i;
    if (flip_y) o = (h - i / w - 1) * w + i % w;
    if (BYTES) {
        unsigned char* q = static_cast<unsigned char*>(out) + (size_t)o * COUT;
        for (int c = 0; c < COUT; c++) {
            const double b = fmin((double)v[c] * 255.0, 255.0);
            q[c] = (unsigned char)(b > 0.0 ? b : 0.0);
        }
    } else {
        float* q = static_cast<float*>(out) + (size_t)o * COUT;
        for (int c = 0; c < COUT; c++) q[c] = v[c];
    }
}

__global__ void clear_counters_kernel(unsigned long long* c) {
    c[0] = 0;
    c[1] = 0;
    c[2] = ~0ull;
    c[3] = 0;
    c[4] = 0;
    c[5] = 0;
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

extern "C" {

cudaError_t rfk_launch_catmull(const double* samples, unsigned sample_size, unsigned nseg, float4* coeff, cudaStream_t s) {
    const unsigned long long n = (unsigned long long)sample_size * nseg;
    if (n == 0) return cudaSuccess;
    catmull_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(samples, sample_size, nseg, coeff);
    return cudaGetLastError();
}

cudaError_t rfk_launch_tonemap_fast(const float4* bins, unsigned size, void* out, int format, float gamma,
                                    float scale_constant, float brightness, float vibrancy, float highlight_power,
                                    unsigned long long* hist, unsigned long long* max_density,
                                    const unsigned long long* q_hits, double q_per_hit, unsigned blocks, cudaStream_t s);

cudaError_t rfk_launch_tonemap(const float4* bins, unsigned size, void* out, int format, int precise, float gamma,
                               float scale_constant, float brightness, float vibrancy, float highlight_power,
                               unsigned long long* hist, unsigned long long* max_density, const unsigned long long* q_hits,
                               double q_per_hit, cudaStream_t s) {
    if (size == 0) return cudaSuccess;
    unsigned blocks = (size + 255) / 256;
    const unsigned cap = (unsigned)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (!precise)
        return rfk_launch_tonemap_fast(bins, size, out, format, gamma, scale_constant, brightness, vibrancy, highlight_power,
                                       hist, max_density, q_hits, q_per_hit, blocks, s);
    switch (format) {
    case 0: rfk_tm::launch<true, 3>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    case 1: rfk_tm::launch<true, 4>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    case 2: rfk_tm::launch<false, 3>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    case 3: rfk_tm::launch<false, 4>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t rfk_launch_density_histogram(const float4* bins, unsigned size, unsigned long long* hist,
                                         unsigned long long* max_density, cudaStream_t s) {
    if (size == 0) return cudaSuccess;
    unsigned blocks = (size + 255) / 256;
    const unsigned cap = (unsigned)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    density_histogram_kernel<<<blocks, 256, 0, s>>>(bins, size, hist, max_density);
    return cudaGetLastError();
}

cudaError_t rfk_launch_de_blur(const float4* in, float4* out, unsigned w, unsigned h, float max_radius, float min_radius,
                               float curve, cudaStream_t s) {
    if (w == 0 || h == 0) return cudaSuccess;
    dim3 grid((w + DE_TILE_X - 1) / DE_TILE_X, (h + DE_TILE_Y - 1) / DE_TILE_Y);
    const int reach = (int)ceilf(max_radius);
    de_blur_kernel<<<grid, DE_TILE_X * DE_TILE_Y / 2, 0, s>>>(in, out, w, h, max_radius, min_radius, curve, reach);
    return cudaGetLastError();
}

cudaError_t rfk_launch_red_v4_probe(float4* buf, unsigned long long n, unsigned iters, unsigned blocks, unsigned threads,
                                    cudaStream_t s) {
    red_v4_probe_kernel<<<blocks, threads, 0, s>>>(buf, n, iters, 12345u);
    return cudaGetLastError();
}

cudaError_t rfk_launch_pipe_probe(float* out, unsigned iters, int pipe, unsigned blocks, unsigned threads,
                                  cudaStream_t s) {
    pipe_probe_kernel<<<blocks, threads, 0, s>>>(out, iters, pipe);
    return cudaGetLastError();
}

cudaError_t rfk_launch_convert(const void* in, int in_channels, void* out, int out_format, unsigned w, unsigned h,
                               int flip_y, int swap, cudaStream_t s) {
    if (w == 0 || h == 0) return cudaSuccess;
    const unsigned blocks = (w * h + 255) / 256;
    const __half* src = static_cast<const __half*>(in);
    // out_format: 2 float3, 3 float4, 4 uchar3, 5 uchar4
    if (in_channels == 3) {
        switch (out_format) {
        case 2: convert_kernel<3, 3, false><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        case 3: convert_kernel<3, 4, false><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        case 4: convert_kernel<3, 3, true><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        case 5: convert_kernel<3, 4, true><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        default: return cudaErrorInvalidValue;
        }
    } else if (in_channels == 4) {
        switch (out_format) {
        case 2: convert_kernel<4, 3, false><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        case 3: convert_kernel<4, 4, false><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        case 4: convert_kernel<4, 3, true><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        case 5: convert_kernel<4, 4, true><<<blocks, 256, 0, s>>>(src, out, w, h, flip_y, swap); break;
        default: return cudaErrorInvalidValue;
        }
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t rfk_launch_clear_counters(unsigned long long* c, cudaStream_t s) {
    clear_counters_kernel<<<1, 1, 0, s>>>(c);
    return cudaGetLastError();
}

}  // extern "C"
