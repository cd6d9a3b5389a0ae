// Memory-bound layers of the denoiser around the tensor-core convolutions.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "unet_kernels.h"

namespace {

using bf16 = __nv_bfloat16;

// 32 pixels x 32 channels through shared memory: reads along channels,
// writes along x, both coalesced.
__global__ void to_chw_kernel(const bf16* __restrict__ in, int h, int w, int cstride, int coff, int c, int dx,
                              bf16* __restrict__ out) {
    __shared__ bf16 t[32][34];
    const int xb = blockIdx.x * 32, ny = blockIdx.y, cb = blockIdx.z * 32;
    const int n = ny / h, y = ny - n * h;
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int x = xb + i, sx = x + dx, ch = cb + threadIdx.x;
        bf16 v = __float2bfloat16(0.0f);
        if (x < w && sx >= 0 && sx < w && ch < c) v = in[((size_t)ny * w + sx) * cstride + coff + ch];
        t[i][threadIdx.x] = v;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int ch = cb + i, x = xb + threadIdx.x;
        if (ch < c && x < w) out[(((size_t)n * c + ch) * h + y) * w + x] = t[threadIdx.x][i];
    }
}

}  // namespace

extern "C" cudaError_t rfk_unet_to_chw(const void* in, int n_img, int h, int w, int cstride, int coff, int c, int dx,
                                       void* out, cudaStream_t s) {
    if (n_img <= 0 || h <= 0 || w <= 0 || c <= 0) return cudaErrorInvalidValue;
    dim3 grid((unsigned)((w + 31) / 32), (unsigned)(n_img * h), (unsigned)((c + 31) / 32));
    to_chw_kernel<<<grid, dim3(32, 8), 0, s>>>(static_cast<const bf16*>(in), h, w, cstride, coff, c, dx,
                                               static_cast<bf16*>(out));
    return cudaGetLastError();
}
