// Fixed device scratch for rfk_prepare_samples_noalloc.
//
// Some callers of this library cannot allocate device memory while they run:
// a host application whose device memory is owned by its own pool (a
// framework's caching allocator, an engine that reserves all memory at start
// and treats any other allocation as a leak or an out-of-memory risk), or a
// real-time loop that must not stall, since cudaMalloc / cudaFree can
// synchronise the whole device. For them the genome preparation step runs in
// this file-scope array instead of temporaries from cudaMalloc.
//
// The array is RFK_NOALLOC_SCRATCH_BYTES (4 MiB) on every device that loads
// the library, held until the process exits. Host code must not use the
// array's name as a device address: it is a host-side stand-in. The device
// address is asked for with cudaGetSymbolAddress on every call, with the
// caller's device current: a cheap lookup once the module is loaded, and
// never stale, also after cudaDeviceReset or any teardown of the primary
// context reloads the module at another address. The first call on a device
// loads the module there, so it should come before any stream capture.
//
// This file is built without FMA contraction (--fmad=false) so that
// fix_rotation_kernel rounds every product and sum as the host fix_rotation
// does (host code is built with -ffp-contract=off).
#include <cuda_runtime.h>

#include "image_kernels.h"

static __device__ __align__(256) unsigned char rfk_noalloc_scratch[RFK_NOALLOC_SCRATCH_BYTES];

namespace {

// FP64 rewrite of every affine's linear columns to (angle, log magnitude),
// unwrapped across the samples, and of the palette hues across +-180 degrees:
// the same arithmetic as the host fix_rotation (genome.cpp). One thread per
// affine index, then one thread per palette entry.
__global__ void fix_rotation_kernel(double* __restrict__ s, unsigned n, unsigned ss, unsigned fs,
                                    const unsigned* __restrict__ aff, unsigned naff) {
    const double pi = 3.14159265358979323846, eps = 1e-10;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < naff) {
        const unsigned idx = aff[i];
        for (unsigned k = 0; k < n; k++) {
            double* o = s + idx + (size_t)k * ss;
            double ax = atan2(o[1], o[0]), mx = sqrt(o[0] * o[0] + o[1] * o[1]);
            double ay = atan2(o[3], o[2]), my = sqrt(o[2] * o[2] + o[3] * o[3]);
            const bool zx = (mx == 0.0), zy = (my == 0.0);
            if (zx && !zy) ax = ay;
            if (zy && !zx) ay = ax;
            o[0] = ax;
            o[1] = ay;
            o[2] = log(mx);
            o[3] = log(my);
        }
        for (unsigned k = 1; k < n; k++)
            for (unsigned j = 0; j < 2; j++) {
                double* me = s + idx + (size_t)k * ss + j;
                const double d = *me - s[idx + (size_t)(k - 1) * ss + j];
                if (d > pi + eps) *me -= 2 * pi;
                else if (d < -(pi - eps)) *me += 2 * pi;
            }
    }
    const unsigned hue = i;  // palette entry
    if (hue < (ss - fs) / 3) {
        const unsigned col = fs + 3 * hue;
        for (unsigned k = 1; k < n; k++) {
            double* me = s + col + (size_t)k * ss;
            const double d = *me - s[col + (size_t)(k - 1) * ss];
            if (d > 180.0 + eps) *me -= 360.0;
            else if (d < -(180.0 - eps)) *me += 360.0;
        }
    }
}

}  // namespace

extern "C" cudaError_t rfk_noalloc_scratch_address(void** addr, size_t* bytes) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, rfk_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *addr = p;
    *bytes = RFK_NOALLOC_SCRATCH_BYTES;
    return cudaSuccess;
}

extern "C" cudaError_t rfk_launch_fix_rotation(double* samples, unsigned n, unsigned sample_size, unsigned flame_size,
                                               const unsigned* aff, unsigned naff, cudaStream_t s) {
    const unsigned entries = (sample_size - flame_size) / 3;
    const unsigned threads = naff > entries ? naff : entries;
    if (threads == 0) return cudaSuccess;
    fix_rotation_kernel<<<(threads + 127) / 128, 128, 0, s>>>(samples, n, sample_size, flame_size, aff, naff);
    return cudaGetLastError();
}
