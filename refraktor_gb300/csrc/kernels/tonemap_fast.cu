// Tonemap under -use_fast_math (see tonemap_impl.cuh): the variant whose
// arithmetic matches the reference's kernel build.
#define RFK_TONEMAP_FAST 1
#include "tonemap_impl.cuh"

extern "C" cudaError_t rfk_launch_tonemap_fast(const float4* bins, unsigned size, void* out, int format, float gamma,
                                               float scale_constant, float brightness, float vibrancy, float highlight_power,
                                               unsigned long long* hist, unsigned long long* max_density,
                                               const unsigned long long* q_hits, double q_per_hit, unsigned blocks,
                                               cudaStream_t s) {
    switch (format) {
    case 0: rfk_tm::launch<true, 3>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    case 1: rfk_tm::launch<true, 4>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    case 2: rfk_tm::launch<false, 3>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    case 3: rfk_tm::launch<false, 4>(blocks, s, bins, out, size, gamma, scale_constant, brightness, vibrancy, highlight_power, hist, max_density, q_hits, q_per_hit); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
