// Internals shared by the librfk runtime translation units (runtime.cpp,
// batch.cpp): error handling, device queries and the handle types behind the
// opaque pointers of rfk.h.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <stdexcept>
#include <string>

#include "../../../include/rfk.h"
#include "codegen.h"
#include "flamedb.h"
#include "genome.h"

namespace rfk::rt {

// Message of the calling thread's last failed call (rfk_last_error).
std::string& error_message();


struct rfk_exception : std::runtime_error {
    rfk_status code;
    rfk_exception(rfk_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(rfk_status c, const std::string& m) { throw rfk_exception(c, m); }

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) fail(RFK_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}


template <typename F>
rfk_status guard(F&& f) {
    try {
        error_message().clear();
        f();
        return RFK_OK;
    } catch (const rfk_exception& e) {
        error_message() = e.what();
        return e.code;
    } catch (const rfk::format_error& e) {
        error_message() = e.what();
        return RFK_E_FORMAT;
    } catch (const rfk::dsl::parse_error& e) {
        error_message() = e.what();
        return RFK_E_FORMAT;
    } catch (const std::bad_alloc&) {
        error_message() = "out of host memory";
        return RFK_E_INVALID;
    } catch (const std::exception& e) {
        error_message() = e.what();
        return RFK_E_INVALID;
    }
}

inline int device_sm_count() {
    int dev = 0, n = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    cuda_check(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    return n;
}

inline std::string device_arch() {
    int dev = 0, major = 0, minor = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) fail(RFK_E_NODEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    cuda_check(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev), "compute capability");
    cuda_check(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev), "compute capability");
    if (major < 10) fail(RFK_E_NODEVICE, "device compute capability " + std::to_string(major) + "." + std::to_string(minor) +
                                             " is below the sm_100 family this library targets");
    return "sm_" + std::to_string(major) + std::to_string(minor) + "a";
}


// Launches an NVRTC-built kernel with the runtime API.
inline void launch(cudaKernel_t fn, unsigned grid, unsigned block, cudaStream_t s, void** args, const char* what) {
    cuda_check(cudaLaunchKernel(reinterpret_cast<const void*>(fn), dim3(grid), dim3(block), args, 0, s), what);
}

}  // namespace rfk::rt

// ------------------------------------------------------------------ handles --
struct rfk_db {
    rfk::flamedb db;
};

struct rfk_flame {
    rfk::flame f;
};

struct kernel_impl {
    rfk::generated_flame gen;
    std::string source;
    std::string log;
    cudaLibrary_t lib = nullptr;
    cudaKernel_t f_prepare = nullptr, f_warmup = nullptr, f_bin = nullptr, f_apply = nullptr, f_bin_batch = nullptr,
                 f_bin_tm = nullptr;
    int block = 256, cpt = 1, flush = 0, sort = 0, grid = 0, regs = 0;
    size_t sample_floats = 0;
    double compile_ms = 0.0;
    double sfu_per_iter = 0.0;
    double fma_per_iter = 0.0;
    uint32_t salt = 0;
    ~kernel_impl() {
        if (lib) cudaLibraryUnload(lib);
    }
};

struct rfk_kernel {
    std::shared_ptr<kernel_impl> impl;
};
