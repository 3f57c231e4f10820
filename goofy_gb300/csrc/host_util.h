// host_util.h -- error reporting and device scoping shared by the host-side
// translation units of the library.
#pragma once
#include <cuda_runtime.h>

#include "../../include/goofy_gpu.h"

#define GOOFY_EXPORT __attribute__((visibility("default")))

namespace goofy_gpu {

// Records `what` and the CUDA error text as the thread's last error and maps
// the CUDA error to a GOOFY_ERR_* status.
int cuda_fail(cudaError_t e, const char* what);

// Records a library-level error message (no CUDA error) and returns `status`.
int fail(int status, const char* what);

// The calling thread's last recorded error message ("" if none).
const char* last_error_text();

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

}  // namespace goofy_gpu

#define GOOFY_CUDA_TRY(call)                                             \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return ::goofy_gpu::cuda_fail(e_, #call); \
    } while (0)
