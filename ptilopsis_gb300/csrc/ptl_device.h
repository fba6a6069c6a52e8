// Current-device handling shared by the C-ABI entry points.
#pragma once

#include <cuda_runtime.h>

namespace ptl {

// Makes `device` current for the life of the scope and then gives the calling thread its
// previous current device back, so an entry point leaves the caller's thread as it found it.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            prev = -1;
            cudaGetLastError();
        }
        if (prev != device) err = cudaSetDevice(device);
    }
    ~DeviceScope() {
        if (prev >= 0 && err == cudaSuccess) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
    bool ok() const { return err == cudaSuccess; }
};

}  // namespace ptl
