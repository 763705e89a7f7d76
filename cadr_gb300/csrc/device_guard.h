// device_guard.h - scoped switch of the calling thread's current CUDA device.
//
// Entry points of the C ABI that allocate, create streams or launch on a
// context's device make that device current for the duration of the call
// and give the calling thread its own current device back on every return
// path, success or error.  A caller that works on several devices therefore
// never finds its current device changed by this library.  This is the only
// place in the library that calls cudaSetDevice on a caller's thread.
#pragma once

#include <cuda_runtime.h>

namespace cadr {

class DeviceGuard {
public:
    explicit DeviceGuard(int device)
    {
        if (cudaGetDevice(&prev_) != cudaSuccess) {
            cudaGetLastError();  // no device current yet: nothing to restore
            prev_ = -1;
        }
        if (prev_ != device) {
            err_ = cudaSetDevice(device);
            switched_ = err_ == cudaSuccess && prev_ >= 0;
        }
    }
    ~DeviceGuard()
    {
        if (switched_) cudaSetDevice(prev_);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
    // cudaSuccess, or the error of switching to the requested device.
    cudaError_t error() const { return err_; }

private:
    int prev_ = -1;
    bool switched_ = false;
    cudaError_t err_ = cudaSuccess;
};

}  // namespace cadr
