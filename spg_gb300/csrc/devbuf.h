// Owning device buffer and upload helpers for the solver handles.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <string>
#include <vector>

#include "api_internal.h"

namespace spgx {

class DevBuf {
public:
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }

    spgx_status alloc(size_t bytes)
    {
        release();
        if (bytes == 0) bytes = 16;
        SPGX_CUDA(cudaMalloc(&ptr_, bytes));
        bytes_ = bytes;
        return SPGX_OK;
    }
    void release()
    {
        if (ptr_) cudaFree(ptr_);
        ptr_ = nullptr;
        bytes_ = 0;
    }
    template <typename T>
    spgx_status upload(const std::vector<T> &v)
    {
        SPGX_TRY_STATUS(alloc(v.size() * sizeof(T)));
        if (!v.empty()) SPGX_CUDA(cudaMemcpy(ptr_, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return SPGX_OK;
    }
    template <typename T>
    T *as() const
    {
        return static_cast<T *>(ptr_);
    }
    size_t bytes() const { return bytes_; }

private:
    void *ptr_{nullptr};
    size_t bytes_{0};
};

// Pinned host staging buffer.
class HostBuf {
public:
    HostBuf() = default;
    HostBuf(const HostBuf &) = delete;
    HostBuf &operator=(const HostBuf &) = delete;
    ~HostBuf()
    {
        if (ptr_) cudaFreeHost(ptr_);
    }
    spgx_status alloc(size_t bytes)
    {
        if (ptr_) cudaFreeHost(ptr_);
        ptr_ = nullptr;
        if (bytes == 0) bytes = 16;
        SPGX_CUDA(cudaMallocHost(&ptr_, bytes));
        bytes_ = bytes;
        return SPGX_OK;
    }
    template <typename T>
    T *as() const
    {
        return static_cast<T *>(ptr_);
    }
    size_t bytes() const { return bytes_; }

private:
    void *ptr_{nullptr};
    size_t bytes_{0};
};

// Checks that the requested device exists and is a compute capability 10.3 part.
inline spgx_status select_device(int device)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return SPGX_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) {
        set_error("invalid CUDA device ordinal");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    SPGX_CUDA(cudaGetDeviceProperties(&prop, device));
    if (!(prop.major == 10 && prop.minor == 3)) {
        set_error("spgx is built for sm_103a (GB300); device " + std::to_string(device) + " is sm_" +
                  std::to_string(prop.major) + std::to_string(prop.minor));
        return SPGX_ERR_NO_DEVICE;
    }
    return SPGX_OK;
}

}  // namespace spgx
