// Owning device buffer used throughout the native library.
#pragma once
#include "internal.h"
#include "common.cuh"
#include <vector>

namespace wt3d {

template <class T>
struct DevVec {
    T *p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        free();
        if (count == 0) return WT3D_OK;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();   // an allocation failure is not sticky: clear it for later checks
            p = nullptr;
            set_error(std::string("cudaMalloc(") + std::to_string(count * sizeof(T)) + " B): " + cudaGetErrorString(e));
            return WT3D_ERR_NOMEM;
        }
        n = count;
        return WT3D_OK;
    }
    int upload(const std::vector<T> &v)
    {
        int rc = alloc(v.size());
        if (rc) return rc;
        if (!v.empty() && cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("upload failed");
            return WT3D_ERR_CUDA;
        }
        return WT3D_OK;
    }
    void free()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevVec() { free(); }
    DevVec() = default;
    DevVec(const DevVec &) = delete;
    DevVec &operator=(const DevVec &) = delete;
};

// Stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync on one
// stream).  Releasing a cudaMalloc buffer with cudaFree waits for the whole
// device, so a per-call temporary of one handle would wait for another
// handle's factorisation; these buffers are released in the order of their
// own stream instead.  The stream must outlive the buffer's release.
template <class T>
struct StreamBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    int alloc(size_t count, cudaStream_t s)
    {
        release();
        st = s;
        if (count == 0) return WT3D_OK;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            set_error(std::string("cudaMallocAsync(") + std::to_string(count * sizeof(T)) +
                      " B): " + cudaGetErrorString(e));
            return WT3D_ERR_NOMEM;
        }
        n = count;
        return WT3D_OK;
    }
    // host vector in (pageable memory: staged before the call returns)
    int upload(const std::vector<T> &v, cudaStream_t s)
    {
        int rc = alloc(v.size(), s);
        if (rc) return rc;
        if (!v.empty() && cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            set_error("upload failed");
            return WT3D_ERR_CUDA;
        }
        return WT3D_OK;
    }
    void release()
    {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
    }
    ~StreamBuf() { release(); }
    StreamBuf() = default;
    StreamBuf(const StreamBuf &) = delete;
    StreamBuf &operator=(const StreamBuf &) = delete;
};

}  // namespace wt3d
