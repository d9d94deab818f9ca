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

}  // namespace wt3d
