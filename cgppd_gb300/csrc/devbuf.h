// devbuf.h -- owning device buffer used by the host-side objects of the library.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "status.h"

namespace cgppd {

template <typename T>
struct DevBuf {
    T *ptr = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        n = 0;
    }
    int alloc(size_t count)
    {
        release();
        n = std::max<size_t>(count, 1);
        return cgppd_check(cudaMalloc(&ptr, n * sizeof(T)), "device allocation");
    }
    int upload(const std::vector<T> &v)
    {
        if (alloc(v.size()) != 0)
            return -1;
        if (v.empty())
            return cgppd_check(cudaMemset(ptr, 0, sizeof(T)), "device memset");
        return cgppd_check(cudaMemcpy(ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "device upload");
    }
    int zero(size_t count)
    {
        if (alloc(count) != 0)
            return -1;
        return cgppd_check(cudaMemset(ptr, 0, n * sizeof(T)), "device memset");
    }
};

}  // namespace cgppd
