// Minimal owning device buffer.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

namespace smc {

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // grow-only; contents are not preserved
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    cudaError_t upload(const T *h, size_t count, cudaStream_t s) {
        cudaError_t e = ensure(count);
        if (e != cudaSuccess) return e;
        if (count == 0) return cudaSuccess;
        return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
    }
    cudaError_t upload(const std::vector<T> &v, cudaStream_t s) { return upload(v.data(), v.size(), s); }
};

}  // namespace smc
