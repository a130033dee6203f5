// device_util.cuh -- CUDA helpers shared by the library's .cu files.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.hpp"

namespace accspmm {

#define ACC_CUDA(call)                                                          \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess)                                                  \
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "%s failed: %s (%s:%d)", #call,       \
                     cudaGetErrorString(e_), __FILE__, __LINE__);               \
    } while (0)

// Checks the launch that was just enqueued.
#define ACC_LAUNCH_CHECK()                                                      \
    do {                                                                        \
        cudaError_t e_ = cudaGetLastError();                                    \
        if (e_ != cudaSuccess)                                                  \
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "kernel launch failed: %s (%s:%d)",    \
                     cudaGetErrorString(e_), __FILE__, __LINE__);               \
    } while (0)

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int sm_count();

// The current device's library memory pool (spmm_host.cpp): it keeps freed
// memory for later allocations instead of returning it at each synchronize.
int library_pool(cudaMemPool_t* pool);

// Stream-ordered device buffer from the library pool that frees itself at
// scope exit.
template <class T>
struct DevBuf {
    T* p = nullptr;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { reset(); }
    cudaError_t alloc(size_t n, cudaStream_t st) {
        reset();
        s = st;
        // a stream being captured into a graph allocates from the device's
        // current pool, as before the library pool existed (creating that
        // pool and its copy streams in the middle of a capture could end
        // the capture); so does a call whose library pool cannot be created
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaMemPool_t pool;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone &&
            library_pool(&pool) == ACCSPMM_SUCCESS)
            return cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), sizeof(T) * (n ? n : 1), pool, st);
        return cudaMallocAsync(reinterpret_cast<void**>(&p), sizeof(T) * (n ? n : 1), st);
    }
    void reset() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
    }
    T* release() {
        T* q = p;
        p = nullptr;
        return q;
    }
};

__host__ __device__ inline uint32_t ceil_div_u32(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace accspmm
