// Shared helpers for the sm_103a PPR / PBR kernels: status codes, the
// per-thread last-error string and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <mutex>
#include <cstdio>
#include <string>

#include "graph_link_gb300.h"

namespace gl {

// Per-thread last error text returned by gl_last_error().
void set_error(const char* fmt, ...);
const char* last_error();

// Maps a CUDA runtime error to a status code and records its text.
inline int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return GL_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA;
}

#define GL_CUDA_TRY(expr)                                                   \
    do {                                                                    \
        cudaError_t _e = (expr);                                            \
        if (_e != cudaSuccess) return ::gl::cuda_status(_e, #expr);         \
    } while (0)

#define GL_LAUNCH_CHECK(what)                                               \
    do {                                                                    \
        cudaError_t _e = cudaGetLastError();                                \
        if (_e != cudaSuccess) return ::gl::cuda_status(_e, what);          \
    } while (0)

#define GL_REQUIRE(cond, code, ...)                                         \
    do {                                                                    \
        if (!(cond)) { ::gl::set_error(__VA_ARGS__); return (code); }       \
    } while (0)

// Per-device caches: one slot per device index, filled the first time that
// device asks (under setup_mutex(), with the device current).
constexpr int kMaxDevices = 64;
inline std::mutex& setup_mutex() {
    static std::mutex m;
    return m;
}

// Runs init(&value) once per device (it may set function attributes, which
// are per device, and returns a GL_* status) and caches the positive value
// it produces in cache[device].
template <typename Init>
int per_device_value(std::atomic<int> (&cache)[kMaxDevices], Init init, int* out) {
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    GL_REQUIRE(dev >= 0 && dev < kMaxDevices, GL_ERR_INVALID_ARGUMENT, "device index %d out of range", dev);
    int v = cache[dev].load(std::memory_order_acquire);
    if (v <= 0) {
        std::lock_guard<std::mutex> lock(setup_mutex());
        v = cache[dev].load(std::memory_order_acquire);
        if (v <= 0) {
            const int rc = init(&v);
            if (rc != GL_OK) return rc;
            if (v <= 0) v = 1;
            cache[dev].store(v, std::memory_order_release);
        }
    }
    *out = v;
    return GL_OK;
}

// SM count of the current device (cached per device).
inline int num_sms() {
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 152;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Warp-wide reductions.
// Exact 64-bit minimum over the lanes of `mask` with two 32-bit reductions
// (redux.sync): the high words as signed, then the low words as unsigned
// among the lanes that hold the smallest high word.
__device__ __forceinline__ int64_t group_min_i64(int64_t v, unsigned mask) {
    const int hi = (int)(v >> 32);
    const int mhi = __reduce_min_sync(mask, hi);
    const unsigned lo = hi == mhi ? (unsigned)(uint64_t)v : 0xffffffffu;
    const unsigned mlo = __reduce_min_sync(mask, lo);
    return (int64_t)(((uint64_t)(uint32_t)mhi << 32) | mlo);
}
__device__ __forceinline__ int64_t warp_min_i64(int64_t v) { return group_min_i64(v, 0xffffffffu); }
__device__ __forceinline__ int64_t warp_max_i64(int64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        int64_t w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ uint64_t group_or_u64(uint64_t v, unsigned mask) {
    const unsigned lo = __reduce_or_sync(mask, (unsigned)v);
    const unsigned hi = __reduce_or_sync(mask, (unsigned)(v >> 32));
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ uint64_t warp_or_u64(uint64_t v) { return group_or_u64(v, 0xffffffffu); }
__device__ __forceinline__ int warp_sum_i32(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int64_t warp_sum_i64(int64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Inclusive scan over the warp.
__device__ __forceinline__ int64_t warp_incl_scan_i64(int64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t w = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += w;
    }
    return v;
}

}  // namespace gl
