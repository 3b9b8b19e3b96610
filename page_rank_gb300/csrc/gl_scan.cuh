// Device-wide exclusive scan (sum or max) used by the PBR builder and the
// teleport index.  Recursive reduce-then-scan: each 2048-element tile is
// reduced, the tile totals are scanned (recursively), then every tile is
// scanned again with its carried-in prefix.  Works in place.
#pragma once

#include "gl_common.cuh"

namespace gl {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

struct OpSum {
    template <typename T> __device__ __forceinline__ T operator()(T a, T b) const { return a + b; }
};
struct OpMax {
    template <typename T> __device__ __forceinline__ T operator()(T a, T b) const { return a > b ? a : b; }
};

template <typename T, typename Op>
__device__ __forceinline__ T block_exclusive_scan(T v, T identity, Op op, T* total) {
    __shared__ T warp_tot[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T w = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl = op(incl, w);
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        T x = lane < kScanThreads / 32 ? warp_tot[lane] : identity;
        T xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T w = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi = op(xi, w);
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = xi;  // inclusive over warps
    }
    __syncthreads();
    T warp_prefix = warp > 0 ? warp_tot[warp - 1] : identity;
    T excl_in_warp = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl_in_warp = identity;
    T result = op(warp_prefix, excl_in_warp);
    if (total) *total = warp_tot[kScanThreads / 32 - 1];
    __syncthreads();
    return result;
}

template <typename T, typename Op>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const T* in, int64_t n, T* sums, T identity, Op op) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    T acc = identity;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) acc = op(acc, in[base + i]);
    T total;
    block_exclusive_scan(acc, identity, op, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <typename T, typename Op>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const T* in, T* out, int64_t n, const T* carry, T identity, Op op) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    T v[kScanItems];
    T acc = identity;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? in[base + i] : identity;
        acc = op(acc, v[i]);
    }
    T prefix = block_exclusive_scan(acc, identity, op, (T*)nullptr);
    if (carry) prefix = op(carry[blockIdx.x], prefix);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = prefix;
        prefix = op(prefix, v[i]);
    }
}

// Elements of scratch that exclusive_scan() needs for n inputs.
inline int64_t scan_scratch_elems(int64_t n) {
    int64_t total = 0;
    while (n > kScanTile) {
        n = ceil_div(n, kScanTile);
        total += n;
    }
    return total + 1;
}

template <typename T, typename Op>
int exclusive_scan(const T* in, T* out, int64_t n, T* scratch, T identity, Op op, cudaStream_t stream) {
    if (n <= 0) return GL_OK;
    if (n <= kScanTile) {
        scan_apply_kernel<T, Op><<<1, kScanThreads, 0, stream>>>(in, out, n, nullptr, identity, op);
        GL_LAUNCH_CHECK("scan_apply_kernel");
        return GL_OK;
    }
    const int64_t nb = ceil_div(n, kScanTile);
    T* sums = scratch;
    scan_reduce_kernel<T, Op><<<(unsigned)nb, kScanThreads, 0, stream>>>(in, n, sums, identity, op);
    GL_LAUNCH_CHECK("scan_reduce_kernel");
    int rc = exclusive_scan<T, Op>(sums, sums, nb, scratch + nb, identity, op, stream);
    if (rc != GL_OK) return rc;
    scan_apply_kernel<T, Op><<<(unsigned)nb, kScanThreads, 0, stream>>>(in, out, n, sums, identity, op);
    GL_LAUNCH_CHECK("scan_apply_kernel");
    return GL_OK;
}

}  // namespace gl
