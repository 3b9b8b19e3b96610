// Launch-shape selection for stripe_kernel (included by the per-type
// translation units stripe_f32.cu / stripe_f64.cu).
#pragma once

#include "stripe_kernel.cuh"

namespace gl {

template <typename S, int BR, int V, int C, bool PPR>
int launch_stripe_shape(const StripeArgs<S>& a0, cudaStream_t stream) {
    StripeArgs<S> a = a0;
    constexpr int T = C * V;
    a.ntiles = (int)ceil_div(a.K, T);
    const int64_t units = (int64_t)a.num_pieces + a.nstripes;
    const int64_t items = units * a.batch * (int64_t)a.ntiles;
    if (items == 0) return GL_OK;
    auto kern = stripe_kernel<S, BR, BR, V, C, PPR>;
    constexpr size_t base = StripeSmem<S, BR, V, C>::bytes;
    // power-iteration steps with up to kCtaSumCols columns gather their
    // per-column sums per CTA (2 * K doubles of shared memory)
    constexpr int64_t kCtaSumCols = 512;
    a.cta_sums = (PPR && a.K <= kCtaSumCols) ? 1 : 0;
#ifndef GL_WINDOW_DRAW
#define GL_WINDOW_DRAW 1
#endif
    // light stripes are drawn window by window (L1 reuse of the diagonal
    // block's X rows within a CTA)
    a.win_draw = (GL_WINDOW_DRAW && a.sched != nullptr) ? 1 : 0;
    const size_t smem = base + (a.cta_sums ? (size_t)(2 * a.K) * sizeof(double) : 0);
    // the shared-memory attribute is per device, so it is set (and the
    // occupancy measured) once for every device that launches this instance
    static std::atomic<int> occ_cache[kMaxDevices];
    int occ = 0;
    const int rc = per_device_value(
        occ_cache,
        [&](int* o) {
            const size_t most = base + (PPR ? (size_t)(2 * kCtaSumCols) * sizeof(double) : 0);
            GL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most));
            GL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, kern, kStripeThreads, most));
            return GL_OK;
        },
        &occ);
    if (rc != GL_OK) return rc;
    int64_t blocks = ceil_div(items, kStripeWarps);
    const int64_t cap = (int64_t)num_sms() * occ;
    if (blocks > cap) blocks = cap;
    kern<<<(unsigned)blocks, kStripeThreads, smem, stream>>>(a);
    GL_LAUNCH_CHECK("stripe_kernel");
    return GL_OK;
}

inline bool aligned_to(const void* p, int bytes) { return (reinterpret_cast<uintptr_t>(p) % bytes) == 0; }

// Vector width and column lanes for K columns.  tile_hint (0 = automatic)
// caps the tile width T = C * V, e.g. 64 instead of 128 for K = 256.
struct Shape {
    int V, C;
};

template <typename S>
Shape pick_shape(int64_t K, int tile_hint, const void* X, const void* Y, bool allow_half_warps = true,
                 int lane_split = 0) {
    auto vec_ok = [&](int v) {
        return K % v == 0 && aligned_to(X, v * (int)sizeof(S)) && aligned_to(Y, v * (int)sizeof(S));
    };
    const int max_v = sizeof(S) == 4 ? 4 : 2;
    int cap = tile_hint > 0 ? tile_hint : 1 << 30;
    if (sizeof(S) == 8 && K < 17) return {1, 1};   // FP64 instantiates only C = 1 below 17 columns
    // 64 <= K < 128 (FP32): two half-warps with float4 lanes each cover 64
    // columns and take alternate nonzeros (the default; lane_split 1 keeps
    // all 32 lanes on each nonzero)
    if (allow_half_warps && lane_split != 1 && sizeof(S) == 4 && K >= 64 && K < 128 && 64 <= cap && vec_ok(4))
        return {4, 16};
    if (K >= 32) {
        for (int v = max_v; v >= 1; v >>= 1)
            if (K >= 32 * v && 32 * v <= cap && vec_ok(v)) return {v, 32};
        return {1, 32};
    }
    int c = 1;
    while (c < K) c <<= 1;   // K <= 31 here: C = next power of two >= K, V = 1
    if (c > 32) c = 32;
    while (c > 1 && c > cap) c >>= 1;
    return {1, c};
}

template <typename S>
int stripe_tile_width(int64_t K, int tile_hint, const void* X, const void* Y) {
    const Shape sh = pick_shape<S>(K, tile_hint, X, Y);
    return sh.V * sh.C;
}

}  // namespace gl
