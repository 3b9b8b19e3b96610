// Launch-shape selection for stripe_kernel (included by the per-type
// translation units stripe_f32.cu / stripe_f64.cu).
#pragma once

#include "stripe_kernel.cuh"

namespace gl {

template <typename S, int BR, int V, int G, bool PPR>
int launch_stripe_shape(const StripeArgs<S>& a0, cudaStream_t stream) {
    StripeArgs<S> a = a0;
    constexpr int T = G * V;
    a.ntiles = (int)ceil_div(a.K, T);
    const int64_t items = a.nstripes * a.batch * (int64_t)a.ntiles;
    if (items == 0) return GL_OK;
    auto kern = stripe_kernel<S, BR, BR, V, G, PPR>;
    static int occ = 0;
    if (occ == 0) {
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, kStripeThreads, 0);
        occ = o > 0 ? o : 1;
    }
    const int64_t groups_per_block = (kStripeThreads / 32) * (32 / G);
    int64_t blocks = ceil_div(items, groups_per_block);
    const int64_t cap = (int64_t)num_sms() * occ;
    if (blocks > cap) blocks = cap;
    kern<<<(unsigned)blocks, kStripeThreads, 0, stream>>>(a);
    GL_LAUNCH_CHECK("stripe_kernel");
    return GL_OK;
}

inline bool aligned_to(const void* p, int bytes) { return (reinterpret_cast<uintptr_t>(p) % bytes) == 0; }

// Widest vector the column count and both pointers allow.
template <typename S>
int pick_vec(const StripeArgs<S>& a, int want) {
    int v = want;
    while (v > 1 && (a.K % v != 0 || !aligned_to(a.X, v * (int)sizeof(S)) || !aligned_to(a.Y, v * (int)sizeof(S))))
        v >>= 1;
    return v;
}

}  // namespace gl
