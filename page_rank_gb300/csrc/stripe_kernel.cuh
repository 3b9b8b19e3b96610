// Stripe-owning fused PBR-block + CSR-remainder kernel (sm_103a).
//
// One "group" of G lanes owns one output stripe (block_rows consecutive rows)
// for one column tile of T = G * V columns; each lane owns V consecutive
// columns and keeps block_rows x V accumulators in registers.  For every
// block of the stripe the lane stages the X rows of the block's active
// columns (one vector load per column) in its own shared-memory slots, then
// walks the set bits of the 64-bit code row by row; the packed values are in
// row-major bit order, so the value index is a running counter.  The CSR
// remainder rows of the stripe are then added by the same lane, and the tile
// is written once: no atomics, no pre-zeroed output, no second stream.
//
// With PPR = true the epilogue is one power-iteration step instead of a plain
// store: X_out = alpha * (A X_in) + scale_k * teleport, the L1 change per
// column and the dangling mass of X_out are accumulated in the same pass.
//
// The reference splits this work over two kernels on two streams with global
// atomics (kernels/pbr_kernel.cu:12-333 block kernels, :421-458 CSR kernel,
// bindings/bindings_kernels.cu:34-80 stream fork/join) and a separate update
// pass (kernels/ppr_kernel.cu:130-168).
#pragma once

#include "gl_common.cuh"

namespace gl {

constexpr int kStripeThreads = 256;

template <typename S, int V>
struct alignas(sizeof(S) * V) Pack {
    S v[V];
};

template <typename S>
struct StripeArgs {
    const int64_t* codes;
    const int32_t* coords;
    const int32_t* offsets;
    const S* bdata;
    const int32_t* rem_ptr;
    const int32_t* rem_col;
    const S* rem_val;
    const int32_t* stripe_ptr;
    int64_t rows, cols, nstripes, batch;
    int32_t K, ntiles;
    const S* X;
    S* Y;
    // power-iteration epilogue
    const int32_t* tp_ptr;
    const int32_t* tp_row;
    const int32_t* tp_col;
    const float* tp_w;
    double alpha, tol;
    int32_t stop_mode, max_iter, step;
    const int32_t* chunk_base;
    double* res_hist;
    double* dang_hist;
    const uint32_t* dbitmap;
};

template <typename S, int V>
__device__ __forceinline__ Pack<S, V> load_pack(const S* p) {
    return *reinterpret_cast<const Pack<S, V>*>(p);
}
template <typename S, int V>
__device__ __forceinline__ void store_pack(S* p, const Pack<S, V>& v) {
    *reinterpret_cast<Pack<S, V>*>(p) = v;
}

template <typename S, int BR, int BC, int V, int G, bool PPR>
__global__ void __launch_bounds__(kStripeThreads)
stripe_kernel(const StripeArgs<S> a) {
    constexpr int T = G * V;            // columns per group
    constexpr int GPW = 32 / G;         // groups per warp
    constexpr uint32_t ROWMASK = (BC >= 32) ? 0xffffffffu : ((1u << BC) - 1u);

    __shared__ Pack<S, V> xs[BC][kStripeThreads];
    __shared__ int s_skip;

    const int lane = threadIdx.x & 31;
    const int gl_lane = lane % G;
    const int64_t gid = ((int64_t)blockIdx.x * (kStripeThreads / 32) + (threadIdx.x >> 5)) * GPW + lane / G;
    const int64_t ngroups = (int64_t)gridDim.x * (kStripeThreads / 32) * GPW;
    const int64_t BT = a.batch * a.ntiles;
    const int64_t items = a.nstripes * BT;

    int t = 0;
    if constexpr (PPR) {
        t = *a.chunk_base + a.step;
        if (t >= a.max_iter) return;
        if (a.stop_mode == GL_PPR_STOP_ALL && t > 0) {
            if (threadIdx.x < 32) {
                double m = 0.0;
                const double* prev = a.res_hist + (int64_t)(t - 1) * a.K;
                for (int k = lane; k < a.K; k += 32) m = fmax(m, prev[k]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
                if (lane == 0) s_skip = (m < a.tol) ? 1 : 0;
            }
            __syncthreads();
            if (s_skip) return;
        }
    }

    const S alpha = static_cast<S>(a.alpha);
    int64_t cur_bt = -1;
    int cur_col = 0;
    bool cur_ok = false;
    S scale[V];
    bool frozen[V];
    float res_acc[V];
    float dang_acc[V];
#pragma unroll
    for (int j = 0; j < V; ++j) { scale[j] = S(0); frozen[j] = false; res_acc[j] = 0.f; dang_acc[j] = 0.f; }

    auto flush = [&]() {
        if constexpr (PPR) {
            if (cur_bt >= 0 && cur_ok) {
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    const int col = cur_col + j;
                    if (res_acc[j] != 0.f) atomicAdd(a.res_hist + (int64_t)t * a.K + col, (double)res_acc[j]);
                    if (a.dbitmap != nullptr && dang_acc[j] != 0.f)
                        atomicAdd(a.dang_hist + (int64_t)(t + 1) * a.K + col, (double)dang_acc[j]);
                    res_acc[j] = 0.f;
                    dang_acc[j] = 0.f;
                }
            }
        }
    };

    for (int64_t item = gid; item < items; item += ngroups) {
        const int64_t s = item / BT;
        const int64_t bt = item - s * BT;
        const int64_t b = bt / a.ntiles;
        const int tile = (int)(bt - b * a.ntiles);
        const int col_base = tile * T + gl_lane * V;
        const bool lane_ok = col_base < a.K;

        if constexpr (PPR) {
            if (bt != cur_bt) {
                flush();
                cur_bt = bt;
                cur_col = col_base;
                cur_ok = lane_ok;
                if (lane_ok) {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const int col = col_base + j;
                        double sc = 1.0 - a.alpha;
                        if (a.dbitmap != nullptr) sc += a.alpha * a.dang_hist[(int64_t)t * a.K + col];
                        scale[j] = static_cast<S>(sc);
                        frozen[j] = (a.stop_mode == GL_PPR_STOP_PER_COLUMN && t > 0 &&
                                     a.res_hist[(int64_t)(t - 1) * a.K + col] < a.tol);
                    }
                }
            }
        }

        S acc[BR][V];
#pragma unroll
        for (int r = 0; r < BR; ++r)
#pragma unroll
            for (int j = 0; j < V; ++j) acc[r][j] = S(0);

        const S* __restrict__ Xb = a.X + b * a.cols * (int64_t)a.K + col_base;

        // ---- PBR blocks of this stripe ------------------------------------
        const int32_t kb0 = a.stripe_ptr[s];
        const int32_t kb1 = a.stripe_ptr[s + 1];
        for (int32_t kb = kb0; kb < kb1; ++kb) {
            const uint64_t code = static_cast<uint64_t>(a.codes[kb]);
            const int64_t col0 = a.coords[2 * (int64_t)kb + 1];
            int32_t k = a.offsets[kb];
            uint32_t colmask = 0;
#pragma unroll
            for (int r = 0; r < BR; ++r) colmask |= (uint32_t)(code >> (r * BC)) & ROWMASK;
            if (lane_ok) {
#pragma unroll
                for (int c = 0; c < BC; ++c)
                    if ((colmask >> c) & 1u)
                        xs[c][threadIdx.x] = load_pack<S, V>(Xb + (col0 + c) * a.K);
            }
#pragma unroll
            for (int r = 0; r < BR; ++r) {
                uint32_t bits = (uint32_t)(code >> (r * BC)) & ROWMASK;
                while (bits) {
                    const int c = __ffs(bits) - 1;
                    bits &= bits - 1u;
                    const S v = a.bdata[k++];
                    if (lane_ok) {
                        const Pack<S, V> x = xs[c][threadIdx.x];
#pragma unroll
                        for (int j = 0; j < V; ++j) acc[r][j] = fma(v, x.v[j], acc[r][j]);
                    }
                }
            }
        }

        // ---- CSR remainder rows of this stripe ------------------------------
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            const int64_t row = s * BR + r;
            if (row < a.rows) {
                int32_t j = a.rem_ptr[row];
                const int32_t je = a.rem_ptr[row + 1];
                for (; j + 4 <= je; j += 4) {
                    const int64_t c0 = a.rem_col[j], c1 = a.rem_col[j + 1];
                    const int64_t c2 = a.rem_col[j + 2], c3 = a.rem_col[j + 3];
                    const S v0 = a.rem_val[j], v1 = a.rem_val[j + 1];
                    const S v2 = a.rem_val[j + 2], v3 = a.rem_val[j + 3];
                    if (lane_ok) {
                        const Pack<S, V> x0 = load_pack<S, V>(Xb + c0 * a.K);
                        const Pack<S, V> x1 = load_pack<S, V>(Xb + c1 * a.K);
                        const Pack<S, V> x2 = load_pack<S, V>(Xb + c2 * a.K);
                        const Pack<S, V> x3 = load_pack<S, V>(Xb + c3 * a.K);
#pragma unroll
                        for (int q = 0; q < V; ++q) {
                            acc[r][q] = fma(v0, x0.v[q], acc[r][q]);
                            acc[r][q] = fma(v1, x1.v[q], acc[r][q]);
                            acc[r][q] = fma(v2, x2.v[q], acc[r][q]);
                            acc[r][q] = fma(v3, x3.v[q], acc[r][q]);
                        }
                    }
                }
                for (; j < je; ++j) {
                    const int64_t c0 = a.rem_col[j];
                    const S v0 = a.rem_val[j];
                    if (lane_ok) {
                        const Pack<S, V> x0 = load_pack<S, V>(Xb + c0 * a.K);
#pragma unroll
                        for (int q = 0; q < V; ++q) acc[r][q] = fma(v0, x0.v[q], acc[r][q]);
                    }
                }
            }
        }

        if (!lane_ok) continue;

        if constexpr (!PPR) {
            S* Yb = a.Y + (b * a.rows) * (int64_t)a.K + col_base;
#pragma unroll
            for (int r = 0; r < BR; ++r) {
                const int64_t row = s * BR + r;
                if (row < a.rows) {
                    Pack<S, V> o;
#pragma unroll
                    for (int j = 0; j < V; ++j) o.v[j] = acc[r][j];
                    store_pack<S, V>(Yb + row * a.K, o);
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < BR; ++r)
#pragma unroll
                for (int j = 0; j < V; ++j) acc[r][j] *= alpha;
            // teleport entries of this stripe that fall in this lane's columns
            const int32_t e0 = a.tp_ptr[s], e1 = a.tp_ptr[s + 1];
            for (int32_t e = e0; e < e1; ++e) {
                const int rr = a.tp_row[e] - (int)(s * BR);
                const int cc = a.tp_col[e] - col_base;
                if (cc >= 0 && cc < V) {
                    const S w = static_cast<S>(a.tp_w[e]);
#pragma unroll
                    for (int r = 0; r < BR; ++r)
#pragma unroll
                        for (int j = 0; j < V; ++j)
                            if (r == rr && j == cc) acc[r][j] = fma(w, scale[j], acc[r][j]);
                }
            }
            const S* Xin = a.X + col_base;
            S* Xout = a.Y + col_base;
#pragma unroll
            for (int r = 0; r < BR; ++r) {
                const int64_t row = s * BR + r;
                if (row < a.rows) {
                    const Pack<S, V> old = load_pack<S, V>(Xin + row * a.K);
                    const bool dang = a.dbitmap != nullptr &&
                                      ((a.dbitmap[row >> 5] >> (row & 31)) & 1u);
                    Pack<S, V> o;
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const S nv = frozen[j] ? old.v[j] : acc[r][j];
                        o.v[j] = nv;
                        res_acc[j] += (float)fabs(nv - old.v[j]);
                        if (dang) dang_acc[j] += (float)nv;
                    }
                    store_pack<S, V>(Xout + row * a.K, o);
                }
            }
        }
    }
    flush();
}

// Host-side launcher for one (S, PPR) family; picks block shape, vector
// width and group width.  Returns a GL_* status.
template <typename S, bool PPR>
int launch_stripe(const StripeArgs<S>& a0, int block_rows, int block_cols, cudaStream_t stream);

}  // namespace gl
