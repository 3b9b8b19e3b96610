// Window-solve warm start: exact solves inside 64-row windows of the node
// order, for the start vector of batched PPR.
//
// The PPR fixed point solves (I - alpha A) x = (1 - alpha) v.  Split A into
// its 64 x 64 diagonal window blocks A_w and the rest M (edges that leave
// their window): with B = I - alpha blockdiag(A_w),
//
//   x = (1 - alpha) sum_k y_k,   y_0 = B^-1 v,   y_k = B^-1 (alpha M y_{k-1}),
//
// a series whose terms are non-negative and whose k-th term carries the mass
// of walks that left their window k times.  Its first few terms are computed
// exactly here (the windows' inverses are dense 64 x 64 matrices, built once
// per graph and damping factor); the mass the truncated series misses is
// placed along a far-field shape supplied by the caller.  The power
// iteration then runs from that vector to the usual certified tolerance, so
// the fixed point does not depend on the start.
//
// B is strictly column diagonally dominant when A's columns sum to at most
// one and alpha < 1 (|1 - alpha a_jj| > alpha sum_{i != j} a_ij), so
// Gauss-Jordan elimination without pivoting is stable and every pivot is
// positive; a pivot that is not (a matrix outside that class) is reported
// through the status word.
//
// The reference has no warm start: its iterate starts from the seed
// indicators (init_ppr_sources_kernel, Backend/graph_link/kernels/
// ppr_kernel.cu:199-209).
#include "gl_common.cuh"

namespace gl {
namespace {

constexpr int kWin = 64;          // window rows (and columns of a window block)
constexpr int kBlk = kWin * kWin;
constexpr int kThreads = 256;

inline unsigned grid_for(int64_t items, int per_sm) {
    const int64_t cap = (int64_t)num_sms() * per_sm;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(items, cap));
}

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gthreads() { return (int64_t)gridDim.x * blockDim.x; }

// blocks[w] = identity
__global__ void window_identity_kernel(float* __restrict__ blocks, int64_t total) {
    for (int64_t i = gtid(); i < total; i += gthreads()) {
        const int e = (int)(i & (kBlk - 1));
        blocks[i] = (e >> 6) == (e & 63) ? 1.0f : 0.0f;
    }
}

// blocks[w][r][c] -= alpha A[row][col] for the entries of a row whose column
// lies in the row's own window; warp per row (duplicate columns add up).
__global__ void window_blocks_kernel(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                     const float* __restrict__ data, int64_t n, float alpha,
                                     float* __restrict__ blocks) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = gthreads() >> 5;
    for (int64_t r = gtid() >> 5; r < n; r += nw) {
        const int64_t w0 = r & ~(int64_t)(kWin - 1);
        float* row = blocks + (r >> 6) * kBlk + (r & (kWin - 1)) * kWin;
        for (int32_t j = indptr[r] + lane; j < indptr[r + 1]; j += 32) {
            const int64_t c = indices[j];
            if (c >= w0 && c < w0 + kWin) atomicAdd(row + (c - w0), -alpha * data[j]);
        }
    }
}

// In-place Gauss-Jordan inversion of each 64 x 64 block, one CTA per block
// at a time.  Per pivot k: scale row k, eliminate column k from the other
// rows, then write column k of the inverse.  The inverse is stored
// transposed (element (r, q) at q * 64 + r), the layout the apply reads:
// for each q, the 64 rows' coefficients are contiguous.
__global__ void __launch_bounds__(kThreads) window_invert_kernel(float* __restrict__ blocks, int64_t windows,
                                                                 int32_t* __restrict__ status) {
    __shared__ float M[kWin][kWin + 1];
    const int t = threadIdx.x;
    for (int64_t w = blockIdx.x; w < windows; w += gridDim.x) {
        float* g = blocks + w * kBlk;
        __syncthreads();
        for (int i = t; i < kBlk; i += kThreads) M[i >> 6][i & 63] = g[i];
        __syncthreads();
        bool bad = false;
        for (int k = 0; k < kWin; ++k) {
            const float p = M[k][k];
            bad |= !(p > 1e-30f) || !isfinite(p);
            const float piv = 1.0f / p;
            if (t < kWin && t != k) M[k][t] *= piv;
            __syncthreads();
            for (int e = t; e < kBlk; e += kThreads) {
                const int i = e >> 6, j = e & 63;
                if (i != k && j != k) M[i][j] = fmaf(-M[i][k], M[k][j], M[i][j]);
            }
            __syncthreads();
            if (t < kWin) M[t][k] = t == k ? piv : -M[t][k] * piv;
            __syncthreads();
        }
        for (int i = t; i < kBlk; i += kThreads) g[i] = M[i & 63][i >> 6];
        if (bad && t == 0) atomicExch(status, 1);
    }
}

struct ApplyArgs {
    const float* inv;      // [windows][64 (q)][64 (r)]: the inverses, transposed
    const float* T;        // [n][K]
    float* Y;              // [n][K] or null
    float* nf;             // near field [n][K] or null
    float* partial;        // [windows][K] column sums of near_scale * Y per window, or null
    int64_t n;
    int K;
    float scale;           // Y = scale * inv_w T_w
    float near_scale;      // nf (+)= near_scale * Y
    int near_init;         // 1: nf = ..., partial = ...; 0: nf += ..., partial += ...
    int vec;               // K % 4 == 0 and T / Y / nf 16-byte aligned
};

// Thread layout of the apply for a column tile of TW columns: 128 threads as
// RG row groups x CG column groups; a thread owns RM rows x CN columns of the
// 64 x TW output tile (with CN = 8 its columns are two runs of four, cg * 4
// and TW / 2 + cg * 4, so a warp's shared-memory reads stay contiguous).
// Tuning (measured on the 2**21-node graph, 256 columns, one apply, same
// box): 64-column tiles (8 x 4 patches) at 6 CTAs per SM 2.25 ms (2.27
// without the row padding); 7 CTAs (register cap 72: a spill) 3.22 ms;
// 32-column tiles at 8 CTAs 2.56 ms; 128-column tiles (8 x 8 patches, 123
// registers, 4 CTAs) 2.70 ms; a cp.async double-buffered 128-column kernel
// (2 CTAs) 3.46 ms, the same at 64 columns (3 CTAs) 2.81 ms: resident warps
// matter more than overlapping one CTA's copies.
#ifndef GL_WIN_APPLY_MAXTW
#define GL_WIN_APPLY_MAXTW 64        // widest column tile used
#endif
#ifndef GL_WIN_APPLY_PAD
#define GL_WIN_APPLY_PAD 4           // floats of padding per shared-memory row
#endif
#ifndef GL_WIN_APPLY_CTAS
#define GL_WIN_APPLY_CTAS 6          // resident CTAs per SM for tiles of <= 64 columns
#endif
constexpr int kApplyThreads = 128;
constexpr int kLdI = kWin + GL_WIN_APPLY_PAD;    // inverse row in shared memory (floats)
template <int TW>
struct ApplyShape {
    static constexpr int CN = TW >= 128 ? 8 : 4;
    static constexpr int CG = TW / CN;
    static constexpr int RG = kApplyThreads / CG;
    static constexpr int RM = kWin / RG;
    static constexpr int LDT = TW + GL_WIN_APPLY_PAD;  // tile row (floats)
    static constexpr int CTAS = TW >= 128 ? 4 : GL_WIN_APPLY_CTAS;
    static constexpr int SMEM = (kWin * kLdI + kWin * LDT) * 4;
    static_assert(CG * CN == TW && RG * CG == kApplyThreads && RM * RG == kWin, "layout");
    static_assert(RG * TW <= kWin * LDT, "column sums fit in the tile");
};

template <int RM>
__device__ __forceinline__ void load_rows(const float* p, float (&a)[RM]) {
    if constexpr (RM % 4 == 0) {
#pragma unroll
        for (int i = 0; i < RM; i += 4) {
            const float4 v = *reinterpret_cast<const float4*>(p + i);
            a[i] = v.x; a[i + 1] = v.y; a[i + 2] = v.z; a[i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < RM; ++i) a[i] = p[i];
    }
}

// Y_w = scale * inv_w @ T_w for every window w and column tile of TW: the
// window's inverse is held transposed in shared memory (invT[q][r]), the
// T tile beside it; each thread accumulates its RM x CN patch over the 64
// rows q of the window, then writes Y / the near field and the tile's
// per-window column sums.
template <int TW>
__global__ void __launch_bounds__(kApplyThreads, ApplyShape<TW>::CTAS) window_apply_kernel(ApplyArgs a,
                                                                                          int64_t windows) {
    using S = ApplyShape<TW>;
    constexpr int RM = S::RM, CN = S::CN, CG = S::CG, RG = S::RG, LDT = S::LDT;
    extern __shared__ __align__(16) float smem[];
    float* invT = smem;                    // [64 q][kLdI]: the inverse, transposed
    float* Ts = smem + kWin * kLdI;        // [64][LDT]; reused for the column sums
    const int t = threadIdx.x, rg = t / CG, cg = t % CG;
    const int64_t K = a.K;
    int cols[CN];
#pragma unroll
    for (int j = 0; j < CN; ++j) cols[j] = (CN == 8 && j >= 4) ? TW / 2 + cg * 4 + (j - 4) : cg * 4 + (j & 3);
    for (int64_t w = blockIdx.x; w < windows; w += gridDim.x) {
        const float* g = a.inv + w * kBlk;
        const int64_t row0 = w * kWin;
        const int rows = (int)min((int64_t)kWin, a.n - row0);
        __syncthreads();                                   // the previous window is done with invT
        for (int i = t * 4; i < kBlk; i += kApplyThreads * 4)
            *reinterpret_cast<float4*>(invT + (i >> 6) * kLdI + (i & 63)) = *reinterpret_cast<const float4*>(g + i);
        for (int64_t c0 = 0; c0 < K; c0 += TW) {
            const int tw = (int)min((int64_t)TW, K - c0);
            __syncthreads();                               // Ts is free, invT is written
            if (a.vec && tw == TW) {
                constexpr int F4 = TW / 4;
                for (int i = t; i < kWin * F4; i += kApplyThreads) {
                    const int q = i / F4, c4 = (i % F4) * 4;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (q < rows) v = *reinterpret_cast<const float4*>(a.T + (row0 + q) * K + c0 + c4);
                    *reinterpret_cast<float4*>(Ts + q * LDT + c4) = v;
                }
            } else {
                for (int i = t; i < kWin * TW; i += kApplyThreads) {
                    const int q = i / TW, c = i % TW;
                    Ts[q * LDT + c] = (q < rows && c < tw) ? a.T[(row0 + q) * K + c0 + c] : 0.0f;
                }
            }
            __syncthreads();
            float acc[RM][CN];
#pragma unroll
            for (int i = 0; i < RM; ++i)
#pragma unroll
                for (int j = 0; j < CN; ++j) acc[i][j] = 0.f;
#pragma unroll 4
            for (int q = 0; q < kWin; ++q) {
                float ar[RM];
                load_rows<RM>(invT + q * kLdI + rg * RM, ar);
                float br[CN];
                const float4 b0 = *reinterpret_cast<const float4*>(Ts + q * LDT + cg * 4);
                br[0] = b0.x; br[1] = b0.y; br[2] = b0.z; br[3] = b0.w;
                if constexpr (CN == 8) {
                    const float4 b1 = *reinterpret_cast<const float4*>(Ts + q * LDT + TW / 2 + cg * 4);
                    br[4] = b1.x; br[5] = b1.y; br[6] = b1.z; br[7] = b1.w;
                }
#pragma unroll
                for (int i = 0; i < RM; ++i)
#pragma unroll
                    for (int j = 0; j < CN; ++j) acc[i][j] = fmaf(ar[i], br[j], acc[i][j]);
            }
            float csum[CN];
#pragma unroll
            for (int j = 0; j < CN; ++j) csum[j] = 0.f;
#pragma unroll
            for (int i = 0; i < RM; ++i) {
                const int r = rg * RM + i;
                if (r >= rows) continue;
                const int64_t base = (row0 + r) * K + c0;
#pragma unroll
                for (int h = 0; h < CN; h += 4) {
                    const int cb = cols[h];
                    float y[4], nv[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        y[j] = a.scale * acc[i][h + j];
                        nv[j] = a.near_scale * y[j];
                    }
                    if (a.vec && cb + 3 < tw) {
                        if (a.Y) *reinterpret_cast<float4*>(a.Y + base + cb) = make_float4(y[0], y[1], y[2], y[3]);
                        if (a.nf) {
                            float4 o = a.near_init ? make_float4(0.f, 0.f, 0.f, 0.f)
                                                   : *reinterpret_cast<const float4*>(a.nf + base + cb);
                            o.x += nv[0]; o.y += nv[1]; o.z += nv[2]; o.w += nv[3];
                            *reinterpret_cast<float4*>(a.nf + base + cb) = o;
                        }
#pragma unroll
                        for (int j = 0; j < 4; ++j) csum[h + j] += nv[j];
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            if (cb + j >= tw) continue;
                            if (a.Y) a.Y[base + cb + j] = y[j];
                            if (a.nf) a.nf[base + cb + j] = a.near_init ? nv[j] : a.nf[base + cb + j] + nv[j];
                            csum[h + j] += nv[j];
                        }
                    }
                }
            }
            if (a.partial) {
                __syncthreads();                           // every thread is done reading Ts
#pragma unroll
                for (int j = 0; j < CN; ++j) Ts[rg * TW + cols[j]] = csum[j];
                __syncthreads();
                for (int c = t; c < tw; c += kApplyThreads) {
                    float sum = 0.f;
#pragma unroll 8
                    for (int r = 0; r < RG; ++r) sum += Ts[r * TW + c];
                    float* p = a.partial + w * K + c0 + c;
                    *p = a.near_init ? sum : *p + sum;
                }
            }
        }
    }
}

template <int TW>
int launch_apply(const ApplyArgs& a, int64_t windows, cudaStream_t stream) {
    using S = ApplyShape<TW>;
    static std::atomic<int> attr_cache[kMaxDevices];
    int attr = 0;
    const int rc = per_device_value(
        attr_cache,
        [&](int* v) {
            GL_CUDA_TRY(cudaFuncSetAttribute(window_apply_kernel<TW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             S::SMEM));
            *v = 1;
            return GL_OK;
        },
        &attr);
    if (rc != GL_OK) return rc;
    window_apply_kernel<TW><<<grid_for(windows, S::CTAS), kApplyThreads, S::SMEM, stream>>>(a, windows);
    GL_LAUNCH_CHECK("window_apply_kernel");
    return GL_OK;
}

// colpart[y][c] = sum of partial[w][c] over the windows w of slice y;
// block (32 columns, 8 window lanes).
__global__ void window_colsum_kernel(const float* __restrict__ partial, int64_t windows, int K,
                                     double* __restrict__ colpart) {
    __shared__ double s[8][33];
    const int c = blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    if (c < K)
        for (int64_t w = (int64_t)blockIdx.y * 8 + threadIdx.y; w < windows; w += (int64_t)gridDim.y * 8)
            acc += partial[w * K + c];
    s[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && c < K) {
        double tot = 0.0;
#pragma unroll
        for (int y = 0; y < 8; ++y) tot += s[y][threadIdx.x];
        colpart[(int64_t)blockIdx.y * K + c] = tot;
    }
}

// missing[c] = max(0, 1 - sum over slices of colpart[.][c])
__global__ void window_missing_kernel(const double* __restrict__ colpart, int slices, int K,
                                      float* __restrict__ missing) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < K; c += gridDim.x * blockDim.x) {
        double tot = 0.0;
        for (int y = 0; y < slices; ++y) tot += colpart[(int64_t)y * K + c];
        missing[c] = (float)fmax(0.0, 1.0 - tot);
    }
}

// nf[i][c] += missing[c] * shape[i]
__global__ void window_finalize_kernel(float* __restrict__ nf, int64_t n, int K, const float* __restrict__ shape,
                                       const float* __restrict__ missing, int vec) {
    if (vec) {
        const int64_t k4 = K / 4, total = n * k4;
        for (int64_t i = gtid(); i < total; i += gthreads()) {
            const int64_t r = i / k4;
            const int c = (int)(i - r * k4) * 4;
            const float s = shape[r];
            float4 o = reinterpret_cast<float4*>(nf)[i];
            o.x += missing[c] * s;
            o.y += missing[c + 1] * s;
            o.z += missing[c + 2] * s;
            o.w += missing[c + 3] * s;
            reinterpret_cast<float4*>(nf)[i] = o;
        }
    } else {
        const int64_t total = n * K;
        for (int64_t i = gtid(); i < total; i += gthreads()) {
            const int64_t r = i / K;
            nf[i] += missing[i - r * K] * shape[r];
        }
    }
}

// Residual of one step from the teleport vector, per column:
// r = || alpha A v - alpha (1 - d(v)) v ||_1 with d(v) the column's mass on
// dangling nodes (the step sends it to v).  Only rows in the seed set and the
// columns' total out-mass enter:
//   r / alpha = sum_s v_s colsum_s - sum_{i in S} (A v)_i + sum_{i in S} |(A v)_i - (1 - d) v_i|.
// Warp per column; lanes over (i, s) seed pairs, A[i][s] by binary search in
// row i (column indices sorted).
__global__ void cold_residual_kernel(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                     const float* __restrict__ data, const double* __restrict__ colsum,
                                     const uint32_t* __restrict__ dangling, int64_t n,
                                     const int32_t* __restrict__ sptr, const int32_t* __restrict__ srows,
                                     const float* __restrict__ sw, int K, float alpha, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = gthreads() >> 5;
    for (int64_t col = gtid() >> 5; col < K; col += nw) {
        const int32_t s0 = sptr[col], s1 = sptr[col + 1];
        const int m = s1 - s0;
        double out_mass = 0.0, dmass = 0.0, bad = 0.0;
        for (int k = lane; k < m; k += 32) {
            const int32_t s = srows[s0 + k];
            if (s < 0 || s >= n) { bad = 1.0; continue; }
            out_mass += (double)sw[s0 + k] * colsum[s];
            if (dangling && ((dangling[s >> 5] >> (s & 31)) & 1u)) dmass += sw[s0 + k];
        }
        for (int o = 16; o > 0; o >>= 1) {
            out_mass += __shfl_xor_sync(0xffffffffu, out_mass, o);
            dmass += __shfl_xor_sync(0xffffffffu, dmass, o);
            bad += __shfl_xor_sync(0xffffffffu, bad, o);
        }
        // (A v)_i for each seed row i, lanes over the seed rows.  Per row the
        // cheaper of two lookups: walk the row and binary-search each entry
        // in the (sorted) seed list, or binary-search each seed in the row
        // (sorted columns); so a column's cost is bounded by the entries of
        // its seed rows, also for a seed set of millions of nodes.
        double in_seed = 0.0, corr = 0.0;
        if (bad == 0.0) {
            int lg_m = 1;
            while ((1 << lg_m) < m) ++lg_m;
            for (int k = lane; k < m; k += 32) {
                const int32_t i = srows[s0 + k];
                const int32_t r0 = indptr[i], r1 = indptr[i + 1];
                const int32_t deg = r1 - r0;
                int lg_d = 1;
                while ((1 << lg_d) < deg) ++lg_d;
                double av = 0.0;
                if ((int64_t)deg * lg_m <= (int64_t)m * lg_d) {
                    for (int32_t j = r0; j < r1; ++j) {
                        const int32_t c = indices[j];
                        int32_t lo = s0, hi = s1;            // c in the seed list?
                        while (lo < hi) {
                            const int32_t mid = lo + ((hi - lo) >> 1);
                            if (srows[mid] < c) lo = mid + 1; else hi = mid;
                        }
                        if (lo < s1 && srows[lo] == c) av += (double)data[j] * sw[lo];
                    }
                } else {
                    for (int q = 0; q < m; ++q) {
                        const int32_t sq = srows[s0 + q];
                        int32_t lo = r0, hi = r1;            // first entry with column >= sq
                        while (lo < hi) {
                            const int32_t mid = lo + ((hi - lo) >> 1);
                            if (indices[mid] < sq) lo = mid + 1; else hi = mid;
                        }
                        for (int32_t j = lo; j < r1 && indices[j] == sq; ++j) av += (double)data[j] * sw[s0 + q];
                    }
                }
                in_seed += av;
                corr += fabs(av - (1.0 - dmass) * (double)sw[s0 + k]);
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            in_seed += __shfl_xor_sync(0xffffffffu, in_seed, o);
            corr += __shfl_xor_sync(0xffffffffu, corr, o);
        }
        if (lane == 0) out[col] = bad != 0.0 ? -1.0 : (double)alpha * (out_mass - in_seed + corr);
    }
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int gl_window_blocks(const int32_t* indptr, const int32_t* indices, const float* data, int64_t n,
                                float alpha, float* blocks, cudaStream_t stream) {
    GL_REQUIRE(n >= 0 && n <= (int64_t)INT32_MAX - 1, GL_ERR_INVALID_ARGUMENT, "n out of range");
    GL_REQUIRE(alpha >= 0.0f && alpha < 1.0f, GL_ERR_INVALID_ARGUMENT, "alpha must be in [0, 1)");
    if (n == 0) return GL_OK;
    GL_REQUIRE(indptr && blocks, GL_ERR_INVALID_ARGUMENT, "indptr / blocks is NULL");
    const int64_t windows = ceil_div(n, kWin);
    window_identity_kernel<<<grid_for(ceil_div(windows * kBlk, kThreads), 16), kThreads, 0, stream>>>(
        blocks, windows * kBlk);
    GL_LAUNCH_CHECK("window_identity_kernel");
    window_blocks_kernel<<<grid_for(ceil_div(n * 32, kThreads), 16), kThreads, 0, stream>>>(indptr, indices, data,
                                                                                           n, alpha, blocks);
    GL_LAUNCH_CHECK("window_blocks_kernel");
    return GL_OK;
}

extern "C" int gl_window_invert(float* blocks, int64_t n, int32_t* status, cudaStream_t stream) {
    GL_REQUIRE(n >= 0, GL_ERR_INVALID_ARGUMENT, "n out of range");
    GL_REQUIRE(status != nullptr, GL_ERR_INVALID_ARGUMENT, "status is NULL");
    GL_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int32_t), stream));
    if (n == 0) return GL_OK;
    GL_REQUIRE(blocks != nullptr, GL_ERR_INVALID_ARGUMENT, "blocks is NULL");
    const int64_t windows = ceil_div(n, kWin);
    window_invert_kernel<<<grid_for(windows, 8), kThreads, 0, stream>>>(blocks, windows, status);
    GL_LAUNCH_CHECK("window_invert_kernel");
    return GL_OK;
}

extern "C" int gl_window_apply(const float* inverses, int64_t n, int32_t K, const float* T, float scale, float* Y,
                               float* near_field, float near_scale, int32_t near_init, float* partial,
                               cudaStream_t stream) {
    GL_REQUIRE(n >= 0 && K >= 0, GL_ERR_INVALID_ARGUMENT, "negative size");
    if (n == 0 || K == 0) return GL_OK;
    GL_REQUIRE(inverses && T, GL_ERR_INVALID_ARGUMENT, "inverses / T is NULL");
    GL_REQUIRE(Y || near_field, GL_ERR_INVALID_ARGUMENT, "nothing to write: Y and near_field are NULL");
    auto al16 = [](const void* p) { return p == nullptr || (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    ApplyArgs a;
    a.inv = inverses;
    a.T = T;
    a.Y = Y;
    a.nf = near_field;
    a.partial = partial;
    a.n = n;
    a.K = K;
    a.scale = scale;
    a.near_scale = near_scale;
    a.near_init = near_init ? 1 : 0;
    a.vec = (K % 4 == 0) && al16(T) && al16(Y) && al16(near_field);
    const int64_t windows = ceil_div(n, kWin);
    // column tile: the widest of GL_WIN_APPLY_MAXTW / 64 / 32 / 16 / 8 that K fills
    if (GL_WIN_APPLY_MAXTW >= 128 && K >= 128) return launch_apply<128>(a, windows, stream);
    if (GL_WIN_APPLY_MAXTW >= 64 && K >= 64) return launch_apply<64>(a, windows, stream);
    if (K >= 32) return launch_apply<32>(a, windows, stream);
    if (K >= 16) return launch_apply<16>(a, windows, stream);
    return launch_apply<8>(a, windows, stream);
}

namespace {
constexpr int kColSlices = 128;
}

extern "C" int64_t gl_window_finalize_workspace_bytes(int64_t n, int32_t K) {
    if (n < 0 || K < 0) return -1;
    return (int64_t)kColSlices * K * (int64_t)sizeof(double) + 4 * (int64_t)K + 16;
}

extern "C" int gl_window_finalize(float* near_field, int64_t n, int32_t K, const float* partial, const float* shape,
                                  void* workspace, int64_t workspace_bytes, cudaStream_t stream) {
    GL_REQUIRE(n >= 0 && K >= 0, GL_ERR_INVALID_ARGUMENT, "negative size");
    if (n == 0 || K == 0) return GL_OK;
    GL_REQUIRE(near_field && partial && shape, GL_ERR_INVALID_ARGUMENT, "near_field / partial / shape is NULL");
    const int64_t need = gl_window_finalize_workspace_bytes(n, K);
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= need, GL_ERR_WORKSPACE,
               "finalize workspace of %lld bytes needed", (long long)need);
    const int64_t windows = ceil_div(n, kWin);
    const int slices = (int)std::min<int64_t>(kColSlices, ceil_div(windows, 64));
    double* colpart = static_cast<double*>(workspace);
    float* missing = reinterpret_cast<float*>(colpart + (int64_t)kColSlices * K);
    window_colsum_kernel<<<dim3((unsigned)ceil_div(K, 32), (unsigned)slices), dim3(32, 8), 0, stream>>>(
        partial, windows, K, colpart);
    GL_LAUNCH_CHECK("window_colsum_kernel");
    window_missing_kernel<<<(unsigned)ceil_div(K, kThreads), kThreads, 0, stream>>>(colpart, slices, K, missing);
    GL_LAUNCH_CHECK("window_missing_kernel");
    const int vec = (K % 4 == 0) && (reinterpret_cast<uintptr_t>(near_field) & 15) == 0;
    const int64_t items = vec ? n * (K / 4) : n * K;
    window_finalize_kernel<<<grid_for(ceil_div(items, kThreads), 16), kThreads, 0, stream>>>(near_field, n, K, shape,
                                                                                            missing, vec);
    GL_LAUNCH_CHECK("window_finalize_kernel");
    return GL_OK;
}

extern "C" int gl_cold_residual(const int32_t* indptr, const int32_t* indices, const float* data,
                                const double* colsum, const uint32_t* dangling_bits, int64_t n,
                                const int32_t* seed_ptr, const int32_t* seed_rows, const float* seed_weights,
                                int32_t K, float alpha, double* out, cudaStream_t stream) {
    GL_REQUIRE(n >= 0 && K >= 0, GL_ERR_INVALID_ARGUMENT, "negative size");
    if (K == 0) return GL_OK;
    GL_REQUIRE(indptr && indices && data && colsum && seed_ptr && seed_rows && seed_weights && out,
               GL_ERR_INVALID_ARGUMENT, "a required pointer is NULL");
    cold_residual_kernel<<<grid_for(ceil_div((int64_t)K * 32, kThreads), 8), kThreads, 0, stream>>>(
        indptr, indices, data, colsum, dangling_bits, n, seed_ptr, seed_rows, seed_weights, K, alpha, out);
    GL_LAUNCH_CHECK("cold_residual_kernel");
    return GL_OK;
}
