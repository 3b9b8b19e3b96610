// Top-k of columns of a row-major [rows][ld] FP32 matrix on the device: the
// k largest values of each selected column with their row indices, sorted
// by value (descending), equal values by row (ascending).  Used to return
// the X highest-ranked nodes of a PPR column instead of all N ranks (the
// reference ships all N ranks and leaves the top-X cut to its frontend,
// Backend/server/app.py:146-158, Frontend/src/lib/ppr/types.ts topX).
//
// Radix select, exact and deterministic:
//   * keys: the float's bits mapped so unsigned order = float order
//     (negative: all bits flipped; positive: sign bit set);
//   * four passes of 8-bit digits from the top: per pass every CTA counts
//     the digits of the keys that still match the column's known prefix in
//     a shared-memory histogram [32 columns][256], adds it to a global one,
//     and one warp per column walks the histogram from the top digit down to
//     fix the next 8 bits of the k-th largest key T and how many keys equal
//     to T are still needed;
//   * a count pass and a write pass over row ranges owned by single warps
//     (lane = column, rows in order): keys above T are all taken, keys equal
//     to T are taken in row order until enough — ties go to the lowest rows;
//   * one CTA per column sorts its k candidates (bitonic, shared memory).
// Six reads of the selected columns in all; no host synchronization.
#include "gl_common.cuh"

namespace gl {
namespace {

constexpr int kTopkThreads = 256;
constexpr int kTopkWarps = kTopkThreads / 32;
constexpr int kTopkUnroll = 8;        // rows in flight per lane
constexpr int kSortThreadsK = 512;

__device__ __forceinline__ uint32_t order_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_value(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

struct TopkArgs {
    const float* X;
    int64_t rows, ld;
    const int32_t* columns;   // [C] or NULL: columns 0..C-1
    int64_t C;
    int32_t k;                // min(k, rows)
    int64_t units;            // row ranges per column group (gridDim.y * kTopkWarps)
    int64_t unit_rows;
    uint32_t* prefix;         // [C] known high bits of T
    int32_t* need;            // [C] keys equal to the prefix bucket still needed
    int32_t* hist;            // [C][256]
    int32_t* cnt_gt;          // [C][units]
    int32_t* cnt_eq;          // [C][units]
    uint32_t* cand_key;       // [C][k]
    int32_t* cand_row;        // [C][k]
};

__device__ __forceinline__ int64_t column_of(const TopkArgs& a, int64_t c) {
    return a.columns ? (int64_t)a.columns[c] : c;
}

// Visits the unit's rows in order with kTopkUnroll loads in flight:
// f(row, key) for each row of this warp's range (lane = column c).
template <typename F>
__device__ __forceinline__ void walk_unit(const TopkArgs& a, int64_t unit, int64_t col, F&& f) {
    const int64_t r0 = unit * a.unit_rows;
    int64_t r1 = r0 + a.unit_rows;
    if (r1 > a.rows) r1 = a.rows;
    int64_t r = r0;
    for (; r + kTopkUnroll <= r1; r += kTopkUnroll) {
        float v[kTopkUnroll];
#pragma unroll
        for (int q = 0; q < kTopkUnroll; ++q) v[q] = a.X[(r + q) * a.ld + col];
#pragma unroll
        for (int q = 0; q < kTopkUnroll; ++q) f(r + q, order_key(v[q]));
    }
    for (; r < r1; ++r) f(r, order_key(a.X[r * a.ld + col]));
}

// Pass `pass` (0..3) of the radix select: digit counts of the keys whose
// high 8 * pass bits equal the column's prefix.
__global__ void __launch_bounds__(kTopkThreads) topk_hist_kernel(TopkArgs a, int pass) {
    __shared__ int32_t h[32][257];   // padded: equal digits of different lanes hit different banks
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int i = t; i < 32 * 257; i += kTopkThreads) (&h[0][0])[i] = 0;
    __syncthreads();
    const int64_t c = (int64_t)blockIdx.x * 32 + lane;
    const int shift = 24 - 8 * pass;
    if (c < a.C && a.k > 0) {
        const int64_t col = column_of(a, c);
        const uint32_t pre = a.prefix[c];
        const int64_t unit = (int64_t)blockIdx.y * kTopkWarps + warp;
        walk_unit(a, unit, col, [&](int64_t, uint32_t key) {
            const bool match = pass == 0 || ((key ^ pre) >> (shift + 8)) == 0u;
            if (match) atomicAdd(&h[lane][(key >> shift) & 255u], 1);
        });
    }
    __syncthreads();
    for (int i = t; i < 32 * 256; i += kTopkThreads) {
        const int cl = i >> 8, d = i & 255;
        const int64_t cc = (int64_t)blockIdx.x * 32 + cl;
        const int32_t v = h[cl][d];
        if (v && cc < a.C) atomicAdd(&a.hist[cc * 256 + d], v);
    }
}

// One warp per column: the digit of T at this pass (walking down from 255)
// and how many keys equal to the new prefix are still needed; clears the
// histogram for the next pass.
__global__ void topk_select_kernel(TopkArgs a, int pass) {
    const int64_t c = blockIdx.x;
    const int lane = threadIdx.x;
    if (c >= a.C || a.k <= 0) return;
    const int shift = 24 - 8 * pass;
    int32_t* hc = a.hist + c * 256;
    const int32_t need = a.need[c];
    // lane l holds digits 255 - 8l .. 248 - 8l (descending)
    int32_t cnt[8];
    int32_t mine = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        cnt[q] = hc[255 - (lane * 8 + q)];
        mine += cnt[q];
    }
    int32_t incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    const int32_t before = incl - mine;   // keys in higher digits than this lane's
    const bool here = before < need && incl >= need;
    if (here) {
        int32_t run = before;
        int q = 0;
        for (; q < 8; ++q) {
            if (run + cnt[q] >= need) break;
            run += cnt[q];
        }
        const uint32_t digit = (uint32_t)(255 - (lane * 8 + q));
        a.prefix[c] |= digit << shift;
        a.need[c] = need - run;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q) hc[lane * 8 + q] = 0;
}

// Per unit: keys above T and keys equal to T.
__global__ void __launch_bounds__(kTopkThreads) topk_count_kernel(TopkArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t c = (int64_t)blockIdx.x * 32 + lane;
    if (c >= a.C || a.k <= 0) return;
    const uint32_t T = a.prefix[c];
    const int64_t unit = (int64_t)blockIdx.y * kTopkWarps + warp;
    int32_t gt = 0, eq = 0;
    walk_unit(a, unit, column_of(a, c), [&](int64_t, uint32_t key) {
        gt += key > T ? 1 : 0;
        eq += key == T ? 1 : 0;
    });
    a.cnt_gt[c * a.units + unit] = gt;
    a.cnt_eq[c * a.units + unit] = eq;
}

// One CTA per column: exclusive scans of the unit counts (in place).
__global__ void __launch_bounds__(1024) topk_unit_scan_kernel(TopkArgs a) {
    __shared__ int32_t warp_tot[2][32];
    __shared__ int32_t carry[2];
    const int64_t c = blockIdx.x;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t < 2) carry[t] = 0;
    __syncthreads();
    int32_t* arr[2] = {a.cnt_gt + c * a.units, a.cnt_eq + c * a.units};
    for (int64_t base = 0; base < a.units; base += 1024) {
        const int64_t i = base + t;
        int32_t x[2], incl[2];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            x[s] = i < a.units ? arr[s][i] : 0;
            incl[s] = x[s];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t u = __shfl_up_sync(0xffffffffu, incl[s], o);
                if (lane >= o) incl[s] += u;
            }
            if (lane == 31) warp_tot[s][warp] = incl[s];
        }
        __syncthreads();
        if (warp < 2) {
            int32_t w = warp_tot[warp][lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t u = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += u;
            }
            warp_tot[warp][lane] = w;
        }
        __syncthreads();
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int32_t prev = warp > 0 ? warp_tot[s][warp - 1] : 0;
            if (i < a.units) arr[s][i] = carry[s] + prev + incl[s] - x[s];
        }
        __syncthreads();
        if (t < 2) carry[t] += warp_tot[t][31];
        __syncthreads();
    }
}

// Per unit, rows in order: keys above T to their slots, keys equal to T to
// theirs while the column still needs ties.
__global__ void __launch_bounds__(kTopkThreads) topk_write_kernel(TopkArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t c = (int64_t)blockIdx.x * 32 + lane;
    if (c >= a.C || a.k <= 0) return;
    const uint32_t T = a.prefix[c];
    const int32_t ties = a.need[c];
    const int32_t above_total = a.k - ties;
    const int64_t unit = (int64_t)blockIdx.y * kTopkWarps + warp;
    int32_t gt = a.cnt_gt[c * a.units + unit];
    int32_t eq = a.cnt_eq[c * a.units + unit];
    uint32_t* ck = a.cand_key + c * a.k;
    int32_t* cr = a.cand_row + c * a.k;
    walk_unit(a, unit, column_of(a, c), [&](int64_t r, uint32_t key) {
        if (key > T) {
            if (gt < above_total) {   // always true by the selection; keeps every store in bounds
                ck[gt] = key;
                cr[gt] = (int32_t)r;
            }
            ++gt;
        } else if (key == T) {
            if (eq < ties) {
                ck[above_total + eq] = key;
                cr[above_total + eq] = (int32_t)r;
            }
            ++eq;
        }
    });
}

// One CTA per column: bitonic sort of the k candidates (key descending, row
// ascending), then values / rows out; slots past the row count get -inf / -1.
__global__ void __launch_bounds__(kSortThreadsK) topk_sort_kernel(TopkArgs a, int32_t k_out, int32_t pow2,
                                                                  float* values, int32_t* indices) {
    extern __shared__ uint64_t sk[];   // (~key << 32 | row): ascending order = the wanted order
    const int64_t c = blockIdx.x;
    const int t = threadIdx.x;
    for (int i = t; i < pow2; i += kSortThreadsK) {
        uint64_t v = ~0ull;
        if (i < a.k) {
            const uint32_t key = a.cand_key[c * a.k + i];
            v = ((uint64_t)(~key) << 32) | (uint32_t)a.cand_row[c * a.k + i];
        }
        sk[i] = v;
    }
    __syncthreads();
    for (int size = 2; size <= pow2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = t; i < pow2; i += kSortThreadsK) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const uint64_t x = sk[i], y = sk[j];
                    if ((x > y) == up) {
                        sk[i] = y;
                        sk[j] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = t; i < k_out; i += kSortThreadsK) {
        float v = -INFINITY;
        int32_t r = -1;
        if (i < a.k) {
            const uint64_t e = sk[i];
            v = key_value(~(uint32_t)(e >> 32));
            r = (int32_t)(e & 0xffffffffu);
        }
        values[c * k_out + i] = v;
        indices[c * k_out + i] = r;
    }
}

__global__ void topk_init_kernel(TopkArgs a) {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.C; c += (int64_t)gridDim.x * blockDim.x) {
        a.prefix[c] = 0u;
        a.need[c] = a.k;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.C * 256;
         i += (int64_t)gridDim.x * blockDim.x)
        a.hist[i] = 0;
}

struct TopkLayout {
    int64_t prefix, need, hist, cnt_gt, cnt_eq, cand_key, cand_row, total;
    int64_t units, unit_rows, ry;
};

TopkLayout topk_layout(int64_t rows, int64_t C, int32_t k) {
    TopkLayout L{};
    const int64_t groups = ceil_div(C, 32);
    // about four CTAs per SM over all column groups, at least 64 rows a unit
    int64_t ry = ceil_div((int64_t)num_sms() * 4, groups);
    const int64_t max_ry = ceil_div(ceil_div(rows > 0 ? rows : 1, 64), kTopkWarps);
    if (ry > max_ry) ry = max_ry;
    if (ry < 1) ry = 1;
    L.ry = ry;
    L.units = ry * kTopkWarps;
    L.unit_rows = ceil_div(rows > 0 ? rows : 1, L.units);
    const int64_t kk = k < rows ? k : rows;
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t at = off;
        off += ((bytes > 0 ? bytes : 1) + 255) & ~int64_t(255);
        return at;
    };
    L.prefix = take(4 * C);
    L.need = take(4 * C);
    L.hist = take(4 * 256 * C);
    L.cnt_gt = take(4 * C * L.units);
    L.cnt_eq = take(4 * C * L.units);
    L.cand_key = take(4 * C * kk);
    L.cand_row = take(4 * C * kk);
    L.total = off;
    return L;
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int64_t gl_topk_workspace_bytes(int64_t rows, int64_t num_columns, int32_t k) {
    if (rows < 0 || rows > (int64_t)INT32_MAX || num_columns < 0 || k < 0 || k > GL_TOPK_MAX) return -1;
    return topk_layout(rows, num_columns, k).total;
}

extern "C" int gl_topk_columns(const float* X, int64_t rows, int64_t ld, const int32_t* columns,
                               int64_t num_columns, int32_t k, float* values, int32_t* indices,
                               void* workspace, int64_t workspace_bytes, cudaStream_t stream) {
    GL_REQUIRE(rows >= 0 && rows <= (int64_t)INT32_MAX && num_columns >= 0 && ld >= 0, GL_ERR_INVALID_ARGUMENT,
               "bad rows / ld / num_columns");
    GL_REQUIRE(k >= 0 && k <= GL_TOPK_MAX, GL_ERR_INVALID_ARGUMENT, "k must be in [0, %d]", GL_TOPK_MAX);
    if (num_columns == 0 || k == 0) return GL_OK;
    GL_REQUIRE(values != nullptr && indices != nullptr, GL_ERR_INVALID_ARGUMENT, "values / indices are NULL");
    GL_REQUIRE(rows == 0 || X != nullptr, GL_ERR_INVALID_ARGUMENT, "X is NULL");
    GL_REQUIRE(columns != nullptr || num_columns <= ld, GL_ERR_INVALID_ARGUMENT,
               "num_columns exceeds the row stride");
    const TopkLayout L = topk_layout(rows, num_columns, k);
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= L.total, GL_ERR_WORKSPACE,
               "top-k workspace too small: need %lld bytes", (long long)L.total);
    char* ws = static_cast<char*>(workspace);
    TopkArgs a{};
    a.X = X;
    a.rows = rows;
    a.ld = ld;
    a.columns = columns;
    a.C = num_columns;
    a.k = (int32_t)(k < rows ? k : rows);
    a.units = L.units;
    a.unit_rows = L.unit_rows;
    a.prefix = reinterpret_cast<uint32_t*>(ws + L.prefix);
    a.need = reinterpret_cast<int32_t*>(ws + L.need);
    a.hist = reinterpret_cast<int32_t*>(ws + L.hist);
    a.cnt_gt = reinterpret_cast<int32_t*>(ws + L.cnt_gt);
    a.cnt_eq = reinterpret_cast<int32_t*>(ws + L.cnt_eq);
    a.cand_key = reinterpret_cast<uint32_t*>(ws + L.cand_key);
    a.cand_row = reinterpret_cast<int32_t*>(ws + L.cand_row);
    const dim3 grid((unsigned)ceil_div(num_columns, 32), (unsigned)L.ry);
    if (a.k > 0) {
        const int64_t init_blocks = ceil_div(num_columns * 256, 256);
        topk_init_kernel<<<(unsigned)(init_blocks < 4096 ? init_blocks : 4096), 256, 0, stream>>>(a);
        GL_LAUNCH_CHECK("topk_init_kernel");
        for (int pass = 0; pass < 4; ++pass) {
            topk_hist_kernel<<<grid, kTopkThreads, 0, stream>>>(a, pass);
            GL_LAUNCH_CHECK("topk_hist_kernel");
            topk_select_kernel<<<(unsigned)num_columns, 32, 0, stream>>>(a, pass);
            GL_LAUNCH_CHECK("topk_select_kernel");
        }
        topk_count_kernel<<<grid, kTopkThreads, 0, stream>>>(a);
        GL_LAUNCH_CHECK("topk_count_kernel");
        topk_unit_scan_kernel<<<(unsigned)num_columns, 1024, 0, stream>>>(a);
        GL_LAUNCH_CHECK("topk_unit_scan_kernel");
        topk_write_kernel<<<grid, kTopkThreads, 0, stream>>>(a);
        GL_LAUNCH_CHECK("topk_write_kernel");
    }
    int32_t pow2 = 1;
    while (pow2 < (a.k > 0 ? a.k : 1)) pow2 <<= 1;
    topk_sort_kernel<<<(unsigned)num_columns, kSortThreadsK, (size_t)pow2 * sizeof(uint64_t), stream>>>(
        a, k, pow2, values, indices);
    GL_LAUNCH_CHECK("topk_sort_kernel");
    return GL_OK;
}
