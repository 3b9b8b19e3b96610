// Stable LSD radix sort of (row, column, value) triples on the device, and
// the small kernels around it (run heads, row pointers by binary search):
// shared by the edge-list pipeline (edges.cu) and the PBR format tools
// (pbr_tools.cu).  Everything here has internal linkage in each translation
// unit that includes it.
#pragma once

#include "gl_common.cuh"
#include "gl_scan.cuh"

namespace gl {
namespace {

constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortRounds = 8;
constexpr int64_t kSortTile = (int64_t)kSortThreads * kSortRounds;
constexpr int kPlainThreads = 256;

inline unsigned plain_grid(int64_t n) {
    const int64_t cap = (int64_t)num_sms() * 8;
    const int64_t b = ceil_div(n > 0 ? n : 1, kPlainThreads);
    return (unsigned)(b < cap ? b : cap);
}

__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }
__device__ __forceinline__ int64_t gindex() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

// Per-tile digit counts, digit-major: hist[d * ntiles + tile].
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const int32_t* __restrict__ key,
                                                                  const int32_t* __restrict__ count, int shift,
                                                                  int64_t ntiles, int32_t* hist) {
    __shared__ int32_t h[256];
    const int t = threadIdx.x;
    if (t < 256) h[t] = 0;
    __syncthreads();
    const int64_t nvalid = *count;
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const int64_t i = base + (int64_t)r * kSortThreads + t;
        if (i < nvalid) atomicAdd(&h[((uint32_t)key[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    if (t < 256) hist[(int64_t)t * ntiles + blockIdx.x] = h[t];
}

// Moves the tile's elements to their sorted positions: scanned digit base of
// the tile + elements of the same digit earlier in the tile (earlier rounds,
// earlier warps of this round, earlier lanes of this warp).  row and val may
// be NULL.
template <typename V>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const int32_t* __restrict__ key, int shift, const int32_t* __restrict__ count, int64_t ntiles,
    const int32_t* __restrict__ hist, const int32_t* __restrict__ row_in, const int32_t* __restrict__ col_in,
    const V* __restrict__ val_in, int32_t* row_out, int32_t* col_out, V* val_out) {
    __shared__ int32_t base[256];
    __shared__ int32_t wcnt[kSortWarps][256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t < 256) base[t] = hist[(int64_t)t * ntiles + blockIdx.x];
    const int64_t nvalid = *count;
    const int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const int64_t r0 = tile0 + (int64_t)r * kSortThreads;
        if (r0 >= nvalid) break;   // uniform over the CTA
        const int64_t i = r0 + t;
        const bool ok = i < nvalid;
        const int d = ok ? (int)(((uint32_t)key[i] >> shift) & 255u) : 256;
        for (int q = lane; q < 256; q += 32) wcnt[warp][q] = 0;
        __syncwarp();
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int lrank = __popc(peers & ((1u << lane) - 1u));
        if (ok && lrank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        int32_t round_total = 0;
        if (t < 256) {   // per digit: exclusive prefix over the warps
#pragma unroll
            for (int w2 = 0; w2 < kSortWarps; ++w2) {
                const int32_t c = wcnt[w2][t];
                wcnt[w2][t] = round_total;
                round_total += c;
            }
        }
        __syncthreads();
        if (ok) {
            const int64_t dst = (int64_t)base[d] + wcnt[warp][d] + lrank;
            if (row_in) row_out[dst] = row_in[i];
            col_out[dst] = col_in[i];
            if (val_in) val_out[dst] = val_in[i];
        }
        __syncthreads();
        if (t < 256) base[t] += round_total;
    }
}

// head[i] = element i starts a run of equal (row, col); head[m] = 0.
__global__ void run_heads_kernel(const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                                 const int32_t* __restrict__ count, int64_t m, int32_t* head) {
    const int64_t nvalid = *count;
    for (int64_t i = gindex(); i <= m; i += gstride()) {
        int32_t h = 0;
        if (i < nvalid) h = (i == 0 || row[i] != row[i - 1] || col[i] != col[i - 1]) ? 1 : 0;
        head[i] = h;
    }
}

// ptr[j] = first index of sorted keys[0, *count) with keys[idx] >= j, j in [0, n].
__global__ void bounds_kernel(const int32_t* __restrict__ keys, const int32_t* __restrict__ count, int64_t n,
                              int32_t* ptr) {
    const int32_t len = *count;
    for (int64_t j = gindex(); j <= n; j += gstride()) {
        int32_t lo = 0, hi = len;
        while (lo < hi) {
            const int32_t mid = lo + ((hi - lo) >> 1);
            if ((int64_t)keys[mid] < j) lo = mid + 1;
            else hi = mid;
        }
        ptr[j] = lo;
    }
}

int bits_for(int64_t max_value) {
    int b = 0;
    while (b < 63 && (max_value >> b) > 0) ++b;
    return b;
}

template <typename V>
struct SortBuf {
    int32_t* row;
    int32_t* col;
    V* val;
};

// Stable sort of buffer `in` by key (row or col digits from bit 0 up to
// `bits`): the first pass writes into `a`, later passes alternate between
// `b` and `a`, so `in` is only read when b is another buffer.  Returns the
// buffer holding the result in *out.  A NULL row means (col, val) pairs, a
// NULL val keys only.
template <typename V>
int radix_sort(SortBuf<V> in, SortBuf<V> a, SortBuf<V> b, bool by_row, int bits, const int32_t* count, int64_t ntiles, int32_t* hist,
               int32_t* scratch, cudaStream_t st, SortBuf<V>* out) {
    SortBuf<V> cur = in, dst = a;
    for (int shift = 0; shift < bits; shift += 8) {
        const int32_t* key = by_row ? cur.row : cur.col;
        radix_hist_kernel<<<(unsigned)ntiles, kSortThreads, 0, st>>>(key, count, shift, ntiles, hist);
        GL_LAUNCH_CHECK("radix_hist_kernel");
        int rc = exclusive_scan<int32_t>(hist, hist, 256 * ntiles, scratch, 0, OpSum{}, st);
        if (rc != GL_OK) return rc;
        radix_scatter_kernel<V><<<(unsigned)ntiles, kSortThreads, 0, st>>>(key, shift, count, ntiles, hist, cur.row,
                                                                         cur.col, cur.val, dst.row, dst.col,
                                                                         dst.val);
        GL_LAUNCH_CHECK("radix_scatter_kernel");
        cur = dst;
        dst = (dst.col == a.col) ? b : a;
    }
    *out = cur;
    return GL_OK;
}

}  // namespace
}  // namespace gl
