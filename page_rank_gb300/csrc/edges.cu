// Edge list -> column-normalized transition matrix (CSR) on the device: the
// request path of the reference service between the JSON body and the PBR
// build (Backend/server/app.py:111-131 builds A[target, source] = weight,
// duplicates summed, then graph_link.normalize_transition_matrix,
// Backend/graph_link/graph_link/__init__.py:184-207), without the reference's
// dense 1/N dangling columns: dangling columns are reported in a mask and the
// PPR step redistributes their mass.
//
// Pipeline (stream-ordered, no host synchronization; counts stay on the
// device and later kernels read them):
//   1. keep edges whose endpoints are in [0, n) and whose weight is finite
//      and > 0 (app.py:114-122); weights rounded to FP32 (round to nearest);
//   2. stable LSD radix sort of (target, source, weight) by source, then by
//      target: 8-bit digits, tiles of 4096 edges, per-tile digit histograms
//      scanned digit-major, stable ranks inside a tile from warp match masks.
//      Duplicate (target, source) pairs end up adjacent in input order;
//   3. duplicate runs summed left to right in FP32;
//   4. column sums: the entries re-sorted stably by column (rows stay
//      increasing inside a column), each column summed the way numpy's
//      add.reduceat sums a segment (scipy's csc.sum(axis=0)): the first
//      entry plus numpy's pairwise sum of the rest; inv = 1 / sum, 0 for a
//      zero sum, which also marks the column dangling;
//   5. value * inv[column] in FP32, exact zeros dropped (scipy's sparse
//      product stores nonzeros only), indptr by binary search over the rows.
// Without normalization steps 4-5 reduce to copying the summed entries.
#include "gl_common.cuh"
#include "gl_scan.cuh"
#include "gl_sort.cuh"

namespace gl {
namespace {

// flag[i] = edge i is kept; flag[m] = 0 (the exclusive scan then leaves the
// kept count there).
__global__ void flag_valid_kernel(const int32_t* __restrict__ source, const int32_t* __restrict__ target,
                                  const double* __restrict__ weight, int64_t m, int64_t n, int32_t* flag) {
    for (int64_t i = gindex(); i <= m; i += gstride()) {
        int32_t f = 0;
        if (i < m) {
            const int64_t s = source[i], t = target[i];
            const double w = weight[i];
            f = (s >= 0 && s < n && t >= 0 && t < n && isfinite(w) && w > 0.0) ? 1 : 0;
        }
        flag[i] = f;
    }
}

__global__ void compact_valid_kernel(const int32_t* __restrict__ source, const int32_t* __restrict__ target,
                                     const double* __restrict__ weight, int64_t m, const int32_t* __restrict__ pos,
                                     int32_t* row, int32_t* col, float* val) {
    for (int64_t i = gindex(); i < m; i += gstride()) {
        const int32_t p = pos[i];
        if (pos[i + 1] != p) {
            row[p] = target[i];
            col[p] = source[i];
            val[p] = __double2float_rn(weight[i]);
        }
    }
}

// One thread per run: the run's weights summed left to right (input order).
__global__ void sum_runs_kernel(const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                                const float* __restrict__ val, const int32_t* __restrict__ count,
                                const int32_t* __restrict__ pos, int32_t* out_row, int32_t* out_col, float* out_val) {
    const int64_t nvalid = *count;
    for (int64_t i = gindex(); i < nvalid; i += gstride()) {
        const int32_t p = pos[i];
        if (pos[i + 1] == p) continue;   // not a run head
        float acc = val[i];
        for (int64_t j = i + 1; j < nvalid && pos[j + 1] == pos[j]; ++j) acc = __fadd_rn(acc, val[j]);
        out_row[p] = row[i];
        out_col[p] = col[i];
        out_val[p] = acc;
    }
}

// numpy's pairwise summation (numpy/_core/src/umath/loops_utils.h.src,
// pairwise_sum) of a[0, n) in FP32: fewer than 8 elements are summed in
// order from 0; up to 128 elements go to 8 interleaved accumulators combined
// as ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7)), then the tail in
// order; longer ranges split at n2 = n / 2 rounded down to a multiple of 8
// and return pairwise(first n2) + pairwise(rest).
__device__ float pairwise_leaf(const float* a, int64_t n) {
    if (n < 8) {
        float res = 0.f;
        for (int64_t i = 0; i < n; ++i) res = __fadd_rn(res, a[i]);
        return res;
    }
    float r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = a[j];
    int64_t i = 8;
    const int64_t stop = n - (n % 8);
    for (; i < stop; i += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = __fadd_rn(r[j], a[i + j]);
    }
    float res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                          __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
    for (; i < n; ++i) res = __fadd_rn(res, a[i]);
    return res;
}

__device__ float pairwise_sum(const float* a, int32_t n) {
    if (n <= 128) return pairwise_leaf(a, n);
    // the recursion as an explicit stack: a child range holds at most
    // n / 2 + 8 elements, so 2^31 elements reach the 128-element leaves
    // within 26 levels
    struct Frame {
        int32_t off, n;
        float left;
        int32_t state;   // 0: left half pending, 1: right half pending
    };
    Frame st[32];
    int sp = 0;
    st[sp++] = Frame{0, n, 0.f, 0};
    float result = 0.f, value = 0.f;
    bool have_value = false;
    while (sp > 0) {
        Frame& f = st[sp - 1];
        const int32_t n2 = (f.n / 2) - (f.n / 2) % 8;
        if (have_value) {   // a child finished
            have_value = false;
            if (f.state == 0) {
                f.left = value;
                f.state = 1;
            } else {
                value = __fadd_rn(f.left, value);
                --sp;
                have_value = true;
                if (sp == 0) result = value;
                continue;
            }
        }
        const int32_t off = f.state == 0 ? f.off : f.off + n2;
        const int32_t len = f.state == 0 ? n2 : f.n - n2;
        if (len <= 128) {
            value = pairwise_leaf(a + off, len);
            have_value = true;
        } else {
            st[sp++] = Frame{off, len, 0.f, 0};
        }
    }
    return result;
}

// One thread per column: sum (first + pairwise(rest)), 1 / sum, dangling.
__global__ void column_sums_kernel(const float* __restrict__ val_by_col, const int32_t* __restrict__ colptr,
                                   int64_t n, float* inv, uint8_t* dangling) {
    for (int64_t j = gindex(); j < n; j += gstride()) {
        const int32_t b = colptr[j], e = colptr[j + 1];
        float s = 0.f;
        if (e > b) s = __fadd_rn(val_by_col[b], pairwise_sum(val_by_col + b + 1, e - b - 1));
        inv[j] = s > 0.f ? __fdiv_rn(1.0f, s) : 0.f;
        if (dangling) dangling[j] = s == 0.f ? 1 : 0;
    }
}

// In CSR order: value * inv[column] (inv NULL: unchanged), keep[i] = the
// entry is stored; keep[m] = 0.
__global__ void scale_kernel(const int32_t* __restrict__ col, float* val, const float* __restrict__ inv,
                             const int32_t* __restrict__ count, int64_t m, int32_t* keep) {
    const int64_t nruns = *count;
    for (int64_t i = gindex(); i <= m; i += gstride()) {
        int32_t k = 0;
        if (i < nruns) {
            if (inv) {
                const float v = __fmul_rn(val[i], inv[col[i]]);
                val[i] = v;
                k = v != 0.f ? 1 : 0;
            } else {
                k = 1;
            }
        }
        keep[i] = k;
    }
}

__global__ void compact_out_kernel(const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                                   const float* __restrict__ val, const int32_t* __restrict__ count,
                                   const int32_t* __restrict__ pos, int32_t* out_row, int32_t* indices,
                                   float* data) {
    const int64_t nruns = *count;
    for (int64_t i = gindex(); i < nruns; i += gstride()) {
        const int32_t p = pos[i];
        if (pos[i + 1] == p) continue;
        out_row[p] = row[i];
        indices[p] = col[i];
        data[p] = val[i];
    }
}

__global__ void store_count_kernel(const int32_t* __restrict__ count, int64_t* out) { *out = *count; }

using Buf = SortBuf<float>;

struct EdgeWorkspace {
    int64_t row[3], col[3], val[3];   // three (row, col, value) buffers; row[2] unused
    int64_t flag, head, keep, hist, scratch, colptr, inv;
    int64_t total;
};

EdgeWorkspace edge_workspace(int64_t n, int64_t m) {
    EdgeWorkspace w{};
    const int64_t ntiles = ceil_div(m > 0 ? m : 1, kSortTile);
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t at = off;
        off += ((bytes > 0 ? bytes : 1) + 255) & ~int64_t(255);
        return at;
    };
    for (int k = 0; k < 3; ++k) {
        w.row[k] = take(4 * m);
        w.col[k] = take(4 * m);
        w.val[k] = take(4 * m);
    }
    w.flag = take(4 * (m + 1));
    w.head = take(4 * (m + 1));
    w.keep = take(4 * (m + 1));
    w.hist = take(4 * 256 * ntiles);
    const int64_t scan_n = (m + 1) > 256 * ntiles ? (m + 1) : 256 * ntiles;
    w.scratch = take(4 * scan_scratch_elems(scan_n));
    w.colptr = take(4 * (n + 1));
    w.inv = take(4 * n);
    w.total = off;
    return w;
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int64_t gl_edges_workspace_bytes(int64_t num_nodes, int64_t num_edges) {
    if (num_nodes < 0 || num_edges < 0 || num_nodes > (int64_t)INT32_MAX - 1 ||
        num_edges > (int64_t)INT32_MAX - 1)
        return -1;
    return edge_workspace(num_nodes, num_edges).total;
}

extern "C" int gl_edges_to_transition(int64_t num_nodes, int64_t num_edges, const int32_t* source,
                                      const int32_t* target, const double* weight, int32_t normalize,
                                      int32_t* indptr, int32_t* indices, float* data, uint8_t* dangling,
                                      int64_t* nnz, void* workspace, int64_t workspace_bytes,
                                      cudaStream_t stream) {
    const int64_t n = num_nodes, m = num_edges;
    GL_REQUIRE(n >= 0 && m >= 0 && n <= (int64_t)INT32_MAX - 1 && m <= (int64_t)INT32_MAX - 1,
               GL_ERR_INVALID_ARGUMENT, "num_nodes / num_edges out of range");
    GL_REQUIRE(indptr != nullptr && nnz != nullptr, GL_ERR_INVALID_ARGUMENT, "indptr / nnz is NULL");
    GL_REQUIRE(m == 0 || (source && target && weight && indices && data), GL_ERR_INVALID_ARGUMENT,
               "edge or output arrays are NULL");
    const EdgeWorkspace w = edge_workspace(n, m);
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= w.total, GL_ERR_WORKSPACE,
               "edge workspace too small: need %lld bytes", (long long)w.total);
    char* ws = static_cast<char*>(workspace);
    auto i32 = [&](int64_t off) { return reinterpret_cast<int32_t*>(ws + off); };
    auto f32 = [&](int64_t off) { return reinterpret_cast<float*>(ws + off); };
    Buf B[3];
    for (int k = 0; k < 3; ++k) B[k] = Buf{k < 2 ? i32(w.row[k]) : nullptr, i32(w.col[k]), f32(w.val[k])};
    int32_t* flag = i32(w.flag);
    int32_t* head = i32(w.head);
    int32_t* keep = i32(w.keep);
    int32_t* hist = i32(w.hist);
    int32_t* scratch = i32(w.scratch);
    const int64_t ntiles = ceil_div(m > 0 ? m : 1, kSortTile);
    const int bits = bits_for(n > 0 ? n - 1 : 0);
    int rc;

    // 1. keep the valid edges (count at flag[m])
    flag_valid_kernel<<<plain_grid(m + 1), kPlainThreads, 0, stream>>>(source, target, weight, m, n, flag);
    GL_LAUNCH_CHECK("flag_valid_kernel");
    rc = exclusive_scan<int32_t>(flag, flag, m + 1, scratch, 0, OpSum{}, stream);
    if (rc != GL_OK) return rc;
    if (m > 0) {
        compact_valid_kernel<<<plain_grid(m), kPlainThreads, 0, stream>>>(source, target, weight, m, flag,
                                                                          B[0].row, B[0].col, B[0].val);
        GL_LAUNCH_CHECK("compact_valid_kernel");
    }
    const int32_t* valid = flag + m;

    // 2. stable sort by (row, col): column digits first
    Buf sorted;
    rc = radix_sort(B[0], B[1], B[0], false, bits, valid, ntiles, hist, scratch, stream, &sorted);
    if (rc != GL_OK) return rc;
    rc = radix_sort(sorted, sorted.row == B[0].row ? B[1] : B[0], sorted, true, bits, valid, ntiles, hist,
                    scratch, stream, &sorted);
    if (rc != GL_OK) return rc;
    const Buf other = sorted.row == B[0].row ? B[1] : B[0];

    // 3. duplicate runs summed (run count at head[m])
    run_heads_kernel<<<plain_grid(m + 1), kPlainThreads, 0, stream>>>(sorted.row, sorted.col, valid, m, head);
    GL_LAUNCH_CHECK("run_heads_kernel");
    rc = exclusive_scan<int32_t>(head, head, m + 1, scratch, 0, OpSum{}, stream);
    if (rc != GL_OK) return rc;
    if (m > 0) {
        sum_runs_kernel<<<plain_grid(m), kPlainThreads, 0, stream>>>(sorted.row, sorted.col, sorted.val, valid,
                                                                     head, other.row, other.col, other.val);
        GL_LAUNCH_CHECK("sum_runs_kernel");
    }
    const int32_t* runs = head + m;
    const Buf summed = other;      // CSR order
    const Buf spare = sorted;      // free from here on

    // 4. column sums over a column-major copy of (col, value)
    float* inv = nullptr;
    if (normalize) {
        inv = f32(w.inv);
        int32_t* colptr = i32(w.colptr);
        Buf by_col;
        // summed stays in CSR order: the passes alternate between spare and B[2]
        rc = radix_sort(Buf{nullptr, summed.col, summed.val}, Buf{nullptr, spare.col, spare.val}, B[2], false,
                        bits, runs, ntiles, hist, scratch, stream, &by_col);
        if (rc != GL_OK) return rc;
        if (n > 0) {
            bounds_kernel<<<plain_grid(n + 1), kPlainThreads, 0, stream>>>(by_col.col, runs, n, colptr);
            GL_LAUNCH_CHECK("bounds_kernel");
            column_sums_kernel<<<plain_grid(n), kPlainThreads, 0, stream>>>(by_col.val, colptr, n, inv, dangling);
            GL_LAUNCH_CHECK("column_sums_kernel");
        }
    } else if (dangling != nullptr && n > 0) {
        GL_CUDA_TRY(cudaMemsetAsync(dangling, 0, (size_t)n, stream));
    }

    // 5. scale, drop exact zeros, compact into the outputs, indptr
    scale_kernel<<<plain_grid(m + 1), kPlainThreads, 0, stream>>>(summed.col, summed.val, inv, runs, m, keep);
    GL_LAUNCH_CHECK("scale_kernel");
    rc = exclusive_scan<int32_t>(keep, keep, m + 1, scratch, 0, OpSum{}, stream);
    if (rc != GL_OK) return rc;
    int32_t* out_row = B[2].col;   // free again once the column sums are done (stream order)
    if (m > 0) {
        compact_out_kernel<<<plain_grid(m), kPlainThreads, 0, stream>>>(summed.row, summed.col, summed.val, runs,
                                                                        keep, out_row, indices, data);
        GL_LAUNCH_CHECK("compact_out_kernel");
    }
    const int32_t* kept = keep + m;
    bounds_kernel<<<plain_grid(n + 1), kPlainThreads, 0, stream>>>(out_row, kept, n, indptr);
    GL_LAUNCH_CHECK("bounds_kernel");
    store_count_kernel<<<1, 1, 0, stream>>>(kept, nnz);
    GL_LAUNCH_CHECK("store_count_kernel");
    return GL_OK;
}
