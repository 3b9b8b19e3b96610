// PBR format tools on the device: PBR -> CSR, and the block-pattern
// histogram behind pbr_analyze_csr.
//
// gl_pbr_to_csr replaces the reference's host pbr_to_csr
// (Backend/graph_link/pbr_matrix/pbr_matrix.cpp:289-338): every stored value
// becomes a (row, column, value) triple — block values pair with their
// code's set bits in row-major bit order, remainder entries with their row —
// the triples are sorted stably by (row, column) with the device radix
// passes, and the row pointers come from a binary search per row.  Unlike
// the reference, a matrix whose row count is not a multiple of the block
// height is handled (the reference throws at pbr_matrix.cpp:308-310).
//
// gl_pbr_block_patterns computes what the reference's pbr_analyze_csr
// (pbr_matrix.cpp:71-156) intends: how often each distinct block code
// occurs, and under the coverage rule (occurrences x bit count >=
// min_nnz_coverage, pbr_matrix.cpp:127-141) the compressed / remainder
// totals.  The codes are sorted as two 32-bit keys (low word, then high
// word) and run-length encoded.
#include "gl_common.cuh"
#include "gl_scan.cuh"
#include "gl_sort.cuh"

namespace gl {
namespace {

__global__ void set_count_kernel(int32_t* count, int32_t v) { *count = v; }

// Block values -> (row, column, value) at the value's own index: thread per
// block, set bits in row-major order (the order block_data is packed in).
template <typename V>
__global__ void expand_blocks_kernel(const uint64_t* __restrict__ codes, const int32_t* __restrict__ coords,
                                     const int32_t* __restrict__ offsets, const V* __restrict__ bdata, int64_t nb,
                                     int br, int bc, int32_t* row, int32_t* col, V* val) {
    for (int64_t b = gindex(); b < nb; b += gstride()) {
        uint64_t code = codes[b];
        const int32_t r0 = coords[2 * b], c0 = coords[2 * b + 1];
        int32_t k = offsets[b];
        while (code) {
            const int bit = __ffsll((long long)code) - 1;
            code &= code - 1;
            row[k] = r0 + bit / bc;
            col[k] = c0 + bit % bc;
            val[k] = bdata[k];
            ++k;
        }
    }
}

// Remainder entries -> triples after the packed values: warp per row.
template <typename V>
__global__ void expand_remainder_kernel(const int32_t* __restrict__ rem_ptr, const int32_t* __restrict__ rem_col,
                                        const V* __restrict__ rem_val, int64_t rows, int64_t packed, int32_t* row,
                                        int32_t* col, V* val) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = gindex() >> 5, nw = gstride() >> 5;
    for (int64_t r = w0; r < rows; r += nw) {
        const int32_t j0 = rem_ptr[r], j1 = rem_ptr[r + 1];
        for (int32_t j = j0 + lane; j < j1; j += 32) {
            row[packed + j] = (int32_t)r;
            col[packed + j] = rem_col[j];
            val[packed + j] = rem_val[j];
        }
    }
}

// Codes -> (high word, low word) sort keys.
__global__ void split_codes_kernel(const uint64_t* __restrict__ codes, int64_t nb, int32_t* hi, int32_t* lo) {
    for (int64_t i = gindex(); i < nb; i += gstride()) {
        const uint64_t c = codes[i];
        hi[i] = (int32_t)(uint32_t)(c >> 32);
        lo[i] = (int32_t)(uint32_t)c;
    }
}

// For every run head i of the sorted keys (pos = exclusive scan of the
// heads): start[pos[i]] = i; start[number of runs] = nb.
__global__ void run_starts_kernel(const int32_t* __restrict__ pos, int64_t nb, int32_t* start) {
    for (int64_t i = gindex(); i <= nb; i += gstride()) {
        if (i == nb) start[pos[nb]] = (int32_t)nb;
        else if (pos[i + 1] != pos[i]) start[pos[i]] = (int32_t)i;
    }
}

// Per distinct code: its value, occurrence count, and the coverage rule's
// totals: [0] nnz in compressed patterns, [1] nnz in the others,
// [2] compressed patterns, [3] blocks of compressed patterns.
__global__ void pattern_totals_kernel(const int32_t* __restrict__ hi, const int32_t* __restrict__ lo,
                                      const int32_t* __restrict__ start, const int32_t* __restrict__ nruns,
                                      int64_t min_cov, uint64_t* codes_out, int64_t* counts_out, int64_t* totals) {
    const int64_t u_n = *nruns;
    for (int64_t u = gindex(); u < u_n; u += gstride()) {
        const int32_t i = start[u];
        const int64_t occ = (int64_t)start[u + 1] - i;
        const uint64_t code = ((uint64_t)(uint32_t)hi[i] << 32) | (uint32_t)lo[i];
        codes_out[u] = code;
        counts_out[u] = occ;
        const int64_t cov = occ * __popcll(code);
        if (cov >= min_cov) {
            atomicAdd(reinterpret_cast<unsigned long long*>(totals + 0), (unsigned long long)cov);
            atomicAdd(reinterpret_cast<unsigned long long*>(totals + 2), 1ull);
            atomicAdd(reinterpret_cast<unsigned long long*>(totals + 3), (unsigned long long)occ);
        } else {
            atomicAdd(reinterpret_cast<unsigned long long*>(totals + 1), (unsigned long long)cov);
        }
    }
}

__global__ void store_runs_kernel(const int32_t* __restrict__ nruns, int64_t* out) { *out = *nruns; }

// Workspace of gl_pbr_to_csr: two (row, col, value) buffers, the radix
// histograms, the scan scratch, the element count.
struct ToCsrWorkspace {
    int64_t row[2], col[2], val[2], hist, scratch, count, total;
};
ToCsrWorkspace to_csr_workspace(int64_t nnz, int64_t elem) {
    ToCsrWorkspace w{};
    const int64_t ntiles = ceil_div(nnz > 0 ? nnz : 1, kSortTile);
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t at = off;
        off += ((bytes > 0 ? bytes : 1) + 255) & ~int64_t(255);
        return at;
    };
    for (int k = 0; k < 2; ++k) {
        w.row[k] = take(4 * nnz);
        w.col[k] = take(4 * nnz);
        w.val[k] = take(elem * nnz);
    }
    w.hist = take(4 * 256 * ntiles);
    w.scratch = take(4 * scan_scratch_elems(256 * ntiles));
    w.count = take(4);
    w.total = off;
    return w;
}

// Workspace of gl_pbr_block_patterns: two key buffers, run heads, run
// starts, histograms, scan scratch, count.
struct PatternWorkspace {
    int64_t hi[2], lo[2], head, start, hist, scratch, count, total;
};
PatternWorkspace pattern_workspace(int64_t nb) {
    PatternWorkspace w{};
    const int64_t ntiles = ceil_div(nb > 0 ? nb : 1, kSortTile);
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t at = off;
        off += ((bytes > 0 ? bytes : 1) + 255) & ~int64_t(255);
        return at;
    };
    for (int k = 0; k < 2; ++k) {
        w.hi[k] = take(4 * nb);
        w.lo[k] = take(4 * nb);
    }
    w.head = take(4 * (nb + 1));
    w.start = take(4 * (nb + 1));
    w.hist = take(4 * 256 * ntiles);
    const int64_t scan_n = (nb + 1) > 256 * ntiles ? (nb + 1) : 256 * ntiles;
    w.scratch = take(4 * scan_scratch_elems(scan_n));
    w.count = take(4);
    w.total = off;
    return w;
}

template <typename V>
int to_csr(const gl_pbr_matrix* A, int32_t* indptr, int32_t* indices, V* data, char* ws, cudaStream_t stream) {
    const int64_t nnz = A->packed_nnz + A->remainder_nnz;
    const ToCsrWorkspace w = to_csr_workspace(nnz, sizeof(V));
    auto i32 = [&](int64_t off) { return reinterpret_cast<int32_t*>(ws + off); };
    SortBuf<V> B[2];
    for (int k = 0; k < 2; ++k) B[k] = SortBuf<V>{i32(w.row[k]), i32(w.col[k]), reinterpret_cast<V*>(ws + w.val[k])};
    int32_t* count = i32(w.count);
    int32_t* hist = i32(w.hist);
    int32_t* scratch = i32(w.scratch);
    set_count_kernel<<<1, 1, 0, stream>>>(count, (int32_t)nnz);
    GL_LAUNCH_CHECK("set_count_kernel");
    if (A->num_blocks > 0) {
        expand_blocks_kernel<V><<<plain_grid(A->num_blocks), kPlainThreads, 0, stream>>>(
            reinterpret_cast<const uint64_t*>(A->block_codes), A->block_coords, A->block_offsets,
            static_cast<const V*>(A->block_data), A->num_blocks, A->block_rows, A->block_cols, B[0].row, B[0].col,
            B[0].val);
        GL_LAUNCH_CHECK("expand_blocks_kernel");
    }
    if (A->remainder_nnz > 0) {
        expand_remainder_kernel<V><<<plain_grid(32 * A->rows), kPlainThreads, 0, stream>>>(
            A->remainder_indptr, A->remainder_col_ind, static_cast<const V*>(A->remainder_data), A->rows,
            A->packed_nnz, B[0].row, B[0].col, B[0].val);
        GL_LAUNCH_CHECK("expand_remainder_kernel");
    }
    const int64_t ntiles = ceil_div(nnz > 0 ? nnz : 1, kSortTile);
    SortBuf<V> sorted = B[0];
    int rc;
    if (nnz > 0) {
        // stable: columns first, then rows
        rc = radix_sort<V>(B[0], B[1], B[0], false, bits_for(A->cols > 0 ? A->cols - 1 : 0), count, ntiles, hist,
                           scratch, stream, &sorted);
        if (rc != GL_OK) return rc;
        const SortBuf<V> other = sorted.col == B[0].col ? B[1] : B[0];
        rc = radix_sort<V>(sorted, other, sorted, true, bits_for(A->rows > 0 ? A->rows - 1 : 0), count, ntiles, hist,
                           scratch, stream, &sorted);
        if (rc != GL_OK) return rc;
        GL_CUDA_TRY(cudaMemcpyAsync(indices, sorted.col, 4 * nnz, cudaMemcpyDeviceToDevice, stream));
        GL_CUDA_TRY(cudaMemcpyAsync(data, sorted.val, sizeof(V) * nnz, cudaMemcpyDeviceToDevice, stream));
    }
    bounds_kernel<<<plain_grid(A->rows + 1), kPlainThreads, 0, stream>>>(sorted.row, count, A->rows, indptr);
    GL_LAUNCH_CHECK("bounds_kernel");
    return GL_OK;
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int64_t gl_pbr_to_csr_workspace_bytes(const gl_pbr_matrix* A) {
    if (A == nullptr || A->packed_nnz < 0 || A->remainder_nnz < 0) return -1;
    const int64_t nnz = A->packed_nnz + A->remainder_nnz;
    if (nnz > (int64_t)INT32_MAX - 1 || A->rows > (int64_t)INT32_MAX - 1 || A->cols > (int64_t)INT32_MAX - 1)
        return -1;
    return to_csr_workspace(nnz, A->value_type == GL_F64 ? 8 : 4).total;
}

extern "C" int gl_pbr_to_csr(const gl_pbr_matrix* A, int32_t* indptr, int32_t* indices, void* data,
                             void* workspace, int64_t workspace_bytes, cudaStream_t stream) {
    GL_REQUIRE(A != nullptr, GL_ERR_INVALID_ARGUMENT, "matrix descriptor is NULL");
    GL_REQUIRE(A->value_type == GL_F32 || A->value_type == GL_F64, GL_ERR_INVALID_ARGUMENT,
               "value_type must be GL_F32 or GL_F64");
    GL_REQUIRE(A->rows >= 0 && A->cols >= 0 && A->block_rows >= 1 && A->block_cols >= 1 &&
                   A->block_rows * A->block_cols <= 64,
               GL_ERR_INVALID_ARGUMENT, "bad sizes in the matrix descriptor");
    const int64_t need = gl_pbr_to_csr_workspace_bytes(A);
    GL_REQUIRE(need >= 0, GL_ERR_INVALID_ARGUMENT, "matrix too large for int32 CSR output");
    GL_REQUIRE(indptr != nullptr, GL_ERR_INVALID_ARGUMENT, "indptr is NULL");
    const int64_t nnz = A->packed_nnz + A->remainder_nnz;
    GL_REQUIRE(nnz == 0 || (indices && data), GL_ERR_INVALID_ARGUMENT, "indices / data is NULL");
    GL_REQUIRE(A->rows == 0 || A->remainder_indptr, GL_ERR_INVALID_ARGUMENT, "remainder_indptr is NULL");
    GL_REQUIRE(A->num_blocks == 0 || (A->block_codes && A->block_coords && A->block_offsets && A->block_data),
               GL_ERR_INVALID_ARGUMENT, "block arrays are NULL");
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= need, GL_ERR_WORKSPACE,
               "pbr_to_csr workspace of %lld bytes needed", (long long)need);
    char* ws = static_cast<char*>(workspace);
    if (A->value_type == GL_F32) return to_csr<float>(A, indptr, indices, static_cast<float*>(data), ws, stream);
    return to_csr<double>(A, indptr, indices, static_cast<double*>(data), ws, stream);
}

extern "C" int64_t gl_pbr_block_patterns_workspace_bytes(int64_t num_blocks) {
    if (num_blocks < 0 || num_blocks > (int64_t)INT32_MAX - 1) return -1;
    return pattern_workspace(num_blocks).total;
}

extern "C" int gl_pbr_block_patterns(const int64_t* block_codes, int64_t num_blocks, int64_t min_nnz_coverage,
                                     uint64_t* unique_codes, int64_t* counts, int64_t* num_unique,
                                     int64_t* totals, void* workspace, int64_t workspace_bytes,
                                     cudaStream_t stream) {
    GL_REQUIRE(num_blocks >= 0 && num_blocks <= (int64_t)INT32_MAX - 1, GL_ERR_INVALID_ARGUMENT,
               "num_blocks out of range");
    GL_REQUIRE(num_unique != nullptr && totals != nullptr, GL_ERR_INVALID_ARGUMENT, "num_unique / totals is NULL");
    GL_REQUIRE(num_blocks == 0 || (block_codes && unique_codes && counts), GL_ERR_INVALID_ARGUMENT,
               "code arrays are NULL");
    const PatternWorkspace w = pattern_workspace(num_blocks);
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= w.total, GL_ERR_WORKSPACE,
               "pattern workspace of %lld bytes needed", (long long)w.total);
    GL_CUDA_TRY(cudaMemsetAsync(totals, 0, 4 * sizeof(int64_t), stream));
    GL_CUDA_TRY(cudaMemsetAsync(num_unique, 0, sizeof(int64_t), stream));
    if (num_blocks == 0) return GL_OK;
    char* ws = static_cast<char*>(workspace);
    auto i32 = [&](int64_t off) { return reinterpret_cast<int32_t*>(ws + off); };
    const int64_t nb = num_blocks;
    int32_t* count = i32(w.count);
    int32_t* hist = i32(w.hist);
    int32_t* scratch = i32(w.scratch);
    int32_t* head = i32(w.head);
    int32_t* start = i32(w.start);
    set_count_kernel<<<1, 1, 0, stream>>>(count, (int32_t)nb);
    GL_LAUNCH_CHECK("set_count_kernel");
    SortBuf<float> K[2] = {{i32(w.hi[0]), i32(w.lo[0]), nullptr}, {i32(w.hi[1]), i32(w.lo[1]), nullptr}};
    split_codes_kernel<<<plain_grid(nb), kPlainThreads, 0, stream>>>(reinterpret_cast<const uint64_t*>(block_codes),
                                                                      nb, K[0].row, K[0].col);
    GL_LAUNCH_CHECK("split_codes_kernel");
    const int64_t ntiles = ceil_div(nb, kSortTile);
    SortBuf<float> sorted;
    int rc = radix_sort<float>(K[0], K[1], K[0], false, 32, count, ntiles, hist, scratch, stream, &sorted);
    if (rc != GL_OK) return rc;
    const SortBuf<float> other = sorted.col == K[0].col ? K[1] : K[0];
    rc = radix_sort<float>(sorted, other, sorted, true, 32, count, ntiles, hist, scratch, stream, &sorted);
    if (rc != GL_OK) return rc;
    run_heads_kernel<<<plain_grid(nb + 1), kPlainThreads, 0, stream>>>(sorted.row, sorted.col, count, nb, head);
    GL_LAUNCH_CHECK("run_heads_kernel");
    rc = exclusive_scan<int32_t>(head, head, nb + 1, scratch, 0, OpSum{}, stream);
    if (rc != GL_OK) return rc;
    run_starts_kernel<<<plain_grid(nb + 1), kPlainThreads, 0, stream>>>(head, nb, start);
    GL_LAUNCH_CHECK("run_starts_kernel");
    pattern_totals_kernel<<<plain_grid(nb), kPlainThreads, 0, stream>>>(sorted.row, sorted.col, start, head + nb,
                                                                         min_nnz_coverage, unique_codes, counts,
                                                                         totals);
    GL_LAUNCH_CHECK("pattern_totals_kernel");
    store_runs_kernel<<<1, 1, 0, stream>>>(head + nb, num_unique);
    GL_LAUNCH_CHECK("store_runs_kernel");
    return GL_OK;
}
