// C ABI: error text, SpMM entry point, stripe index, and the personalized
// PageRank entry points (teleport index, init, fused step).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "gl_common.cuh"
#include "gl_scan.cuh"
#include "stripe_kernel.cuh"

namespace gl {

namespace {
thread_local char g_last_error[1024] = {0};
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

const char* last_error() { return g_last_error; }

namespace {

int check_matrix(const gl_pbr_matrix* A) {
    GL_REQUIRE(A != nullptr, GL_ERR_INVALID_ARGUMENT, "matrix descriptor is NULL");
    GL_REQUIRE(A->rows >= 0 && A->cols >= 0, GL_ERR_INVALID_ARGUMENT, "negative matrix size");
    GL_REQUIRE(A->value_type == GL_F32 || A->value_type == GL_F64, GL_ERR_INVALID_ARGUMENT,
               "value_type must be GL_F32 or GL_F64");
    const bool ok_block = (A->block_rows == A->block_cols) &&
                          (A->block_rows == 2 || A->block_rows == 4 || A->block_rows == 8);
    GL_REQUIRE(ok_block, GL_ERR_UNSUPPORTED_BLOCK,
               "Unsupported block size for PBR SpMM. Only 2x2, 4x4, and 8x8 are supported.");
    GL_REQUIRE(A->rows == 0 || (A->stripe_block_ptr && A->remainder_indptr), GL_ERR_INVALID_ARGUMENT,
               "stripe_block_ptr / remainder_indptr are NULL");
    return GL_OK;
}

template <typename S>
StripeArgs<S> make_args(const gl_pbr_matrix* A) {
    StripeArgs<S> a{};
    a.codes = A->block_codes;
    a.coords = A->block_coords;
    a.offsets = A->block_offsets;
    a.bdata = static_cast<const S*>(A->block_data);
    a.rem_ptr = A->remainder_indptr;
    a.rem_col = A->remainder_col_ind;
    a.rem_val = static_cast<const S*>(A->remainder_data);
    a.stripe_ptr = A->stripe_block_ptr;
    a.rows = A->rows;
    a.cols = A->cols;
    a.nstripes = ceil_div(A->rows, A->block_rows);
    a.batch = 1;
    a.num_pieces = A->num_pieces > 0 && A->heavy_of ? A->num_pieces : 0;
    a.piece_work = A->piece_work;
    a.heavy_of = a.num_pieces ? A->heavy_of : nullptr;
    a.heavy_stripe = A->heavy_stripe;
    a.heavy_first = A->heavy_first;
    a.piece_heavy = A->piece_heavy;
    a.piece_range = a.num_pieces ? A->piece_range : nullptr;
    a.variant = A->kernel;
    return a;
}

// Default piece size of the load-balance schedule: stripes above twice this
// many stored entries are cut into pieces.  192 keeps every other stripe
// within the window kernel's 384-entry lists.
constexpr int32_t kDefaultPieceWork = 192;

int64_t workspace_bytes(const gl_pbr_matrix* A, int64_t batch, int64_t K) {
    return workspace_layout(A, batch, K).total;
}

// Points the kernel's scheduler / counter / partial buffers into the
// caller's workspace.  Without a workspace the launch distributes stripes
// statically, which is only possible when no stripe is cut into pieces.
template <typename S>
int bind_workspace(StripeArgs<S>& a, const gl_pbr_matrix* A, int64_t batch, int64_t K, void* ws,
                   int64_t ws_bytes) {
    const WorkspaceLayout w = workspace_layout(A, batch, K);
    if (ws == nullptr && a.num_pieces == 0) {
        a.sched = nullptr;
        return GL_OK;
    }
    GL_REQUIRE(ws != nullptr && ws_bytes >= w.total, GL_ERR_WORKSPACE,
               "SpMM workspace of %lld bytes needed (gl_pbr_spmm_workspace_bytes)", (long long)w.total);
    char* base = static_cast<char*>(ws);
    a.sched = reinterpret_cast<unsigned long long*>(base);
    a.counters = reinterpret_cast<int32_t*>(base + w.counters);
    a.partial = reinterpret_cast<S*>(base + w.partial);
    return GL_OK;
}

// Block and remainder range of every piece of a heavy stripe: the stripe's
// stored entries (packed values, then remainder entries) cut every W
// entries, the block range rounded to whole blocks by the first block whose
// offset reaches the cut (so a block belongs to the piece its first value
// falls in).
__global__ void piece_range_kernel(const int32_t* stripe_ptr, const int32_t* offsets, const int32_t* rem_ptr,
                                   int64_t rows, int br, const int32_t* piece_heavy, const int32_t* heavy_stripe,
                                   const int32_t* heavy_first, int64_t np, int32_t W, int32_t* range) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int32_t h = piece_heavy[p];
    const int64_t s = heavy_stripe[h];
    const int32_t pidx = (int32_t)(p - heavy_first[h]);
    const int32_t sb0 = stripe_ptr[s], sb1 = stripe_ptr[s + 1];
    const int64_t pk0 = offsets[sb0];
    const int64_t pw = (int64_t)offsets[sb1] - pk0;
    const int64_t last_row = (s * br + br < rows) ? s * br + br : rows;
    const int32_t rj0 = rem_ptr[s * br], rj1 = rem_ptr[last_row];
    const int64_t total = pw + (rj1 - rj0);
    const int64_t u0 = (int64_t)pidx * W;
    const int64_t u1 = (u0 + W < total) ? u0 + W : total;
    range[4 * p + 0] = lower_bound_i32(offsets, sb0, sb1, pk0 + u0);
    range[4 * p + 1] = (u1 >= pw) ? sb1 : lower_bound_i32(offsets, sb0, sb1, pk0 + u1);
    range[4 * p + 2] = rj0 + (int32_t)(u0 > pw ? u0 - pw : 0);
    range[4 * p + 3] = rj0 + (int32_t)(u1 > pw ? u1 - pw : 0);
}

__global__ void stripe_work_kernel(const int32_t* stripe_ptr, const int32_t* offsets, const int32_t* rem_ptr,
                                   int64_t rows, int br, int64_t ns, int32_t* work) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const int64_t last = (s * br + br < rows) ? s * br + br : rows;
    const int64_t w = (int64_t)offsets[stripe_ptr[s + 1]] - offsets[stripe_ptr[s]] +
                      (int64_t)rem_ptr[last] - rem_ptr[s * br];
    work[s] = (int32_t)(w < INT32_MAX ? w : INT32_MAX);
}

// Consistency of PBR arrays that did not come from this library's builder
// (error bits: 1 offsets / popcounts, 2 block coordinates, 4 bits past the
// matrix edge, 8 remainder row pointers, 16 remainder columns, 32 stripe
// pointers).  Only reads inside the arrays' declared sizes.
__global__ void validate_pbr_kernel(const uint64_t* codes, const int32_t* coords, const int32_t* offsets,
                                    int64_t nb, int64_t packed, const int32_t* rem_ptr, const int32_t* rem_col,
                                    int64_t rem, const int32_t* stripe_ptr, int64_t rows, int64_t cols, int br,
                                    int bc, int32_t* flag) {
    const int64_t ns = ceil_div(rows, br);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t bad = 0;
    if (i0 == 0) {
        if (nb > 0 && (offsets[0] != 0 || offsets[nb] != packed)) bad |= 1;
        if (nb == 0 && packed != 0) bad |= 1;
        if (rem_ptr[0] != 0 || rem_ptr[rows] != rem) bad |= 8;
        if (stripe_ptr && (stripe_ptr[0] != 0 || stripe_ptr[ns] != nb)) bad |= 32;
    }
    const uint32_t rowmask = bc >= 32 ? 0xffffffffu : ((1u << bc) - 1u);
    for (int64_t b = i0; b < nb; b += stride) {
        const uint64_t code = codes[b];
        if ((int64_t)offsets[b + 1] - offsets[b] != __popcll(code)) bad |= 1;
        const int64_t r0 = coords[2 * b], c0 = coords[2 * b + 1];
        if (r0 < 0 || r0 >= rows || c0 < 0 || c0 >= cols || r0 % br != 0 || c0 % bc != 0) {
            bad |= 2;
            continue;
        }
        uint32_t colbits = 0;
        for (int r = 0; r < br; ++r) {
            const uint32_t rb = (uint32_t)(code >> (r * bc)) & rowmask;
            if (rb && r0 + r >= rows) bad |= 4;
            colbits |= rb;
        }
        if (br * bc < 64 && (code >> (br * bc)) != 0) bad |= 4;
        if (colbits && c0 + (31 - __clz(colbits)) >= cols) bad |= 4;
        if (stripe_ptr) {
            const int64_t s = r0 / br;
            if (!(b >= stripe_ptr[s] && b < stripe_ptr[s + 1])) bad |= 32;
        }
    }
    for (int64_t r = i0; r < rows; r += stride)
        if (rem_ptr[r + 1] < rem_ptr[r]) bad |= 8;
    for (int64_t j = i0; j < rem; j += stride) {
        const int32_t c = rem_col[j];
        if (c < 0 || c >= cols) bad |= 16;
    }
    if (stripe_ptr)
        for (int64_t s = i0; s < ns; s += stride)
            if (stripe_ptr[s + 1] < stripe_ptr[s]) bad |= 32;
    if (bad) atomicOr(flag, bad);
}

__global__ void stripe_index_kernel(const int32_t* coords, int64_t nb, int64_t rows, int br, int64_t ns,
                                    int32_t* ptr, int32_t* flag) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b > nb) return;
    int64_t s_cur;
    if (b < nb) {
        const int64_t r0 = coords[2 * b];
        if (r0 < 0 || r0 >= rows || r0 % br != 0) {
            atomicOr(flag, 1);
            return;
        }
        s_cur = r0 / br;
    } else {
        s_cur = ns;
    }
    int64_t s_prev = -1;
    if (b > 0) {
        const int64_t rp = coords[2 * (b - 1)];
        s_prev = (rp >= 0 && rp < rows) ? rp / br : -1;
    }
    if (s_cur < s_prev) {
        atomicOr(flag, 1);
        return;
    }
    for (int64_t s = s_prev + 1; s <= s_cur; ++s) ptr[s] = (int32_t)b;
}

// One thread per seed entry (grid-stride): its column is found by binary
// search in seed_ptr, so a column with millions of seeds (a uniform teleport
// vector) is spread over the whole grid instead of one thread.  Pass 1
// counts the entries of each stripe; pass 2 scatters them.  Slots within a
// stripe come from atomics, so their order is unspecified; the step's
// epilogue adds each entry to its own (row, column) element, so results do
// not depend on it unless a (seed, column) pair repeats.
__global__ void teleport_count_kernel(int64_t K, const int32_t* seed_ptr, const int32_t* seed_idx,
                                      int64_t num_seeds, int64_t rows, int br, int32_t* counters, int64_t ns,
                                      int32_t* stripe_ptr, int32_t* row, int32_t* col, float* weight,
                                      const float* seed_w, bool scatter) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < num_seeds;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = K;                 // last column k with seed_ptr[k] <= e
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (seed_ptr[mid] <= e) lo = mid; else hi = mid;
        }
        const int64_t k = lo;
        const int32_t e0 = seed_ptr[k], e1 = seed_ptr[k + 1];
        if (e < e0 || e >= e1) {                // seed_ptr not covering [0, num_seeds)
            atomicOr(&counters[ns], 2);
            continue;
        }
        const int64_t r = seed_idx[e];
        if (r < 0 || r >= rows) {
            atomicOr(&counters[ns], 1);
            continue;
        }
        const int64_t s = r / br;
        if (!scatter) {
            atomicAdd(&counters[s], 1);
        } else {
            const int32_t slot = stripe_ptr[s] + atomicAdd(&counters[s], 1);
            row[slot] = (int32_t)r;
            col[slot] = (int32_t)k;
            weight[slot] = seed_w ? seed_w[e] : 1.0f / (float)(e1 - e0);
        }
    }
}

template <typename S>
__global__ void ppr_init_kernel(const int32_t* row, const int32_t* col, const float* w, int64_t n, int64_t K, S* X,
                                const uint32_t* bitmap, double* d0) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int64_t r = row[e], k = col[e];
    atomicAdd(X + r * K + k, (S)w[e]);
    if (bitmap && ((bitmap[r >> 5] >> (r & 31)) & 1u)) atomicAdd(d0 + k, (double)w[e]);
}

template <typename S>
__global__ void dangling_mass_kernel(const S* X, int64_t rows, int64_t K, const uint32_t* bitmap, double* out,
                                     int64_t rows_per_block) {
    const int64_t k = (int64_t)blockIdx.y * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t r1 = r0 + rows_per_block < rows ? r0 + rows_per_block : rows;
    double acc = 0.0;
    for (int64_t r = r0; r < r1; ++r)
        if ((bitmap[r >> 5] >> (r & 31)) & 1u) acc += (double)X[r * K + k];
    if (acc != 0.0) atomicAdd(out + k, acc);
}

__global__ void counter_add_kernel(int32_t* c, int32_t d) { *c += d; }

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" const char* gl_last_error(void) { return last_error(); }
extern "C" int gl_version(void) { return 102; }

extern "C" int64_t gl_pbr_matrix_bytes(void) { return (int64_t)sizeof(gl_pbr_matrix); }

extern "C" int64_t gl_struct_bytes(const char* name) {
    if (name == nullptr) return -1;
    const std::string n(name);
    if (n == "gl_pbr_matrix") return (int64_t)sizeof(gl_pbr_matrix);
    if (n == "gl_pbr_build_counts") return (int64_t)sizeof(gl_pbr_build_counts);
    if (n == "gl_teleport") return (int64_t)sizeof(gl_teleport);
    if (n == "gl_ppr_step_params") return (int64_t)sizeof(gl_ppr_step_params);
    if (n == "gl_ppr_run_result") return (int64_t)sizeof(gl_ppr_run_result);
    return -1;
}

extern "C" int64_t gl_pbr_spmm_workspace_bytes(const gl_pbr_matrix* A, int64_t batch, int64_t features) {
    if (A == nullptr || batch < 0 || features < 0) return -1;
    return workspace_bytes(A, batch, features);
}

extern "C" int64_t gl_pbr_schedule_elems(const gl_pbr_matrix* A, int32_t piece_work) {
    if (A == nullptr || A->block_rows < 1) return -1;
    const int64_t w = piece_work > 0 ? piece_work : kDefaultPieceWork;
    const int64_t ns = ceil_div(A->rows, A->block_rows);
    // heavy_of [ns], heavy_stripe [H], heavy_first [H + 1], piece_heavy [NP],
    // 16-byte padding, piece_range [4 NP]; H <= ns, NP <= (packed + rem) / w + H
    return 8 * ns + 16 + 5 * ((A->packed_nnz + A->remainder_nnz) / w);
}

extern "C" int gl_pbr_schedule_build(gl_pbr_matrix* A, int32_t piece_work, int32_t* buffer, int64_t buffer_elems,
                                     cudaStream_t stream) {
    GL_REQUIRE(A != nullptr && A->block_rows >= 1, GL_ERR_INVALID_ARGUMENT, "bad matrix");
    const int32_t W = piece_work > 0 ? piece_work : kDefaultPieceWork;
    const int64_t need = gl_pbr_schedule_elems(A, W);
    GL_REQUIRE(buffer != nullptr && buffer_elems >= need, GL_ERR_WORKSPACE, "schedule buffer of %lld int32 needed",
               (long long)need);
    const int64_t ns = ceil_div(A->rows, A->block_rows);
    A->num_heavy = 0;
    A->num_pieces = 0;
    A->piece_work = W;
    A->heavy_of = nullptr;
    A->piece_range = nullptr;
    if (ns == 0) return GL_OK;
    stripe_work_kernel<<<(unsigned)ceil_div(ns, 256), 256, 0, stream>>>(A->stripe_block_ptr, A->block_offsets,
                                                                        A->remainder_indptr, A->rows, A->block_rows,
                                                                        ns, buffer);
    GL_LAUNCH_CHECK("stripe_work_kernel");
    std::vector<int32_t> work(ns);
    GL_CUDA_TRY(cudaMemcpyAsync(work.data(), buffer, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    std::vector<int32_t> heavy_of(ns, -1), heavy_stripe, heavy_first(1, 0), piece_heavy;
    for (int64_t s = 0; s < ns; ++s) {
        if (work[s] > 2 * W) {
            const int32_t h = (int32_t)heavy_stripe.size();
            const int32_t np = (int32_t)ceil_div(work[s], W);
            heavy_of[s] = h;
            heavy_stripe.push_back((int32_t)s);
            for (int32_t q = 0; q < np; ++q) piece_heavy.push_back(h);
            heavy_first.push_back((int32_t)piece_heavy.size());
        }
    }
    const int64_t H = (int64_t)heavy_stripe.size(), NP = (int64_t)piece_heavy.size();
    if (H == 0) return GL_OK;
    const int64_t range_off = (ns + H + (H + 1) + NP + 3) / 4 * 4;   // 16-byte aligned (int4 loads)
    GL_REQUIRE(range_off + 4 * NP <= buffer_elems, GL_ERR_WORKSPACE, "schedule buffer too small");
    GL_REQUIRE(reinterpret_cast<uintptr_t>(buffer) % 16 == 0, GL_ERR_INVALID_ARGUMENT,
               "schedule buffer must be 16-byte aligned");
    int32_t* d_heavy_of = buffer;
    int32_t* d_heavy_stripe = d_heavy_of + ns;
    int32_t* d_heavy_first = d_heavy_stripe + H;
    int32_t* d_piece_heavy = d_heavy_first + H + 1;
    int32_t* d_piece_range = buffer + range_off;
    GL_CUDA_TRY(cudaMemcpyAsync(d_heavy_of, heavy_of.data(), 4 * ns, cudaMemcpyHostToDevice, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(d_heavy_stripe, heavy_stripe.data(), 4 * H, cudaMemcpyHostToDevice, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(d_heavy_first, heavy_first.data(), 4 * (H + 1), cudaMemcpyHostToDevice, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(d_piece_heavy, piece_heavy.data(), 4 * NP, cudaMemcpyHostToDevice, stream));
    piece_range_kernel<<<(unsigned)ceil_div(NP, 256), 256, 0, stream>>>(
        A->stripe_block_ptr, A->block_offsets, A->remainder_indptr, A->rows, A->block_rows, d_piece_heavy,
        d_heavy_stripe, d_heavy_first, NP, W, d_piece_range);
    GL_LAUNCH_CHECK("piece_range_kernel");
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    A->num_heavy = (int32_t)H;
    A->num_pieces = (int32_t)NP;
    A->heavy_of = d_heavy_of;
    A->heavy_stripe = d_heavy_stripe;
    A->heavy_first = d_heavy_first;
    A->piece_heavy = d_piece_heavy;
    A->piece_range = d_piece_range;
    return GL_OK;
}

extern "C" int gl_pbr_spmm(const gl_pbr_matrix* A, const void* X, void* Y, int64_t batch, int64_t features,
                           void* workspace, int64_t workspace_bytes, cudaStream_t stream) {
    int rc = check_matrix(A);
    if (rc != GL_OK) return rc;
    GL_REQUIRE(batch >= 0 && features >= 0, GL_ERR_INVALID_ARGUMENT, "negative batch / features");
    GL_REQUIRE(features < (int64_t)INT32_MAX, GL_ERR_INVALID_ARGUMENT, "too many features");
    if (batch == 0 || features == 0 || A->rows == 0) return GL_OK;
    GL_REQUIRE(X != nullptr && Y != nullptr, GL_ERR_INVALID_ARGUMENT, "X / Y is NULL");
    if (A->value_type == GL_F32) {
        StripeArgs<float> a = make_args<float>(A);
        a.batch = batch;
        a.K = (int32_t)features;
        a.X = static_cast<const float*>(X);
        a.Y = static_cast<float*>(Y);
        if ((rc = bind_workspace(a, A, batch, features, workspace, workspace_bytes)) != GL_OK) return rc;
        return launch_stripe<float, false>(a, A->block_rows, A->block_cols, A->column_tile, A->lane_split, stream);
    }
    StripeArgs<double> a = make_args<double>(A);
    a.batch = batch;
    a.K = (int32_t)features;
    a.X = static_cast<const double*>(X);
    a.Y = static_cast<double*>(Y);
    if ((rc = bind_workspace(a, A, batch, features, workspace, workspace_bytes)) != GL_OK) return rc;
    return launch_stripe<double, false>(a, A->block_rows, A->block_cols, A->column_tile, A->lane_split, stream);
}

extern "C" int gl_spmm_workspace_error(void* workspace, cudaStream_t stream) {
    GL_REQUIRE(workspace != nullptr, GL_ERR_INVALID_ARGUMENT, "workspace is NULL");
    int32_t* word = reinterpret_cast<int32_t*>(static_cast<char*>(workspace) + 16);
    int32_t v = 0;
    GL_CUDA_TRY(cudaMemcpyAsync(&v, word, sizeof(v), cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaMemsetAsync(word, 0, sizeof(v), stream));
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    if (v != GL_OK) set_error("a window-kernel launch on this workspace reported status %d", v);
    return v;
}

extern "C" int gl_pbr_stripe_index(const int32_t* block_coords, int64_t num_blocks, int64_t rows, int32_t block_rows,
                                   int32_t* stripe_block_ptr, int32_t* flag_scratch, cudaStream_t stream) {
    GL_REQUIRE(num_blocks >= 0 && rows >= 0 && block_rows >= 1, GL_ERR_INVALID_ARGUMENT, "bad sizes");
    GL_REQUIRE(stripe_block_ptr && flag_scratch, GL_ERR_INVALID_ARGUMENT, "NULL output");
    const int64_t ns = ceil_div(rows, block_rows);
    GL_CUDA_TRY(cudaMemsetAsync(flag_scratch, 0, sizeof(int32_t), stream));
    GL_CUDA_TRY(cudaMemsetAsync(stripe_block_ptr, 0, sizeof(int32_t) * (ns + 1), stream));
    stripe_index_kernel<<<(unsigned)ceil_div(num_blocks + 1, 256), 256, 0, stream>>>(
        block_coords, num_blocks, rows, block_rows, ns, stripe_block_ptr, flag_scratch);
    GL_LAUNCH_CHECK("stripe_index_kernel");
    int32_t flag = 0;
    GL_CUDA_TRY(cudaMemcpyAsync(&flag, flag_scratch, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    GL_REQUIRE(flag == 0, GL_ERR_INVALID_ARGUMENT,
               "PBR blocks must be stored stripe-major with row origins that are multiples of block_rows");
    return GL_OK;
}

extern "C" int gl_pbr_validate(const gl_pbr_matrix* A, int32_t* flag_scratch, cudaStream_t stream) {
    GL_REQUIRE(A != nullptr && flag_scratch != nullptr, GL_ERR_INVALID_ARGUMENT, "NULL argument");
    GL_REQUIRE(A->rows >= 0 && A->cols >= 0 && A->block_rows >= 1 && A->block_cols >= 1 &&
                   A->block_rows * A->block_cols <= 64 && A->num_blocks >= 0 && A->packed_nnz >= 0 &&
                   A->remainder_nnz >= 0,
               GL_ERR_INVALID_ARGUMENT, "bad sizes in the matrix descriptor");
    GL_REQUIRE(A->remainder_indptr != nullptr, GL_ERR_INVALID_ARGUMENT, "remainder_indptr is NULL");
    GL_REQUIRE(A->num_blocks == 0 || (A->block_codes && A->block_coords && A->block_offsets),
               GL_ERR_INVALID_ARGUMENT, "block arrays are NULL");
    GL_REQUIRE(A->remainder_nnz == 0 || A->remainder_col_ind, GL_ERR_INVALID_ARGUMENT, "remainder_col_ind is NULL");
    GL_CUDA_TRY(cudaMemsetAsync(flag_scratch, 0, sizeof(int32_t), stream));
    const int64_t work = std::max<int64_t>(std::max<int64_t>(A->num_blocks, A->rows), A->remainder_nnz) + 1;
    const int64_t cap = (int64_t)num_sms() * 8;
    const int64_t grid = std::min<int64_t>(ceil_div(work, 256), cap);
    validate_pbr_kernel<<<(unsigned)grid, 256, 0, stream>>>(
        reinterpret_cast<const uint64_t*>(A->block_codes), A->block_coords, A->block_offsets, A->num_blocks,
        A->packed_nnz, A->remainder_indptr, A->remainder_col_ind, A->remainder_nnz, A->stripe_block_ptr, A->rows,
        A->cols, A->block_rows, A->block_cols, flag_scratch);
    GL_LAUNCH_CHECK("validate_pbr_kernel");
    int32_t flag = 0;
    GL_CUDA_TRY(cudaMemcpyAsync(&flag, flag_scratch, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    GL_REQUIRE(!(flag & 1), GL_ERR_INVALID_ARGUMENT, "PBR block_offsets do not match the block codes' bit counts");
    GL_REQUIRE(!(flag & 2), GL_ERR_INVALID_ARGUMENT, "PBR block coordinates are off the block grid or the matrix");
    GL_REQUIRE(!(flag & 4), GL_ERR_INVALID_ARGUMENT, "a PBR block code has bits past the matrix edge");
    GL_REQUIRE(!(flag & 8), GL_ERR_INVALID_ARGUMENT, "PBR remainder_indptr is not a valid row pointer array");
    GL_REQUIRE(!(flag & 16), GL_ERR_INVALID_ARGUMENT, "a PBR remainder column index is out of range");
    GL_REQUIRE(!(flag & 32), GL_ERR_INVALID_ARGUMENT, "stripe_block_ptr does not index the blocks stripe by stripe");
    return GL_OK;
}

extern "C" int gl_ppr_teleport_index(int64_t rows, int32_t block_rows, int64_t num_columns, const int32_t* seed_ptr,
                                     const int32_t* seed_idx, const float* seed_weight, int64_t num_seeds,
                                     int32_t* stripe_ptr, int32_t* row, int32_t* col, float* weight,
                                     int32_t* counter_scratch, cudaStream_t stream) {
    GL_REQUIRE(rows >= 0 && block_rows >= 1 && num_columns >= 0 && num_seeds >= 0, GL_ERR_INVALID_ARGUMENT,
               "bad sizes");
    GL_REQUIRE(stripe_ptr && counter_scratch, GL_ERR_INVALID_ARGUMENT, "NULL output");
    const int64_t ns = ceil_div(rows, block_rows);
    GL_CUDA_TRY(cudaMemsetAsync(counter_scratch, 0, sizeof(int32_t) * (ns + 1), stream));
    const int64_t work = num_columns > 0 ? num_seeds : 0;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(work, 256),
                                                                           (int64_t)num_sms() * 8));
    if (work > 0) {
        teleport_count_kernel<<<grid, 256, 0, stream>>>(num_columns, seed_ptr, seed_idx, num_seeds, rows,
                                                        block_rows, counter_scratch, ns, nullptr, nullptr, nullptr,
                                                        nullptr, nullptr, false);
        GL_LAUNCH_CHECK("teleport_count_kernel");
    }
    int32_t bad = 0;
    GL_CUDA_TRY(cudaMemcpyAsync(&bad, counter_scratch + ns, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    GL_REQUIRE(!(bad & 2), GL_ERR_INVALID_ARGUMENT, "seed_ptr does not cover the %lld seeds", (long long)num_seeds);
    GL_REQUIRE(bad == 0, GL_ERR_INVALID_ARGUMENT, "seed node index out of range [0, %lld)", (long long)rows);
    // Per-stripe counts -> stripe_ptr (exclusive scan).  The counters are
    // free once copied, so they double as the scan's scratch (it needs at
    // most ns + 1 elements).
    {
        GL_CUDA_TRY(cudaMemcpyAsync(stripe_ptr, counter_scratch, sizeof(int32_t) * ns, cudaMemcpyDeviceToDevice,
                                    stream));
        GL_CUDA_TRY(cudaMemsetAsync(stripe_ptr + ns, 0, sizeof(int32_t), stream));
        int rc = exclusive_scan<int32_t, OpSum>(stripe_ptr, stripe_ptr, ns + 1, counter_scratch, 0, OpSum(), stream);
        if (rc != GL_OK) return rc;
    }
    GL_CUDA_TRY(cudaMemsetAsync(counter_scratch, 0, sizeof(int32_t) * (ns + 1), stream));
    if (work > 0) {
        teleport_count_kernel<<<grid, 256, 0, stream>>>(num_columns, seed_ptr, seed_idx, num_seeds, rows,
                                                        block_rows, counter_scratch, ns, stripe_ptr, row, col,
                                                        weight, seed_weight, true);
        GL_LAUNCH_CHECK("teleport_count_kernel");
    }
    return GL_OK;
}

extern "C" int gl_ppr_init(const gl_teleport* tp, int64_t rows, int64_t K, int32_t value_type, void* X0,
                           const uint32_t* dangling_bitmap, double* dangling0, cudaStream_t stream) {
    GL_REQUIRE(tp != nullptr && rows >= 0 && K >= 0, GL_ERR_INVALID_ARGUMENT, "bad arguments");
    GL_REQUIRE(value_type == GL_F32 || value_type == GL_F64, GL_ERR_INVALID_ARGUMENT, "bad value_type");
    const size_t es = value_type == GL_F32 ? 4 : 8;
    if (rows * K > 0) GL_CUDA_TRY(cudaMemsetAsync(X0, 0, es * rows * K, stream));
    if (tp->num_entries == 0) return GL_OK;
    const unsigned grid = (unsigned)ceil_div(tp->num_entries, 256);
    const uint32_t* bm = dangling0 ? dangling_bitmap : nullptr;
    if (value_type == GL_F32)
        ppr_init_kernel<float><<<grid, 256, 0, stream>>>(tp->row, tp->col, tp->weight, tp->num_entries, K,
                                                         static_cast<float*>(X0), bm, dangling0);
    else
        ppr_init_kernel<double><<<grid, 256, 0, stream>>>(tp->row, tp->col, tp->weight, tp->num_entries, K,
                                                          static_cast<double*>(X0), bm, dangling0);
    GL_LAUNCH_CHECK("ppr_init_kernel");
    return GL_OK;
}

extern "C" int gl_ppr_dangling_mass(const void* X, int64_t rows, int64_t K, int32_t value_type,
                                    const uint32_t* dangling_bitmap, double* out, cudaStream_t stream) {
    GL_REQUIRE(rows >= 0 && K >= 0 && dangling_bitmap && out, GL_ERR_INVALID_ARGUMENT, "bad arguments");
    if (rows == 0 || K == 0) return GL_OK;
    const int64_t rpb = 4096;
    dim3 grid((unsigned)ceil_div(rows, rpb), (unsigned)ceil_div(K, 128));
    if (value_type == GL_F32)
        dangling_mass_kernel<float><<<grid, 128, 0, stream>>>(static_cast<const float*>(X), rows, K, dangling_bitmap,
                                                              out, rpb);
    else
        dangling_mass_kernel<double><<<grid, 128, 0, stream>>>(static_cast<const double*>(X), rows, K,
                                                               dangling_bitmap, out, rpb);
    GL_LAUNCH_CHECK("dangling_mass_kernel");
    return GL_OK;
}

extern "C" int gl_ppr_step(const gl_pbr_matrix* A, const gl_teleport* tp, const void* X_in, void* X_out, int64_t K,
                           const gl_ppr_step_params* p, void* workspace, int64_t workspace_bytes,
                           cudaStream_t stream) {
    int rc = check_matrix(A);
    if (rc != GL_OK) return rc;
    GL_REQUIRE(tp != nullptr && p != nullptr, GL_ERR_INVALID_ARGUMENT, "NULL teleport / params");
    GL_REQUIRE(A->rows == A->cols, GL_ERR_INVALID_ARGUMENT, "PPR needs a square matrix");
    GL_REQUIRE(K >= 0 && K < (int64_t)INT32_MAX, GL_ERR_INVALID_ARGUMENT, "bad K");
    GL_REQUIRE(p->chunk_base && p->residual_hist && p->dangling_hist, GL_ERR_INVALID_ARGUMENT,
               "NULL iteration buffers");
    GL_REQUIRE(p->stop_mode == GL_PPR_STOP_ALL || p->stop_mode == GL_PPR_STOP_PER_COLUMN, GL_ERR_INVALID_ARGUMENT,
               "bad stop_mode");
    GL_REQUIRE(X_in != X_out, GL_ERR_INVALID_ARGUMENT, "X_in and X_out must be different buffers");
    GL_REQUIRE(p->dangling_target == GL_DANGLING_TO_TELEPORT || p->dangling_target == GL_DANGLING_UNIFORM,
               GL_ERR_INVALID_ARGUMENT, "bad dangling_target");
    if (K == 0 || A->rows == 0) return GL_OK;
    GL_REQUIRE(tp->num_entries == 0 || tp->stripe_ptr, GL_ERR_INVALID_ARGUMENT, "teleport index missing");
#define GL_FILL_PPR(a)                                     \
    (a).batch = 1;                                         \
    (a).K = (int32_t)K;                                    \
    (a).tp_ptr = tp->stripe_ptr;                           \
    (a).tp_row = tp->row;                                  \
    (a).tp_col = tp->col;                                  \
    (a).tp_w = tp->weight;                                 \
    (a).alpha = p->alpha;                                  \
    (a).tol = p->tol;                                      \
    (a).stop_mode = p->stop_mode;                          \
    (a).max_iter = p->max_iterations;                      \
    (a).step = p->step_in_chunk;                           \
    (a).chunk_base = p->chunk_base;                        \
    (a).res_hist = p->residual_hist;                       \
    (a).dang_hist = p->dangling_hist;                      \
    (a).dbitmap = p->dangling_bitmap;                      \
    (a).dang_uniform = p->dangling_target == GL_DANGLING_UNIFORM; \
    (a).col_alpha = p->column_alpha;                       \
    (a).col_tol = p->column_tol
    if (A->value_type == GL_F32) {
        StripeArgs<float> a = make_args<float>(A);
        GL_FILL_PPR(a);
        a.X = static_cast<const float*>(X_in);
        a.Y = static_cast<float*>(X_out);
        if ((rc = bind_workspace(a, A, 1, K, workspace, workspace_bytes)) != GL_OK) return rc;
        return launch_stripe<float, true>(a, A->block_rows, A->block_cols, A->column_tile, A->lane_split, stream);
    }
    StripeArgs<double> a = make_args<double>(A);
    GL_FILL_PPR(a);
    a.X = static_cast<const double*>(X_in);
    a.Y = static_cast<double*>(X_out);
    if ((rc = bind_workspace(a, A, 1, K, workspace, workspace_bytes)) != GL_OK) return rc;
    return launch_stripe<double, true>(a, A->block_rows, A->block_cols, A->column_tile, A->lane_split, stream);
#undef GL_FILL_PPR
}

extern "C" int gl_counter_add(int32_t* counter, int32_t delta, cudaStream_t stream) {
    GL_REQUIRE(counter != nullptr, GL_ERR_INVALID_ARGUMENT, "NULL counter");
    counter_add_kernel<<<1, 1, 0, stream>>>(counter, delta);
    GL_LAUNCH_CHECK("counter_add_kernel");
    return GL_OK;
}

// The whole power iteration behind one call: chunks of `chunk` fused steps
// (gl_ppr_step; step t reads buffer t % 2 and writes the other), one read of
// the chunk's residual rows per chunk, the stop rule checked on the host.
// Steps past the stop (STOP_ALL) or past max_iterations are no-ops on the
// device, so a chunk is always launched whole.
extern "C" int gl_ppr_run(const gl_pbr_matrix* A, const gl_teleport* tp, void* X0, void* X1, int64_t K,
                          const gl_ppr_step_params* params, int32_t init_from_teleport, int32_t chunk,
                          void* workspace, int64_t workspace_bytes, int32_t* column_iterations,
                          gl_ppr_run_result* result, cudaStream_t stream) {
    GL_REQUIRE(A && tp && X0 && X1 && params && result, GL_ERR_INVALID_ARGUMENT, "NULL argument");
    GL_REQUIRE(X0 != X1, GL_ERR_INVALID_ARGUMENT, "X0 and X1 must be different buffers");
    GL_REQUIRE(K >= 0 && K < (int64_t)INT32_MAX && chunk >= 1 && params->max_iterations >= 0,
               GL_ERR_INVALID_ARGUMENT, "bad K / chunk / max_iterations");
    gl_ppr_step_params p = *params;
    GL_REQUIRE(p.chunk_base && p.residual_hist && p.dangling_hist, GL_ERR_INVALID_ARGUMENT,
               "NULL iteration buffers");
    const int32_t max_it = p.max_iterations;
    const int64_t rows = A->rows;
    result->iterations = max_it;
    result->converged = 0;
    result->result_in_x1 = 0;
    GL_CUDA_TRY(cudaMemsetAsync(p.residual_hist, 0, sizeof(double) * (size_t)(max_it > 0 ? max_it : 1) * K, stream));
    GL_CUDA_TRY(cudaMemsetAsync(p.dangling_hist, 0, sizeof(double) * (size_t)(max_it + 1) * K, stream));
    GL_CUDA_TRY(cudaMemsetAsync(const_cast<int32_t*>(p.chunk_base), 0, sizeof(int32_t), stream));
    int rc = GL_OK;
    if (init_from_teleport)
        rc = gl_ppr_init(tp, rows, K, A->value_type, X0, p.dangling_bitmap,
                         p.dangling_bitmap ? p.dangling_hist : nullptr, stream);
    else if (p.dangling_bitmap)
        rc = gl_ppr_dangling_mass(X0, rows, K, A->value_type, p.dangling_bitmap, p.dangling_hist, stream);
    if (rc != GL_OK) return rc;
    std::vector<double> thr((size_t)K, p.tol);
    if (p.stop_mode == GL_PPR_STOP_PER_COLUMN && p.column_tol && K > 0)
        GL_CUDA_TRY(cudaMemcpyAsync(thr.data(), p.column_tol, sizeof(double) * K, cudaMemcpyDeviceToHost, stream));
    std::vector<double> res((size_t)chunk * (size_t)K);
    std::vector<int32_t> first((size_t)K, -1);
    void* bufs[2] = {X0, X1};
    int64_t done = 0, written = max_it;
    int64_t finished = 0;
    bool stop = K == 0 || rows == 0;
    if (stop) {
        result->iterations = 0;
        result->converged = 1;
        written = 0;
    }
    while (!stop && done < max_it) {
        for (int32_t i = 0; i < chunk; ++i) {
            p.step_in_chunk = i;
            rc = gl_ppr_step(A, tp, bufs[(done + i) & 1], bufs[(done + i + 1) & 1], K, &p, workspace,
                             workspace_bytes, stream);
            if (rc != GL_OK) return rc;
        }
        rc = gl_counter_add(const_cast<int32_t*>(p.chunk_base), chunk, stream);
        if (rc != GL_OK) return rc;
        const int64_t n = std::min<int64_t>(chunk, max_it - done);
        GL_CUDA_TRY(cudaMemcpyAsync(res.data(), p.residual_hist + done * K, sizeof(double) * (size_t)(n * K),
                                    cudaMemcpyDeviceToHost, stream));
        GL_CUDA_TRY(cudaStreamSynchronize(stream));
        for (int64_t t = 0; t < n && !stop; ++t) {
            const double* row = res.data() + t * K;
            double worst = 0.0;
            for (int64_t k = 0; k < K; ++k) {
                worst = std::max(worst, row[k]);
                if (first[k] < 0 && row[k] < thr[k]) {
                    first[k] = (int32_t)(done + t + 1);
                    ++finished;
                }
            }
            if (p.stop_mode == GL_PPR_STOP_ALL ? worst < p.tol : finished == K) {
                result->iterations = (int32_t)(done + t + 1);
                result->converged = 1;
                // STOP_ALL: the steps after the stop wrote nothing; per column,
                // stopped columns are carried into every later buffer
                written = p.stop_mode == GL_PPR_STOP_ALL ? done + t + 1 : std::min<int64_t>(done + chunk, max_it);
                stop = true;
            }
        }
        done += chunk;
    }
    result->result_in_x1 = (int32_t)(written & 1);
    if (column_iterations && K > 0) std::copy(first.begin(), first.end(), column_iterations);
    return GL_OK;
}
