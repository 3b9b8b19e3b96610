/*
 * graph_link_gb300 — C ABI of the GB300 (sm_103a) Personalized-PageRank engine.
 *
 * Plain extern "C" functions over raw device pointers, sizes and a
 * cudaStream_t.  No torch types cross this boundary.  Every function returns a
 * status code (GL_OK == 0); gl_last_error() gives the text of the last failure
 * on the calling thread.  Outputs are owned by the caller.  Nothing here
 * synchronizes the stream unless its comment says so.
 *
 * The reference (Dayan135/Page_Rank, package graph_link) has no C ABI: its
 * native layer is the pybind11 module `graph_link_core`.  Each entry point
 * below names the reference function or kernel launcher it replaces.
 */
#ifndef GRAPH_LINK_GB300_H
#define GRAPH_LINK_GB300_H

#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GL_OK                    0
#define GL_ERR_INVALID_ARGUMENT  1  /* maps to ValueError                      */
#define GL_ERR_UNSUPPORTED_BLOCK 2  /* maps to ValueError (pbr_kernel.cu:392)  */
#define GL_ERR_OOM               3  /* maps to MemoryError / RuntimeError      */
#define GL_ERR_CUDA              4  /* maps to RuntimeError                    */
#define GL_ERR_TIMEOUT           5  /* bounded device wait gave up             */
#define GL_ERR_NONCANONICAL      6  /* CSR row not strictly increasing         */
#define GL_ERR_WORKSPACE         7  /* workspace too small                     */

/* ---- element types ------------------------------------------------------ */
#define GL_I32 0
#define GL_I64 1
#define GL_F32 0
#define GL_F64 1

/* Text of the last error raised on the calling thread ("" when none). */
const char* gl_last_error(void);
/* ABI version of this library (major * 100 + minor). */
int gl_version(void);
/* sizeof(gl_pbr_matrix) in this library: a binding that declares the
 * descriptor itself (ctypes, cgo, JNI) checks its own size against it. */
int64_t gl_pbr_matrix_bytes(void);
/* sizeof of any struct this header declares, by name ("gl_pbr_matrix",
 * "gl_pbr_build_counts", "gl_teleport", "gl_ppr_step_params",
 * "gl_ppr_run_result"); -1 for another name. */
int64_t gl_struct_bytes(const char* name);

/*
 * A PBR matrix resident in device memory.  Field meaning follows the
 * reference's pbr_matrix_t (Backend/graph_link/pbr_matrix/pbr_matrix.hpp:98-167)
 * and the seven tensors its `.to()` uploads (graph_link/__init__.py:43-51):
 * block codes as int64 bit patterns, int32 (row0, col0) coordinate pairs,
 * int32 offsets into block_data (num_blocks + 1 entries), packed values in
 * row-major bit order, and a CSR remainder with int32 indices.
 *
 * stripe_block_ptr has no reference counterpart: entry s is the first block
 * of stripe s (blocks are stored stripe-major, as the reference builder emits
 * them), with ceil(rows / block_rows) + 1 entries.  gl_pbr_stripe_index()
 * derives it from block_coords.
 *
 * The load-balance schedule (no reference counterpart) is optional: with
 * num_pieces == 0 every stripe is one work unit.  gl_pbr_schedule_build()
 * fills it: stripes holding more than 2 * piece_work stored entries are cut
 * into pieces of piece_work entries, processed independently and reduced in
 * piece order.  column_tile caps the columns one warp covers (0: automatic).
 * lane_split picks how a warp's lanes share a stripe for 64..127 columns:
 * 0 automatic (half-warps for the SpMM), 1 all 32 lanes on each nonzero, 2 two half-warps taking
 * alternate nonzeros (float4 lanes).
 */
typedef struct gl_pbr_matrix {
    int64_t rows, cols;
    int32_t block_rows, block_cols;
    int64_t num_blocks, packed_nnz, remainder_nnz;
    int32_t value_type;                 /* GL_F32 or GL_F64                  */
    const int64_t* block_codes;         /* [num_blocks]                      */
    const int32_t* block_coords;        /* [2 * num_blocks]                  */
    const int32_t* block_offsets;       /* [num_blocks + 1]                  */
    const void*    block_data;          /* [packed_nnz]                      */
    const int32_t* remainder_indptr;    /* [rows + 1]                        */
    const int32_t* remainder_col_ind;   /* [remainder_nnz]                   */
    const void*    remainder_data;      /* [remainder_nnz]                   */
    const int32_t* stripe_block_ptr;    /* [ceil(rows/block_rows) + 1]       */
    /* load-balance schedule (see above) */
    int32_t num_heavy, num_pieces, piece_work, column_tile, lane_split;
    const int32_t* heavy_of;            /* [num_stripes]: heavy index or -1  */
    const int32_t* heavy_stripe;        /* [num_heavy]                       */
    const int32_t* heavy_first;         /* [num_heavy + 1]: first piece      */
    const int32_t* piece_heavy;         /* [num_pieces]: owning heavy index  */
    /* SpMM kernel: 0 automatic, 1 the stripe kernel, 2 the window kernel
     * (see gl_pbr_spmm; falls back to the stripe kernel where it does not
     * apply).  Added in ABI version 101. */
    int32_t kernel;
    /* [num_pieces][4]: each piece's first and end block and first and end
     * remainder entry, filled by gl_pbr_schedule_build (NULL: the kernels
     * find them by binary search).  Added in ABI version 101. */
    const int32_t* piece_range;
} gl_pbr_matrix;

/* ======================================================================== */
/* Edge list -> transition matrix on the device                             */
/* Replaces the request path of the reference service between the JSON body
 * and csr_to_pbr: the COO -> CSR construction of A[target, source] = weight
 * (Backend/server/app.py:111-131) and normalize_transition_matrix
 * (graph_link/__init__.py:184-207), except that a dangling column stays
 * empty and is flagged in `dangling` instead of becoming N values of 1/N.  */
/* ======================================================================== */
/* Device workspace (bytes) for gl_edges_to_transition; -1 for sizes above
 * INT32_MAX - 1. */
int64_t gl_edges_workspace_bytes(int64_t num_nodes, int64_t num_edges);

/* Edges i with 0 <= source[i], target[i] < num_nodes and a finite weight > 0
 * are kept (others skipped, as app.py:114-122 does); A[target, source] sums
 * their FP32-rounded weights, duplicates left to right in input order.  With
 * normalize != 0 every column is divided by its FP32 sum, computed as scipy's
 * csc.sum(axis=0) does (first entry + numpy pairwise sum of the rest, rows
 * increasing); exact-zero products are dropped and dangling[j] (may be NULL)
 * = 1 for a zero column sum.  Outputs: indptr [num_nodes + 1] int32,
 * indices / data with room for num_edges entries, *nnz (device int64) the
 * stored count.  Rows come out sorted by column.  Asynchronous on `stream`.
 * The result equals the reference's bit for bit whenever scipy's per-row sort
 * keeps duplicate edges in input order (rows of at most 16 entries, at most
 * two copies of a pair, or equal weights); otherwise a sum of three or more
 * duplicates may differ in rounding. */
int gl_edges_to_transition(int64_t num_nodes, int64_t num_edges, const int32_t* source,
                           const int32_t* target, const double* weight, int32_t normalize,
                           int32_t* indptr, int32_t* indices, float* data, uint8_t* dangling,
                           int64_t* nnz, void* workspace, int64_t workspace_bytes,
                           cudaStream_t stream);

/* ======================================================================== */
/* PBR builder on the device                                                */
/* Replaces csr_to_pbr<index_t, scalar_t> (pbr_matrix/pbr_matrix.cpp:340-477,
 * bound at bindings/bindings.cpp:70-73).  Output is bit-identical to the
 * reference builder for canonical CSR input (sorted, duplicate-free rows),
 * including the order of the blocks inside each stripe.                    */
/* ======================================================================== */
typedef struct gl_pbr_build_counts {
    int64_t num_blocks;          /* kept blocks                              */
    int64_t packed_nnz;          /* length of block_data                     */
    int64_t remainder_nnz;       /* length of remainder_col_ind / _data      */
    int64_t max_stripe_blocks;   /* most distinct blocks in one stripe       */
    int64_t distinct_blocks;     /* distinct blocks over all stripes         */
} gl_pbr_build_counts;

/* Device workspace (bytes) the two build phases need. */
int64_t gl_pbr_build_workspace_bytes(int64_t rows, int64_t cols, int64_t nnz,
                                     int32_t block_rows, int32_t block_cols);

/* Phase 1: validates the CSR (indices in range, rows strictly increasing),
 * counts blocks / packed values / remainder entries per stripe and row and
 * scans them.  Synchronizes `stream` to return the totals in *counts.  Both
 * phases run on the current device, whose stream `stream` must be.
 * index_type: GL_I32 or GL_I64 for indptr and indices.
 * Errors: GL_ERR_INVALID_ARGUMENT (block_rows * block_cols > 64, an index out
 * of range, min_nnz outside 0..255, 2^30 or more stripes),
 * GL_ERR_NONCANONICAL, GL_ERR_WORKSPACE. */
int gl_pbr_build_count(const void* indptr, const void* indices, int32_t index_type,
                       int64_t rows, int64_t cols, int64_t nnz,
                       int32_t block_rows, int32_t block_cols, int32_t min_nnz_per_block,
                       void* workspace, int64_t workspace_bytes,
                       gl_pbr_build_counts* counts, cudaStream_t stream);

/* Phase 2: writes the PBR arrays.  Index outputs use index_type (the
 * reference's PBRMatrixInt32* / PBRMatrixInt64* variants), values use
 * value_type.  block_codes receives the raw 64-bit masks.  stripe_block_ptr
 * (int32, ceil(rows/block_rows)+1 entries) may be NULL.  Must follow
 * gl_pbr_build_count with the same arguments and the workspace as the count
 * left it (the fill reads the count's per-stripe results there); it may be
 * repeated after one count (it resets the counters its kernels draw stripes
 * from).  Synchronizes `stream`. */
int gl_pbr_build_fill(const void* indptr, const void* indices, const void* values,
                      int32_t index_type, int32_t value_type,
                      int64_t rows, int64_t cols, int64_t nnz,
                      int32_t block_rows, int32_t block_cols, int32_t min_nnz_per_block,
                      void* workspace, int64_t workspace_bytes,
                      const gl_pbr_build_counts* counts,
                      uint64_t* block_codes, void* block_coords, void* block_offsets,
                      void* block_data, void* remainder_indptr, void* remainder_col_ind,
                      void* remainder_data, int32_t* stripe_block_ptr, cudaStream_t stream);

/* Derives stripe_block_ptr from block_coords for PBR arrays built elsewhere
 * (e.g. uploaded from the reference builder) and checks that the blocks are
 * stripe-major.  flag_scratch: one device int32.  Synchronizes `stream`.
 * Errors: GL_ERR_INVALID_ARGUMENT when blocks are not stripe-major. */
int gl_pbr_stripe_index(const int32_t* block_coords, int64_t num_blocks, int64_t rows,
                        int32_t block_rows, int32_t* stripe_block_ptr,
                        int32_t* flag_scratch, cudaStream_t stream);

/* Checks PBR arrays built elsewhere (for example by the reference's host
 * builder, pbr_matrix.cpp:340-477, or read from a file) before they reach a
 * kernel: offsets start at 0, end at packed_nnz and step by each code's bit
 * count; block origins lie on the block grid inside the matrix; no code has
 * bits past the matrix edge; remainder_indptr is a row pointer array ending
 * at remainder_nnz with columns in range; stripe_block_ptr (when set)
 * indexes the blocks stripe by stripe.  Reads only inside the declared
 * sizes.  flag_scratch: one device int32.  Synchronizes `stream`.
 * Errors: GL_ERR_INVALID_ARGUMENT naming the first failed property. */
int gl_pbr_validate(const gl_pbr_matrix* A, int32_t* flag_scratch, cudaStream_t stream);

/* int32 elements of the buffer gl_pbr_schedule_build() needs. */
int64_t gl_pbr_schedule_elems(const gl_pbr_matrix* A, int32_t piece_work);

/* Builds the load-balance schedule of A into `buffer` (device int32,
 * gl_pbr_schedule_elems() entries) and sets A's schedule fields to point into
 * it.  piece_work <= 0 selects the default (192).  Synchronizes `stream`. */
int gl_pbr_schedule_build(gl_pbr_matrix* A, int32_t piece_work, int32_t* buffer, int64_t buffer_elems,
                          cudaStream_t stream);

/* ======================================================================== */
/* PBR format tools                                                         */
/* ======================================================================== */
/* Device workspace (bytes) for gl_pbr_to_csr; -1 when the CSR would not fit
 * int32 indices. */
int64_t gl_pbr_to_csr_workspace_bytes(const gl_pbr_matrix* A);

/* PBR -> CSR on the device.  Replaces pbr_to_csr (pbr_matrix/pbr_matrix.cpp:
 * 289-338, bound at bindings/bindings.cpp:75-78): every block value pairs with
 * its code's set bits in row-major bit order, remainder entries keep their
 * rows, and each row comes out sorted by column.  indptr: [rows + 1],
 * indices / data: [packed_nnz + remainder_nnz] (data of A->value_type).
 * Rows that are not a multiple of block_rows are handled (the reference
 * throws there, pbr_matrix.cpp:308-310).  Only stripe_block_ptr and the
 * schedule fields of A are not read.  Asynchronous on `stream`. */
int gl_pbr_to_csr(const gl_pbr_matrix* A, int32_t* indptr, int32_t* indices, void* data,
                  void* workspace, int64_t workspace_bytes, cudaStream_t stream);

/* Device workspace (bytes) for gl_pbr_block_patterns; -1 for too many blocks. */
int64_t gl_pbr_block_patterns_workspace_bytes(int64_t num_blocks);

/* Block-pattern histogram (what the reference's pbr_analyze_csr,
 * pbr_matrix.cpp:71-156, computes from a stripe walk): the distinct codes
 * among block_codes, ascending as unsigned 64-bit values, into
 * unique_codes / counts (room for num_blocks each), their number into
 * *num_unique (device int64), and under the coverage rule "occurrences x bit
 * count >= min_nnz_coverage" (pbr_matrix.cpp:127-141) the device int64
 * totals[4] = { nnz of compressed patterns, nnz of the others, compressed
 * patterns, blocks of compressed patterns }.  Asynchronous on `stream`. */
int gl_pbr_block_patterns(const int64_t* block_codes, int64_t num_blocks, int64_t min_nnz_coverage,
                          uint64_t* unique_codes, int64_t* counts, int64_t* num_unique,
                          int64_t* totals, void* workspace, int64_t workspace_bytes,
                          cudaStream_t stream);

/* ======================================================================== */
/* Fused PBR-block + CSR-remainder SpMM                                     */
/* Replaces pbr_spmm_cuda_dispatch (bindings/bindings_kernels.cu:13-83) and
 * the kernels it launches, launch_pbr_spmm (kernels/pbr_kernel.cu:336-396)
 * and launch_csr_spmm (kernels/pbr_kernel.cu:460-478).  One launch, no
 * atomics, no second stream; Y is overwritten (no pre-zeroing needed).      */
/* ======================================================================== */
/* X: [batch][cols][features], Y: [batch][rows][features], both contiguous,
 * element type A->value_type.  Supported blocks: 2x2, 4x4, 8x8 (others give
 * GL_ERR_UNSUPPORTED_BLOCK, as the reference throws std::invalid_argument).
 *
 * Two kernels implement it.  The window kernel (FP32, features % 4 == 0 and
 * >= 64, 16-byte aligned X and Y, a workspace, a schedule built with
 * piece_work <= 192, cols * features / 4 < 2^29) stages the 64 X rows of each 64-row window
 * in shared memory with bulk asynchronous copies and reads the nonzeros of
 * the window's diagonal block from there; every other case runs the stripe
 * kernel.  A->kernel selects one explicitly.  The window kernel records a
 * bounded wait that gave up, or a unit too large for its lists, in the
 * workspace (gl_spmm_workspace_error). */
/* Workspace (bytes) of gl_pbr_spmm / gl_ppr_step for A's schedule: partial
 * tiles of the heavy-stripe pieces plus one counter per heavy stripe and
 * tile.  It must be zero-filled before its first use; every call leaves the
 * counters at zero again, so it can be reused (not concurrently). */
int64_t gl_pbr_spmm_workspace_bytes(const gl_pbr_matrix* A, int64_t batch, int64_t features);

int gl_pbr_spmm(const gl_pbr_matrix* A, const void* X, void* Y,
                int64_t batch, int64_t features, void* workspace, int64_t workspace_bytes,
                cudaStream_t stream);

/* Reads and clears the error word a window-kernel launch leaves in its
 * workspace: GL_OK, GL_ERR_TIMEOUT (a bounded wait gave up) or
 * GL_ERR_INVALID_ARGUMENT (a unit had more entries than its list; the
 * schedule did not match the matrix).  Synchronizes `stream`.  No
 * counterpart in the reference. */
int gl_spmm_workspace_error(void* workspace, cudaStream_t stream);

/* gl_pbr_spmm for callers that cannot allocate device memory when they call
 * it (a host program whose device memory is all owned by its own allocator,
 * or a latency-critical loop that must not wait on cudaMalloc / cudaFree).
 * No counterpart in the reference.  Same arguments and result as gl_pbr_spmm
 * without the workspace: the scratch lives in a static device array of
 * GL_SPMM_STATIC_SCRATCH_BYTES that every GPU loading this library holds
 * until exit.  Calls needing more scratch than that (see
 * gl_pbr_spmm_workspace_bytes) fail with GL_ERR_WORKSPACE before launching.
 * All calls on a device share the array, so calls that overlap on the GPU
 * race; the array keeps the last call's contents (the call clears what must
 * start at zero).  The first call on a device looks up the array's address
 * with cudaGetSymbolAddress, so make it before any stream capture. */
#define GL_SPMM_STATIC_SCRATCH_BYTES (16u * 1024u * 1024u)
int gl_pbr_spmm_static(const gl_pbr_matrix* A, const void* X, void* Y,
                       int64_t batch, int64_t features, cudaStream_t stream);

/* ======================================================================== */
/* Personalized PageRank                                                    */
/* ======================================================================== */
/*
 * Teleport (personalization) vectors, indexed by stripe so the fused
 * iteration can add them in its epilogue.  Entry e puts weight[e] on
 * (row[e], column col[e]); stripe s owns entries stripe_ptr[s] .. stripe_ptr[s+1].
 */
typedef struct gl_teleport {
    const int32_t* stripe_ptr;   /* [ceil(rows/block_rows) + 1] */
    const int32_t* row;          /* [num_entries]               */
    const int32_t* col;          /* [num_entries]               */
    const float*   weight;       /* [num_entries]               */
    int64_t num_entries;
} gl_teleport;

/* Builds a gl_teleport from per-column seed sets (column k has seeds
 * seed_idx[seed_ptr[k] .. seed_ptr[k+1]) ).  seed_weight NULL gives each
 * seed of column k the weight 1/|S_k| (uniform personalization over the set;
 * the reference's one-seed-per-column case, init_ppr_sources_kernel at
 * kernels/ppr_kernel.cu:199-209, is |S_k| = 1).  Outputs: stripe_ptr
 * (num_stripes + 1), row/col/weight (num_seeds); the order of the entries
 * within a stripe is unspecified (each adds into its own (row, column)
 * element, so results do not depend on it unless a (seed, column) pair
 * repeats).  counter_scratch: device int32[num_stripes + 1].  seed_ptr must
 * be non-decreasing with seed_ptr[0] = 0 and seed_ptr[num_columns] =
 * num_seeds.  Errors: GL_ERR_INVALID_ARGUMENT for a seed outside [0, rows)
 * or a seed_ptr that does not cover the seeds — checked on the device and
 * reported after a stream sync. */
int gl_ppr_teleport_index(int64_t rows, int32_t block_rows, int64_t num_columns,
                          const int32_t* seed_ptr, const int32_t* seed_idx,
                          const float* seed_weight, int64_t num_seeds,
                          int32_t* stripe_ptr, int32_t* row, int32_t* col, float* weight,
                          int32_t* counter_scratch, cudaStream_t stream);

/* X0 = teleport vectors (zero elsewhere), plus the dangling mass of X0 per
 * column into dangling0[K] (double, accumulated: zero it first) when
 * dangling_bitmap is not NULL.  Replaces launch_init_ppr
 * (kernels/ppr_kernel.cu:211-216).  X0: [rows][K] of value_type. */
int gl_ppr_init(const gl_teleport* tp, int64_t rows, int64_t K, int32_t value_type,
                void* X0, const uint32_t* dangling_bitmap, double* dangling0,
                cudaStream_t stream);

/* Dangling mass of a given X per column: out[k] += sum over rows i with
 * bit i set in dangling_bitmap of X[i][k] (for warm starts). */
int gl_ppr_dangling_mass(const void* X, int64_t rows, int64_t K, int32_t value_type,
                         const uint32_t* dangling_bitmap, double* out, cudaStream_t stream);

#define GL_PPR_STOP_ALL        0  /* stop every column when max_k residual < tol */
#define GL_PPR_STOP_PER_COLUMN 1  /* freeze column k once its residual < tol     */

#define GL_DANGLING_TO_TELEPORT 0 /* dangling mass returns through v_k          */
#define GL_DANGLING_UNIFORM     1 /* dangling mass spreads as 1/rows over rows   */

/*
 * One fused power-iteration step (SpMM + alpha-scaling + teleport + dangling
 * mass + per-column L1 residual in one pass):
 *
 *   X_out[:, k] = alpha * A X_in[:, k] + ((1 - alpha) + alpha * d_t[k]) * v_k
 *   residual[t][k] = sum_i |X_out[i, k] - X_in[i, k]|
 *   d_{t+1}[k]     = sum over dangling rows i of X_out[i, k]
 *
 * or, with dangling_target == GL_DANGLING_UNIFORM, the dangling mass is spread
 * evenly instead: X_out[:, k] = alpha * A X_in[:, k] + alpha * d_t[k] / rows
 * + (1 - alpha) * v_k — the same fixed point as the reference's
 * normalize_transition_matrix (graph_link/__init__.py:200-206), which stores a
 * dense 1/N column per dangling node, without storing those columns.
 *
 * where v_k is the teleport vector of column k and d_t the dangling mass of
 * X_in (zero when dangling_bitmap is NULL — the column-stochastic case of the
 * reference update, ppr_update_normalized_kernel at kernels/ppr_kernel.cu:
 * 130-168; with the bitmap it is the missing-mass update of
 * batched_ppr_update_kernel, kernels/ppr_kernel.cu:57-97).
 *
 * The iteration number is t = *chunk_base + step_in_chunk, read on the device
 * so a CUDA graph of several steps can be replayed.  residual_hist is
 * [max_iterations][K] doubles and dangling_hist [max_iterations + 1][K]
 * doubles, both zeroed before the first step; step t accumulates row t of
 * residual_hist and row t + 1 of dangling_hist and reads row t of
 * dangling_hist.  A step is a no-op when t >= max_iterations, or (STOP_ALL)
 * when max_k residual_hist[t-1][k] < tol.  Under STOP_PER_COLUMN, a column
 * whose residual_hist[t-1][k] < tol is copied unchanged and adds 0; a column
 * tile whose columns all stopped is not recomputed (copied once, then left
 * as both iterate buffers already hold it), and the dangling entries of
 * stopped columns are not accumulated.
 * workspace: as for gl_pbr_spmm with batch 1 and K features.
 */
typedef struct gl_ppr_step_params {
    double  alpha;
    double  tol;
    int32_t stop_mode;
    int32_t max_iterations;
    int32_t step_in_chunk;
    const int32_t*  chunk_base;       /* device int32                        */
    double*         residual_hist;    /* device [max_iterations][K]          */
    double*         dangling_hist;    /* device [max_iterations + 1][K]      */
    const uint32_t* dangling_bitmap;  /* device, ceil(rows/32) words, or NULL */
    int32_t         dangling_target;  /* GL_DANGLING_TO_TELEPORT / _UNIFORM  */
    const double*   column_alpha;     /* device [K]: alpha of each column, or
                                         NULL: alpha for every column         */
    const double*   column_tol;       /* device [K]: STOP_PER_COLUMN threshold
                                         of each column, or NULL: tol         */
} gl_ppr_step_params;

int gl_ppr_step(const gl_pbr_matrix* A, const gl_teleport* tp,
                const void* X_in, void* X_out, int64_t K,
                const gl_ppr_step_params* params, void* workspace, int64_t workspace_bytes,
                cudaStream_t stream);

/* Adds `delta` to the device int32 at `counter` (stream-ordered; the node
 * that advances chunk_base at the end of a captured chunk of steps). */
int gl_counter_add(int32_t* counter, int32_t delta, cudaStream_t stream);

typedef struct gl_ppr_run_result {
    int32_t iterations;    /* steps until the stop rule held (max_iterations if it never did) */
    int32_t converged;     /* 1 when the stop rule held                                      */
    int32_t result_in_x1;  /* 1: the final iterate is in X1; 0: in X0                         */
} gl_ppr_run_result;

/* The whole power iteration in one call (the loop of run_personalized_pagerank,
 * graph_link/__init__.py:210-271, which reads the residual back after every
 * step; here once per chunk of `chunk` steps): gl_ppr_step until the stop
 * rule of params->stop_mode holds or params->max_iterations steps ran.
 * params as for gl_ppr_step (step_in_chunk is set here; residual_hist,
 * dangling_hist and *chunk_base are zeroed here).  X0 holds the start
 * [rows][K] (init_from_teleport = 1: X0 is first set to the teleport
 * vectors), X1 is the second iterate buffer; result->result_in_x1 says which
 * holds the answer.  column_iterations (host, K entries, or NULL) receives
 * each column's first step below its threshold (-1: none).  Synchronizes
 * the stream once per chunk. */
int gl_ppr_run(const gl_pbr_matrix* A, const gl_teleport* tp, void* X0, void* X1, int64_t K,
               const gl_ppr_step_params* params, int32_t init_from_teleport, int32_t chunk,
               void* workspace, int64_t workspace_bytes, int32_t* column_iterations,
               gl_ppr_run_result* result, cudaStream_t stream);

/* ======================================================================== */
/* Top-k of PPR columns                                                     */
/* The reference returns all N ranks and leaves the top-X cut to its        */
/* frontend (Backend/server/app.py:146-158); this selects the k highest     */
/* entries of each column on the device, so a caller copies k pairs back.   */
/* ======================================================================== */
#define GL_TOPK_MAX 2048

/* Device workspace (bytes) for gl_topk_columns; -1 for k outside [0,
 * GL_TOPK_MAX] or rows above INT32_MAX. */
int64_t gl_topk_workspace_bytes(int64_t rows, int64_t num_columns, int32_t k);

/* For each selected column c (columns[c], or c itself when columns is NULL)
 * of the row-major FP32 matrix X [rows][ld]: its k largest entries, sorted by
 * value descending and equal values by row ascending, into values [C][k] and
 * indices [C][k] (row numbers); with rows < k the slots past rows hold -inf
 * and -1.  Exact and deterministic (radix select on the values' bits; +0.0
 * ranks above -0.0, a NaN with the sign bit clear above +inf).
 * Asynchronous on `stream`. */
int gl_topk_columns(const float* X, int64_t rows, int64_t ld, const int32_t* columns,
                    int64_t num_columns, int32_t k, float* values, int32_t* indices,
                    void* workspace, int64_t workspace_bytes, cudaStream_t stream);

/* ======================================================================== */
/* Learned warm start: 2-layer MLP kernels                                  */
/* No counterpart in the reference.  f_in inputs (<= GL_MLP_MAX_IN) ->      */
/* GL_MLP_HIDDEN ReLU units -> 1 output.  W1 [hidden][f_in] and w2 [hidden] */
/* are BF16 (uint16 bit patterns); biases, inputs and accumulation FP32.    */
/* ======================================================================== */
#define GL_MLP_MAX_IN 16
#define GL_MLP_HIDDEN 128

/* out[e] = w2 . relu(W1 x_e + b1) + b2 for the n rows x_e of X [n][f_in]. */
int gl_mlp_forward(const float* X, int64_t n, int32_t f_in, const uint16_t* W1, const float* b1,
                   const uint16_t* w2, float b2, float* out, cudaStream_t stream);

/* Gradient of sum_e (out_e - target_e)^2 / 2, added into grad
 * ([W1 | b1 | w2 | b2] in FP32, hidden*f_in + 2*hidden + 1 entries; zero it
 * first) and the loss added into *loss_sum (may be NULL). */
int gl_mlp_backward(const float* X, const float* target, int64_t n, int32_t f_in, const uint16_t* W1,
                    const float* b1, const uint16_t* w2, float b2, float* grad, double* loss_sum,
                    cudaStream_t stream);

/* One Adam step on the FP32 master parameters (same layout as grad, scaled
 * by grad_scale first); refreshes the BF16 copies of W1 and w2.  step >= 1. */
int gl_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t count, float lr,
                float beta1, float beta2, float eps, float grad_scale, int32_t step,
                uint16_t* W1_bf16, uint16_t* w2_bf16, int32_t f_in, cudaStream_t stream);

/* ======================================================================== */
/* Window-solve warm start                                                  */
/* No counterpart in the reference (its iterate starts from the seed        */
/* indicators, Backend/graph_link/kernels/ppr_kernel.cu:199-209).  The node */
/* order is cut into windows of 64 rows; B = I - alpha blockdiag(A_w) over  */
/* the 64 x 64 diagonal window blocks A_w of the transition matrix, stored  */
/* as ceil(n / 64) dense row-major FP32 blocks (rows past n are identity).  */
/* ======================================================================== */

/* blocks[w] = I - alpha A_w from the device CSR of A (int32 indptr /
 * indices, FP32 data; entries of a row whose column is outside the row's
 * window are skipped).  alpha in [0, 1). */
int gl_window_blocks(const int32_t* indptr, const int32_t* indices, const float* data, int64_t n, float alpha,
                     float* blocks, cudaStream_t stream);

/* Inverts every block in place (Gauss-Jordan without pivoting, valid for
 * strictly column diagonally dominant blocks: columns of A summing to at
 * most 1) and stores each inverse transposed: entry (r, q) of block w at
 * blocks[w * 4096 + q * 64 + r].  *status (device int32) is set to 0, then
 * to 1 if a pivot was not positive and finite; the caller reads it after
 * the stream. */
int gl_window_invert(float* blocks, int64_t n, int32_t* status, cudaStream_t stream);

/* Y = scale * B^-1 T window by window (inverses as gl_window_invert leaves
 * them; T, Y, near_field: [n][K] row-major
 * FP32); near_field = near_scale * Y (near_init = 1) or += (near_init = 0),
 * and partial[w][K] = (or +=) the column sums of near_scale * Y over window w
 * (partial may be NULL).  Y or near_field may be NULL, not both. */
int gl_window_apply(const float* inverses, int64_t n, int32_t K, const float* T, float scale, float* Y,
                    float* near_field, float near_scale, int32_t near_init, float* partial, cudaStream_t stream);

/* Device workspace (bytes) for gl_window_finalize; -1 for negative sizes. */
int64_t gl_window_finalize_workspace_bytes(int64_t n, int32_t K);

/* near_field[i][c] += max(0, 1 - sum_w partial[w][c]) * shape[i]: the mass a
 * truncated near field misses, placed along shape (FP32 [n], summing to 1). */
int gl_window_finalize(float* near_field, int64_t n, int32_t K, const float* partial, const float* shape,
                       void* workspace, int64_t workspace_bytes, cudaStream_t stream);

/* Residual of one PPR step from the teleport vector, per column:
 * out[c] = || P(v_c) - v_c ||_1 for P(x) = alpha A x + ((1 - alpha) +
 * alpha d(x)) v_c, d(x) the mass on dangling nodes (bitmap, may be NULL).
 * colsum[j] = sum_i A[i][j] (FP64).  The seed sets are the teleport index
 * (seed_ptr [K + 1], seed_rows unique and increasing within each column,
 * seed_weights); A's column indices must be sorted within each row.  Work
 * per column is bounded by the entries of its seed rows.  A seed outside
 * [0, n) gives -1. */
int gl_cold_residual(const int32_t* indptr, const int32_t* indices, const float* data, const double* colsum,
                     const uint32_t* dangling_bits, int64_t n, const int32_t* seed_ptr, const int32_t* seed_rows,
                     const float* seed_weights, int32_t K, float alpha, double* out, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GRAPH_LINK_GB300_H */
