// gl_pbr_spmm_static: the fused PBR + CSR-remainder SpMM with its scratch
// memory in a fixed device array instead of a caller-provided workspace.
//
// Who needs it: a caller that must not allocate device memory when it calls
// the SpMM.  Typical cases are a host program that owns every byte of device
// memory through its own allocator (a framework's caching pool or a fixed
// per-tenant budget, where an extra driver allocation fails or fragments the
// pool) and passes this library only its input and output buffers, and a
// latency-critical request loop where a cudaMalloc / cudaFree would stall on
// a device-wide synchronization.  Such a caller passes X and Y and nothing
// else; the work scheduler and the partial tiles of the heavy-stripe pieces
// live in g_spmm_scratch below, whose size is fixed at build time.
//
// Costs and limits:
//   * every GPU that loads this library holds GL_SPMM_STATIC_SCRATCH_BYTES
//     of device memory for g_spmm_scratch until the process exits;
//   * each call clears the scratch's scheduler and counter words with one
//     cudaMemsetAsync on the caller's stream before the launch;
//   * a call whose scratch need (gl_pbr_spmm_workspace_bytes) exceeds that
//     size is rejected with GL_ERR_WORKSPACE before anything is launched;
//   * all calls on a device share the one array, which keeps whatever the
//     last call left in it: calls whose kernels overlap on the GPU (for
//     example, issued on two different streams) race on it and must be
//     serialized by the caller;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current); make that first call
//     before any stream capture on that device.
#include <mutex>

#include "gl_common.cuh"
#include "stripe_kernel.cuh"

namespace gl {
namespace {

static __device__ __align__(256) unsigned char g_spmm_scratch[GL_SPMM_STATIC_SCRATCH_BYTES];

void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_spmm_scratch on the current device (set up once per
// device).  In host code the array's name is only a stand-in for the device
// object, so its address must come from the runtime.
int scratch_address(void** out) {
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    GL_REQUIRE(dev >= 0 && dev < kMaxDevices, GL_ERR_INVALID_ARGUMENT, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(setup_mutex());
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_spmm_scratch);
        if (e != cudaSuccess || p == nullptr)
            return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress(g_spmm_scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GL_OK;
}

template <typename S>
StripeArgs<S> static_args(const gl_pbr_matrix* A, const void* X, void* Y, int64_t batch, int64_t features) {
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
    a.batch = batch;
    a.K = (int32_t)features;
    a.X = static_cast<const S*>(X);
    a.Y = static_cast<S*>(Y);
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

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int gl_pbr_spmm_static(const gl_pbr_matrix* A, const void* X, void* Y, int64_t batch,
                                  int64_t features, cudaStream_t stream) {
    GL_REQUIRE(A != nullptr, GL_ERR_INVALID_ARGUMENT, "matrix descriptor is NULL");
    GL_REQUIRE(A->value_type == GL_F32 || A->value_type == GL_F64, GL_ERR_INVALID_ARGUMENT,
               "value_type must be GL_F32 or GL_F64");
    const bool ok_block = (A->block_rows == A->block_cols) &&
                          (A->block_rows == 2 || A->block_rows == 4 || A->block_rows == 8);
    GL_REQUIRE(ok_block, GL_ERR_UNSUPPORTED_BLOCK,
               "Unsupported block size for PBR SpMM. Only 2x2, 4x4, and 8x8 are supported.");
    GL_REQUIRE(batch >= 0 && features >= 0 && features < (int64_t)INT32_MAX, GL_ERR_INVALID_ARGUMENT,
               "bad batch / features");
    const int64_t need = gl_pbr_spmm_workspace_bytes(A, batch, features);
    GL_REQUIRE(need >= 0 && need <= (int64_t)GL_SPMM_STATIC_SCRATCH_BYTES, GL_ERR_WORKSPACE,
               "this SpMM needs %lld bytes of scratch but the static scratch holds %lld bytes; "
               "use gl_pbr_spmm with a caller-provided workspace",
               (long long)need, (long long)GL_SPMM_STATIC_SCRATCH_BYTES);
    if (batch == 0 || features == 0 || A->rows == 0) return GL_OK;
    GL_REQUIRE(X != nullptr && Y != nullptr, GL_ERR_INVALID_ARGUMENT, "X / Y is NULL");
    GL_REQUIRE(A->stripe_block_ptr && A->remainder_indptr, GL_ERR_INVALID_ARGUMENT,
               "stripe_block_ptr / remainder_indptr are NULL");
    // same layout as gl_pbr_spmm's workspace; the scheduler and the counters
    // are cleared here (a launch that never ran to completion cannot leave
    // them dirty for the next call)
    const WorkspaceLayout w = workspace_layout(A, batch, features);
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != GL_OK) return rc;
    GL_CUDA_TRY(cudaMemsetAsync(scratch, 0, (size_t)w.zero_bytes, stream));
    char* base = static_cast<char*>(scratch);
    if (A->value_type == GL_F32) {
        StripeArgs<float> a = static_args<float>(A, X, Y, batch, features);
        a.sched = reinterpret_cast<unsigned long long*>(base);
        a.counters = reinterpret_cast<int32_t*>(base + w.counters);
        a.partial = reinterpret_cast<float*>(base + w.partial);
        return launch_stripe<float, false>(a, A->block_rows, A->block_cols, A->column_tile, A->lane_split, stream);
    }
    StripeArgs<double> a = static_args<double>(A, X, Y, batch, features);
    a.sched = reinterpret_cast<unsigned long long*>(base);
    a.counters = reinterpret_cast<int32_t*>(base + w.counters);
    a.partial = reinterpret_cast<double*>(base + w.partial);
    return launch_stripe<double, false>(a, A->block_rows, A->block_cols, A->column_tile, A->lane_split, stream);
}
