// Warm-start network kernels: a 2-layer MLP (f_in inputs -> 128 ReLU units ->
// 1 output) with BF16 weight matrices, FP32 biases and FP32 accumulation.
// It predicts log-PPR per (node, query) from cheap graph features; the
// predicted vector starts the power iteration (the fixed point is unchanged).
//
//   forward : one thread per example; the weights are expanded from BF16 to
//             FP32 once per CTA into shared memory and read as broadcasts.
//   backward: loss = sum_e (y_e - t_e)^2 / 2.  A persistent CTA takes chunks
//             of 128 examples: phase 1 (thread per example) recomputes the
//             hidden activations into shared memory; phase 2 reduces the
//             chunk into per-thread gradient registers as a small GEMM
//             (dW1 = (dy * 1[h > 0] * w2)^T X, db1, dw2 = dy^T H, db2); the
//             registers are added to the global FP32 gradient once per CTA.
//   adam    : FP32 master weights, BF16 copies rounded to nearest even.
//
// No counterpart in the reference (the learned warm start is new).
#include <cuda_bf16.h>

#include "gl_common.cuh"

namespace gl {
namespace {

constexpr int H = GL_MLP_HIDDEN;
constexpr int FMAX = GL_MLP_MAX_IN;
constexpr int kFwdThreads = 256;
constexpr int kBwdThreads = 256;
constexpr int kChunk = 128;

__device__ __forceinline__ float bf16_to_f32(uint16_t b) { return __uint_as_float(((uint32_t)b) << 16); }

__global__ void __launch_bounds__(kFwdThreads) mlp_forward_kernel(const float* __restrict__ X, int64_t n, int f_in,
                                                                   const uint16_t* __restrict__ W1,
                                                                   const float* __restrict__ b1,
                                                                   const uint16_t* __restrict__ w2, float b2,
                                                                   float* __restrict__ out) {
    __shared__ float sW1[H * FMAX];
    __shared__ float sb1[H];
    __shared__ float sw2[H];
    for (int i = threadIdx.x; i < H * f_in; i += blockDim.x) sW1[i] = bf16_to_f32(W1[i]);
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        sb1[i] = b1[i];
        sw2[i] = bf16_to_f32(w2[i]);
    }
    __syncthreads();
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float x[FMAX];
#pragma unroll
        for (int i = 0; i < FMAX; ++i) x[i] = i < f_in ? X[e * f_in + i] : 0.f;
        float y = b2;
        for (int j = 0; j < H; ++j) {
            float h = sb1[j];
#pragma unroll
            for (int i = 0; i < FMAX; ++i)
                if (i < f_in) h = fmaf(sW1[j * f_in + i], x[i], h);
            y = fmaf(sw2[j], fmaxf(h, 0.f), y);
        }
        out[e] = y;
    }
}

// Gradient layout (FP32): [W1: H * f_in][b1: H][w2: H][b2: 1].
__global__ void __launch_bounds__(kBwdThreads) mlp_backward_kernel(const float* __restrict__ X,
                                                                    const float* __restrict__ target, int64_t n,
                                                                    int f_in, const uint16_t* __restrict__ W1,
                                                                    const float* __restrict__ b1,
                                                                    const uint16_t* __restrict__ w2, float b2,
                                                                    float* __restrict__ grad, double* loss_sum) {
    extern __shared__ __align__(16) float smem[];
    float* sW1 = smem;                    // H * FMAX
    float* sb1 = sW1 + H * FMAX;          // H
    float* sw2 = sb1 + H;                 // H
    float* sH = sw2 + H;                  // kChunk * H   (ReLU outputs)
    float* sX = sH + kChunk * H;          // kChunk * FMAX
    float* sdy = sX + kChunk * FMAX;      // kChunk
    __shared__ double s_loss[kBwdThreads / 32];

    for (int i = threadIdx.x; i < H * f_in; i += blockDim.x) sW1[i] = bf16_to_f32(W1[i]);
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        sb1[i] = b1[i];
        sw2[i] = bf16_to_f32(w2[i]);
    }
    // phase-2 ownership: thread t owns hidden unit j = t % H and the half
    // (t / H) of the input features (plus db1[j] for the first half, dw2[j]
    // for the second), so every gradient entry has exactly one owner.
    const int j = threadIdx.x % H;
    const int half = threadIdx.x / H;                      // 0 or 1
    const int i_lo = half * ((f_in + 1) / 2);
    const int i_hi = half == 0 ? (f_in + 1) / 2 : f_in;
    float gW[(FMAX + 1) / 2];
#pragma unroll
    for (int q = 0; q < (FMAX + 1) / 2; ++q) gW[q] = 0.f;
    float gB = 0.f;      // db1[j] (half 0) or dw2[j] (half 1)
    float gb2 = 0.f;
    double loss = 0.0;
    __syncthreads();

    for (int64_t c0 = (int64_t)blockIdx.x * kChunk; c0 < n; c0 += (int64_t)gridDim.x * kChunk) {
        const int cn = (int)((n - c0) < kChunk ? (n - c0) : kChunk);
        // phase 1: thread e < cn recomputes example c0 + e
        if (threadIdx.x < kChunk) {
            const int e = threadIdx.x;
            if (e < cn) {
                float x[FMAX];
#pragma unroll
                for (int i = 0; i < FMAX; ++i) {
                    x[i] = i < f_in ? X[(c0 + e) * f_in + i] : 0.f;
                    sX[e * FMAX + i] = x[i];
                }
                float y = b2;
                for (int jj = 0; jj < H; ++jj) {
                    float h = sb1[jj];
#pragma unroll
                    for (int i = 0; i < FMAX; ++i)
                        if (i < f_in) h = fmaf(sW1[jj * f_in + i], x[i], h);
                    h = fmaxf(h, 0.f);
                    sH[e * H + jj] = h;
                    y = fmaf(sw2[jj], h, y);
                }
                const float dy = y - target[c0 + e];
                sdy[e] = dy;
                loss += 0.5 * (double)dy * (double)dy;
            } else {
                sdy[e] = 0.f;
            }
        }
        __syncthreads();
        // phase 2: reduce the chunk
        const float w2j = sw2[j];
        for (int e = 0; e < cn; ++e) {
            const float dy = sdy[e];
            const float h = sH[e * H + j];
            const float g = (h > 0.f) ? dy * w2j : 0.f;   // d loss / d pre-activation j
            if (half == 0) gB += g;
            else gB = fmaf(dy, h, gB);
#pragma unroll
            for (int q = 0; q < (FMAX + 1) / 2; ++q) {
                const int i = i_lo + q;
                if (i < i_hi) gW[q] = fmaf(g, sX[e * FMAX + i], gW[q]);
            }
            if (threadIdx.x == 0) gb2 += dy;
        }
        __syncthreads();
    }
    // one global add per gradient entry per CTA
#pragma unroll
    for (int q = 0; q < (FMAX + 1) / 2; ++q) {
        const int i = i_lo + q;
        if (i < i_hi && gW[q] != 0.f) atomicAdd(grad + j * f_in + i, gW[q]);
    }
    if (gB != 0.f) atomicAdd(grad + H * f_in + (half == 0 ? 0 : H) + j, gB);
    if (threadIdx.x == 0 && gb2 != 0.f) atomicAdd(grad + H * f_in + 2 * H, gb2);
    // loss: warp then CTA reduction
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBwdThreads / 32; ++w) t += s_loss[w];
        if (loss_sum && t != 0.0) atomicAdd(loss_sum, t);
    }
}

__device__ __forceinline__ uint16_t f32_to_bf16_rne(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

__global__ void mlp_adam_kernel(float* params, const float* grad, float* m, float* v, int64_t count, float lr,
                                float beta1, float beta2, float eps, float grad_scale, float bc1, float bc2,
                                uint16_t* W1_bf16, uint16_t* w2_bf16, int f_in) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    const float g = grad[p] * grad_scale;
    const float mp = beta1 * m[p] + (1.f - beta1) * g;
    const float vp = beta2 * v[p] + (1.f - beta2) * g * g;
    m[p] = mp;
    v[p] = vp;
    const float upd = lr * (mp / bc1) / (sqrtf(vp / bc2) + eps);
    const float w = params[p] - upd;
    params[p] = w;
    const int64_t nW1 = (int64_t)H * f_in;
    if (p < nW1) W1_bf16[p] = f32_to_bf16_rne(w);
    else if (p >= nW1 + H && p < nW1 + 2 * H) w2_bf16[p - nW1 - H] = f32_to_bf16_rne(w);
}

int check_mlp(int64_t n, int f_in) {
    GL_REQUIRE(n >= 0, GL_ERR_INVALID_ARGUMENT, "negative example count");
    GL_REQUIRE(f_in >= 1 && f_in <= FMAX, GL_ERR_INVALID_ARGUMENT, "f_in must be in 1..%d", FMAX);
    return GL_OK;
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int gl_mlp_forward(const float* X, int64_t n, int32_t f_in, const uint16_t* W1, const float* b1,
                              const uint16_t* w2, float b2, float* out, cudaStream_t stream) {
    int rc = check_mlp(n, f_in);
    if (rc != GL_OK) return rc;
    if (n == 0) return GL_OK;
    int64_t blocks = ceil_div(n, kFwdThreads);
    const int64_t cap = (int64_t)num_sms() * 8;
    if (blocks > cap) blocks = cap;
    mlp_forward_kernel<<<(unsigned)blocks, kFwdThreads, 0, stream>>>(X, n, f_in, W1, b1, w2, b2, out);
    GL_LAUNCH_CHECK("mlp_forward_kernel");
    return GL_OK;
}

extern "C" int gl_mlp_backward(const float* X, const float* target, int64_t n, int32_t f_in, const uint16_t* W1,
                               const float* b1, const uint16_t* w2, float b2, float* grad, double* loss_sum,
                               cudaStream_t stream) {
    int rc = check_mlp(n, f_in);
    if (rc != GL_OK) return rc;
    GL_REQUIRE(grad != nullptr, GL_ERR_INVALID_ARGUMENT, "grad is NULL");
    if (n == 0) return GL_OK;
    const size_t smem = sizeof(float) * (H * FMAX + 2 * H + kChunk * H + kChunk * FMAX + kChunk);
    // the shared-memory attribute is per device: set once on every device
    static std::atomic<int> attr_cache[kMaxDevices];
    int attr = 0;
    rc = per_device_value(
        attr_cache,
        [&](int* v) {
            GL_CUDA_TRY(
                cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            *v = 1;
            return GL_OK;
        },
        &attr);
    if (rc != GL_OK) return rc;
    int64_t blocks = ceil_div(n, kChunk);
    const int64_t cap = (int64_t)num_sms() * 2;
    if (blocks > cap) blocks = cap;
    mlp_backward_kernel<<<(unsigned)blocks, kBwdThreads, smem, stream>>>(X, target, n, f_in, W1, b1, w2, b2, grad,
                                                                         loss_sum);
    GL_LAUNCH_CHECK("mlp_backward_kernel");
    return GL_OK;
}

extern "C" int gl_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t count, float lr, float beta1,
                           float beta2, float eps, float grad_scale, int32_t step, uint16_t* W1_bf16,
                           uint16_t* w2_bf16, int32_t f_in, cudaStream_t stream) {
    GL_REQUIRE(f_in >= 1 && f_in <= FMAX, GL_ERR_INVALID_ARGUMENT, "f_in must be in 1..%d", FMAX);
    GL_REQUIRE(count == (int64_t)H * f_in + 2 * H + 1, GL_ERR_INVALID_ARGUMENT, "parameter count mismatch");
    GL_REQUIRE(step >= 1, GL_ERR_INVALID_ARGUMENT, "step counts from 1");
    const float bc1 = 1.f - powf(beta1, (float)step);
    const float bc2 = 1.f - powf(beta2, (float)step);
    mlp_adam_kernel<<<(unsigned)ceil_div(count, 256), 256, 0, stream>>>(params, grad, m, v, count, lr, beta1, beta2,
                                                                        eps, grad_scale, bc1, bc2, W1_bf16, w2_bf16,
                                                                        f_in);
    GL_LAUNCH_CHECK("mlp_adam_kernel");
    return GL_OK;
}
