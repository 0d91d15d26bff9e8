// nz_mlp.cu -- MLP surrogate of the canonical curves: forward, backward, Adam.
//
// A fully connected network with GELU hidden activations (erf form) and a
// linear output layer.  Every GEMM takes BF16 operands -- activations and
// gradients are rounded to BF16 (round-to-nearest-even) where they enter a
// product -- and accumulates in FP32; biases, activations, the loss and the
// optimizer state are FP32.  (The surrogate has no counterpart in the
// reference; it serves the p-grid placement and the choice of the next
// lattice size, with the Monte Carlo estimate as its fallback and judge.)
//
// Parameter layout (one flat FP32 buffer, mirrored as BF16 for products):
// for layer l = 0..n_layers-1: W_l [in_l][out_l] row-major, then b_l [out_l].
#include <cstdint>
#include <cuda_bf16.h>

#include "nz_common.cuh"
#include "nz_internal.cuh"

namespace nz {

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

constexpr int kTile = 64;
constexpr int kKc = 16;

// C[m][n] = sum_k A(m, k) * B(k, n) (+ bias[n]); A(m, k) = A[m * sam + k * sak],
// B(k, n) = Bm[k * sbk + n * sbn]; operands read as BF16-rounded FP32 (A) or
// BF16 (B when b_bf16 != nullptr); FP32 accumulation.
// epilogue 0: C = acc (+bias); 1: Z = acc + bias, C = GELU(Z) (Z stored).
__global__ void __launch_bounds__(256) mlp_gemm_kernel(int M, int N, int K, const float *A, int sam, int sak,
                                                       const float *Bf, const __nv_bfloat16 *Bh, int sbk, int sbn,
                                                       const float *bias, int epilogue, float *Z, float *C,
                                                       int ldc, int accumulate) {
    __shared__ float sA[kKc][kTile + 1];
    __shared__ float sB[kKc][kTile + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kKc) {
        for (int i = threadIdx.x; i < kKc * kTile; i += 256) {
            const int kk = i / kTile, mm = i % kTile;
            const int m = m0 + mm, k = k0 + kk;
            sA[kk][mm] = (m < M && k < K) ? bf16r(A[(size_t)m * sam + (size_t)k * sak]) : 0.0f;
            const int n = n0 + mm;
            float b = 0.0f;
            if (n < N && k < K) {
                const size_t idx = (size_t)k * sbk + (size_t)n * sbn;
                b = Bh ? __bfloat162float(Bh[idx]) : bf16r(Bf[idx]);
            }
            sB[kk][mm] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kKc; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) { a[i] = sA[kk][ty * 4 + i]; b[i] = sB[kk][tx * 4 + i]; }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx * 4 + j;
            if (n >= N) continue;
            float v = acc[i][j] + (bias ? bias[n] : 0.0f);
            const size_t o = (size_t)m * ldc + n;
            if (epilogue == 1) { Z[o] = v; v = gelu(v); }
            C[o] = accumulate ? C[o] + v : v;
        }
    }
}

static void gemm(int M, int N, int K, const float *A, int sam, int sak, const float *Bf, const __nv_bfloat16 *Bh,
                 int sbk, int sbn, const float *bias, int epilogue, float *Z, float *C, int ldc, int accumulate,
                 cudaStream_t s) {
    dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
    mlp_gemm_kernel<<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, Bf, Bh, sbk, sbn, bias, epilogue, Z, C, ldc,
                                         accumulate);
}

__global__ void to_bf16_kernel(const float *a, __nv_bfloat16 *b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16_rn(a[i]);
}

// dZ = dH * GELU'(Z)
__global__ void gelu_back_kernel(const float *Z, const float *dH, float *dZ, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dZ[i] = dH[i] * gelu_grad(Z[i]);
}

// db[o] = sum_b dZ[b][o]
__global__ void bias_grad_kernel(const float *dZ, int B, int N, float *db) {
    const int o = blockIdx.x;
    float s = 0.0f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) s += dZ[(size_t)b * N + o];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < (unsigned)off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[o] = red[0];
}

// Weighted squared error: loss = sum_{b,o} w[b][o] (y - t)^2 / B ; dY = 2 w (y - t) / B
__global__ void mse_kernel(const float *Y, const float *T, const float *Wt, int B, int N, float *dY,
                           float *loss_parts) {
    float s = 0.0f;
    const int64_t n = (int64_t)B * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float w = Wt ? Wt[i] : 1.0f;
        const float d = Y[i] - T[i];
        s += w * d * d;
        dY[i] = 2.0f * w * d / (float)B;
    }
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < (unsigned)off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_parts[blockIdx.x] = red[0] / (float)B;
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, __nv_bfloat16 *pb, int64_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16_rn(pi);
    }
}

}  // namespace nz

using namespace nz;

namespace {
int param_offsets(const int32_t *widths, int32_t n_layers, int64_t *w_off, int64_t *b_off) {
    int64_t o = 0;
    for (int l = 0; l < n_layers; ++l) {
        if (widths[l] <= 0 || widths[l + 1] <= 0 || widths[l] > 4096 || widths[l + 1] > 4096) return NZ_ERR_INVALID;
        w_off[l] = o;
        o += (int64_t)widths[l] * widths[l + 1];
        b_off[l] = o;
        o += widths[l + 1];
    }
    return NZ_OK;
}
constexpr int kMaxLayers = 16;
inline int blocks_for(int64_t n) { int64_t b = (n + 255) / 256; return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b)); }
}  // namespace

extern "C" {

int64_t nz_mlp_param_count(const int32_t *widths, int32_t n_layers) {
    if (!widths || n_layers <= 0 || n_layers > kMaxLayers) return -1;
    int64_t w[kMaxLayers], b[kMaxLayers];
    if (param_offsets(widths, n_layers, w, b) != NZ_OK) return -1;
    return b[n_layers - 1] + widths[n_layers];
}

int64_t nz_mlp_activation_count(const int32_t *widths, int32_t n_layers, int32_t batch) {
    if (!widths || n_layers <= 0 || n_layers > kMaxLayers || batch <= 0) return -1;
    int64_t s = 0;
    for (int l = 1; l <= n_layers; ++l) s += (int64_t)batch * widths[l];
    return s;
}

int nz_mlp_params_to_bf16(const float *params, int64_t count, void *params_bf16, void *stream) {
    if (!params || !params_bf16 || count <= 0) return NZ_ERR_INVALID;
    to_bf16_kernel<<<blocks_for(count), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        params, reinterpret_cast<__nv_bfloat16 *>(params_bf16), count);
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

int nz_mlp_forward(const int32_t *widths, int32_t n_layers, int32_t batch, const float *x, const float *params,
                   const void *params_bf16, float *z, float *h, float *y, void *stream) {
    if (!widths || n_layers <= 0 || n_layers > kMaxLayers || batch <= 0 || !x || !params || !params_bf16 || !z ||
        !h || !y)
        return NZ_ERR_INVALID;
    int64_t wo[kMaxLayers], bo[kMaxLayers];
    if (param_offsets(widths, n_layers, wo, bo) != NZ_OK) return NZ_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const __nv_bfloat16 *pb = reinterpret_cast<const __nv_bfloat16 *>(params_bf16);
    const float *in = x;
    int64_t act = 0;
    for (int l = 0; l < n_layers; ++l) {
        const int K = widths[l], N = widths[l + 1];
        const bool last = l == n_layers - 1;
        float *zl = z + act, *hl = last ? y : h + act;
        gemm(batch, N, K, in, K, 1, nullptr, pb + wo[l], N, 1, params + bo[l], last ? 0 : 1, zl, hl, N, 0, s);
        if (last) cudaMemcpyAsync(zl, y, sizeof(float) * (size_t)batch * N, cudaMemcpyDeviceToDevice, s);
        in = hl;
        act += (int64_t)batch * N;
    }
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

int nz_mlp_loss(const float *y, const float *target, const float *weight, int32_t batch, int32_t n_out,
                float *dy, float *loss_parts, int32_t n_parts, void *stream) {
    if (!y || !target || !dy || !loss_parts || batch <= 0 || n_out <= 0 || n_parts <= 0) return NZ_ERR_INVALID;
    mse_kernel<<<n_parts, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(y, target, weight, batch, n_out, dy,
                                                                            loss_parts);
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

// dy: gradient of the loss w.r.t. the output [batch][n_out]; z, h from the
// forward pass; grads: flat FP32 gradient (same layout as params);
// scratch: 2 * batch * max(width) floats.
int nz_mlp_backward(const int32_t *widths, int32_t n_layers, int32_t batch, const float *x, const void *params_bf16,
                    const float *z, const float *h, const float *dy, float *grads, float *scratch, void *stream) {
    if (!widths || n_layers <= 0 || n_layers > kMaxLayers || batch <= 0 || !x || !params_bf16 || !z || !h ||
        !dy || !grads || !scratch)
        return NZ_ERR_INVALID;
    int64_t wo[kMaxLayers], bo[kMaxLayers];
    if (param_offsets(widths, n_layers, wo, bo) != NZ_OK) return NZ_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const __nv_bfloat16 *pb = reinterpret_cast<const __nv_bfloat16 *>(params_bf16);
    int wmax = 0;
    for (int l = 0; l <= n_layers; ++l) wmax = widths[l] > wmax ? widths[l] : wmax;
    float *dZ = scratch, *dA = scratch + (size_t)batch * wmax;
    int64_t act_off[kMaxLayers];
    int64_t a = 0;
    for (int l = 0; l < n_layers; ++l) { act_off[l] = a; a += (int64_t)batch * widths[l + 1]; }
    // dZ of the last (linear) layer = dy
    cudaMemcpyAsync(dZ, dy, sizeof(float) * (size_t)batch * widths[n_layers], cudaMemcpyDeviceToDevice, s);
    for (int l = n_layers - 1; l >= 0; --l) {
        const int K = widths[l], N = widths[l + 1];
        const float *A = l == 0 ? x : h + act_off[l - 1];
        // dW[K][N] = A^T dZ  (reduction over the batch)
        gemm(K, N, batch, A, 1, K, dZ, nullptr, N, 1, nullptr, 0, nullptr, grads + wo[l], N, 0, s);
        bias_grad_kernel<<<N, 256, 0, s>>>(dZ, batch, N, grads + bo[l]);
        if (l == 0) break;
        // dA[batch][K] = dZ W^T  (W[K][N]: B(k=n, n=k) = W[k][n] -> sbk = 1, sbn = N)
        gemm(batch, K, N, dZ, N, 1, nullptr, pb + wo[l], 1, N, nullptr, 0, nullptr, dA, K, 0, s);
        const int64_t cnt = (int64_t)batch * K;
        gelu_back_kernel<<<blocks_for(cnt), 256, 0, s>>>(z + act_off[l - 1], dA, dZ, cnt);
    }
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

int nz_mlp_adam(float *params, const float *grads, float *m, float *v, void *params_bf16, int64_t count,
                float lr, float beta1, float beta2, float eps, int32_t step, void *stream) {
    if (!params || !grads || !m || !v || !params_bf16 || count <= 0 || step <= 0) return NZ_ERR_INVALID;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    adam_kernel<<<blocks_for(count), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        params, grads, m, v, reinterpret_cast<__nv_bfloat16 *>(params_bf16), count, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

}  // extern "C"
