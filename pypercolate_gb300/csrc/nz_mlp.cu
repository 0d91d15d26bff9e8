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
#include "nz_tc.cuh"

namespace nz {

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ---------------------------------------------------------------------
// GEMM on the tensor cores: tcgen05.mma kind::f16 with BF16 operands and an
// FP32 accumulator in TMEM
// ---------------------------------------------------------------------
// C[m][n] = sum_k A(m, k) B(k, n) (+ bias[n]); A(m, k) = A[m * sam + k * sak]
// (FP32, rounded to BF16 as it is staged), B(k, n) = B[k * sbk + n * sbn]
// (BF16, or FP32 rounded to BF16).  epilogue 0: C = acc (+ bias); 1: Z = acc
// + bias, C = GELU(Z).  accumulate: C += instead of C =.
//
// One CTA of 128 threads per 128 x ntile tile of C (ntile <= 128, a multiple
// of 16): the threads stage 64-deep K chunks of A (128 rows) and B (ntile
// rows) into shared memory as BF16 in the canonical no-swizzle K-major
// layout (8-row x 16-byte core matrices, K-adjacent ones 128 bytes apart,
// 8-row groups 1 KB apart), double-buffered; one thread issues four
// 128 x ntile x 16 MMAs per chunk and commits them to the chunk's mbarrier;
// thread t reads row t of the accumulator out of TMEM (tcgen05.ld, lane t)
// for the epilogue.  Every mbarrier wait gives up after 1 s: the tile is
// then written as NaN and counted in g_mlp_errors (nz_mlp_take_errors).
constexpr int kGM = 128;   // rows of C per CTA (TMEM lanes)
constexpr int kGK = 64;    // K per staged chunk: 4 MMAs of K = 16
constexpr int kGN = 128;   // largest column tile
constexpr uint32_t kGSbo = (kGK / 8) * tc::kCoreBytes;

struct GemmSmem {
    __nv_bfloat16 a[2][kGM * kGK];
    __nv_bfloat16 b[2][kGN * kGK];
    uint64_t mbar[2];
    uint32_t tmem;
};

__device__ uint32_t g_mlp_errors;  // tiles whose mbarrier waits gave up

// element (row, k) of a staged K-major operand, in BF16 units
__device__ __forceinline__ int kmajor_idx(int row, int k) {
    return (row >> 3) * (int)(kGSbo / 2) + (k >> 3) * 64 + (row & 7) * 8 + (k & 7);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t bf16_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kGM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__global__ void __launch_bounds__(kGM) mlp_gemm_kernel(int M, int N, int K, const float *A, int sam, int sak,
                                                       const float *Bf, const __nv_bfloat16 *Bh, int sbk, int sbn,
                                                       const float *bias, int epilogue, float *Z, float *C,
                                                       int ldc, int accumulate, int ntile, int k_split) {
    extern __shared__ __align__(1024) uint8_t gemm_smem[];
    GemmSmem &sh = *reinterpret_cast<GemmSmem *>(gemm_smem);
    const int t = threadIdx.x, warp = t >> 5;
    const int m0 = blockIdx.y * kGM, n0 = blockIdx.x * ntile;
    // split-K: this CTA's K range [kb, kb + k_split); its tile goes to slice
    // blockIdx.z of C (M x ldc floats per slice)
    const int kb = blockIdx.z * k_split;
    if (gridDim.z > 1) {
        K = min(K - kb, k_split);
        C += (size_t)blockIdx.z * M * ldc;
    }
    const uint32_t cols = ntile <= 32 ? 32u : (ntile <= 64 ? 64u : 128u);  // TMEM: power of two >= 32
    if (warp == 0) tc::tmem_alloc(tc::smem_u32(&sh.tmem), cols);
    if (t == 0) {
        tc::mbar_init(tc::smem_u32(&sh.mbar[0]));
        tc::mbar_init(tc::smem_u32(&sh.mbar[1]));
        tc::mbar_init_fence();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = sh.tmem;
    const int nch = (K + kGK - 1) / kGK;
    // thread index -> element: K fastest when K is the contiguous dimension
    // of the source, else rows fastest (coalesced global loads either way)
    const bool a_kfast = sak == 1, b_kfast = sbk == 1;
    auto stage = [&](int c, int buf) {
        const int k0 = c * kGK;
        __nv_bfloat16 *sa = sh.a[buf], *sb = sh.b[buf];
        for (int i = t; i < kGM * kGK; i += kGM) {
            const int r = a_kfast ? i / kGK : i % kGM;
            const int k = a_kfast ? i % kGK : i / kGM;
            const int gm = m0 + r, gk = k0 + k;
            const float v = (gm < M && gk < K) ? A[(size_t)gm * sam + (size_t)(kb + gk) * sak] : 0.0f;
            sa[kmajor_idx(r, k)] = __float2bfloat16_rn(v);
        }
        for (int i = t; i < ntile * kGK; i += kGM) {
            const int r = b_kfast ? i / kGK : i % ntile;
            const int k = b_kfast ? i % kGK : i / ntile;
            const int gn = n0 + r, gk = k0 + k;
            __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
            if (gn < N && gk < K) {
                const size_t idx = (size_t)(kb + gk) * sbk + (size_t)gn * sbn;
                v = Bh ? Bh[idx] : __float2bfloat16_rn(Bf[idx]);
            }
            sb[kmajor_idx(r, k)] = v;
        }
    };
    stage(0, 0);
    bool bad = false;
    int c = 0;
    for (; c < nch; ++c) {
        const int buf = c & 1;
        tc::fence_async_smem();
        tc::fence_before();
        if (__syncthreads_or(bad)) break;  // a wait below gave up
        if (t == 0) {
            tc::fence_after();
            const uint32_t a0 = tc::smem_u32(sh.a[buf]), b0 = tc::smem_u32(sh.b[buf]);
#pragma unroll
            for (int ks = 0; ks < kGK / 16; ++ks) {
                const uint32_t o = (uint32_t)ks * 2 * tc::kCoreBytes;  // K = 16: two core matrices
                mma_bf16(tmem, tc::smem_desc(a0 + o, tc::kCoreBytes, kGSbo),
                         tc::smem_desc(b0 + o, tc::kCoreBytes, kGSbo), bf16_idesc(ntile),
                         (c > 0 || ks > 0) ? 1u : 0u);
            }
            tc::mma_commit(tc::smem_u32(&sh.mbar[buf]));
        }
        if (c + 1 < nch) {
            // the other buffer is free once the MMAs of chunk c - 1 are done
            if (c >= 1) bad = !tc::mbar_wait(tc::smem_u32(&sh.mbar[(c - 1) & 1]), ((c - 1) >> 1) & 1);
            if (!bad) stage(c + 1, (c + 1) & 1);
        }
    }
    // MMAs complete in order: the last chunk issued covers them all
    if (c > 0 && !tc::mbar_wait(tc::smem_u32(&sh.mbar[(c - 1) & 1]), ((c - 1) >> 1) & 1)) bad = true;
    tc::fence_before();
    const bool any_bad = __syncthreads_or(bad) || c < nch;
    tc::fence_after();
    const int m = m0 + t;
    if (!any_bad) {
        for (int j0 = 0; j0 < ntile; j0 += 32) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j0, v);
            if (m < M) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int n = n0 + j0 + j;
                    if (j0 + j >= ntile || n >= N) continue;
                    float x = v[j] + (bias ? bias[n] : 0.0f);
                    const size_t o = (size_t)m * ldc + n;
                    if (epilogue == 1) { Z[o] = x; x = gelu(x); }
                    C[o] = accumulate ? C[o] + x : x;
                }
            }
        }
    } else {
        if (m < M)
            for (int j = 0; j < ntile && n0 + j < N; ++j) C[(size_t)m * ldc + n0 + j] = __int_as_float(0x7fc00000);
        if (t == 0) atomicAdd(&g_mlp_errors, 1u);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, cols);
    }
}

// slices[z][m][n] summed over z in order into C (deterministic split-K)
__global__ void splitk_sum_kernel(const float *slices, int splits, int M, int N, int ldc, float *C) {
    const int64_t total = (int64_t)M * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int m = (int)(i / N), n = (int)(i % N);
        float acc = 0.0f;
        for (int z = 0; z < splits; ++z) acc += slices[(size_t)z * M * ldc + (size_t)m * ldc + n];
        C[(size_t)m * ldc + n] = acc;
    }
}

// C = A B (+ bias, epilogue).  With `partial` (room for `splits` x M x ldc
// floats) and splits > 1, K is split over that many CTAs per tile, for GEMMs
// with few output tiles and a long K (the weight gradients: K = batch); the
// slices are then summed in order (no bias, no epilogue, C overwritten).
static void gemm(int M, int N, int K, const float *A, int sam, int sak, const float *Bf, const __nv_bfloat16 *Bh,
                 int sbk, int sbn, const float *bias, int epilogue, float *Z, float *C, int ldc, int accumulate,
                 cudaStream_t s, float *partial = nullptr, int splits = 1) {
    if (M <= 0 || N <= 0) return;
    const int ntile = N >= kGN ? kGN : ((N + 15) / 16) * 16;
    int k_split = K;
    if (partial && splits > 1) {
        k_split = ((K + splits - 1) / splits + kGK - 1) / kGK * kGK;
        splits = (K + k_split - 1) / k_split;
    }
    if (splits < 2) { partial = nullptr; splits = 1; k_split = K; }
    // above 48 KB of dynamic shared memory the launch needs the attribute,
    // which belongs to the function in the current device's context
    cudaFuncSetAttribute(mlp_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GemmSmem));
    dim3 grid((N + ntile - 1) / ntile, (M + kGM - 1) / kGM, splits);
    mlp_gemm_kernel<<<grid, kGM, sizeof(GemmSmem), s>>>(M, N, K, A, sam, sak, Bf, Bh, sbk, sbn,
                                                         partial ? nullptr : bias, partial ? 0 : epilogue, Z,
                                                         partial ? partial : C, ldc, partial ? 0 : accumulate,
                                                         ntile, k_split);
    if (partial) {
        const int64_t total = (int64_t)M * N;
        const int blocks = (int)((total + 255) / 256 > 1024 ? 1024 : (total + 255) / 256);
        splitk_sum_kernel<<<blocks, 256, 0, s>>>(partial, splits, M, N, ldc, C);
    }
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
        // dW[K][N] = A^T dZ  (reduction over the batch), split over the batch
        // into slices held in the dA half of the scratch (free until the dA
        // GEMM below): splits * K * N <= batch * wmax floats
        const int64_t room = (int64_t)batch * wmax / ((int64_t)K * N);
        const int splits = (int)(room < 32 ? room : 32);
        gemm(K, N, batch, A, 1, K, dZ, nullptr, N, 1, nullptr, 0, nullptr, grads + wo[l], N, 0, s, dA, splits);
        bias_grad_kernel<<<N, 256, 0, s>>>(dZ, batch, N, grads + bo[l]);
        if (l == 0) break;
        // dA[batch][K] = dZ W^T  (W[K][N]: B(k=n, n=k) = W[k][n] -> sbk = 1, sbn = N)
        gemm(batch, K, N, dZ, N, 1, nullptr, pb + wo[l], 1, N, nullptr, 0, nullptr, dA, K, 0, s);
        const int64_t cnt = (int64_t)batch * K;
        gelu_back_kernel<<<blocks_for(cnt), 256, 0, s>>>(z + act_off[l - 1], dA, dZ, cnt);
    }
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

int nz_mlp_take_errors(uint32_t *count) {
    if (!count) return NZ_ERR_INVALID;
    const uint32_t zero = 0;
    if (cudaMemcpyFromSymbol(count, g_mlp_errors, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_mlp_errors, &zero, sizeof(uint32_t)) != cudaSuccess)
        return NZ_ERR_CUDA;
    return NZ_OK;
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
