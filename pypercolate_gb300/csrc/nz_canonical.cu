// nz_canonical.cu -- canonical (binomial-convolution) stage, averages and
// confidence intervals.
//
// Replaces percolate/percolate.py:1067-1109 (_binomial_pmf),
// percolate/hpc.py:443-515 (bond_canonical_statistics), :561-635
// (bond_initialize_canonical_averages), :638-702 (bond_reduce) and :752-834
// (finalize_canonical_averages), plus the microcanonical run-reductions whose
// semantics are percolate/percolate.py:450-705.
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "nz_common.cuh"
#include "nz_internal.cuh"
#include "nz_math.cuh"
#include "nz_records.cuh"

namespace nz {

// =====================================================================
// Binomial weights
// =====================================================================
// Log B(M, n, p) up to an n-independent constant, from lgamma; used only to
// locate the band edges (its absolute error does not reach the weights).
__device__ __forceinline__ double log_binom_shape(uint32_t M, uint32_t n, double lp, double lq) {
    return -lgamma((double)n + 1.0) - lgamma((double)(M - n) + 1.0) + (double)n * lp + (double)(M - n) * lq;
}

// One CTA per p.  Band = {n : log B(n) >= log B(mode) - cutoff}, found by
// bisection on each side of the mode (log B is concave in n).  The weights
// are then built from the ratio recursion of Newman & Ziff Eq. (10),
//   log B(n) - log B(n-1) = log(M - n + 1) - log(n) + log(p) - log(1 - p),
// summed by a block-wide prefix scan from the band's low edge, shifted by the
// maximum, exponentiated and normalised by their FP64 sum (as the reference
// normalises by ret.sum()).  Writes wp[0, cap) and returns (lo, len) to all
// threads of the block.
template <int BLOCK>
__device__ void band_weights_block(uint32_t M, double p, double cutoff, int32_t cap, double *wp, uint32_t &lo_out,
                                   uint32_t &len_out, bool &overflow) {
    __shared__ double s_scan[BLOCK];
    __shared__ double s_red[BLOCK];
    __shared__ uint32_t s_lo, s_hi;
    if (threadIdx.x == 0) {
        uint32_t lo, hi;
        if (!(p > 0.0)) { lo = hi = 0; }
        else if (!(p < 1.0)) { lo = hi = M; }
        else {
            const double lp = log(p), lq = log1p(-p);
            uint32_t mode = (uint32_t)floor((double)(M + 1) * p);
            if (mode > M) mode = M;
            const double lm = log_binom_shape(M, mode, lp, lq) - cutoff;
            // smallest n <= mode with shape(n) >= lm
            uint32_t a = 0, b = mode;
            if (log_binom_shape(M, 0, lp, lq) >= lm) b = 0;
            else while (b - a > 1) { uint32_t c = a + (b - a) / 2; if (log_binom_shape(M, c, lp, lq) >= lm) b = c; else a = c; }
            lo = b;
            // largest n >= mode with shape(n) >= lm
            a = mode; b = M;
            if (log_binom_shape(M, M, lp, lq) >= lm) a = M;
            else while (b - a > 1) { uint32_t c = a + (b - a) / 2; if (log_binom_shape(M, c, lp, lq) >= lm) a = c; else b = c; }
            hi = a;
        }
        s_lo = lo; s_hi = hi;
    }
    __syncthreads();
    const uint32_t lo = s_lo;
    uint32_t len = s_hi - s_lo + 1;
    overflow = len > (uint32_t)cap;
    if (overflow) len = cap;
    lo_out = lo;
    len_out = len;
    if (len == 1) {
        for (int j = threadIdx.x; j < cap; j += BLOCK) wp[j] = (j == 0) ? 1.0 : 0.0;
        __syncthreads();
        return;
    }
    const double lpq = log(p) - log1p(-p);
    // pass 1: log weights relative to the low edge (prefix scan of log ratios)
    double carry = 0.0;
    double vmax = -INFINITY;
    for (uint32_t base = 0; base < len; base += BLOCK) {
        const uint32_t j = base + threadIdx.x;
        double x = 0.0;
        if (j > 0 && j < len) {
            const double n = (double)(lo + j);
            x = log((double)M - n + 1.0) - log(n) + lpq;
        }
        s_scan[threadIdx.x] = x;
        __syncthreads();
        for (int off = 1; off < BLOCK; off <<= 1) {  // Hillis-Steele inclusive scan
            double y = threadIdx.x >= (unsigned)off ? s_scan[threadIdx.x - off] : 0.0;
            __syncthreads();
            s_scan[threadIdx.x] += y;
            __syncthreads();
        }
        const double lv = carry + s_scan[threadIdx.x];
        if (j < len) { wp[j] = lv; vmax = fmax(vmax, lv); }
        carry += s_scan[BLOCK - 1];
        __syncthreads();
    }
    s_red[threadIdx.x] = vmax;
    __syncthreads();
    for (int off = BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < (unsigned)off) s_red[threadIdx.x] = fmax(s_red[threadIdx.x], s_red[threadIdx.x + off]);
        __syncthreads();
    }
    vmax = s_red[0];
    __syncthreads();
    // pass 2: exponentiate and sum
    double sum = 0.0;
    for (uint32_t j = threadIdx.x; j < len; j += BLOCK) {
        const double e = exp(wp[j] - vmax);
        wp[j] = e;
        sum += e;
    }
    s_red[threadIdx.x] = sum;
    __syncthreads();
    for (int off = BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < (unsigned)off) s_red[threadIdx.x] += s_red[threadIdx.x + off];
        __syncthreads();
    }
    const double inv = 1.0 / s_red[0];
    for (uint32_t j = threadIdx.x; j < (uint32_t)cap; j += BLOCK) wp[j] = (j < len) ? wp[j] * inv : 0.0;
    __syncthreads();
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) binomial_weights_kernel(uint32_t M, const double *ps, double cutoff,
                                                                 int32_t cap, uint32_t *band_lo,
                                                                 uint32_t *band_len, double *w,
                                                                 int32_t *overflow) {
    const int pi = blockIdx.x;
    uint32_t lo, len;
    bool ovf;
    band_weights_block<BLOCK>(M, ps[pi], cutoff, cap, w + (size_t)pi * cap, lo, len, ovf);
    if (threadIdx.x == 0) {
        band_lo[pi] = lo;
        band_len[pi] = len;
        if (ovf && overflow) atomicExch(overflow, 1);
    }
}

// Full-length pmf rows out[pi][0..M]: band weights computed at the row start,
// then shifted in place to their offset and the rest zeroed.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) binomial_pmf_kernel(uint32_t M, const double *ps, double cutoff,
                                                             double *out) {
    const int pi = blockIdx.x;
    double *row = out + (size_t)pi * (M + 1);
    uint32_t lo, len;
    bool ovf;
    band_weights_block<BLOCK>(M, ps[pi], cutoff, (int32_t)(M + 1), row, lo, len, ovf);
    if (lo > 0) {
        // move [0, len) to [lo, lo + len), highest block first
        for (int64_t top = (int64_t)len; top > 0; top -= BLOCK) {
            const int64_t j = top - BLOCK + threadIdx.x;
            double v = 0.0;
            if (j >= 0) v = row[j];
            __syncthreads();
            if (j >= 0) row[j + lo] = v;
            __syncthreads();
        }
        for (uint32_t j = threadIdx.x; j < lo; j += BLOCK) row[j] = 0.0;
    }
}

void launch_binomial_weights(uint32_t M, const double *ps, int32_t P, double cutoff, int32_t cap,
                             uint32_t *band_lo, uint32_t *band_len, double *w, int32_t *overflow,
                             cudaStream_t s) {
    if (P <= 0) return;
    binomial_weights_kernel<256><<<P, 256, 0, s>>>(M, ps, cutoff, cap, band_lo, band_len, w, overflow);
}

void launch_binomial_pmf(uint32_t M, const double *ps, int32_t P, double cutoff, double *out, cudaStream_t s) {
    if (P <= 0) return;
    binomial_pmf_kernel<256><<<P, 256, 0, s>>>(M, ps, cutoff, out);
}

// =====================================================================
// bond_canonical_statistics on the reference's packed rows (FP64)
// =====================================================================
__device__ __forceinline__ uint64_t ld_bytes(const uint8_t *p, int n) {
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)p[i] << (8 * i);
    return v;
}

// grid: (factor set); each CTA reduces over the M+1 rows.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) canonical_rows_kernel(const uint8_t *rows, uint32_t M, int32_t spanning,
                                                               const double *factors, double *out) {
    const int set = blockIdx.x;
    const double *f = factors + (size_t)set * (M + 1);
    const uint32_t rb = spanning ? 53u : 52u;
    const int o = spanning ? 9 : 8;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (uint32_t n = threadIdx.x; n <= M; n += BLOCK) {
        const uint8_t *r = rows + (size_t)n * rb;
        const double fn = f[n];
        if (spanning) acc[0] += fn * (double)(r[8] != 0);
        acc[1] += fn * (double)(uint32_t)ld_bytes(r + o, 4);
#pragma unroll
        for (int k = 0; k < 5; ++k) acc[2 + k] += fn * (double)ld_bytes(r + o + 4 + 8 * k, 8);
    }
    __shared__ double s_red[7][BLOCK];
#pragma unroll
    for (int k = 0; k < 7; ++k) s_red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int off = BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < (unsigned)off)
#pragma unroll
            for (int k = 0; k < 7; ++k) s_red[k][threadIdx.x] += s_red[k][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x < 7) out[(size_t)set * 7 + threadIdx.x] = (threadIdx.x == 0 && !spanning) ? 0.0 : s_red[threadIdx.x][0];
}

void launch_canonical_rows(const uint8_t *rows, uint32_t M, int32_t spanning, const double *factors,
                           int32_t n_sets, double *out, cudaStream_t s) {
    if (n_sets <= 0) return;
    canonical_rows_kernel<256><<<n_sets, 256, 0, s>>>(rows, M, spanning, factors, out);
}

// =====================================================================
// Classic canonical averages: binomial weights times microcanonical arrays
// =====================================================================
// out[i][c] = sum_j w[i][j] V[lo_i + j][c] for the band of p_i (FP64): the
// sums percolate/percolate.py:1171-1221 (canonical_averages) forms with the
// full-length pmf, over the rows where the pmf does not underflow.  One CTA
// per (p, group of 32 columns): lane c of every warp owns column c (a row
// of V is one coalesced load per warp), warps stride over the band's rows,
// and the warps' partial sums are added in a fixed order (deterministic).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) band_dot_kernel(const uint32_t *band_lo, const uint32_t *band_len,
                                                         const double *w, int32_t cap, const double *V,
                                                         uint32_t rows, int32_t cols, double *out) {
    __shared__ double part[BLOCK / 32][32];
    const int pi = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.y * 32 + lane;
    const uint32_t lo = band_lo[pi];
    uint32_t len = min(band_len[pi], (uint32_t)cap);
    if (lo >= rows) len = 0;
    else len = min(len, rows - lo);
    const double *wp = w + (size_t)pi * cap;
    double acc = 0.0;
    if (c < cols)
        for (uint32_t j = warp; j < len; j += BLOCK / 32) acc = fma(wp[j], V[(size_t)(lo + j) * cols + c], acc);
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && c < cols) {
        double t = 0.0;
        for (int k = 0; k < BLOCK / 32; ++k) t += part[k][lane];
        out[(size_t)pi * cols + c] = t;
    }
}

void launch_band_dot(const uint32_t *band_lo, const uint32_t *band_len, const double *w, int32_t cap, int32_t P,
                     const double *V, uint32_t rows, int32_t cols, double *out, cudaStream_t s) {
    if (P <= 0 || cols <= 0) return;
    dim3 g(P, (cols + 31) / 32);
    band_dot_kernel<256><<<g, 256, 0, s>>>(band_lo, band_len, w, cap, V, rows, cols, out);
}

// =====================================================================
// Banded convolution of record windows (ensemble path)
// =====================================================================
constexpr int kConvRuns = 128;         // runs per CTA (one per thread)
// probabilities per CTA of the FP32 / FP64 window kernels: 8 by default
// (8 gave 544 ms, 16 587 ms, 32 1025 ms per 100,000-run step with the
// earlier FP64-accumulated kernels); 16 is an autotuner candidate for the
// m0 / m3 / m4 kernel
constexpr int kConvPT = 8;
constexpr int kConvChunk = 128;  // rows staged per step, summed in FP32 before the TwoSum add
// 16 record loads in flight per thread: over the FP32 band (weights >= e^-30
// of the mode) 1047 against 1052 ms per 100,000-run L = 256 step with 8
// (over the full e^-80 band 8 had been better: 479 against 512 ms); 32
// measured 1229 against 1211 ms (same box)
#ifndef NZ_CONV_BATCH
#define NZ_CONV_BATCH 16
#endif
constexpr int kConvBatch = NZ_CONV_BATCH;  // record loads in flight per thread

// Window accumulator of one canonical value.  FP64 path: an FP64 sum.  FP32
// path: the FP32 partial sums of the row chunks are added into an FP32
// (sum, compensation) pair by an error-free addition -- as accurate as an
// FP64 sum of them, without the FP64 pipe, which runs at 1/64 of the FP32
// rate on this chip.
template <int PRECISION>
struct ConvAcc {
    double v = 0.0;
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ double value() const { return v; }
};
template <>
struct ConvAcc<1> {
    float s = 0.0f, c = 0.0f;
    // chunk sums and the running sum are >= 0: Fast2Sum on the operands
    // ordered by size is exact (3 additions and a max / min, not TwoSum's 6)
    __device__ __forceinline__ void add(float x) {
        const float a = fmaxf(s, x), b = fminf(s, x);
        const float t = __fadd_rn(a, b);
        c = __fadd_rn(c, __fsub_rn(b, __fsub_rn(t, a)));
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// grid: (run tiles, p tiles, 7 statistics).  Each thread accumulates the
// kConvPT canonical values of its run for one statistic over the window's
// rows, with the tile's weights staged in shared memory (zero outside each
// p's band).  PRECISION 0: FP64 products and sums.  PRECISION 1: FP32
// products summed in FP32 over kConvChunk rows, then added into a TwoSum
// pair (ConvAcc<1>).
template <int PRECISION, int S, bool SITE, int kConvPT>
__device__ __forceinline__ void conv_rows(const ConvParams &p, uint32_t c0, uint32_t cn, int r,
                                          const typename std::conditional<PRECISION == 0, double, float>::type (*s_w)[kConvPT],
                                          ConvAcc<PRECISION> *acc) {
    using wtype = typename std::conditional<PRECISION == 0, double, float>::type;
    wtype part[kConvPT];
#pragma unroll
    for (int j = 0; j < kConvPT; ++j) part[j] = 0;
    const size_t base = (size_t)(c0 - p.n_begin) * p.rec.run_stride + r;
    // m1 = (sites in clusters) - max: N for bond records, n for site records
    auto value = [&](uint32_t i) -> wtype {
        const size_t off = base + (size_t)i * p.rec.run_stride;
        const uint32_t held = (S == 3 && SITE) ? c0 + i : p.N;
        return PRECISION == 0 ? (wtype)record_value<S>(p.rec, off, held)
                              : (wtype)record_value_f<S>(p.rec, off, held);
    };
    // the records of kConvBatch rows are loaded before their products so that
    // that many loads are in flight per thread; each accumulator still adds
    // the rows in increasing order
    uint32_t i = 0;
    for (; i + kConvBatch <= cn; i += kConvBatch) {
        wtype q[kConvBatch];
#pragma unroll
        for (int b = 0; b < kConvBatch; ++b) q[b] = value(i + b);
#pragma unroll
        for (int b = 0; b < kConvBatch; ++b)
#pragma unroll
            for (int j = 0; j < kConvPT; ++j) part[j] = fma(s_w[i + b][j], q[b], part[j]);
    }
    for (; i < cn; ++i) {
        const wtype q = value(i);
#pragma unroll
        for (int j = 0; j < kConvPT; ++j) part[j] = fma(s_w[i][j], q, part[j]);
    }
#pragma unroll
    for (int j = 0; j < kConvPT; ++j) acc[j].add(part[j]);
}

// Statistics 0 (spanning), 1 (max) and 3 (m1 = held - max) all come from the
// max_span plane: one pass loads each word once and feeds the three sets of
// products (each accumulator adds the same values in the same order as a
// pass per statistic would).
template <int PRECISION, bool SITE, int kConvPT>
__device__ __forceinline__ void conv_rows_max(const ConvParams &p, uint32_t c0, uint32_t cn, int r,
                                              const typename std::conditional<PRECISION == 0, double, float>::type (*s_w)[kConvPT],
                                              ConvAcc<PRECISION> *acc0, ConvAcc<PRECISION> *acc1,
                                              ConvAcc<PRECISION> *acc3) {
    using wtype = typename std::conditional<PRECISION == 0, double, float>::type;
    wtype p0[kConvPT], p1[kConvPT], p3[kConvPT];
#pragma unroll
    for (int j = 0; j < kConvPT; ++j) p0[j] = p1[j] = p3[j] = 0;
    const size_t base = (size_t)(c0 - p.n_begin) * p.rec.run_stride + r;
    auto step = [&](uint32_t i, uint32_t ms) {
        const uint32_t held = SITE ? c0 + i : p.N;
        const uint32_t mx = ms & ~kSpanBit;
        const wtype q0 = (ms & kSpanBit) ? (wtype)1 : (wtype)0;
        const wtype q1 = (wtype)mx, q3 = (wtype)(held - mx);
#pragma unroll
        for (int j = 0; j < kConvPT; ++j) {
            const wtype w = s_w[i][j];
            p0[j] = fma(w, q0, p0[j]);  // (dropped at the end without a spanning statistic)
            p1[j] = fma(w, q1, p1[j]);
            p3[j] = fma(w, q3, p3[j]);
        }
    };
    uint32_t i = 0;
    for (; i + kConvBatch <= cn; i += kConvBatch) {
        uint32_t ms[kConvBatch];
#pragma unroll
        for (int b = 0; b < kConvBatch; ++b) ms[b] = p.rec.max_span[base + (size_t)(i + b) * p.rec.run_stride];
#pragma unroll
        for (int b = 0; b < kConvBatch; ++b) step(i + b, ms[b]);
    }
    for (; i < cn; ++i) step(i, p.rec.max_span[base + (size_t)i * p.rec.run_stride]);
#pragma unroll
    for (int j = 0; j < kConvPT; ++j) {
        acc0[j].add(p0[j]);
        acc1[j].add(p1[j]);
        acc3[j].add(p3[j]);
    }
}

// Each thread accumulates the kConvPT canonical values of its run over the
// window's rows, with the tile's weights staged in shared memory (zero
// outside each p's band).  PRECISION 0: FP64 products and sums.  PRECISION 1:
// FP32 products summed in FP32 over kConvChunk rows, then added into a
// TwoSum pair (ConvAcc<1>).
// MAXSET: grid (run tiles, p tiles, 1), statistics 0, 1 and 3 from the
// max_span plane in one pass; otherwise grid (run tiles, p tiles, 4),
// statistics 2, 4, 5, 6 (one per z) -- on the FP32 path (run tiles, p
// tiles, 3), statistics 2, 5, 6, with m2 (4) in conv_m2_comp_kernel.
#ifdef NZ_CONV_MIN_BLOCKS
#define NZ_CONV_BOUNDS __launch_bounds__(kConvRuns, NZ_CONV_MIN_BLOCKS)
#else
#define NZ_CONV_BOUNDS __launch_bounds__(kConvRuns)
#endif
template <int PRECISION, bool SITE, bool MAXSET, int kConvPT>
__global__ void NZ_CONV_BOUNDS conv_window_kernel(ConvParams p) {
    using wtype = typename std::conditional<PRECISION == 0, double, float>::type;
    __shared__ wtype s_w[kConvChunk][kConvPT];
    __shared__ uint32_t s_lo[kConvPT], s_len[kConvPT];
    __shared__ uint32_t s_range[2];
    const int r = blockIdx.x * kConvRuns + threadIdx.x;
    const int p0 = blockIdx.y * kConvPT;
    // FP64: statistics 2, 4, 5, 6; FP32: 2, 5, 6 (m2 has its compensated kernel)
    constexpr int kOther[4] = {2, 4, 5, 6};
    constexpr int kOther32[3] = {2, 5, 6};
    const int s = MAXSET ? 1 : (PRECISION == 0 ? kOther[blockIdx.z] : kOther32[blockIdx.z]);
    if (threadIdx.x < kConvPT) {
        const int pi = p0 + threadIdx.x;
        s_lo[threadIdx.x] = pi < p.P ? p.band_lo[pi] : 0u;
        s_len[threadIdx.x] = pi < p.P ? p.band_len[pi] : 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0xffffffffu, b = 0;
        for (int j = 0; j < kConvPT; ++j)
            if (s_len[j]) { a = min(a, s_lo[j]); b = max(b, s_lo[j] + s_len[j]); }
        a = max(a, p.n_begin);
        b = min(b, p.n_end);
        s_range[0] = a; s_range[1] = b;
    }
    __syncthreads();
    const uint32_t nlo = s_range[0], nhi = s_range[1];
    if (nlo >= nhi) return;
    ConvAcc<PRECISION> acc[kConvPT], acc0[MAXSET ? kConvPT : 1], acc3[MAXSET ? kConvPT : 1];
    for (uint32_t c0 = nlo; c0 < nhi; c0 += kConvChunk) {
        const uint32_t cn = min((uint32_t)kConvChunk, nhi - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < kConvChunk * kConvPT; i += kConvRuns) {
            const int row = i / kConvPT, j = i % kConvPT;
            const uint32_t n = c0 + row;
            wtype v = 0;
            if (row < (int)cn && n >= s_lo[j] && n < s_lo[j] + s_len[j]) {
                const size_t widx = (size_t)(p0 + j) * p.cap + (n - s_lo[j]);
                v = PRECISION == 0 ? (wtype)p.w64[widx] : (wtype)p.w32[widx];
            }
            s_w[row][j] = v;
        }
        __syncthreads();
        if (r < p.n_runs) {
            if (MAXSET) {
                conv_rows_max<PRECISION, SITE, kConvPT>(p, c0, cn, r, s_w, acc0, acc, acc3);
            } else {
                switch (s) {
                    case 2:
                        if (p.rec.narrow) conv_rows<PRECISION, 8, SITE, kConvPT>(p, c0, cn, r, s_w, acc);
                        else conv_rows<PRECISION, 2, SITE, kConvPT>(p, c0, cn, r, s_w, acc);
                        break;
                    case 4:
                        if (p.rec.narrow) conv_rows<PRECISION, 9, SITE, kConvPT>(p, c0, cn, r, s_w, acc);
                        else conv_rows<PRECISION, 4, SITE, kConvPT>(p, c0, cn, r, s_w, acc);
                        break;
                    case 5: conv_rows<PRECISION, 5, SITE, kConvPT>(p, c0, cn, r, s_w, acc); break;
                    default:
                        if (p.rec.m4_hi) conv_rows<PRECISION, 6, SITE, kConvPT>(p, c0, cn, r, s_w, acc);
                        else conv_rows<PRECISION, 7, SITE, kConvPT>(p, c0, cn, r, s_w, acc);
                        break;
                }
            }
        }
    }
    if (r < p.n_runs) {
#pragma unroll
        for (int j = 0; j < kConvPT; ++j) {
            const int pi = p0 + j;
            if (pi >= p.P) continue;
            double *o = p.acc + ((size_t)r * p.P + pi) * 7;
            o[s] += acc[j].value();
            if (MAXSET) {
                if (p.spanning) o[0] += acc0[j].value();
                o[3] += acc3[j].value();
            }
        }
    }
}

// ---------------------------------------------------------------------
// m2 with compensated FP32 arithmetic
// ---------------------------------------------------------------------
// sum' s^2 / N is the susceptibility curve: up to ~2e4 at L = 1024, and its
// canonical value must come within 1e-6 absolute of the FP64 convolution,
// i.e. ~5e-11 relative per run.  Plain FP32 sums of 128 products carry
// ~1e-7, and FP32 weights alone ~2e-9.  So every term is computed from exact
// two-part operands and summed with its rounding errors kept, after Dot2 of
// Ogita, Rump & Oishi (2005, "Accurate sum and dot product"):
//   w = wh + wl        (wh = FP32(w64), wl = FP32(w64 - wh): ~2^-48 relative)
//   q = qh + ql        (qh = q rounded toward zero to 24 bits, ql = q - qh,
//                       both exact in FP32 for q < 2^48)
//   ph = wh qh, eh = fma(wh, qh, -ph)     (TwoProduct: ph + eh = wh qh exactly)
//   (s, e) = Fast2Sum(max(s, ph), min(s, ph))  (s + e = old s + ph exactly)
//   c += e + eh + wh ql + wl qh           (wl ql, ~2^-48 of the term, dropped)
// The run's value is s + c (FP64), about 2^-44 relative; the statistic's
// curve then inherits FP64-level accuracy from the FP64 run reduction.
// Only the band's core -- the rows whose weight is >= e^-8 of the mode, +-4
// standard deviations -- needs this: the tails hold < 1e-4 of the weight,
// and plain FP32 products summed per chunk keep their error near 1e-11 of
// the value.  Chunks of rows outside every core of a tile (about a third of
// a tile's rows) take the plain path.
struct Dot2Acc {
    float s = 0.0f, c = 0.0f, tail = 0.0f;
    // a compensated term.  Every term and the running sum are >= 0, so
    // ordering the two operands by size (max / min, on the integer pipe)
    // makes Dekker's Fast2Sum exact: 3 additions instead of TwoSum's 6.
    __device__ __forceinline__ void add(float wh, float wl, float qh, float ql) {
        const float ph = __fmul_rn(wh, qh);
        const float eh = __fmaf_rn(wh, qh, -ph);
        const float a = fmaxf(s, ph), b = fminf(s, ph);
        const float t = __fadd_rn(a, b);
        const float e = __fsub_rn(b, __fsub_rn(t, a));
        s = t;
        c = __fadd_rn(c, __fadd_rn(e, eh));
        c = __fmaf_rn(wh, ql, c);
        c = __fmaf_rn(wl, qh, c);
    }
    // a term of a chunk outside every core: plain FP32 product and sum,
    // added into the running sum once per chunk by Fast2Sum (so the
    // compensation stays of the size of the rounding errors it collects)
    __device__ __forceinline__ void add_tail(float wh, float q) { tail = __fmaf_rn(wh, q, tail); }
    __device__ __forceinline__ void flush_tail() {
        const float a = fmaxf(s, tail), b = fminf(s, tail);
        const float t = __fadd_rn(a, b);
        c = __fadd_rn(c, __fsub_rn(b, __fsub_rn(t, a)));
        s = t;
        tail = 0.0f;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// q (< 2^48) as qh + ql, both exact in FP32
__device__ __forceinline__ void split_u64(uint64_t q, float &qh, float &ql) {
    qh = __ull2float_rz(q);
    ql = (float)(int64_t)(q - (uint64_t)qh);
}
__device__ __forceinline__ void split_u32(uint32_t q, float &qh, float &ql) {
    qh = __uint2float_rz(q);
    ql = (float)(int32_t)(q - (uint32_t)qh);
}


// grid (run tiles, tiles of kM2PT probabilities): each thread the kM2PT m2
// values of its run.  A chunk of rows that meets the core of any of the
// tile's probabilities runs the compensated arithmetic on all its rows
// (branch-free, so the kM2PT accumulator chains interleave); a chunk
// entirely in the tails runs plain FP32 products.
// record loads in flight per thread of the compensated m2 kernel: 32
// against 16, 1092 against 1099 ms per 100,000-run L = 256 step (same box,
// the convolution stream 801 against 838 ms)
#ifndef NZ_M2_BATCH
#define NZ_M2_BATCH 32
#endif
constexpr int kM2Batch = NZ_M2_BATCH;

// kM2PT probabilities per CTA (the tuned m2_tile, 8 or 16; 8 by default:
// on the same box 8 gave 1085.8 and 1204.7 ms per 100,000-run L = 256 step
// against 1108.8 and 1224.7 ms for 16 (two boxes); 32 measured 1285 against
// 1128 ms for 16)
template <bool NARROW, int kM2PT>
__global__ void NZ_CONV_BOUNDS conv_m2_comp_kernel(ConvParams p) {
    __shared__ float s_wh[kConvChunk][kM2PT], s_wl[kConvChunk][kM2PT];
    __shared__ uint32_t s_lo[kM2PT], s_len[kM2PT], s_clo[kM2PT], s_clen[kM2PT];
    __shared__ uint32_t s_range[2];
    const int r = blockIdx.x * kConvRuns + threadIdx.x;
    const int p0 = blockIdx.y * kM2PT;
    if (threadIdx.x < kM2PT) {
        const int pi = p0 + threadIdx.x;
        s_lo[threadIdx.x] = pi < p.P ? p.band_lo[pi] : 0u;
        s_len[threadIdx.x] = pi < p.P ? p.band_len[pi] : 0u;
        s_clo[threadIdx.x] = pi < p.P ? p.core_lo[pi] : 0u;
        s_clen[threadIdx.x] = pi < p.P ? p.core_len[pi] : 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0xffffffffu, b = 0;
        for (int j = 0; j < kM2PT; ++j)
            if (s_len[j]) { a = min(a, s_lo[j]); b = max(b, s_lo[j] + s_len[j]); }
        s_range[0] = max(a, p.n_begin);
        s_range[1] = min(b, p.n_end);
    }
    __syncthreads();
    const uint32_t nlo = s_range[0], nhi = s_range[1];
    if (nlo >= nhi) return;
    Dot2Acc acc[kM2PT];
    const uint32_t *m2n = reinterpret_cast<const uint32_t *>(p.rec.m2);
    for (uint32_t c0 = nlo; c0 < nhi; c0 += kConvChunk) {
        const uint32_t cn = min((uint32_t)kConvChunk, nhi - c0);
        // does the chunk meet a core?  (uniform over the CTA)
        bool core = false;
#pragma unroll
        for (int j = 0; j < kM2PT; ++j)
            core |= s_clen[j] && s_clo[j] < c0 + cn && c0 < s_clo[j] + s_clen[j];
        __syncthreads();
        for (int i = threadIdx.x; i < kConvChunk * kM2PT; i += kConvRuns) {
            const int rw = i / kM2PT, j = i % kM2PT;
            const uint32_t n = c0 + rw;
            float vh = 0.0f, vl = 0.0f;
            if (rw < (int)cn && n >= s_lo[j] && n < s_lo[j] + s_len[j]) {
                const size_t widx = (size_t)(p0 + j) * p.cap + (n - s_lo[j]);
                vh = p.w32[widx];
                vl = p.w32lo[widx];
            }
            s_wh[rw][j] = vh;
            s_wl[rw][j] = vl;
        }
        __syncthreads();
        if (r >= p.n_runs) continue;
        const size_t base = (size_t)(c0 - p.n_begin) * p.rec.run_stride + r;
        // raw m2 words of kM2Batch rows are loaded before any is split and
        // used, so that many loads are in flight per thread
        using raw_t = typename std::conditional<NARROW, uint32_t, uint64_t>::type;
        const raw_t *plane = NARROW ? reinterpret_cast<const raw_t *>(m2n)
                                    : reinterpret_cast<const raw_t *>(p.rec.m2);
        auto split = [&](raw_t w, float &qh, float &ql) {
            if constexpr (NARROW) split_u32(w, qh, ql);
            else split_u64(w, qh, ql);
        };
        uint32_t i = 0;
        if (core) {
            for (; i + kM2Batch <= cn; i += kM2Batch) {
                raw_t w[kM2Batch];
#pragma unroll
                for (int b = 0; b < kM2Batch; ++b) w[b] = plane[base + (size_t)(i + b) * p.rec.run_stride];
#pragma unroll
                for (int b = 0; b < kM2Batch; ++b) {
                    float qh, ql;
                    split(w[b], qh, ql);
#pragma unroll
                    for (int j = 0; j < kM2PT; ++j) acc[j].add(s_wh[i + b][j], s_wl[i + b][j], qh, ql);
                }
            }
            for (; i < cn; ++i) {
                float qh, ql;
                split(plane[base + (size_t)i * p.rec.run_stride], qh, ql);
#pragma unroll
                for (int j = 0; j < kM2PT; ++j) acc[j].add(s_wh[i][j], s_wl[i][j], qh, ql);
            }
        } else {
            for (; i + kM2Batch <= cn; i += kM2Batch) {
                raw_t w[kM2Batch];
#pragma unroll
                for (int b = 0; b < kM2Batch; ++b) w[b] = plane[base + (size_t)(i + b) * p.rec.run_stride];
#pragma unroll
                for (int b = 0; b < kM2Batch; ++b) {
                    float qh, ql;
                    split(w[b], qh, ql);
                    const float q = __fadd_rn(qh, ql);
#pragma unroll
                    for (int j = 0; j < kM2PT; ++j) acc[j].add_tail(s_wh[i + b][j], q);
                }
            }
            for (; i < cn; ++i) {
                float qh, ql;
                split(plane[base + (size_t)i * p.rec.run_stride], qh, ql);
                const float q = __fadd_rn(qh, ql);
#pragma unroll
                for (int j = 0; j < kM2PT; ++j) acc[j].add_tail(s_wh[i][j], q);
            }
#pragma unroll
            for (int j = 0; j < kM2PT; ++j) acc[j].flush_tail();
        }
    }
    if (r < p.n_runs) {
#pragma unroll
        for (int j = 0; j < kM2PT; ++j) {
            const int pi = p0 + j;
            if (pi >= p.P) continue;
            p.acc[((size_t)r * p.P + pi) * 7 + 4] += acc[j].value();
        }
    }
}

void launch_conv_m2_comp(const ConvParams &p, cudaStream_t s) {
    if (p.n_runs <= 0 || p.P <= 0) return;
    const int pt = p.m2_tile == 16 ? 16 : 8;
    dim3 g((p.n_runs + kConvRuns - 1) / kConvRuns, (p.P + pt - 1) / pt, 1);
    if (pt == 8) {
        if (p.rec.narrow) conv_m2_comp_kernel<true, 8><<<g, kConvRuns, 0, s>>>(p);
        else conv_m2_comp_kernel<false, 8><<<g, kConvRuns, 0, s>>>(p);
    } else {
        if (p.rec.narrow) conv_m2_comp_kernel<true, 16><<<g, kConvRuns, 0, s>>>(p);
        else conv_m2_comp_kernel<false, 16><<<g, kConvRuns, 0, s>>>(p);
    }
}

bool conv_grid_fits(int32_t n_runs, int32_t P) {
    // grid.y (p tiles) is limited to 65535
    return n_runs > 0 && P > 0 && (P + kConvPT - 1) / kConvPT <= 65535;
}

// PT_OTHER: probabilities per CTA of the other statistics' kernel (m0, m3,
// m4: 18 of the 26 record bytes at L = 256); the max-set kernel keeps 8 (16
// takes it to 201 registers beside the union-find)
template <int PT_OTHER>
static void launch_conv_window_pt(const ConvParams &p, int precision, cudaStream_t s) {
    // (run tiles, p tiles, statistics); launching the p tiles of one run tile
    // back to back (for L2 reuse of its records) measured slower
    dim3 gmax((p.n_runs + kConvRuns - 1) / kConvRuns, (p.P + kConvPT - 1) / kConvPT, 1);
    dim3 gother(gmax.x, (p.P + PT_OTHER - 1) / PT_OTHER, precision == 0 ? 4 : 3);
    // the record model is a template parameter: a run-time test in the row
    // loop cost 17 % of the kernel's time
    if (p.rec.site) {
        if (precision == 0) {
            conv_window_kernel<0, true, true, kConvPT><<<gmax, kConvRuns, 0, s>>>(p);
            conv_window_kernel<0, true, false, kConvPT><<<gother, kConvRuns, 0, s>>>(p);
        } else {
            conv_window_kernel<1, true, true, kConvPT><<<gmax, kConvRuns, 0, s>>>(p);
            conv_window_kernel<1, true, false, PT_OTHER><<<gother, kConvRuns, 0, s>>>(p);
            launch_conv_m2_comp(p, s);
        }
    } else {
        if (precision == 0) {
            conv_window_kernel<0, false, true, kConvPT><<<gmax, kConvRuns, 0, s>>>(p);
            conv_window_kernel<0, false, false, kConvPT><<<gother, kConvRuns, 0, s>>>(p);
        } else {
            conv_window_kernel<1, false, true, kConvPT><<<gmax, kConvRuns, 0, s>>>(p);
            conv_window_kernel<1, false, false, PT_OTHER><<<gother, kConvRuns, 0, s>>>(p);
            launch_conv_m2_comp(p, s);
        }
    }
}

void launch_conv_window(const ConvParams &p, int precision, cudaStream_t s) {
    if (p.n_runs <= 0 || p.P <= 0) return;
    // the FP64 path keeps 8 probabilities per CTA (its accumulators are
    // twice as wide)
    if (precision != 0 && p.conv_tile == 16) launch_conv_window_pt<16>(p, precision, s);
    else launch_conv_window_pt<kConvPT>(p, precision, s);
}

// Weights of the FP32 convolution: the part of each p's band whose weights
// are at least `rel` times the band's largest, converted to FP32 and re-based
// at its own low edge (w32[i * cap + j] is the weight of row lo32[i] + j).
// The band of the FP64 path reaches weights e^-80 below its mode; at rel =
// e^-30 (7.7 standard deviations from the mode) the weights left out sum to
// less than 1e-13, far below the FP32 rounding of the sums, and the rows each
// p reads shrink by 40 %.  Band weights are unimodal, so the kept part is one
// run of rows.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) narrow_weights_f32_kernel(const double *w64, const uint32_t *band_lo,
                                                                   const uint32_t *band_len, int32_t cap, double rel,
                                                                   double rel_core, float *w32, float *w32lo,
                                                                   uint32_t *lo32, uint32_t *len32,
                                                                   uint32_t *core_lo, uint32_t *core_len) {
    __shared__ double s_max[BLOCK / 32];
    __shared__ uint32_t s_a[BLOCK / 32], s_b[BLOCK / 32], s_ca[BLOCK / 32], s_cb[BLOCK / 32];
    const int pi = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double *w = w64 + (size_t)pi * cap;
    const uint32_t len = min(band_len[pi], (uint32_t)cap);
    double m = 0.0;
    for (uint32_t j = threadIdx.x; j < len; j += BLOCK) m = fmax(m, w[j]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) s_max[warp] = m;
    __syncthreads();
    m = s_max[0];
    for (int k = 1; k < BLOCK / 32; ++k) m = fmax(m, s_max[k]);
    const double thr = m * rel, thr_core = m * rel_core;
    uint32_t a = 0xffffffffu, b = 0, ca = 0xffffffffu, cb = 0;
    for (uint32_t j = threadIdx.x; j < len; j += BLOCK) {
        if (w[j] >= thr) { a = min(a, j); b = max(b, j + 1); }
        if (w[j] >= thr_core) { ca = min(ca, j); cb = max(cb, j + 1); }
    }
    for (int o = 16; o > 0; o >>= 1) {
        a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
        ca = min(ca, __shfl_xor_sync(0xffffffffu, ca, o));
        cb = max(cb, __shfl_xor_sync(0xffffffffu, cb, o));
    }
    if (lane == 0) { s_a[warp] = a; s_b[warp] = b; s_ca[warp] = ca; s_cb[warp] = cb; }
    __syncthreads();
    a = s_a[0]; b = s_b[0]; ca = s_ca[0]; cb = s_cb[0];
    for (int k = 1; k < BLOCK / 32; ++k) {
        a = min(a, s_a[k]); b = max(b, s_b[k]);
        ca = min(ca, s_ca[k]); cb = max(cb, s_cb[k]);
    }
    if (b <= a) a = b = 0;  // an empty band stays empty
    if (cb <= ca) ca = cb = 0;
    if (threadIdx.x == 0) {
        lo32[pi] = band_lo[pi] + a;
        len32[pi] = b - a;
        core_lo[pi] = band_lo[pi] + ca;
        core_len[pi] = cb - ca;
    }
    float *o = w32 + (size_t)pi * cap;
    float *ol = w32lo + (size_t)pi * cap;
    for (uint32_t j = threadIdx.x; j < (uint32_t)cap; j += BLOCK) {
        const double v = j < b - a ? w[a + j] : 0.0;
        const float hi = (float)v;
        o[j] = hi;
        ol[j] = (float)(v - (double)hi);  // exact difference; its FP32 rounding is 2^-24 of 2^-24 w
    }
}

void launch_narrow_weights_f32(const double *w64, const uint32_t *band_lo, const uint32_t *band_len, int32_t P,
                               int32_t cap, double rel, double rel_core, float *w32, float *w32lo, uint32_t *lo32,
                               uint32_t *len32, uint32_t *core_lo, uint32_t *core_len, cudaStream_t s) {
    if (P <= 0) return;
    narrow_weights_f32_kernel<256><<<P, 256, 0, s>>>(w64, band_lo, band_len, cap, rel, rel_core, w32, w32lo, lo32,
                                                     len32, core_lo, core_len);
}

// =====================================================================
// Pairwise (n, mean, M2) reduction over runs
// =====================================================================
// Chan, Golub & LeVeque (1979) pairwise update, the formula simoa's
// online_variance applies in bond_reduce (percolate/hpc.py:674-692).
__device__ __forceinline__ void chan_merge(double &na, double &ma, double &sa, double nb, double mb, double sb) {
    if (nb == 0.0) return;
    if (na == 0.0) { na = nb; ma = mb; sa = sb; return; }
    const double n = na + nb;
    const double d = mb - ma;
    ma += d * nb / n;
    sa += sb + d * d * na * nb / n;
    na = n;
}

// stats [n_runs][P*7]: one thread per column, looping over a slice of runs;
// partial (n, mean, M2) go to `part` [slices][cols][3].
__global__ void reduce_runs_partial_kernel(const double *stats, int32_t n_runs, int32_t cols, int32_t slice,
                                           double *part) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int sl = blockIdx.y;
    if (c >= cols) return;
    const int r0 = sl * slice, r1 = min(n_runs, r0 + slice);
    // sums of the deviations from the slice's first value, x0: mean = x0 +
    // S1 / n, M2 = S2 - S1^2 / n (the shift keeps the difference free of
    // cancellation).  Welford's update needs an FP64 division per value, and
    // FP64 runs at 1/64 of the FP32 rate on this chip.
    double x0 = 0.0, s1 = 0.0, s2 = 0.0;
    if (r0 < r1) x0 = stats[(size_t)r0 * cols + c];
    for (int r = r0 + 1; r < r1; ++r) {
        const double d = stats[(size_t)r * cols + c] - x0;
        s1 += d;
        s2 = fma(d, d, s2);
    }
    const double n = (double)max(r1 - r0, 0);
    double *o = part + ((size_t)sl * cols + c) * 3;
    o[0] = n;
    o[1] = n > 0 ? x0 + s1 / n : 0.0;
    o[2] = n > 0 ? fmax(s2 - s1 * s1 / n, 0.0) : 0.0;
}

__global__ void reduce_runs_final_kernel(const double *part, int32_t cols, int32_t slices, const uint64_t *acc_count,
                                         double *acc_mean, double *acc_m2) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    double n = 0, mean = 0, m2 = 0;
    for (int sl = 0; sl < slices; ++sl) {
        const double *o = part + ((size_t)sl * cols + c) * 3;
        chan_merge(n, mean, m2, o[0], o[1], o[2]);
    }
    double na = (double)*acc_count, ma = acc_mean[c], sa = acc_m2[c];
    chan_merge(na, ma, sa, n, mean, m2);
    acc_mean[c] = ma;
    acc_m2[c] = sa;
}

__global__ void add_count_kernel(uint64_t *count, int32_t n) { *count += (uint64_t)n; }

void launch_reduce_runs(const double *stats, int32_t n_runs, int32_t P, uint64_t *acc_count, double *acc_mean,
                           double *acc_m2, double *part, int32_t slices, cudaStream_t s) {
    const int cols = P * 7;
    const int slice = (n_runs + slices - 1) / slices;
    dim3 grid((cols + 127) / 128, slices);
    reduce_runs_partial_kernel<<<grid, 128, 0, s>>>(stats, n_runs, cols, slice, part);
    reduce_runs_final_kernel<<<(cols + 127) / 128, 128, 0, s>>>(part, cols, slices, acc_count, acc_mean, acc_m2);
    add_count_kernel<<<1, 1, 0, s>>>(acc_count, n_runs);
}

// =====================================================================
// Microcanonical run-reductions (fused over a window of records)
// =====================================================================
// Per (row n, statistic): exact integer sum over runs and the sum of squared
// deviations, merged into the accumulators with the pairwise formula.
// Statistics: 0 max, 1 m0, 2 m1 (= N - max), 3 m2, 4 m3, 5 m4; block 6
// counts the spanning runs.  Deviations are taken from run 0's value x0:
//   max, m0, m1 (< 2^21) and m2 (< 2^42): d = x - x0 as int64, d^2 summed
//     exactly (u64 / u128), and M2 = (R * sum d^2 - (sum d)^2) / R from the
//     exact 128-bit numerator;
//   m3, m4: d exact as a 128-bit integer; |d| 2^-e as two FP32 parts (its
//     top 48 bits, 2^-47 relative), squared with an exact FP32 product and
//     summed as an FP32 (sum, compensation) pair per thread, then in FP64
//     across threads (the shift keeps the sum free of cancellation; the
//     power-of-two scale 2^-e, e from N, keeps squares and sums inside FP32's
//     range).  FP64 runs at 1/64 of the FP32 rate on this chip, and the FP64
//     squares were most of this kernel's time.
typedef unsigned __int128 u128;
typedef __int128 i128;

__device__ __forceinline__ u128 shfl_down_u128(u128 v, int off) {
    uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
    lo = __shfl_down_sync(0xffffffffu, lo, off);
    hi = __shfl_down_sync(0xffffffffu, hi, off);
    return ((u128)hi << 64) | lo;
}

template <int BLOCK>
__device__ __forceinline__ u128 block_sum_u128(u128 v, u128 *s_tmp) {
    for (int off = 16; off > 0; off >>= 1) v += shfl_down_u128(v, off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_tmp[warp] = v;
    __syncthreads();
    u128 t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < BLOCK / 32; ++w) t += s_tmp[w];
    return t;  // valid in thread 0
}

template <int BLOCK>
__device__ __forceinline__ double block_sum_f64(double v, double *s_tmp) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_tmp[warp] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < BLOCK / 32; ++w) t += s_tmp[w];
    return t;
}

__device__ __forceinline__ double u128_to_f64(u128 x) {
    return fma((double)(uint64_t)(x >> 64), 18446744073709551616.0, (double)(uint64_t)x);
}

__device__ __forceinline__ double i128_to_f64(i128 x) {
    return x < 0 ? -u128_to_f64((u128)(-x)) : u128_to_f64((u128)x);
}

// Per-thread partial sums of one row: for every statistic the exact sum of
// x, the exact sum of d = x - x0 and the sum of d^2 (exact integers for
// max, m0, m2; FP64 for m3, m4), plus the spanning count.
struct MicroPart {
    uint64_t sx_max, sx_m0, sx_m2;  // max, m0 < 2^21; m2 < 2^42 (per-thread sums fit)
    u128 sx_m3, sx_m4;
    int64_t sd_max, sd_m0, sd_m2;
    i128 sd_m3, sd_m4;
    uint64_t sq_max, sq_m0;
    u128 sq_m2;
    float fs_m3, fc_m3, fs_m4, fc_m4;  // scaled sum of d^2 and its compensation
    uint32_t span;
};

__device__ __forceinline__ float exp2i(int k) { return __int_as_float((127 + k) << 23); }  // -126 <= k <= 127

// x (< 2^96, as 64-bit halves) times 2^-e as yh + yl: yh = x's top 24
// significant bits, yl = the next 24 (both exact in FP32; the bits below are
// truncated: 2^-47 relative), so yh^2 carries the square and yl only small
// corrections.
__device__ __forceinline__ void scaled_split(uint64_t lo, uint64_t hi, int e, float &yh, float &yl) {
    const int nb = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);
    const int s2 = nb > 48 ? nb - 48 : 0;  // y = x >> s2 keeps min(nb, 48) bits
    uint64_t y;
    if (s2 == 0) y = lo;
    else if (s2 < 64) y = (lo >> s2) | (hi << (64 - s2));
    else y = hi >> (s2 - 64);
    const int sh = nb > 24 ? nb - s2 - 24 : 0;  // y's top 24 bits sit above bit sh
    const uint64_t top = y >> sh;
    const int k = s2 - e;
    yh = (float)(uint32_t)top * exp2i(sh + k);
    yl = (float)(uint32_t)(y - (top << sh)) * exp2i(k);
}

// (s, c) += (yh + yl)^2: the exact product yh^2 (TwoProd by FMA), TwoSum of
// the running sum, the cross and low terms into the compensation.
__device__ __forceinline__ void add_square(float &s, float &c, float yh, float yl) {
    const float p = __fmul_rn(yh, yh);
    const float pe = fmaf(yh, yh, -p);
    const float cross = fmaf(2.0f * yh, yl, __fmul_rn(yl, yl));
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, __fadd_rn(pe, cross)));
}

template <int BLOCK>
__device__ __forceinline__ uint64_t bsum_u64(uint64_t v, uint64_t *s_tmp) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = v;
    __syncthreads();
    uint64_t t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < BLOCK / 32; ++w) t += s_tmp[w];
    return t;
}

// 3 resident blocks of 256 threads per SM (at most 80 registers, a few
// hundred bytes of spills): beside the union-find of the next window this
// measured 1364 against 1394 ms per 100,000-run L = 256 step at 100
// registers.
#ifndef NZ_MICRO_MIN_BLOCKS
#define NZ_MICRO_MIN_BLOCKS 3
#endif
// records in flight per thread: 2 against 1 took the kernel from 400 to
// 179 ms per 100,000-run L = 256 step inside the pipeline; 4 (with a few
// hundred bytes of spills at the 80-register cap) gave the same step time
// (1076.2 against 1076.0 ms, same box)
#ifndef NZ_MICRO_INFLIGHT
#define NZ_MICRO_INFLIGHT 2
#endif
constexpr int kMicroInflight = NZ_MICRO_INFLIGHT;
#define NZ_MICRO_BOUNDS __launch_bounds__(BLOCK, NZ_MICRO_MIN_BLOCKS)

// One block per row n: reduces all statistics of that row over the runs and
// merges them into the accumulators (pairwise formula for M2).
template <int BLOCK>
__global__ void NZ_MICRO_BOUNDS micro_window_kernel(MicroParams p) {
    const uint32_t n = p.n_begin + blockIdx.x;
    const size_t row = (size_t)(n - p.n_begin) * p.rec.run_stride;
    const NzRecords &rec = p.rec;
    __shared__ u128 s_u[BLOCK / 32];
    __shared__ double s_f[BLOCK / 32];
    __shared__ uint64_t s_w[BLOCK / 32];
    const uint32_t x0_max = rec.max_span[row] & ~kSpanBit;
    const uint32_t x0_m0 = record_m0(rec, row);
    const uint64_t x0_m2 = record_m2(rec, row), x0_m3 = rec.m3[row];
    const bool has_hi = rec.m4_hi != nullptr;  // without the plane the high words are zero
    const u128 x0_m4 = ((u128)(has_hi ? rec.m4_hi[row] : 0u) << 64) | rec.m4_lo[row];
    // scales: m3 < N^3 and m4 < N^4 (< 2^96); |d| 2^-e <= 2^40, so squares
    // stay below 2^80 and sums below 2^111, and |d| >= 1 keeps its square
    // above 2^-88 (FP32 normal)
    const int nbits = 32 - __clz((int)p.N);
    const int e3 = max(0, 3 * nbits - 40), e4 = max(0, min(4 * nbits, 96) - 40);
    MicroPart a = {};
    struct Rec {
        uint32_t ms, m0, m4_hi;
        uint64_t m2, m3, m4_lo;
    };
    auto load = [&](int r) -> Rec {
        const size_t off = row + r;
        return Rec{rec.max_span[off], record_m0(rec, off), has_hi ? rec.m4_hi[off] : 0u,
                   record_m2(rec, off), rec.m3[off],     rec.m4_lo[off]};
    };
    auto add = [&](const Rec &q) {
        const uint32_t mx = q.ms & ~kSpanBit;
        const u128 m4 = ((u128)q.m4_hi << 64) | q.m4_lo;
        a.span += q.ms >> 31;
        a.sx_max += mx;
        a.sx_m0 += q.m0;
        a.sx_m2 += q.m2;
        a.sx_m3 += q.m3;
        a.sx_m4 += m4;
        const int64_t dmax = (int64_t)mx - (int64_t)x0_max;
        const int64_t dm0 = (int64_t)q.m0 - (int64_t)x0_m0;
        const int64_t dm2 = (int64_t)q.m2 - (int64_t)x0_m2;
        const int64_t dm3 = (int64_t)(q.m3 - x0_m3);  // |m3 - x0| < 2^63
        const i128 dm4 = (i128)(m4 - x0_m4);
        a.sd_max += dmax;
        a.sd_m0 += dm0;
        a.sd_m2 += dm2;
        a.sd_m3 += dm3;
        a.sd_m4 += dm4;
        a.sq_max += (uint64_t)(dmax * dmax);
        a.sq_m0 += (uint64_t)(dm0 * dm0);
        const uint64_t ad2 = (uint64_t)(dm2 < 0 ? -dm2 : dm2);
        a.sq_m2 += (u128)ad2 * ad2;
        float yh, yl;
        scaled_split((uint64_t)(dm3 < 0 ? -dm3 : dm3), 0, e3, yh, yl);
        add_square(a.fs_m3, a.fc_m3, yh, yl);
        const u128 ad4 = (u128)(dm4 < 0 ? -dm4 : dm4);
        scaled_split((uint64_t)ad4, (uint64_t)(ad4 >> 64), e4, yh, yl);
        add_square(a.fs_m4, a.fc_m4, yh, yl);
    };
    // the records of NZ_MICRO_INFLIGHT runs are loaded before any is added,
    // so each thread keeps that many records' loads in flight
    int r = threadIdx.x;
    for (; r + (kMicroInflight - 1) * BLOCK < p.n_runs; r += kMicroInflight * BLOCK) {
        Rec q[kMicroInflight];
#pragma unroll
        for (int k = 0; k < kMicroInflight; ++k) q[k] = load(r + k * BLOCK);
#pragma unroll
        for (int k = 0; k < kMicroInflight; ++k) add(q[k]);
    }
    for (; r < p.n_runs; r += BLOCK) add(load(r));
    // block sums (results valid in thread 0)
    const uint64_t span = bsum_u64<BLOCK>(a.span, s_w);
    const uint64_t sx_max = bsum_u64<BLOCK>(a.sx_max, s_w);
    const uint64_t sx_m0 = bsum_u64<BLOCK>(a.sx_m0, s_w);
    const u128 sx_m2 = block_sum_u128<BLOCK>(a.sx_m2, s_u);
    const u128 sx_m3 = block_sum_u128<BLOCK>(a.sx_m3, s_u);
    const u128 sx_m4 = block_sum_u128<BLOCK>(a.sx_m4, s_u);
    const i128 sd_max = (i128)block_sum_u128<BLOCK>((u128)(i128)a.sd_max, s_u);
    const i128 sd_m0 = (i128)block_sum_u128<BLOCK>((u128)(i128)a.sd_m0, s_u);
    const i128 sd_m2 = (i128)block_sum_u128<BLOCK>((u128)(i128)a.sd_m2, s_u);
    const i128 sd_m3 = (i128)block_sum_u128<BLOCK>((u128)a.sd_m3, s_u);
    const i128 sd_m4 = (i128)block_sum_u128<BLOCK>((u128)a.sd_m4, s_u);
    const u128 sq_max = block_sum_u128<BLOCK>(a.sq_max, s_u);
    const u128 sq_m0 = block_sum_u128<BLOCK>(a.sq_m0, s_u);
    const u128 sq_m2 = block_sum_u128<BLOCK>(a.sq_m2, s_u);
    const double fq_m3 = ldexp(block_sum_f64<BLOCK>((double)a.fs_m3 + (double)a.fc_m3, s_f), 2 * e3);
    const double fq_m4 = ldexp(block_sum_f64<BLOCK>((double)a.fs_m4 + (double)a.fc_m4, s_f), 2 * e4);
    if (threadIdx.x != 0) return;
    const double R = (double)p.n_runs;
    const uint64_t Rn = (uint64_t)p.n_runs;
    // exact M2 numerator R * sum d^2 - (sum d)^2 when it fits in 128 bits
    auto m2_exact = [&](u128 sq, i128 sd) -> double {
        const u128 ad = (u128)(sd < 0 ? -sd : sd);
        if ((sq >> 103) == 0 && (ad >> 63) == 0) return u128_to_f64(Rn * sq - ad * ad) / R;
        const double f = u128_to_f64(ad);
        const double v = u128_to_f64(sq) - f * f / R;
        return v > 0.0 ? v : 0.0;
    };
    auto m2_float = [&](double fq, i128 sd) -> double {
        const double f = i128_to_f64(sd);
        const double v = fq - f * f / R;
        return v > 0.0 ? v : 0.0;
    };
    // statistic order 0 max, 1 m0, 2 m1 (= N - max: same M2 as max), 3 m2, 4 m3, 5 m4
    const u128 held = rec.site ? n : p.N;  // sites in clusters: all N (bond) or the n occupied (site)
    const u128 sx[6] = {sx_max, sx_m0, (u128)Rn * held - sx_max, sx_m2, sx_m3, sx_m4};
    const double m2b_max = m2_exact(sq_max, sd_max);
    const double m2b[6] = {m2b_max, m2_exact(sq_m0, sd_m0), m2b_max, m2_exact(sq_m2, sd_m2),
                           m2_float(fq_m3, sd_m3), m2_float(fq_m4, sd_m4)};
    const double na = (double)*p.count_before;
    for (int k = 0; k < 6; ++k) {
        const size_t idx = (size_t)k * (p.M + 1) + n;
        const u128 acc = ((u128)p.acc.sum_hi[idx] << 64) | p.acc.sum_lo[idx];
        const double mean_a = na > 0 ? u128_to_f64(acc) / na : 0.0;
        double nn = na, mm = mean_a, ss = p.acc.m2[idx];
        chan_merge(nn, mm, ss, R, u128_to_f64(sx[k]) / R, m2b[k]);
        const u128 t = acc + sx[k];
        p.acc.sum_lo[idx] = (uint64_t)t;
        p.acc.sum_hi[idx] = (uint64_t)(t >> 64);
        p.acc.m2[idx] = ss;
    }
    p.acc.span_count[n] += span;
}

void launch_micro_window(const MicroParams &p, cudaStream_t s) {
    const uint32_t rows = p.n_end - p.n_begin;
    if (rows == 0 || p.n_runs <= 0) return;
    micro_window_kernel<256><<<rows, 256, 0, s>>>(p);
}

void launch_micro_count(uint64_t *count, int32_t n_runs, cudaStream_t s) {
    add_count_kernel<<<1, 1, 0, s>>>(count, n_runs);
}

// ------------------------------------------------ merging two accumulators
// dst <- dst (+) src for running (count, mean, M2) columns sharing one count
// each side: the pairwise update of percolate/hpc.py:638-702.
__global__ void canonical_merge_kernel(const uint64_t *dst_count, double *dst_mean, double *dst_m2,
                                       const uint64_t *src_count, const double *src_mean,
                                       const double *src_m2, int32_t cols) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    double na = (double)*dst_count, ma = dst_mean[c], sa = dst_m2[c];
    chan_merge(na, ma, sa, (double)*src_count, src_mean[c], src_m2[c]);
    dst_mean[c] = ma;
    dst_m2[c] = sa;
}

// Microcanonical accumulators of rows = M + 1 rows: exact 128-bit sums and
// spanning counts add; M2 merges pairwise with the means taken from the
// exact sums, as micro_window_kernel merges a batch.
__global__ void micro_merge_kernel(NzMicroAccum dst, NzMicroAccum src, uint32_t rows) {
    const size_t total = (size_t)6 * rows;
    const double na = (double)*dst.count, nb = (double)*src.count;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total + rows;
         i += (size_t)gridDim.x * blockDim.x) {
        if (i >= total) {
            dst.span_count[i - total] += src.span_count[i - total];
            continue;
        }
        const u128 a = ((u128)dst.sum_hi[i] << 64) | dst.sum_lo[i];
        const u128 b = ((u128)src.sum_hi[i] << 64) | src.sum_lo[i];
        double nn = na, mm = na > 0 ? u128_to_f64(a) / na : 0.0, ss = dst.m2[i];
        chan_merge(nn, mm, ss, nb, nb > 0 ? u128_to_f64(b) / nb : 0.0, src.m2[i]);
        const u128 t = a + b;
        dst.sum_lo[i] = (uint64_t)t;
        dst.sum_hi[i] = (uint64_t)(t >> 64);
        dst.m2[i] = ss;
    }
}

__global__ void add_counts_kernel(uint64_t *dst, const uint64_t *src) { *dst += *src; }

// the counts are read by the merge kernels, so they are added afterwards
void launch_canonical_merge(uint64_t *dst_count, double *dst_mean, double *dst_m2, const uint64_t *src_count,
                            const double *src_mean, const double *src_m2, int32_t cols, cudaStream_t s) {
    if (cols > 0)
        canonical_merge_kernel<<<(cols + 255) / 256, 256, 0, s>>>(dst_count, dst_mean, dst_m2, src_count,
                                                                  src_mean, src_m2, cols);
    add_counts_kernel<<<1, 1, 0, s>>>(dst_count, src_count);
}

void launch_micro_merge(const NzMicroAccum &dst, const NzMicroAccum &src, uint32_t rows, cudaStream_t s) {
    const size_t work = (size_t)7 * rows;
    const unsigned grid = (unsigned)((work + 255) / 256 < 4096 ? (work + 255) / 256 : 4096);
    micro_merge_kernel<<<grid, 256, 0, s>>>(dst, src, rows);
    add_counts_kernel<<<1, 1, 0, s>>>(dst.count, src.count);
}

// =====================================================================
// Row-format kernels: initialize / reduce / finalize
// =====================================================================
// Packed structured rows with 4-byte alignment: doubles are moved as two words.
__device__ __forceinline__ double ld_f64(const uint8_t *p) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(p);
    return __hiloint2double((int)w[1], (int)w[0]);
}
__device__ __forceinline__ void st_f64(uint8_t *p, double v) {
    uint32_t *w = reinterpret_cast<uint32_t *>(p);
    w[0] = (uint32_t)__double2loint(v);
    w[1] = (uint32_t)__double2hiint(v);
}

// canonical_statistics_dtype (hpc.py:407-440): [pp f8] max f8 moments 5*f8
// canonical_averages_dtype  (hpc.py:518-558): n u4 [pp_mean pp_m2] max_mean max_m2
//                                             moments_mean 5*f8 moments_m2 5*f8
__global__ void init_avg_kernel(const uint8_t *canon, int32_t P, int32_t spanning, uint8_t *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int nst = spanning ? 7 : 6;
    const uint8_t *c = canon + (size_t)i * nst * 8;
    uint8_t *o = out + (size_t)i * (4 + nst * 16);
    *reinterpret_cast<uint32_t *>(o) = 1u;
    int k = 0;
    if (spanning) { st_f64(o + 4, ld_f64(c)); st_f64(o + 12, 0.0); k = 1; }
    const int base = 4 + k * 16;
    st_f64(o + base, ld_f64(c + k * 8));
    st_f64(o + base + 8, 0.0);
    for (int m = 0; m < 5; ++m) {
        st_f64(o + base + 16 + 8 * m, ld_f64(c + (k + 1 + m) * 8));
        st_f64(o + base + 56 + 8 * m, 0.0);
    }
}

void launch_init_avg(const uint8_t *canon_rows, int32_t P, int32_t spanning, uint8_t *out, cudaStream_t s) {
    if (P > 0) init_avg_kernel<<<(P + 127) / 128, 128, 0, s>>>(canon_rows, P, spanning, out);
}

__global__ void bond_reduce_kernel(const uint8_t *a, const uint8_t *b, int32_t P, int32_t spanning, uint8_t *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int nst = spanning ? 7 : 6;
    const size_t rb = 4 + nst * 16;
    const uint8_t *ra = a + i * rb, *rbp = b + i * rb;
    uint8_t *o = out + i * rb;
    const uint32_t na = *reinterpret_cast<const uint32_t *>(ra);
    const uint32_t nb = *reinterpret_cast<const uint32_t *>(rbp);
    // (mean offset, m2 offset) pairs
    int mo[7], so[7], cnt = 0;
    int off = 4;
    if (spanning) { mo[cnt] = off; so[cnt] = off + 8; ++cnt; off += 16; }
    mo[cnt] = off; so[cnt] = off + 8; ++cnt; off += 16;
    for (int m = 0; m < 5; ++m) { mo[cnt] = off + 8 * m; so[cnt] = off + 40 + 8 * m; ++cnt; }
    for (int k = 0; k < cnt; ++k) {
        double n1 = (double)na, m1 = ld_f64(ra + mo[k]), s1 = ld_f64(ra + so[k]);
        const double n2 = (double)nb, m2 = ld_f64(rbp + mo[k]), s2 = ld_f64(rbp + so[k]);
        const double n = n1 + n2;
        const double d = m2 - m1;
        const double mean = m1 + d * n2 / n;
        const double ss = s1 + s2 + d * d * n1 * n2 / n;
        st_f64(o + mo[k], mean);
        st_f64(o + so[k], ss);
    }
    *reinterpret_cast<uint32_t *>(o) = na + nb;
}

void launch_bond_reduce(const uint8_t *a, const uint8_t *b, int32_t P, int32_t spanning, uint8_t *out,
                        cudaStream_t s) {
    if (P > 0) bond_reduce_kernel<<<(P + 127) / 128, 128, 0, s>>>(a, b, P, spanning, out);
}

// finalized_canonical_averages_dtype (hpc.py:705-749):
//   n u4, p f8, alpha f8, [pp_mean, pp_std, pp_ci 2*f8], strength_mean, strength_std,
//   strength_ci 2*f8, moments_mean 5*f8, moments_std 5*f8, moments_ci 5*2*f8
// Student-t quantiles ppf((1 - conf)/2, df) and ppf((1 + conf)/2, df) for
// the rows of a block: threads 0 and 1 evaluate them once for df0 (the df of
// the block's first row) and share them; a row with another df evaluates its
// own.  Every thread of the block must call this (it synchronises).
struct TPair { double lo, hi; };

__device__ TPair t_pair_block(double conf, double df0, double df, bool active) {
    __shared__ double s_q[2];
    if (threadIdx.x < 2)
        s_q[threadIdx.x] = student_t_quantile(threadIdx.x == 0 ? (1.0 - conf) / 2.0 : (1.0 + conf) / 2.0, df0);
    __syncthreads();
    TPair r;
    if (df == df0) { r.lo = s_q[0]; r.hi = s_q[1]; }
    else if (active) {
        r.lo = student_t_quantile((1.0 - conf) / 2.0, df);
        r.hi = student_t_quantile((1.0 + conf) / 2.0, df);
    } else { r.lo = r.hi = NAN; }
    return r;
}

__device__ void t_interval(const TPair &q, double df, double loc, double scale, double &lo, double &hi) {
    // scipy.stats.t.interval: loc + scale * ppf((1 -+ conf)/2); NaN unless
    // scale > 0 and df > 0.
    if (!(scale > 0.0) || !(df > 0.0) || isnan(loc)) { lo = NAN; hi = NAN; return; }
    lo = loc + scale * q.lo;
    hi = loc + scale * q.hi;
}

__global__ void finalize_kernel(const uint8_t *avg, int32_t P, int32_t spanning, double N, const double *ps,
                                double alpha, uint8_t *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nst = spanning ? 7 : 6;
    const size_t in_row = 4 + nst * 16;
    const double conf = 1.0 - alpha;
    // numpy uint32 arithmetic: n - 1 wraps for n = 0
    const uint32_t nu0 = *reinterpret_cast<const uint32_t *>(avg + (size_t)blockIdx.x * blockDim.x * in_row);
    const uint32_t nu_i = i < P ? *reinterpret_cast<const uint32_t *>(avg + (size_t)i * in_row) : nu0;
    const TPair tq = t_pair_block(conf, (double)(uint32_t)(nu0 - 1u), (double)(uint32_t)(nu_i - 1u), i < P);
    if (i >= P) return;
    const uint8_t *a = avg + (size_t)i * in_row;
    uint8_t *o = out + (size_t)i * (spanning ? 244 : 212);
    const uint32_t nu = nu_i;
    const double n = (double)nu;
    const double nm1 = (double)(uint32_t)(nu - 1u);
    const double sqrt_n = sqrt(n);
    *reinterpret_cast<uint32_t *>(o) = nu;
    st_f64(o + 4, ps[i]);
    st_f64(o + 12, alpha);
    int ai = 4, oi = 20;
    auto transform = [&](double mean, double m2, bool normalize, uint8_t *pm, uint8_t *pstd, uint8_t *pci) {
        double mu = mean, sd = sqrt(m2 / nm1);
        if (normalize) { mu /= N; sd /= N; }
        st_f64(pm, mu);
        st_f64(pstd, sd);
        double lo, hi;
        t_interval(tq, nm1, mu, sd / sqrt_n, lo, hi);
        st_f64(pci, lo);
        st_f64(pci + 8, hi);
    };
    if (spanning) {
        transform(ld_f64(a + ai), ld_f64(a + ai + 8), false, o + oi, o + oi + 8, o + oi + 16);
        ai += 16; oi += 32;
    }
    transform(ld_f64(a + ai), ld_f64(a + ai + 8), true, o + oi, o + oi + 8, o + oi + 16);
    ai += 16; oi += 32;
    for (int m = 0; m < 5; ++m)
        transform(ld_f64(a + ai + 8 * m), ld_f64(a + ai + 40 + 8 * m), true, o + oi + 8 * m, o + oi + 40 + 8 * m,
                  o + oi + 80 + 16 * m);
}

void launch_finalize(const uint8_t *avg, int32_t P, int32_t spanning, double N, const double *ps, double alpha,
                     uint8_t *out, cudaStream_t s) {
    if (P > 0) finalize_kernel<<<(P + 63) / 64, 64, 0, s>>>(avg, P, spanning, N, ps, alpha, out);
}

// Microcanonical averages from the run-reduction accumulators, per row n
// (percolate/percolate.py:450-705 and :968-1064): spanning -> Bayesian
// posterior mean (k+1)/(R+2) with Beta(k+1, R-k+1) quantiles at alpha/2 and
// 1 - alpha/2; max and moments -> mean and Student-t interval with scale
// std/sqrt(R), std with ddof 1, (mean, mean) where std == 0; max and moments
// divided by N as microcanonical_averages_arrays returns them.
// out[n * 21 + ...]: span (mean, lo, hi), max (mean, lo, hi), m0..m4 (mean, lo, hi).
// Two threads per row n: half 0 the spanning mean, the lower Beta bound and
// statistics max, m0, m1; half 1 the upper Beta bound and m2, m3, m4 -- the
// Beta quantiles (iterative, FP64) are most of the work, and rows where some
// but not all runs span are contiguous, so splitting them doubles the
// threads working on those rows.
__global__ void micro_finalize_kernel(NzMicroAccum acc, uint32_t N, uint32_t M, int32_t spanning, double alpha,
                                      int32_t normalize, double *out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = t >> 1, half = t & 1u;
    const double R = (double)*acc.count;
    // every row has R runs: one pair of t quantiles per block
    const TPair tq = t_pair_block(1.0 - alpha, R - 1.0, R - 1.0, n <= M);
    if (n > M) return;
    // value j of row n: out[n * 21 + j], or out[j * (M + 1) + n] field-major
    const bool fields = (normalize & NZ_MICRO_FIELD_MAJOR) != 0;
    auto put = [&](int j, double v) { out[fields ? (size_t)j * (M + 1) + n : (size_t)n * 21 + j] = v; };
    if (spanning) {
        const double k = (double)acc.span_count[n];
        if (half == 0) {
            put(0, (k + 1.0) / (R + 2.0));
            put(1, beta_quantile(alpha / 2.0, k + 1.0, R - k + 1.0));
        } else {
            put(2, beta_quantile(1.0 - alpha / 2.0, k + 1.0, R - k + 1.0));
        }
    } else if (half == 0) {
        put(0, NAN); put(1, NAN); put(2, NAN);
    }
    const int map[6] = {0, 1, 2, 3, 4, 5};  // max, m0, m1, m2, m3, m4
    for (int j = 3 * (int)half; j < 3 * (int)half + 3; ++j) {
        const size_t idx = (size_t)map[j] * (M + 1) + n;
        const double mean = fma((double)acc.sum_hi[idx], 18446744073709551616.0, (double)acc.sum_lo[idx]) / R;
        const double m2 = acc.m2[idx];
        const double sd = R > 1.0 ? sqrt(m2 / (R - 1.0)) : NAN;
        double lo = mean, hi = mean;
        if (sd > 0.0) {
            const double sc = sd / sqrt(R);
            lo = mean + sc * tq.lo;
            hi = mean + sc * tq.hi;
        }
        const double scale = (normalize & 1) ? (double)N : 1.0;
        put(3 + 3 * j, mean / scale);
        put(4 + 3 * j, lo / scale);
        put(5 + 3 * j, hi / scale);
    }
}

void launch_micro_finalize(const NzMicroAccum &acc, uint32_t N, uint32_t M, int32_t spanning, double alpha,
                           int32_t normalize, double *out, cudaStream_t s) {
    const uint64_t threads = 2ull * ((uint64_t)M + 1);
    micro_finalize_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(acc, N, M, spanning, alpha, normalize,
                                                                          out);
}

__global__ void t_quantile_kernel(const double *q, const double *df, int32_t count, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = student_t_quantile(q[i], df[i]);
}

void launch_t_quantile(const double *q, const double *df, int32_t count, double *out, cudaStream_t s) {
    if (count > 0) t_quantile_kernel<<<(count + 127) / 128, 128, 0, s>>>(q, df, count, out);
}

}  // namespace nz
