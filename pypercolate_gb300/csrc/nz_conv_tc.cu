// Canonical convolution of record windows on the tensor cores: tcgen05.mma
// kind::tf32 with three split products per term ("3xTF32").
//
// For one statistic, a window of records Q[n][run] and the FP32 weights
// W[p][n] of each probability's band, every CTA computes
//   C[run][p] += sum_n Q[n][run] W[p][n]
// for 128 runs (M, one TMEM lane each) and 32 probabilities (N) over the
// rows its probabilities' bands share with the window (K), in chunks of 16
// rows.  The CTA's threads load the records of a chunk (thread t = run t,
// coalesced across the warp), convert them to FP32 and split each value into
// TF32 hi + lo parts (round to nearest: x = hi + lo to 2^-22 relative), do the
// same for the weights, and write both into shared memory in the canonical
// no-swizzle K-major layout; one thread then issues
//   D  = A_hi B_hi + A_hi B_lo + A_lo B_hi
// as 3 x 2 MMAs of 128 x 32 x 8 into an FP32 TMEM accumulator and commits
// them to an mbarrier.  While those run, the threads stage the next chunk;
// afterwards they read the chunk's 32 sums of their run out of TMEM and add
// them into FP32 TwoSum pairs (value + compensation: the sums over the whole
// band keep ~2^-44 relative accuracy without FP64, whose rate on this chip is
// 1/64 of FP32).  Shared memory and TMEM accumulators are double-buffered.
// m2 (the susceptibility, which needs ~5e-11 relative per run) is not done
// here: the launcher adds the compensated SIMT kernel of nz_canonical.cu.
//
// Reference: the products and sums of bond_canonical_statistics
// (percolate/hpc.py:443-515), sum_n B(M, n, p) Q_n per statistic.
#include <cstdint>
#include <type_traits>

#include "nz_common.cuh"
#include "nz_internal.cuh"
#include "nz_records.cuh"
#include "nz_tc.cuh"

namespace nz {
namespace {

constexpr int kTcRuns = 128;  // M: runs per CTA
constexpr int kTcP = 32;      // N: probabilities per CTA
// 16-row chunks: 165 registers and 41 KB of shared memory per CTA, against
// 231-255 and 82 KB with 32 (1216 vs 1234 ms per 100,000-run L = 256 step)
#ifndef NZ_TC_K
#define NZ_TC_K 16
#endif
constexpr int kTcK = NZ_TC_K;  // rows per chunk (16 or 32): kTcK / 8 MMAs of K = 8
static_assert(kTcK == 16 || kTcK == 32, "chunk of 16 or 32 rows");
// TMEM columns: for each of two periods in flight, a main accumulator (the
// hi x hi products) and a correction accumulator (hi x lo + lo x hi)
constexpr uint32_t kTcCols = 4 * kTcP;
// chunks accumulated in TMEM (FP32) before the threads drain them into their
// (sum, compensation) pairs.  The tensor cores' FP32 accumulation rounds
// toward zero, so its error grows with the accumulation steps between
// drains: with all three products in one accumulator, 8 chunks (48 steps)
// left every curve ~2e-6 relative low (the strength 1.7e-6 absolute at
// L = 256), one chunk (6 steps) within 2.3e-7.  With the corrections (~2^-11
// of the main terms) in their own accumulator, the main one takes 2 steps
// per chunk: 4 chunks are 8 steps, and a drain every 4 chunks costs the
// threads a quarter of a drain every chunk
#ifndef NZ_TC_DRAIN
#define NZ_TC_DRAIN 4
#endif
constexpr uint32_t kTcDrain = NZ_TC_DRAIN;
constexpr uint32_t kCoreBytes = 128;                  // core matrix: 8 rows x 16 bytes
constexpr uint32_t kSbo = (kTcK / 4) * kCoreBytes;    // between 8-row groups

struct TcShared {
    float a[2][2][kTcRuns * kTcK];  // [stage][hi, lo] records
    float b[2][2][kTcP * kTcK];     // [stage][hi, lo] weights
    uint64_t mbar[2];               // MMAs of the chunk in each stage done
    uint32_t tmem;                  // TMEM base address
    uint32_t lo[kTcP], len[kTcP];   // FP32 bands of the CTA's probabilities
    uint32_t range[2];
};

// Instruction descriptor of tcgen05.mma kind::tf32: D FP32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcP >> 3) << 17) |
                            ((uint32_t)(kTcRuns >> 4) << 24);

using tc::fence_async_smem;
using tc::mbar_wait;
using tc::mma_commit;
using tc::smem_u32;
using tc::tmem_ld32;
__device__ __forceinline__ void tc_fence_before() { tc::fence_before(); }
__device__ __forceinline__ void tc_fence_after() { tc::fence_after(); }

// descriptor of one operand stage: core matrices adjacent in K 128 bytes
// apart, 8-row groups kSbo apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) { return tc::smem_desc(addr, kCoreBytes, kSbo); }

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// x = hi + lo with both parts TF32 (10 explicit mantissa bits each)
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    hi = to_tf32(x);
    lo = to_tf32(__fsub_rn(x, hi));
}

// s + x = t + err exactly, err collected in c.  The chunk sums and the
// running sum are >= 0, so Dekker's Fast2Sum on the operands ordered by size
// (max / min) is exact: 3 additions instead of Knuth's TwoSum's 6.
__device__ __forceinline__ void two_sum_add(float &s, float &c, float x) {
    const float a = fmaxf(s, x), b = fminf(s, x);
    const float t = __fadd_rn(a, b);
    c = __fadd_rn(c, __fsub_rn(b, __fsub_rn(t, a)));
    s = t;
}

// Raw record words of one chunk's rows: the plane statistic S reads (m4_lo
// for S = 6, whose m4_hi words go to `hi`; S = 8 and 9: m0 and m2 of narrow
// records, uint16 and uint32).
template <int S>
using raw_word = typename std::conditional<
    S == 8, uint16_t,
    typename std::conditional<(S >= 4 && S != 9), uint64_t, uint32_t>::type>::type;

template <int S>
__device__ __forceinline__ const raw_word<S> *raw_plane(const NzRecords &rec) {
    if constexpr (S == 0 || S == 1 || S == 3) return rec.max_span;
    else if constexpr (S == 2) return rec.m0;
    else if constexpr (S == 4) return rec.m2;
    else if constexpr (S == 5) return rec.m3;
    else if constexpr (S == 8) return reinterpret_cast<const uint16_t *>(rec.m0);
    else if constexpr (S == 9) return reinterpret_cast<const uint32_t *>(rec.m2);
    else return rec.m4_lo;
}

// Loads of chunk rows [k0, k0 + 32) relative to the CTA's first row, each
// clamped to the last row so that every load is in bounds and unconditional
// (all 32 in flight at once); rows past the end are zeroed on conversion.
template <int S>
__device__ __forceinline__ void load_chunk(const NzRecords &rec, size_t base, size_t stride, uint32_t k0,
                                           uint32_t last, raw_word<S> (&raw)[kTcK],
                                           uint64_t (&hi)[S == 6 ? kTcK : 1]) {
    const raw_word<S> *plane = raw_plane<S>(rec);
#pragma unroll
    for (int k = 0; k < kTcK; ++k) {
        const size_t off = base + (size_t)min(k0 + (uint32_t)k, last) * stride;
        raw[k] = plane[off];
        if constexpr (S == 6) hi[k] = rec.m4_hi[off];
    }
}

template <int S>
__device__ __forceinline__ float raw_value(raw_word<S> w, uint64_t hi, uint32_t held) {
    if constexpr (S == 0) return (w & kSpanBit) ? 1.0f : 0.0f;
    else if constexpr (S == 1) return (float)(w & ~kSpanBit);
    else if constexpr (S == 2 || S == 8 || S == 9) return (float)w;
    else if constexpr (S == 3) return (float)(held - (w & ~kSpanBit));
    else if constexpr (S == 6) return fmaf((float)hi, 18446744073709551616.0f, u64_to_f32(w));
    else return u64_to_f32(w);
}

// One CTA's tile for statistic S (7 = m4 without its high-word plane).
template <int S, bool SITE>
__device__ __forceinline__ void conv_tc_tile(const ConvParams &p, TcShared &sh, int p0, uint32_t nlo, uint32_t nhi) {
    const int t = threadIdx.x, warp = t >> 5;
    const int r = blockIdx.x * kTcRuns + t;
    const bool live = r < p.n_runs;
    if (warp == 0) {
        tc::tmem_alloc(smem_u32(&sh.tmem), kTcCols);
    }
    if (t == 0) {
        tc::mbar_init(smem_u32(&sh.mbar[0]));
        tc::mbar_init(smem_u32(&sh.mbar[1]));
        tc::mbar_init_fence();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem;
    const uint32_t rows = nhi - nlo, last = rows - 1;
    const uint32_t nchunks = (rows + kTcK - 1) / kTcK;
    const size_t stride = p.rec.run_stride;
    const size_t base = (size_t)(nlo - p.n_begin) * stride + (size_t)(live ? r : 0);
    // thread t's row of A: 8-row group t / 8, row t % 8 of each core matrix
    const int a_off = (t >> 3) * (int)(kSbo / 4) + (t & 7) * 4;
    // weights staged by thread t: probability j = t / 4, rows (t % 4) kTcK / 4
    // .. + kTcK / 4 - 1
    constexpr int kWRows = kTcK / 4;
    const int wj = t >> 2, wk = (t & 3) * kWRows;
    const int b_off = (wj >> 3) * (int)(kSbo / 4) + (wj & 7) * 4 + (wk / 4) * 32;
    const uint32_t wlo = sh.lo[wj], wlen = sh.len[wj];
    const float *wrow = p.w32 + (size_t)(p0 + wj) * p.cap;
    float acc_s[kTcP], acc_c[kTcP];
#pragma unroll
    for (int j = 0; j < kTcP; ++j) acc_s[j] = acc_c[j] = 0.0f;
    // a period's sums of this thread's run (TMEM lane t): the main terms
    // into the (sum, compensation) pairs, the corrections into the
    // compensation
    auto drain = [&](uint32_t q) {
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16) + q * 2 * kTcP;
        float v[kTcP];
        tmem_ld32(lane_base, v);
#pragma unroll
        for (int j = 0; j < kTcP; ++j) two_sum_add(acc_s[j], acc_c[j], v[j]);
        tmem_ld32(lane_base + kTcP, v);
#pragma unroll
        for (int j = 0; j < kTcP; ++j) acc_c[j] = __fadd_rn(acc_c[j], v[j]);
    };
    raw_word<S> raw[kTcK];
    uint64_t raw_hi[S == 6 ? kTcK : 1];
    load_chunk<S>(p.rec, base, stride, 0, last, raw, raw_hi);
    bool bad = false;
    uint32_t ch = 0;
    for (; ch < nchunks; ++ch) {
        const int st = ch & 1;
        const uint32_t c0 = nlo + ch * kTcK;
        {
            float v[kTcK];
#pragma unroll
            for (int k = 0; k < kTcK; ++k) {
                const uint32_t n = c0 + k;
                const uint32_t held = (S == 3 && SITE) ? n : p.N;
                v[k] = (live && n < nhi) ? raw_value<S>(raw[k], S == 6 ? raw_hi[k] : 0, held) : 0.0f;
            }
            // the next chunk's loads fly while this one is staged, multiplied
            // and drained
            if (ch + 1 < nchunks) load_chunk<S>(p.rec, base, stride, (ch + 1) * kTcK, last, raw, raw_hi);
            float *ah = sh.a[st][0] + a_off, *al = sh.a[st][1] + a_off;
#pragma unroll
            for (int kb = 0; kb < kTcK / 4; ++kb) {
                float4 h, l;
                split_tf32(v[4 * kb + 0], h.x, l.x);
                split_tf32(v[4 * kb + 1], h.y, l.y);
                split_tf32(v[4 * kb + 2], h.z, l.z);
                split_tf32(v[4 * kb + 3], h.w, l.w);
                *reinterpret_cast<float4 *>(ah + kb * 32) = h;
                *reinterpret_cast<float4 *>(al + kb * 32) = l;
            }
        }
        {
            float w[kWRows];
#pragma unroll
            for (int q = 0; q < kWRows; ++q) {
                const uint32_t n = c0 + wk + q;
                w[q] = (n < nhi && n - wlo < wlen) ? wrow[n - wlo] : 0.0f;
            }
            float *bh = sh.b[st][0] + b_off, *bl = sh.b[st][1] + b_off;
#pragma unroll
            for (int h2 = 0; h2 < kWRows / 4; ++h2) {
                float4 h, l;
                split_tf32(w[4 * h2 + 0], h.x, l.x);
                split_tf32(w[4 * h2 + 1], h.y, l.y);
                split_tf32(w[4 * h2 + 2], h.z, l.z);
                split_tf32(w[4 * h2 + 3], h.w, l.w);
                *reinterpret_cast<float4 *>(bh + h2 * 32) = h;
                *reinterpret_cast<float4 *>(bl + h2 * 32) = l;
            }
        }
        fence_async_smem();
        tc_fence_before();
        if (__syncthreads_or(bad)) break;  // a wait below gave up
        if (t == 0) {
            tc_fence_after();
            // accumulators of this chunk's period of kTcDrain chunks; a
            // period's first chunk overwrites them
            const uint32_t d = tmem + (uint32_t)(((ch / kTcDrain) & 1) * 2 * kTcP), dc = d + kTcP;
            const bool fresh = ch % kTcDrain == 0;
            const uint32_t ah = smem_u32(sh.a[st][0]), al = smem_u32(sh.a[st][1]);
            const uint32_t bh = smem_u32(sh.b[st][0]), bl = smem_u32(sh.b[st][1]);
#pragma unroll
            for (int ks = 0; ks < kTcK / 8; ++ks) {
                const uint32_t o = (uint32_t)ks * 2 * kCoreBytes;  // K = 8: two core matrices
                const uint32_t acc = (ks > 0 || !fresh) ? 1u : 0u;
                mma_tf32(d, smem_desc(ah + o), smem_desc(bh + o), acc);
                mma_tf32(dc, smem_desc(ah + o), smem_desc(bl + o), acc);
                if (S != 0) mma_tf32(dc, smem_desc(al + o), smem_desc(bh + o), 1u);  // spanning: lo = 0
            }
            mma_commit(smem_u32(&sh.mbar[st]));
        }
        if (ch > 0) {
            const uint32_t pc = ch - 1;
            // chunk ch - 1's MMAs done: its shared-memory stage is free, and
            // if it closed a period, that period's accumulator is complete
            // (warp-uniform: tcgen05.ld is executed by the whole warp)
            bad = !__all_sync(0xffffffffu, mbar_wait(smem_u32(&sh.mbar[pc & 1]), (pc >> 1) & 1));
            if (!bad && pc % kTcDrain == kTcDrain - 1) {
                tc_fence_after();
                drain((pc / kTcDrain) & 1);
            }
        }
    }
    // the last chunk issued (all of them unless a wait gave up)
    const uint32_t issued = ch;
    if (issued > 0) {
        const uint32_t pc = issued - 1;
        const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&sh.mbar[pc & 1]), (pc >> 1) & 1));
        // the last period: the loop drains a period when it waits for the
        // chunk after it, which the last one does not have
        if (ok && !__any_sync(0xffffffffu, bad)) {
            tc_fence_after();
            drain((pc / kTcDrain) & 1);
        } else if (!ok) {
            bad = true;
        }
    }
    tc_fence_before();
    const bool any_bad = __syncthreads_or(bad);
    if (warp == 0) {
        tc_fence_after();
        tc::tmem_dealloc(tmem, kTcCols);
    }
    if (any_bad) {
        if (t == 0 && p.errors) atomicAdd(p.errors, 1u);
        return;
    }
    if (live) {
        constexpr int out = S == 7 ? 6 : (S == 8 ? 2 : (S == 9 ? 4 : S));
        double *o = p.acc + (size_t)r * p.P * 7;
#pragma unroll
        for (int j = 0; j < kTcP; ++j)
            if (p0 + j < p.P) o[(size_t)(p0 + j) * 7 + out] += (double)acc_s[j] + (double)acc_c[j];
    }
}

// grid (run tiles, probability tiles of 32, statistics): HI = false: the
// statistics 0, 1, 2, 3, 5, 6, or 0, 1, 2, 3, 5 when the records carry m4
// high words; HI = true: m4 with its high words alone (its wider loads would
// otherwise set the register count of every statistic's code).  m2 (4) runs
// on the compensated SIMT kernel.
template <bool SITE, bool HI>
__global__ void __launch_bounds__(kTcRuns) conv_tc_kernel(ConvParams p) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    TcShared &sh = *reinterpret_cast<TcShared *>(tc_smem);
    // statistic of this z: m2 (4) runs on the compensated SIMT kernel
    // (conv_m2_comp_kernel) instead
    constexpr int kStat[6] = {0, 1, 2, 3, 5, 6};
    const int z = kStat[blockIdx.z];
    if (!HI && z == 0 && !p.spanning) return;
    const int p0 = blockIdx.y * kTcP;
    if (threadIdx.x < kTcP) {
        const int pi = p0 + threadIdx.x;
        sh.lo[threadIdx.x] = pi < p.P ? p.band_lo[pi] : 0u;
        sh.len[threadIdx.x] = pi < p.P ? p.band_len[pi] : 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0xffffffffu, b = 0;
        for (int j = 0; j < kTcP; ++j)
            if (sh.len[j]) { a = min(a, sh.lo[j]); b = max(b, sh.lo[j] + sh.len[j]); }
        sh.range[0] = max(a, p.n_begin);
        sh.range[1] = min(b, p.n_end);
    }
    __syncthreads();
    const uint32_t nlo = sh.range[0], nhi = sh.range[1];
    if (nlo >= nhi) return;
    if (HI) {
        conv_tc_tile<6, SITE>(p, sh, p0, nlo, nhi);
        return;
    }
    switch (z) {
        case 0: conv_tc_tile<0, SITE>(p, sh, p0, nlo, nhi); break;
        case 1: conv_tc_tile<1, SITE>(p, sh, p0, nlo, nhi); break;
        case 2:
            if (p.rec.narrow) conv_tc_tile<8, SITE>(p, sh, p0, nlo, nhi);
            else conv_tc_tile<2, SITE>(p, sh, p0, nlo, nhi);
            break;
        case 3: conv_tc_tile<3, SITE>(p, sh, p0, nlo, nhi); break;
        case 5: conv_tc_tile<5, SITE>(p, sh, p0, nlo, nhi); break;
        default: conv_tc_tile<7, SITE>(p, sh, p0, nlo, nhi); break;
    }
}

template <bool SITE, bool HI>
cudaError_t launch_tc_k(const ConvParams &p, unsigned stats, cudaStream_t s) {
    // above 48 KB of dynamic shared memory (32-row chunks) the launch needs
    // the attribute, which belongs to the function in the current device's
    // context: set it before every such launch
    if constexpr (sizeof(TcShared) > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(conv_tc_kernel<SITE, HI>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcShared));
        if (e != cudaSuccess) return e;
    }
    dim3 grid((p.n_runs + kTcRuns - 1) / kTcRuns, (p.P + kTcP - 1) / kTcP, stats);
    conv_tc_kernel<SITE, HI><<<grid, kTcRuns, sizeof(TcShared), s>>>(p);
    return cudaGetLastError();
}

template <bool SITE>
cudaError_t launch_tc(const ConvParams &p, cudaStream_t s) {
    if (!p.rec.m4_hi) return launch_tc_k<SITE, false>(p, 6, s);
    const cudaError_t e = launch_tc_k<SITE, false>(p, 5, s);
    return e != cudaSuccess ? e : launch_tc_k<SITE, true>(p, 1, s);
}

}  // namespace

bool conv_tc_grid_fits(int32_t n_runs, int32_t P) {
    return n_runs > 0 && P > 0 && (P + kTcP - 1) / kTcP <= 65535;
}

int launch_conv_window_tc(const ConvParams &p, cudaStream_t s) {
    if (p.n_runs <= 0 || p.P <= 0) return 0;
    const cudaError_t e = p.rec.site ? launch_tc<true>(p, s) : launch_tc<false>(p, s);
    if (e != cudaSuccess) return -1;
    // m2 needs ~5e-11 relative per run (the susceptibility curve within 1e-6
    // absolute of FP64 at L = 1024), beyond FP32 tensor-core accumulation:
    // it runs on the compensated SIMT kernel
    launch_conv_m2_comp(p, s);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace nz
