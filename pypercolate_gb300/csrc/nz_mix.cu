// nz_mix.cu -- batched uneven ensembles in one persistent launch.
//
// n_runs independent runs whose substrate is drawn per run: with probability
// chain_share a spanning_1d_chain(l), l log-uniform in [chain_min, chain_max],
// otherwise a spanning_2d_grid(L), L log-uniform in [grid_min, grid_max]
// (percolate/percolate.py:899-965).  The draw and the bond permutation of
// run r both come from Philox-4x32-10 keyed by `key` at counter r.
//
// Pipeline (all on the caller's stream, no host synchronisation):
//   1. mix_class_kernel   : class of every run (threshold tables, no libm),
//                           histogram of classes;
//   2. mix_offsets_kernel : classes ordered by node words S descending
//                           (longest-first scheduling) -> segment offsets;
//                           S = l for a chain, grid_slots(L) >= L^2 for a
//                           grid, whose sites sit in 4 x 2 blocks per sector;
//   3. mix_scatter_kernel : run ids bucketed into a queue sorted by S desc;
//   4. mix_slots_kernel   : node-slot offsets of the T persistent threads;
//   5. mix_uf_kernel      : persistent union-find.  Thread t runs queue[t]
//      first (its node slot is sized for it), then claims further items with
//      an atomic counter; S only decreases along the queue, so every later
//      item fits the slot.  Small items (S words <= smem slot) run in shared
//      memory.  At F evenly spaced occupation checkpoints
//      n_j = floor(j M / (F - 1)) each run either writes its exact
//      statistics (records) or, with the fused reduction, adds them and
//      their squares into its class's cell j itself (integer atomics of
//      32-bit limbs: exact, and independent of the order the runs finish in);
//   6. mix_reduce_kernel  : per (class, checkpoint) exact integer sums of x
//      and x^2 (up to 192 bits) over the class's records -> mean and M2
//      (percolate/percolate.py:450-705 semantics at those n); or
//      mix_finalize_kernel: the same sums and M2 from the fused cells.
//   Both reductions give identical results; which is faster depends on the
//   mix of lattices (many runs per lattice favour the fused one).
#include <cmath>
#include <cstdint>

#include "nz_common.cuh"
#include "nz_internal.cuh"

namespace nz {

typedef unsigned __int128 u128;
constexpr uint32_t kSizeTag = 0x53495A45u;  // "SIZE"


__device__ __forceinline__ uint32_t class_of_run(const MixDev &m, uint64_t key, uint64_t r) {
    uint32_t c[4] = {(uint32_t)r, (uint32_t)(r >> 32), 0u, kSizeTag};
    philox4x32_10(c, (uint32_t)key, (uint32_t)(key >> 32));
    const bool chain = c[0] < m.chain_share;
    const uint32_t *thr = chain ? m.thr_chain : m.thr_grid;
    const uint32_t n = chain ? m.n_chain : m.n_grid;
    // largest i with thr[i] <= u (thr[0] == 0)
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (thr[mid] <= c[1]) lo = mid; else hi = mid;
    }
    return chain ? m.n_grid + lo : lo;
}

__device__ __forceinline__ void class_graph(const MixDev &m, uint32_t cls, uint32_t &kind, uint32_t &L,
                                            uint32_t &N, uint32_t &M) {
    if (cls < m.n_grid) {
        kind = NZ_GRAPH_GRID2D; L = m.grid_min + cls; N = L * L; M = 2u * L * (L - 1u);
    } else {
        kind = NZ_GRAPH_CHAIN1D; L = m.chain_min + (cls - m.n_grid); N = L; M = L - 1u;
    }
}

// node words a run of class cls needs: grid_slots(L) (the tiled layout) or l
__device__ __forceinline__ uint32_t class_slots(const MixDev &m, uint32_t cls) {
    return cls < m.n_grid ? grid_slots(m.grid_min + cls) : m.chain_min + (cls - m.n_grid);
}

__global__ void mix_class_kernel(MixDev m, uint32_t *cls, uint32_t *counts) {
    const uint64_t key = *m.key_ptr;
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m.n_runs; r += gridDim.x * blockDim.x) {
        const uint32_t c = class_of_run(m, key, (uint64_t)r);
        cls[r] = c;
        atomicAdd(&counts[c], 1u);
    }
}

// Position of every class in the order "node words S descending, grids
// before chains on equal S" (grid S = grid_slots(L) and chain S = l are
// non-decreasing in the length).  Ordering by the words a run needs -- not
// by M -- is what makes the persistent threads' node slots safe: every item
// after position t needs at most the words of item t.
__global__ void mix_order_kernel(MixDev m, uint32_t *order) {
    const uint32_t n_classes = m.n_grid + m.n_chain;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n_classes; c += gridDim.x * blockDim.x) {
        uint32_t rank;
        if (c < m.n_grid) {
            const uint64_t Nc = grid_slots(m.grid_min + c);
            // chains with more words: l >= Nc + 1
            const uint64_t lo = Nc + 1u;
            const uint32_t more = lo > m.chain_max ? 0u
                                : (uint32_t)(m.chain_max - (lo > m.chain_min ? lo : (uint64_t)m.chain_min) + 1u);
            rank = (m.n_grid - 1u - c) + more;
        } else {
            const uint32_t k = c - m.n_grid;
            const uint64_t Nk = (uint64_t)m.chain_min + k;
            // grids with at least as many words: smallest L in range with
            // grid_slots(L) >= Nk
            uint32_t a = m.grid_min, b = m.grid_max + 1u;
            while (a < b) {
                const uint32_t mid = (a + b) >> 1;
                if ((uint64_t)grid_slots(mid) >= Nk) b = mid; else a = mid + 1u;
            }
            rank = (m.n_chain - 1u - k) + (m.grid_max + 1u - a);
        }
        order[rank] = c;
    }
}

__global__ void mix_head_kernel(uint32_t *head, uint32_t v) { *head = v; }

// Single block: exclusive scan of counts taken in the order `order` (classes
// by N descending) -> offsets[c]; also the cursor copy used by the scatter.
__global__ void mix_offsets_kernel(const uint32_t *counts, const uint32_t *order, uint32_t n_classes,
                                   uint32_t *offsets, uint32_t *cursor) {
    __shared__ uint32_t s[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n_classes; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < n_classes ? counts[order[i]] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const uint32_t y = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0u;
            __syncthreads();
            s[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < n_classes) {
            const uint32_t ex = carry + s[threadIdx.x] - v;
            offsets[order[i]] = ex;
            cursor[order[i]] = ex;
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
    }
}

__global__ void mix_scatter_kernel(int32_t n_runs, const uint32_t *cls, uint32_t *cursor, uint32_t *queue) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_runs; r += gridDim.x * blockDim.x)
        queue[atomicAdd(&cursor[cls[r]], 1u)] = (uint32_t)r;
}

// Node-slot offsets (in words) of the T persistent threads: exclusive scan of
// the words of queue[t]'s class for t < T (single block).
__global__ void mix_slots_kernel(MixDev m, const uint32_t *queue, const uint32_t *cls, int32_t T,
                                 uint64_t *slot_off) {
    __shared__ uint64_t s[1024];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int32_t base = 0; base < T; base += 1024) {
        const int32_t t = base + threadIdx.x;
        uint64_t v = 0;
        if (t < T && t < m.n_runs) v = class_slots(m, cls[queue[t]]);
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const uint64_t y = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0ull;
            __syncthreads();
            s[threadIdx.x] += y;
            __syncthreads();
        }
        if (t < T) slot_off[t] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
        if (threadIdx.x == 0 && base + 1024 >= T) slot_off[T] = carry;
    }
}


__device__ __forceinline__ void add128m(uint64_t &lo, uint64_t &hi, uint64_t blo, uint64_t bhi) {
    const uint64_t nlo = lo + blo;
    hi += bhi + (nlo < lo ? 1ull : 0ull);
    lo = nlo;
}

// ------------------------------------------------------- fused reduction
// Cell words.  Each word sums one 32-bit limb over the class's runs: at most
// NZ_MAX_RUNS = 2^24 limbs < 2^32, so no word can overflow.  With N <= 2^21:
// max, m0 < 2^21, m2 < 2^42, m3 < 2^63, m4 < 2^84.
//   0 runs with a spanning cluster
//   sums of x:   1 max, 2 m0, 3-4 m2, 5-6 m3, 7-9 m4
//   sums of x^2: 10-11 max, 12-13 m0, 14-16 m2, 17-20 m3, 21-26 m4
// (m1 = N - max follows from the max sums.)
constexpr int kCellSpan = 0, kSxMax = 1, kSxM0 = 2, kSxM2 = 3, kSxM3 = 5, kSxM4 = 7;
constexpr int kSqMax = 10, kSqM0 = 12, kSqM2 = 14, kSqM3 = 17, kSqM4 = 21;
static_assert(kSqM4 + 6 == kMixCellWords, "cell layout");

// Adds 32-bit limbs into the words of one cell.  When every active lane of
// the warp adds into the same cell (runs of one lattice reach their
// checkpoints together), the lanes' limbs are summed first (redux.sync on
// 16-bit halves, so 32 lanes' sums fit 32 bits) and one lane issues the
// atomic: 27 atomics per warp and checkpoint instead of up to 27 x 32.
struct CellAdder {
    uint64_t *cell;
    unsigned mask;
    bool warp, leader;
    __device__ __forceinline__ explicit CellAdder(uint64_t *c) : cell(c) {
        mask = __activemask();
        warp = __match_any_sync(mask, (unsigned long long)(uintptr_t)c) == mask;
        leader = (threadIdx.x & 31u) == (unsigned)(__ffs(mask) - 1);
    }
    __device__ __forceinline__ void limb(int k, uint32_t v) const {
        if (warp) {
            const uint32_t lo = __reduce_add_sync(mask, v & 0xffffu);
            const uint32_t hi = __reduce_add_sync(mask, v >> 16);
            const uint64_t sum = (uint64_t)lo + ((uint64_t)hi << 16);
            if (leader && sum) atomicAdd(reinterpret_cast<unsigned long long *>(cell + k), (unsigned long long)sum);
        } else if (v) {
            atomicAdd(reinterpret_cast<unsigned long long *>(cell + k), (unsigned long long)v);
        }
    }
    __device__ __forceinline__ void u64(int k, uint64_t v) const {
        limb(k, (uint32_t)v);
        limb(k + 1, (uint32_t)(v >> 32));
    }
    template <int LIMBS>
    __device__ __forceinline__ void wide(int k, u128 v) const {
#pragma unroll
        for (int i = 0; i < LIMBS; ++i) limb(k + i, (uint32_t)(v >> (32 * i)));
    }
};

// One run's statistics at one checkpoint into its class's cell.
__device__ __forceinline__ void mix_checkpoint(uint64_t *cell, uint32_t mx, bool span, uint32_t m0, uint64_t m2,
                                               uint64_t m3, uint64_t m4lo, uint32_t m4hi) {
    const CellAdder a(cell);
    a.limb(kCellSpan, span ? 1u : 0u);
    a.limb(kSxMax, mx);
    a.limb(kSxM0, m0);
    a.u64(kSxM2, m2);
    a.u64(kSxM3, m3);
    a.u64(kSxM4, m4lo);
    a.limb(kSxM4 + 2, m4hi);
    a.u64(kSqMax, (uint64_t)mx * mx);
    a.u64(kSqM0, (uint64_t)m0 * m0);
    a.wide<3>(kSqM2, (u128)m2 * m2);
    a.wide<4>(kSqM3, (u128)m3 * m3);
    // m4^2 = lo^2 + 2 lo hi 2^64 + hi^2 2^128 (< 2^168) as three 64-bit words
    const u128 ll = (u128)m4lo * m4lo;
    const u128 mid = ((u128)m4lo * m4hi) << 1;  // < 2^85
    const u128 t = (ll >> 64) + (uint64_t)mid;  // < 2^65
    a.u64(kSqM4, (uint64_t)ll);
    a.u64(kSqM4 + 2, (uint64_t)t);
    a.u64(kSqM4 + 4, (uint64_t)(t >> 64) + (uint64_t)(mid >> 64) + (uint64_t)m4hi * m4hi);
}

// Where a run's checkpoints go: its records (queue position `pos`, F
// entries) or its class's F cells.
template <bool FUSED>
struct MixSink {
    MixRec rec;
    size_t rec_base;
    uint64_t *cells;
    __device__ __forceinline__ void put(uint32_t j, uint32_t mx, bool span, uint32_t m0, uint64_t m2, uint64_t m3,
                                        uint64_t m4lo, uint32_t m4hi) const {
        if (FUSED) {
            mix_checkpoint(cells + (size_t)j * kMixCellWords, mx, span, m0, m2, m3, m4lo, m4hi);
        } else {
            const size_t off = rec_base + j;
            rec.max_span[off] = mx | (span ? kSpanBit : 0u);
            rec.m0[off] = m0;
            rec.m2[off] = m2;
            rec.m3[off] = m3;
            rec.m4_lo[off] = m4lo;
            rec.m4_hi[off] = m4hi;
        }
    }
};

// One complete run in `node` (global or shared), delivering its checkpoints.
template <int KIND, bool FUSED>
__device__ void mix_run(const MixDev &m, uint64_t key, uint32_t run, uint32_t L, uint32_t N, uint32_t M, uint32_t *node,
                        const MixSink<FUSED> &out) {
    GraphDev g;
    g.kind = KIND; g.site = 0; g.wrap = 0; g.L = L; g.N = N; g.M = M;
    g.tile_cols = KIND == NZ_GRAPH_GRID2D ? (L + 3u) >> 2 : 0u;  // grids in the tiled layout
    g.slots = KIND == NZ_GRAPH_GRID2D ? grid_slots(L) : N;
    g.two_l_m1 = KIND == NZ_GRAPH_GRID2D ? 2u * L - 1u : 1u;
    g.row_edges = KIND == NZ_GRAPH_GRID2D ? (L - 1u) * g.two_l_m1 : 0u;
    g.inv_two_l_m1 = 1.0f / (float)g.two_l_m1;
    g.eu = g.ev = nullptr; g.side = nullptr;
    for (uint32_t i = 0; i < N; ++i) node[node_slot<KIND>(g, i)] = make_root(1u, node_sides<KIND>(g, i));
    FeistelPerm fp;
    fp.init(key, run, M);
    uint64_t t2 = N, t3 = N, t4lo = N, t4hi = 0;
    uint32_t t0 = N, mx = 1;
    uint64_t mx2 = 1, mx3 = 1, mx4lo = 1, mx4hi = 0;
    bool span = false;
    const uint32_t Fm1 = (uint32_t)m.F - 1u;
    uint32_t j = 0;
    // checkpoint j is the row n_j = floor(j * M / (F - 1))
    auto next_row = [&](uint32_t jj) -> uint32_t {
        return (uint32_t)(((uint64_t)jj * M) / Fm1);
    };
    uint32_t target = next_row(0);
    for (uint32_t n = 0; n <= M; ++n) {
        if (n > 0) {
            const uint32_t e = fp.at(n - 1u);
            uint32_t u, v;
            decode_edge_slots<KIND>(g, e, u, v);
            uint32_t xu = u, xv = v;
            uint32_t wu = node[xu], wv = node[xv];
            for (int hops = 0; !(is_root(wu) && is_root(wv)); ++hops) {
                if (hops >= 64) { wu = wv = make_root(0, 0); xu = xv; break; }
                if (!is_root(wu)) {
                    const uint32_t nu = node[wu];
                    if (!is_root(nu)) node[xu] = nu;
                    xu = wu; wu = nu;
                }
                if (!is_root(wv)) {
                    const uint32_t nv = node[wv];
                    if (!is_root(nv)) node[xv] = nv;
                    xv = wv; wv = nv;
                }
            }
            if (xu != xv) {
                const uint32_t a = root_size(wu), b = root_size(wv);
                const uint32_t sides = root_sides(wu) | root_sides(wv);
                const uint32_t s = a + b;
                uint32_t big = xu, small = xv;
                if (a < b) { big = xv; small = xu; }
                node[small] = big;
                node[big] = make_root(s, sides);
                t0 -= 1u;
                const uint64_t ab = (uint64_t)a * b;
                t2 += 2ull * ab;
                t3 += 3ull * ab * s;
                const uint64_t q = 4ull * a * a + 6ull * ab + 4ull * b * b;
                add128m(t4lo, t4hi, ab * q, __umul64hi(ab, q));
                if (s > mx) {
                    mx = s; mx2 = (uint64_t)mx * mx; mx3 = mx2 * mx;
                    mx4lo = mx3 * mx; mx4hi = __umul64hi(mx3, (uint64_t)mx);
                }
                if (sides == 3u) span = true;
            }
        }
        if (n == target) {
            const uint64_t m4lo = t4lo - mx4lo;
            const uint32_t m4hi = (uint32_t)(t4hi - mx4hi - (t4lo < mx4lo ? 1ull : 0ull));
            // several checkpoints share row n when F - 1 > M
            while (j < (uint32_t)m.F && n == target) {
                out.put(j, mx, span, t0 - 1u, t2 - mx2, t3 - mx3, m4lo, m4hi);
                ++j;
                if (j < (uint32_t)m.F) target = next_row(j);
            }
        }
    }
}

// (256, 3): at most 85 registers (80 used by either reduction), so that 6
// CTAs of 128 threads stay resident per SM
template <bool FUSED>
__global__ void __launch_bounds__(256, 3) mix_uf_kernel(MixDev m, const uint32_t *queue, const uint32_t *cls,
                                                        int32_t T, const uint64_t *slot_off, uint32_t *nodes,
                                                        uint32_t smem_words, uint32_t *head, MixRec rec,
                                                        uint64_t *cells, uint32_t *errors) {
    extern __shared__ uint32_t s_nodes[];
    const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T || t >= m.n_runs) return;
    const uint64_t key = *m.key_ptr;
    uint32_t *gslot = nodes + slot_off[t];
    const uint64_t slot_words = slot_off[t + 1] - slot_off[t];
    uint32_t *sslot = smem_words ? s_nodes + (size_t)threadIdx.x * smem_words : nullptr;
    uint32_t pos = (uint32_t)t;
    while (pos < (uint32_t)m.n_runs) {
        const uint32_t run = queue[pos];
        uint32_t kind, L, N, M;
        class_graph(m, cls[run], kind, L, N, M);
        const uint32_t words = class_slots(m, cls[run]);
        uint32_t *node = (sslot && words <= smem_words) ? sslot : gslot;
        if (node == gslot && words > slot_words) {  // cannot happen with the words-descending queue
            atomicAdd(errors, 1u);
            pos = atomicAdd(head, 1u);
            continue;
        }
        MixSink<FUSED> out;
        out.rec = rec;
        out.rec_base = (size_t)pos * (uint32_t)m.F;
        out.cells = cells + (size_t)cls[run] * (uint32_t)m.F * kMixCellWords;
        if (kind == NZ_GRAPH_GRID2D) mix_run<NZ_GRAPH_GRID2D, FUSED>(m, key, run, L, N, M, node, out);
        else mix_run<NZ_GRAPH_CHAIN1D, FUSED>(m, key, run, L, N, M, node, out);
        pos = atomicAdd(head, 1u);
    }
}

// ---------------------------------------------------------------- reduction
// Unsigned 256-bit helpers (4 little-endian 64-bit limbs).
struct U256 { uint64_t w[4]; };

__device__ __forceinline__ void u256_add(U256 &a, const U256 &b) {
    uint64_t c = 0;
    for (int i = 0; i < 4; ++i) {
        const uint64_t s = a.w[i] + b.w[i];
        const uint64_t c1 = s < a.w[i];
        const uint64_t s2 = s + c;
        const uint64_t c2 = s2 < s;
        a.w[i] = s2;
        c = c1 | c2;
    }
}
__device__ __forceinline__ U256 u256_from_u128(u128 x) {
    U256 r = {{(uint64_t)x, (uint64_t)(x >> 64), 0, 0}};
    return r;
}
// a (< 2^128) squared
__device__ __forceinline__ U256 u128_sq(u128 a) {
    const uint64_t lo = (uint64_t)a, hi = (uint64_t)(a >> 64);
    const u128 ll = (u128)lo * lo, lh = (u128)lo * hi, hh = (u128)hi * hi;
    U256 r = u256_from_u128(ll);
    U256 mid = {{0, (uint64_t)lh, (uint64_t)(lh >> 64), 0}};
    u256_add(r, mid);
    u256_add(r, mid);
    U256 top = {{0, 0, (uint64_t)hh, (uint64_t)(hh >> 64)}};
    u256_add(r, top);
    return r;
}
// a * k for k < 2^64
__device__ __forceinline__ U256 u256_mul64(const U256 &a, uint64_t k) {
    U256 r = {{0, 0, 0, 0}};
    u128 carry = 0;
    for (int i = 0; i < 4; ++i) {
        const u128 p = (u128)a.w[i] * k + carry;
        r.w[i] = (uint64_t)p;
        carry = p >> 64;
    }
    return r;
}
// a - b (a >= b)
__device__ __forceinline__ U256 u256_sub(const U256 &a, const U256 &b) {
    U256 r;
    uint64_t borrow = 0;
    for (int i = 0; i < 4; ++i) {
        const uint64_t d = a.w[i] - b.w[i];
        const uint64_t b1 = a.w[i] < b.w[i];
        const uint64_t d2 = d - borrow;
        const uint64_t b2 = d < borrow;
        r.w[i] = d2;
        borrow = b1 | b2;
    }
    return r;
}
__device__ __forceinline__ double u256_to_f64(const U256 &a) {
    const double t64 = 18446744073709551616.0;
    return ((a.w[3] * t64 + (double)a.w[2]) * t64 + (double)a.w[1]) * t64 + (double)a.w[0];
}
__device__ __forceinline__ double u128_f64(u128 x) {
    return fma((double)(uint64_t)(x >> 64), 18446744073709551616.0, (double)(uint64_t)x);
}


// grid (classes, ceil(F / 32)); thread = checkpoint j; loop over the class's runs.
__global__ void mix_reduce_kernel(MixDev m, const uint32_t *counts, const uint32_t *offsets, MixRec rec,
                                  MixAccum acc, uint32_t n_classes) {
    const uint32_t c = blockIdx.x;
    const uint32_t j = blockIdx.y * blockDim.x + threadIdx.x;
    if (c >= n_classes || j >= (uint32_t)m.F) return;
    const uint32_t cnt = counts[c], off = offsets[c];
    uint32_t kind, L, N, M;
    class_graph(m, c, kind, L, N, M);
    (void)kind; (void)L; (void)M;
    uint32_t span = 0;
    u128 sx[6] = {0, 0, 0, 0, 0, 0};
    U256 sq[6];
    for (int k = 0; k < 6; ++k) sq[k] = U256{{0, 0, 0, 0}};
    for (uint32_t i = 0; i < cnt; ++i) {
        const size_t o = (size_t)(off + i) * (uint32_t)m.F + j;
        const uint32_t ms = rec.max_span[o];
        const uint32_t mxv = ms & ~kSpanBit;
        span += ms >> 31;
        const u128 x[6] = {mxv, rec.m0[o], (u128)(N - mxv), rec.m2[o], rec.m3[o],
                           ((u128)rec.m4_hi[o] << 64) | rec.m4_lo[o]};
        for (int k = 0; k < 6; ++k) {
            sx[k] += x[k];
            u256_add(sq[k], u128_sq(x[k]));
        }
    }
    const size_t cj = (size_t)c * (uint32_t)m.F + j;
    const size_t plane = (size_t)n_classes * (uint32_t)m.F;
    if (j == 0) acc.count[c] = cnt;
    acc.span[cj] = span;
    for (int k = 0; k < 6; ++k) {
        acc.sum_lo[k * plane + cj] = (uint64_t)sx[k];
        acc.sum_hi[k * plane + cj] = (uint64_t)(sx[k] >> 64);
        // M2 = (cnt * sum x^2 - (sum x)^2) / cnt, numerator exact in 256 bits
        double m2 = 0.0;
        if (cnt > 0) {
            const U256 num = u256_sub(u256_mul64(sq[k], cnt), u128_sq(sx[k]));
            m2 = u256_to_f64(num) / (double)cnt;
        }
        acc.m2[k * plane + cj] = m2;
    }
}

// a + (w << (32 k)) for a cell word w < 2^64
__device__ __forceinline__ void u256_add_limb(U256 &a, uint64_t w, int k) {
    U256 t = {{0, 0, 0, 0}};
    const int q = k >> 1;
    if (k & 1) {
        t.w[q] = w << 32;
        if (q + 1 < 4) t.w[q + 1] = w >> 32;
    } else {
        t.w[q] = w;
    }
    u256_add(a, t);
}
__device__ __forceinline__ U256 cell_sum(const uint64_t *w, int limbs) {
    U256 r = {{0, 0, 0, 0}};
    for (int k = 0; k < limbs; ++k) u256_add_limb(r, w[k], k);
    return r;
}

// thread = cell (class c, checkpoint j): the fused limb sums -> exact sums
// of x and M2 = (cnt * sum x^2 - (sum x)^2) / cnt from the exact 256-bit
// numerator, as mix_reduce_kernel computes them from the records.
__global__ void mix_finalize_kernel(MixDev m, const uint32_t *counts, const uint64_t *cells, MixAccum acc,
                                    uint32_t n_classes) {
    const size_t plane = (size_t)n_classes * (uint32_t)m.F;
    const size_t cj = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cj >= plane) return;
    const uint32_t c = (uint32_t)(cj / (uint32_t)m.F), j = (uint32_t)(cj % (uint32_t)m.F);
    const uint32_t cnt = counts[c];
    uint32_t kind, L, N, M;
    class_graph(m, c, kind, L, N, M);
    (void)kind; (void)L; (void)M;
    const uint64_t *w = cells + cj * kMixCellWords;
    const u128 sx_max = cell_sum(w + kSxMax, 1).w[0];
    const U256 sq_max = cell_sum(w + kSqMax, 2);
    // m1 = N - max: sum (N - x) = cnt N - sum x; sum (N - x)^2 = cnt N^2 - 2 N sum x + sum x^2 (< 2^67)
    const u128 sq_max128 = ((u128)sq_max.w[1] << 64) | sq_max.w[0];
    const u128 sx_m1 = (u128)cnt * N - sx_max;
    const u128 sq_m1 = (u128)cnt * N * N + sq_max128 - (u128)(2ull * N) * sx_max;
    U256 sx[6], sq[6];
    sx[0] = cell_sum(w + kSxMax, 1);  sq[0] = sq_max;
    sx[1] = cell_sum(w + kSxM0, 1);   sq[1] = cell_sum(w + kSqM0, 2);
    sx[2] = u256_from_u128(sx_m1);    sq[2] = u256_from_u128(sq_m1);
    sx[3] = cell_sum(w + kSxM2, 2);   sq[3] = cell_sum(w + kSqM2, 3);
    sx[4] = cell_sum(w + kSxM3, 2);   sq[4] = cell_sum(w + kSqM3, 4);
    sx[5] = cell_sum(w + kSxM4, 3);   sq[5] = cell_sum(w + kSqM4, 6);
    if (j == 0) acc.count[c] = cnt;
    acc.span[cj] = (uint32_t)w[kCellSpan];
    for (int k = 0; k < 6; ++k) {
        const u128 sum = ((u128)sx[k].w[1] << 64) | sx[k].w[0];  // < 2^108
        acc.sum_lo[k * plane + cj] = (uint64_t)sum;
        acc.sum_hi[k * plane + cj] = (uint64_t)(sum >> 64);
        double m2 = 0.0;
        if (cnt > 0) {
            const U256 num = u256_sub(u256_mul64(sq[k], cnt), u128_sq(sum));
            m2 = u256_to_f64(num) / (double)cnt;
        }
        acc.m2[k * plane + cj] = m2;
    }
}

// ---------------------------------------------------------------- launchers

int launch_mix(const MixLaunch &p, cudaStream_t s) {
    const uint32_t n_classes = p.m.n_grid + p.m.n_chain;
    if (cudaMemsetAsync(p.counts, 0, sizeof(uint32_t) * n_classes, s) != cudaSuccess) return NZ_ERR_CUDA;
    if (cudaMemsetAsync(p.acc.errors, 0, sizeof(uint32_t), s) != cudaSuccess) return NZ_ERR_CUDA;
    int blocks = (p.m.n_runs + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    mix_class_kernel<<<blocks, 256, 0, s>>>(p.m, p.cls, p.counts);
    mix_order_kernel<<<(n_classes + 255) / 256, 256, 0, s>>>(p.m, p.order);
    mix_offsets_kernel<<<1, 1024, 0, s>>>(p.counts, p.order, n_classes, p.offsets, p.cursor);
    mix_scatter_kernel<<<blocks, 256, 0, s>>>(p.m.n_runs, p.cls, p.cursor, p.queue);
    mix_slots_kernel<<<1, 1024, 0, s>>>(p.m, p.queue, p.cls, p.T, p.slot_off);
    const uint32_t first_free = (uint32_t)(p.T < p.m.n_runs ? p.T : p.m.n_runs);
    mix_head_kernel<<<1, 1, 0, s>>>(p.head, first_free);
    const size_t smem = (size_t)p.smem_words * 4u * (size_t)p.block;
    const unsigned grid = (unsigned)((p.T + p.block - 1) / p.block);
    if (p.fused) {
        const size_t cells = (size_t)n_classes * (uint32_t)p.m.F;
        if (cudaMemsetAsync(p.cells, 0, cells * kMixCellWords * sizeof(uint64_t), s) != cudaSuccess)
            return NZ_ERR_CUDA;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(mix_uf_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
            return NZ_ERR_INVALID;
        mix_uf_kernel<true><<<grid, p.block, smem, s>>>(p.m, p.queue, p.cls, p.T, p.slot_off, p.nodes, p.smem_words,
                                                        p.head, p.rec, p.cells, p.acc.errors);
        mix_finalize_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(p.m, p.counts, p.cells, p.acc,
                                                                            n_classes);
    } else {
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(mix_uf_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
            return NZ_ERR_INVALID;
        mix_uf_kernel<false><<<grid, p.block, smem, s>>>(p.m, p.queue, p.cls, p.T, p.slot_off, p.nodes,
                                                         p.smem_words, p.head, p.rec, p.cells, p.acc.errors);
        dim3 rg(n_classes, (p.m.F + 31) / 32);
        mix_reduce_kernel<<<rg, 32, 0, s>>>(p.m, p.counts, p.offsets, p.rec, p.acc, n_classes);
    }
    return cudaGetLastError() == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

}  // namespace nz
