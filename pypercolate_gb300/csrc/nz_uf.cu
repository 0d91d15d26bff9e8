// nz_uf.cu -- Newman-Ziff union-find kernels (microcanonical statistics).
//
// Replaces the hot loop of percolate/hpc.py:249-307 (bond_sample_states).
// One thread owns one run: its node words live in HBM (run-major, 4 bytes
// per node), and its loop adds the bonds of its permutation one at a time.
//
// Per step, instead of the reference's "subtract the merged clusters, add the
// merged one, keep track of the largest" bookkeeping (hpc.py:283-305), the
// kernel keeps the exact totals T_k = sum over ALL clusters of s^k, updated
// by (a+b)^k - a^k - b^k on a merge of sizes a and b, and the largest size
// S.  The reference's moments are then T_k - S^k (the primed sum excludes
// exactly one largest cluster), which is the same integer regardless of
// union-find tie-breaking.  T_4 is 128-bit; the reference's uint64 field is
// its low 64 bits.
//
// Spanning (hpc.py:224-274): each root carries the two-bit set of sides its
// cluster touches; the run's flag is set at the first union that produces a
// root touching both sides (or at the first union at all if some node
// touches both sides from the start), and stays set -- exactly when the
// reference's auxiliary union-find first connects its two side roots.
#include <cstdint>

#include "nz_common.cuh"
#include "nz_internal.cuh"
#include "nz_records.cuh"

namespace nz {

__device__ __forceinline__ void add128(uint64_t &lo, uint64_t &hi, uint64_t blo, uint64_t bhi) {
    uint64_t nlo = lo + blo;
    hi += bhi + (nlo < lo ? 1ull : 0ull);
    lo = nlo;
}

// ------------------------------------------------------------ initialisers
// Initial word of node slot j: every node a singleton root with its spanning
// sides.  Slots are written in order (coalesced) and mapped back to their
// node; padding slots of the tiled grid layout (never read) get 0.
template <int KIND>
__device__ __forceinline__ uint32_t init_word(const GraphDev &g, uint32_t j) {
    uint32_t k = j;
    if (KIND == NZ_GRAPH_GRID2D && kGridTiled) {
        const uint32_t tile = j >> 3, w = j & 7u;
        const uint32_t tr = tile / g.tile_cols, tc = tile - tr * g.tile_cols;
        const uint32_t r = 2u * tr + (w >> 2), c = 4u * tc + (w & 3u);
        if (r >= g.L || c >= g.L) return 0u;
        k = r * g.L + c;
    }
    if (k >= g.N) return 0u;
    return make_root(1u, node_sides<KIND>(g, k));
}

// block b: chunk b % chunks (kInitChunk slots) of run b / chunks
constexpr uint32_t kInitChunk = 4096;
template <int KIND>
__global__ void init_nodes_kernel(GraphDev g, uint64_t blocks, uint32_t chunks, uint32_t *nodes) {
    for (uint64_t b = blockIdx.x; b < blocks; b += gridDim.x) {
        const uint64_t r = b / chunks;
        const uint32_t ch = (uint32_t)(b - r * chunks);
        uint32_t *row = nodes + r * g.slots;
        const uint32_t j1 = min(g.slots, (ch + 1u) * kInitChunk);
        for (uint32_t j = ch * kInitChunk + threadIdx.x; j < j1; j += blockDim.x) row[j] = init_word<KIND>(g, j);
    }
}

__global__ void any_both_sides_kernel(GraphDev g, uint32_t *flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < g.N; i += gridDim.x * blockDim.x)
        if (g.side && (g.side[i] & 3u) == 3u) *flag = kFlagInitBoth;
}

__global__ void init_state_kernel(int32_t n_runs, uint32_t N, const uint32_t *init_flag,
                                  RunState *state) {
    int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_runs) return;
    RunState s;
    s.t2 = N; s.t3 = N; s.t4_lo = N; s.t4_hi = 0;
    s.t0 = N; s.max = 1; s.flags = init_flag ? *init_flag : 0u; s.pad = 0;
    state[r] = s;
}

// ------------------------------------------------------------ main kernel
// 9 resident CTAs of 128 threads per SM: at most 56 registers.  In the
// ensemble pipeline the union-find shares the SMs with the consumers of the
// previous window; a smaller register footprint leaves them more warps: 1491
// ms per 100,000-run L = 256 step against 1636 ms at 70 registers and 1515 ms
// when forced to 48 (with spills).  Since the next permutation element is
// computed during the first loads, the kernel needs 48 without spills.
#ifndef NZ_UF_MIN_BLOCKS
#define NZ_UF_MIN_BLOCKS 9
#endif
#define NZ_UF_BOUNDS __launch_bounds__(128, NZ_UF_MIN_BLOCKS)
template <int KIND, int PERM, bool SPAN>
__global__ void NZ_UF_BOUNDS uf_window_kernel(UfParams p) {
    const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= p.n_runs) return;
    const GraphDev &g = p.g;
    uint32_t *node = p.nodes + (size_t)r * g.slots;
    RunState st = p.state[r];

    FeistelPerm fp;
    const uint32_t *perm = nullptr;
    if (PERM == NZ_PERM_PHILOX) fp.init(p.key, p.run0 + (uint64_t)r, g.M);
    else perm = p.perms + (size_t)r * g.M;

    const NzRecords rec = p.rec;
    uint32_t mx = st.max;
    // the permutation element of the next step is computed while this
    // step's first node loads are in flight
    uint32_t e_next = 0;
    {
        const uint32_t first = p.n_begin > 0 ? p.n_begin - 1u : 0u;
        if (first < g.M) e_next = (PERM == NZ_PERM_PHILOX) ? fp.at(first) : __ldg(perm + first);
    }
    for (uint32_t n = p.n_begin; n < p.n_end; ++n) {
        uint32_t e = 0;
        if (n > 0) {
            const uint32_t idx = n - 1u;
            e = e_next;
            uint32_t u, v;
            if (PERM != NZ_PERM_PHILOX && e >= g.M) {
                u = v = 0;  // caller-supplied index out of range: no bond added
            } else {
                decode_edge_slots<KIND>(g, e, u, v);
                if (KIND == NZ_GRAPH_EDGES && (u >= g.N || v >= g.N)) u = v = 0;  // invalid edge list
            }
            // two interleaved finds with path splitting
            uint32_t xu = u, xv = v;
            uint32_t wu = node[xu], wv = node[xv];
            if (idx + 1u < g.M)
                e_next = (PERM == NZ_PERM_PHILOX) ? fp.at(idx + 1u) : __ldg(perm + idx + 1u);
            // union by size keeps every tree at most log2(N) <= 21 levels deep;
            // the hop limit only guards against corrupted input state
            for (int hops = 0; !(is_root(wu) && is_root(wv)); ++hops) {
                if (hops >= 64) { st.flags |= kFlagCorrupt; wu = wv = make_root(0, 0); xu = xv; break; }
                if (!is_root(wu)) {
                    uint32_t nu = node[wu];
                    if (!is_root(nu)) node[xu] = nu;
                    xu = wu; wu = nu;
                }
                if (!is_root(wv)) {
                    uint32_t nv = node[wv];
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
                st.t0 -= 1u;
                const uint64_t ab = (uint64_t)a * b;
                st.t2 += 2ull * ab;
                st.t3 += 3ull * ab * s;
                const uint64_t q = 4ull * a * a + 6ull * ab + 4ull * b * b;
                add128(st.t4_lo, st.t4_hi, ab * q, __umul64hi(ab, q));
                if (s > mx) mx = s;
                if (SPAN && (sides == 3u || (st.flags & kFlagInitBoth))) st.flags |= kFlagSpan;
            }
        }
        // row n: moments = T_k - max^k
        const size_t off = (size_t)(n - p.n_begin) * rec.run_stride + r;
        // powers of the largest size, recomputed per row (a few integer
        // multiplies) rather than kept live: at the 56-register cap the
        // kernel then needs no spills
        const uint64_t mx2 = (uint64_t)mx * mx, mx3 = mx2 * mx;
        const uint64_t mx4_lo = mx3 * mx, mx4_hi = __umul64hi(mx3, (uint64_t)mx);
        if (rec.max_span) rec.max_span[off] = mx | ((SPAN && (st.flags & kFlagSpan)) ? kSpanBit : 0u);
        put_m0_m2(rec, off, st.t0 - 1u, st.t2 - mx2);
        if (rec.m3) rec.m3[off] = st.t3 - mx3;
        const uint64_t m4_lo = st.t4_lo - mx4_lo;
        const uint64_t m4_hi = st.t4_hi - mx4_hi - (st.t4_lo < mx4_lo ? 1ull : 0ull);
        if (rec.m4_lo) rec.m4_lo[off] = m4_lo;
        if (rec.m4_hi) rec.m4_hi[off] = (uint32_t)m4_hi;
        if (rec.edge) rec.edge[off] = e;
    }
    st.max = mx;
    p.state[r] = st;
    // a find that exceeded the depth bound (only possible with corrupted
    // state: union by size keeps trees log2 N deep) is reported once per run
    if (p.errors && (st.flags & kFlagCorrupt) && p.n_end == g.M + 1u) atomicAdd(p.errors, 1u);
}

// ------------------------------------------------------- permutation kernels
__global__ void philox_perm_kernel(uint32_t M, int32_t n_runs, uint64_t key, uint64_t run0,
                                   uint32_t *out) {
    const uint64_t total = (uint64_t)n_runs * M;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t r = (uint32_t)(i / M), n = (uint32_t)(i % M);
        FeistelPerm fp;
        fp.init(key, run0 + r, M);
        out[i] = fp.at(n);
    }
}

// MT19937 (Matsumoto & Nishimura 1998) with the authors' init_genrand and
// init_by_array seeding; then the Fisher-Yates shuffle with masked rejection
// that numpy's legacy RandomState.permutation(M) performs.  One thread per
// run; the 624-word state lives in local memory.
struct Mt19937 {
    uint32_t mt[624];
    int mti;

    __device__ void init_genrand(uint32_t seed) {
        mt[0] = seed;
        for (int i = 1; i < 624; ++i) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
        mti = 624;
    }
    __device__ void init_by_array(const uint32_t *key, int len) {
        init_genrand(19650218u);
        int i = 1, j = 0;
        for (int k = (624 > len ? 624 : len); k; --k) {
            mt[i] = (mt[i] ^ ((mt[i - 1] ^ (mt[i - 1] >> 30)) * 1664525u)) + key[j] + (uint32_t)j;
            ++i; ++j;
            if (i >= 624) { mt[0] = mt[623]; i = 1; }
            if (j >= len) j = 0;
        }
        for (int k = 623; k; --k) {
            mt[i] = (mt[i] ^ ((mt[i - 1] ^ (mt[i - 1] >> 30)) * 1566083941u)) - (uint32_t)i;
            ++i;
            if (i >= 624) { mt[0] = mt[623]; i = 1; }
        }
        mt[0] = 0x80000000u;
        mti = 624;
    }
    __device__ uint32_t next() {
        if (mti >= 624) {
            for (int kk = 0; kk < 624; ++kk) {
                uint32_t y = (mt[kk] & 0x80000000u) | (mt[kk + 1 < 624 ? kk + 1 : 0] & 0x7fffffffu);
                int src = kk + 397 < 624 ? kk + 397 : kk + 397 - 624;
                mt[kk] = mt[src] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            mti = 0;
        }
        uint32_t y = mt[mti++];
        y ^= (y >> 11);
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= (y >> 18);
        return y;
    }
};

__global__ void mt_perm_kernel(uint32_t M, int32_t n_runs, const uint32_t *seed_words,
                               const int32_t *seed_len, int32_t stride, uint32_t *out) {
    const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_runs) return;
    Mt19937 g;
    const int len = seed_len[r];
    const uint32_t *w = seed_words + (size_t)r * stride;
    if (len == 0) g.init_genrand(w[0]);
    else g.init_by_array(w, len);
    uint32_t *o = out + (size_t)r * M;
    for (uint32_t i = 0; i < M; ++i) o[i] = i;
    for (int64_t i = (int64_t)M - 1; i >= 1; --i) {
        uint32_t mx = (uint32_t)i, mask = mx;
        mask |= mask >> 1; mask |= mask >> 2; mask |= mask >> 4; mask |= mask >> 8; mask |= mask >> 16;
        uint32_t j;
        do { j = g.next() & mask; } while (j > mx);
        uint32_t t = o[i]; o[i] = o[j]; o[j] = t;
    }
}

// Continuation of one MT19937 stream (numpy's global RandomState): the state
// (624 words + position) is loaded, n_runs permutations of range(M) are drawn
// one after another exactly as np.random.permutation(M) would draw them
// (percolate/percolate.py:270, once per run in run order), and the advanced
// state is stored back.  One thread: the stream is sequential by nature.
__global__ void mt_stream_perm_kernel(const uint32_t *state_in, uint32_t M, int32_t n_runs, uint32_t *out,
                                      uint32_t *state_out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    Mt19937 g;
    for (int i = 0; i < 624; ++i) g.mt[i] = state_in[i];
    g.mti = (int)state_in[624];
    for (int32_t r = 0; r < n_runs; ++r) {
        uint32_t *o = out + (size_t)r * M;
        for (uint32_t i = 0; i < M; ++i) o[i] = i;
        for (int64_t i = (int64_t)M - 1; i >= 1; --i) {
            uint32_t mx = (uint32_t)i, mask = mx;
            mask |= mask >> 1; mask |= mask >> 2; mask |= mask >> 4; mask |= mask >> 8; mask |= mask >> 16;
            uint32_t j;
            do { j = g.next() & mask; } while (j > mx);
            uint32_t t = o[i]; o[i] = o[j]; o[j] = t;
        }
    }
    for (int i = 0; i < 624; ++i) state_out[i] = g.mt[i];
    state_out[624] = (uint32_t)g.mti;
}

void launch_mt_stream_perms(const uint32_t *state_in, uint32_t M, int32_t n_runs, uint32_t *out,
                            uint32_t *state_out, cudaStream_t s) {
    mt_stream_perm_kernel<<<1, 1, 0, s>>>(state_in, M, n_runs, out, state_out);
}

// ---------------------------------------------------------------- packing
// Reference row layout (packed little-endian), percolate/hpc.py:34-70:
//   n u32 | edge u32 | [has_spanning_cluster u8] | max_cluster_size u32 | moments 5 x u64
__device__ __forceinline__ void put_bytes(uint8_t *dst, uint64_t v, int nbytes) {
    for (int i = 0; i < nbytes; ++i) dst[i] = (uint8_t)(v >> (8 * i));
}

__global__ void pack_rows_kernel(NzRecords rec, int32_t run, uint32_t N, uint32_t M, int32_t spanning,
                                 uint8_t *rows) {
    const uint32_t row_bytes = spanning ? 53u : 52u;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n <= M; n += gridDim.x * blockDim.x) {
        const size_t off = (size_t)n * rec.run_stride + run;
        uint8_t *d = rows + (size_t)n * row_bytes;
        const uint32_t ms = rec.max_span[off];
        const uint32_t mx = ms & ~kSpanBit;
        put_bytes(d, n, 4);
        put_bytes(d + 4, rec.edge ? rec.edge[off] : 0u, 4);
        int o = 8;
        if (spanning) { d[8] = (ms & kSpanBit) ? 1 : 0; o = 9; }
        put_bytes(d + o, mx, 4);
        put_bytes(d + o + 4, record_m0(rec, off), 8);
        put_bytes(d + o + 12, (uint64_t)((rec.site ? n : N) - mx), 8);
        put_bytes(d + o + 20, record_m2(rec, off), 8);
        put_bytes(d + o + 28, rec.m3[off], 8);
        put_bytes(d + o + 36, rec.m4_lo[off], 8);
    }
}

// ------------------------------------------------------------ launchers
template <int KIND>
static void launch_init_nodes_k(const GraphDev &g, int32_t n_runs, uint32_t *nodes, cudaStream_t s) {
    const uint32_t chunks = (g.slots + kInitChunk - 1) / kInitChunk;
    const uint64_t blocks = (uint64_t)n_runs * chunks;
    if (blocks == 0) return;
    const uint64_t grid = blocks < 152ull * 256 ? blocks : 152ull * 256;
    init_nodes_kernel<KIND><<<(unsigned)grid, 256, 0, s>>>(g, blocks, chunks, nodes);
}

void launch_init_runs(const GraphDev &g, int32_t n_runs, uint32_t *nodes, RunState *state,
                      uint32_t *flag_scratch, cudaStream_t s) {
    if (lattice_extension(g)) { launch_init_lattice_runs(g, n_runs, nodes, state, s); return; }
    if (g.kind == NZ_GRAPH_GRID2D) launch_init_nodes_k<NZ_GRAPH_GRID2D>(g, n_runs, nodes, s);
    else if (g.kind == NZ_GRAPH_CHAIN1D) launch_init_nodes_k<NZ_GRAPH_CHAIN1D>(g, n_runs, nodes, s);
    else launch_init_nodes_k<NZ_GRAPH_EDGES>(g, n_runs, nodes, s);
    const uint32_t *flag = nullptr;
    if (g.kind == NZ_GRAPH_EDGES && flag_scratch) {
        cudaMemsetAsync(flag_scratch, 0, sizeof(uint32_t), s);
        any_both_sides_kernel<<<(g.N + 255) / 256 < 1024 ? (g.N + 255) / 256 : 1024, 256, 0, s>>>(g, flag_scratch);
        flag = flag_scratch;
    }
    init_state_kernel<<<(n_runs + 255) / 256, 256, 0, s>>>(n_runs, g.N, flag, state);
}

template <int KIND, int PERM>
static void launch_uf_k(const UfParams &p, bool span, int block, cudaStream_t s) {
    dim3 grid((p.n_runs + block - 1) / block);
    if (span) uf_window_kernel<KIND, PERM, true><<<grid, block, 0, s>>>(p);
    else uf_window_kernel<KIND, PERM, false><<<grid, block, 0, s>>>(p);
}

template <int KIND>
static void launch_uf_kind(const UfParams &p, int perm_mode, bool span, int block, cudaStream_t s) {
    if (perm_mode == NZ_PERM_PHILOX) launch_uf_k<KIND, NZ_PERM_PHILOX>(p, span, block, s);
    else launch_uf_k<KIND, NZ_PERM_GIVEN>(p, span, block, s);
}

void launch_uf_window(const UfParams &p, int perm_mode, bool span, int block, cudaStream_t s) {
    if (lattice_extension(p.g)) { launch_lattice_window(p, perm_mode, span, block, s); return; }
    if (p.g.kind == NZ_GRAPH_GRID2D) launch_uf_kind<NZ_GRAPH_GRID2D>(p, perm_mode, span, block, s);
    else if (p.g.kind == NZ_GRAPH_CHAIN1D) launch_uf_kind<NZ_GRAPH_CHAIN1D>(p, perm_mode, span, block, s);
    else launch_uf_kind<NZ_GRAPH_EDGES>(p, perm_mode, span, block, s);
}

void launch_philox_perms(uint32_t M, int32_t n_runs, uint64_t key, uint64_t run0, uint32_t *out,
                         cudaStream_t s) {
    uint64_t total = (uint64_t)n_runs * M;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152ull * 64) blocks = 152ull * 64;
    if (blocks == 0) return;
    philox_perm_kernel<<<(unsigned)blocks, 256, 0, s>>>(M, n_runs, key, run0, out);
}

void launch_mt_perms(uint32_t M, int32_t n_runs, const uint32_t *seed_words, const int32_t *seed_len,
                     int32_t stride, uint32_t *out, cudaStream_t s) {
    if (n_runs <= 0) return;
    mt_perm_kernel<<<(n_runs + 63) / 64, 64, 0, s>>>(M, n_runs, seed_words, seed_len, stride, out);
}

void launch_pack_rows(const NzRecords &rec, int32_t run, uint32_t N, uint32_t M, int32_t spanning,
                      uint8_t *rows, cudaStream_t s) {
    uint32_t blocks = (M + 1 + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    pack_rows_kernel<<<blocks, 256, 0, s>>>(rec, run, N, M, spanning, rows);
}

}  // namespace nz
