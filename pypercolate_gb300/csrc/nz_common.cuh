// nz_common.cuh -- device building blocks shared by the GB300 kernels.
//
//  * Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the project's
//    Philox-keyed Feistel permutation of [0, M) (8 rounds, cycle walking);
//    host and device evaluate the identical function.
//  * Implicit substrate lattices: spanning_2d_grid(L) and spanning_1d_chain(l)
//    of percolate/percolate.py:899-965, numbered in the order networkx lists
//    perc_graph.edges() (node-major; per node the edge to the next row, then
//    the edge to the next column).
//  * Union-find node words: one uint32 per node.
//      root     : bit 31 set, bits 29..30 = sides touched, bits 0..28 = size
//      non-root : bit 31 clear, bits 0..30 = parent index
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nz_gb300.h"

namespace nz {

constexpr uint32_t kRoot = 0x80000000u;
constexpr uint32_t kSideShift = 29;
constexpr uint32_t kSizeMask = (1u << 29) - 1u;
constexpr uint32_t kSpanBit = 0x80000000u;  // in NzRecords::max_span

__host__ __device__ __forceinline__ bool is_root(uint32_t w) { return (w & kRoot) != 0; }
__host__ __device__ __forceinline__ uint32_t root_size(uint32_t w) { return w & kSizeMask; }
__host__ __device__ __forceinline__ uint32_t root_sides(uint32_t w) { return (w >> kSideShift) & 3u; }
__host__ __device__ __forceinline__ uint32_t make_root(uint32_t size, uint32_t sides) {
    return kRoot | (sides << kSideShift) | size;
}

// ---------------------------------------------------------------- Philox
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(kPhiloxM0, c[0], hi0, lo0);
        mulhilo32(kPhiloxM1, c[2], hi1, lo1);
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += kPhiloxW0; k1 += kPhiloxW1;
    }
}

// ------------------------------------------------------- Feistel permutation
// Alternating Feistel network on exactly b = bits(M - 1) bits, split into a
// left part of floor(b/2) bits and a right part of the remaining bits; round
// i xors one part with a keyed hash of the other (even rounds update the
// left part, odd rounds the right part), 8 rounds, round keys from two
// Philox-4x32-10 blocks.  The round function is the top bits of
// lowbias32(v ^ k), C. Wellons' two-multiply xorshift integer hash
// (hash-prospector, 2018), whose output bits all depend on all input bits: a
// single multiply-high instead makes the network nearly affine, and the
// permutation then over-represents parts of the edge range in its prefixes
// (7x the hypergeometric spread of the horizontal-bond share of a torus).
// Values >= M are re-encrypted (cycle walking); the domain is < 2M so fewer
// than 2 walks are needed on average, and about one for
// spanning_2d_grid(2^k), whose M = 2L(L-1) lies just below 2^b.
constexpr int kFeistelRounds = 8;
constexpr uint32_t kPermTag = 0x5045524Du;  // "PERM"

__host__ __device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__host__ __device__ __forceinline__ uint32_t feistel_f(uint32_t v, uint32_t obits, uint32_t k) {
    return obits ? (lowbias32(v ^ k) >> (32u - obits)) : 0u;
}

struct FeistelPerm {
    uint32_t M, hl, hr, maskL, maskR;
    uint32_t k[kFeistelRounds];

    __host__ __device__ void init(uint64_t key, uint64_t run_id, uint32_t m) {
        uint32_t bits = 0;
        if (m > 1) {
            uint32_t x = m - 1;
            while (x) { ++bits; x >>= 1; }
        }
        M = m;
        hl = bits / 2;
        hr = bits - hl;
        maskL = (1u << hl) - 1u;
        maskR = (1u << hr) - 1u;
#pragma unroll
        for (uint32_t half = 0; half < 2; ++half) {
            uint32_t c[4] = {(uint32_t)run_id, (uint32_t)(run_id >> 32), half, kPermTag};
            philox4x32_10(c, (uint32_t)key, (uint32_t)(key >> 32));
#pragma unroll
            for (int i = 0; i < 4; ++i) k[4 * half + i] = c[i];
        }
    }

    __host__ __device__ __forceinline__ uint32_t encrypt(uint32_t x) const {
        uint32_t L = x >> hr, R = x & maskR;
#pragma unroll
        for (int i = 0; i < kFeistelRounds; i += 2) {
            L ^= feistel_f(R, hl, k[i]) & maskL;
            R ^= feistel_f(L, hr, k[i + 1]) & maskR;
        }
        return (L << hr) | R;
    }

    // n-th element of the permutation of [0, M) (requires n < M).
    __host__ __device__ __forceinline__ uint32_t at(uint32_t n) const {
        uint32_t x = n;
        do { x = encrypt(x); } while (x >= M);
        return x;
    }
};

// ------------------------------------------------------------- graphs
struct GraphDev {
    int32_t kind;         // NZ_GRAPH_* without flags
    uint32_t site;        // NZ_MODEL_SITE given: M = N steps occupy sites
    uint32_t wrap;        // torus: NZ_WRAP_* >> 9 (0 either, 1 x, 2 y, 3 both)
    uint32_t L, N, M;
    uint32_t slots;       // union-find words per run (>= N: layout padding, torus cells)
    uint32_t tile_cols;   // grid: 4 x 2 site blocks per block row, (L+3)/4
    uint32_t row_edges;   // grid: (L-1)*(2L-1) edges in rows 0..L-2
    uint32_t two_l_m1;    // grid: 2L-1
    float inv_two_l_m1;   // grid: 1/(2L-1)
    const uint32_t *eu, *ev;
    const uint8_t *side;
};

// The square grid (bond and site percolation) keeps its node words in blocks
// of 4 x 2 sites, one block per 32-byte sector (block rows of (L+3)/4 blocks),
// instead of row-major: both ends of a random bond then share a sector 5/8 of
// the time instead of 7/16, and small clusters span fewer sectors.  Node
// words hold these slot indices as parents; the records do not depend on the
// layout.
#ifndef NZ_GRID_TILED
#define NZ_GRID_TILED 1
#endif
constexpr bool kGridTiled = NZ_GRID_TILED != 0;

__host__ __device__ __forceinline__ uint32_t grid_slot(uint32_t tile_cols, uint32_t r, uint32_t c) {
    return ((r >> 1) * tile_cols + (c >> 2)) * 8u + ((r & 1u) << 2) + (c & 3u);
}

// node words of an L x L grid in that layout (>= L^2, non-decreasing in L)
__host__ __device__ __forceinline__ uint32_t grid_slots(uint32_t L) {
    return kGridTiled ? ((L + 1u) >> 1) * ((L + 3u) >> 2) * 8u : L * L;
}

inline int graph_size_base(const NzGraph &g, int kind, uint32_t &N, uint32_t &M);

inline int graph_size(const NzGraph &g, uint32_t &N, uint32_t &M) {
    const int kind = g.kind & NZ_KIND_MASK, flags = g.kind & ~NZ_KIND_MASK;
    if (flags & ~(NZ_MODEL_SITE | NZ_WRAP_BOTH)) return NZ_ERR_INVALID;
    if ((flags & NZ_WRAP_BOTH) && kind != NZ_GRAPH_TORUS2D) return NZ_ERR_INVALID;
    if ((flags & NZ_MODEL_SITE) && kind == NZ_GRAPH_EDGES) return NZ_ERR_INVALID;
    const int st = graph_size_base(g, kind, N, M);
    if (st == NZ_OK && (flags & NZ_MODEL_SITE)) M = N;
    return st;
}

inline int graph_size_base(const NzGraph &g, int kind, uint32_t &N, uint32_t &M) {
    if (kind == NZ_GRAPH_TORUS2D) {
        if (g.length == 0) return NZ_ERR_INVALID;
        if ((uint64_t)g.length * g.length > NZ_MAX_NODES) return NZ_ERR_TOO_LARGE;
        N = g.length * g.length;
        M = 2u * N;
        return NZ_OK;
    }
    if (kind == NZ_GRAPH_GRID2D) {
        if (g.length == 0 || (uint64_t)g.length * g.length > NZ_MAX_NODES) return NZ_ERR_TOO_LARGE;
        N = g.length * g.length;
        M = 2u * g.length * (g.length - 1u);
        return NZ_OK;
    }
    if (kind == NZ_GRAPH_CHAIN1D) {
        if (g.length == 0) return NZ_ERR_INVALID;
        if (g.length > NZ_MAX_NODES) return NZ_ERR_TOO_LARGE;
        N = g.length;
        M = g.length - 1u;
        return NZ_OK;
    }
    if (kind == NZ_GRAPH_EDGES) {
        if (g.num_nodes == 0) return NZ_ERR_INVALID;
        if (g.num_nodes > NZ_MAX_NODES || g.num_edges > 2u * NZ_MAX_NODES) return NZ_ERR_TOO_LARGE;
        if (g.num_edges > 0 && (!g.edge_u || !g.edge_v)) return NZ_ERR_INVALID;
        N = g.num_nodes;
        M = g.num_edges;
        return NZ_OK;
    }
    return NZ_ERR_INVALID;
}

inline GraphDev make_graph_dev(const NzGraph &g, uint32_t N, uint32_t M) {
    GraphDev d;
    d.kind = g.kind & NZ_KIND_MASK;
    d.site = (g.kind & NZ_MODEL_SITE) ? 1u : 0u;
    d.wrap = (uint32_t)(g.kind & NZ_WRAP_BOTH) >> 9;
    d.L = g.length;
    d.N = N;
    d.M = M;
    d.row_edges = 0;
    d.two_l_m1 = 1;
    d.inv_two_l_m1 = 1.0f;
    d.tile_cols = 0;
    d.slots = N;
    if (d.kind == NZ_GRAPH_GRID2D) {
        d.two_l_m1 = 2u * g.length - 1u;
        d.row_edges = (g.length - 1u) * d.two_l_m1;
        d.inv_two_l_m1 = 1.0f / (float)d.two_l_m1;
        d.tile_cols = (g.length + 3u) >> 2;
        d.slots = grid_slots(g.length);
    }
    if (d.kind == NZ_GRAPH_TORUS2D) d.slots = 4u * N;
    d.eu = g.edge_u;
    d.ev = g.edge_v;
    d.side = g.node_side;
    return d;
}

// Exact e / d for e < 2^23, d < 2^12 using a float reciprocal and one fix-up.
__device__ __forceinline__ uint32_t div_small(uint32_t e, uint32_t d, float inv) {
    uint32_t q = __float2uint_rz(__uint2float_rz(e) * inv);
    int32_t r = (int32_t)(e - q * d);
    if (r < 0) { --q; } else if ((uint32_t)r >= d) { ++q; }
    return q;
}

template <int KIND>
__device__ __forceinline__ void decode_edge(const GraphDev &g, uint32_t e, uint32_t &u, uint32_t &v) {
    if (KIND == NZ_GRAPH_GRID2D) {
        if (e < g.row_edges) {
            uint32_t r = div_small(e, g.two_l_m1, g.inv_two_l_m1);
            uint32_t w = e - r * g.two_l_m1;
            u = r * g.L + (w >> 1);
            v = (w & 1u) ? u + 1u : u + g.L;
        } else {
            u = (g.L - 1u) * g.L + (e - g.row_edges);
            v = u + 1u;
        }
    } else if (KIND == NZ_GRAPH_CHAIN1D) {
        u = e;
        v = e + 1u;
    } else {
        u = __ldg(g.eu + e);
        v = __ldg(g.ev + e);
    }
}

// Ends of edge e as slots of the run's node array (grid_slot on the tiled
// square grid, the node ids otherwise).
template <int KIND>
__device__ __forceinline__ void decode_edge_slots(const GraphDev &g, uint32_t e, uint32_t &u, uint32_t &v) {
    if (KIND == NZ_GRAPH_GRID2D && kGridTiled) {
        uint32_t r, c;
        bool right;
        if (e < g.row_edges) {
            r = div_small(e, g.two_l_m1, g.inv_two_l_m1);
            const uint32_t w = e - r * g.two_l_m1;
            c = w >> 1;
            right = (w & 1u) != 0;
        } else {
            r = g.L - 1u;
            c = e - g.row_edges;
            right = true;
        }
        u = grid_slot(g.tile_cols, r, c);
        v = right ? grid_slot(g.tile_cols, r, c + 1u) : grid_slot(g.tile_cols, r + 1u, c);
    } else {
        decode_edge<KIND>(g, e, u, v);
    }
}

// slot of node i (see decode_edge_slots)
template <int KIND>
__device__ __forceinline__ uint32_t node_slot(const GraphDev &g, uint32_t i) {
    if (KIND == NZ_GRAPH_GRID2D && kGridTiled) {
        const uint32_t r = i / g.L;
        return grid_slot(g.tile_cols, r, i - r * g.L);
    }
    return i;
}

template <int KIND>
__device__ __forceinline__ uint32_t node_sides(const GraphDev &g, uint32_t i) {
    if (KIND == NZ_GRAPH_GRID2D) {
        uint32_t r = i / g.L;
        return (r == 0 ? 1u : 0u) | (r == g.L - 1u ? 2u : 0u);
    } else if (KIND == NZ_GRAPH_CHAIN1D) {
        return (i == 0 ? 1u : 0u) | (i == g.L - 1u ? 2u : 0u);
    } else {
        return g.side ? (uint32_t)(g.side[i] & 3u) : 0u;
    }
}

// Per-run state carried between windows of steps.
struct __align__(16) RunState {
    uint64_t t2, t3;        // sum over all clusters of s^2, s^3
    uint64_t t4_lo, t4_hi;  // sum over all clusters of s^4 (128-bit)
    uint32_t t0;            // number of clusters
    uint32_t max;           // largest cluster size
    uint32_t flags;         // bit 0: spanning cluster seen; bit 1: a node touches both sides
    uint32_t pad;
};

constexpr uint32_t kFlagSpan = 1u;
constexpr uint32_t kFlagInitBoth = 2u;
constexpr uint32_t kFlagCorrupt = 4u;   // a find exceeded the depth bound (never in valid use)
constexpr uint32_t kFlagWrapX = 8u;     // torus: a cluster wraps along x
constexpr uint32_t kFlagWrapY = 16u;    // torus: a cluster wraps along y


}  // namespace nz
