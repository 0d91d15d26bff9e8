// nz_lattice.cu -- site percolation, and wrapping on the periodic square lattice.
//
// Extensions that the reference lists as to-do (percolate/__init__.py:68-78;
// percolate/percolate.py:210-211 rejects every model but 'bond'), built on
// the union-find of nz_uf.cu and writing the same per-step records, so the
// fused microcanonical reductions, the canonical convolution and every other
// consumer of records apply unchanged.
//
// Site percolation (Newman & Ziff, Phys. Rev. Lett. 85, 4104 (2000); Phys.
// Rev. E 64, 016706 (2001), Sec. II): step n occupies the n-th site of a
// permutation of the N sites -- a new cluster of one site -- and joins it to
// each occupied neighbour.  An unoccupied site holds the root word of size 0.
// The statistics count occupied sites only (T_k over occupied clusters, so
// m1 = n - max; m0 = clusters - 1, or 0 while no site is occupied).
//
// Wrapping (NZ 2001, Sec. III.B): on the L x L torus every node keeps, next to
// its union-find word, its displacement (dx, dy) from its parent, so a find
// returns the root and the node's position relative to it.  Joining u to
// v = u + delta inside one cluster closes a loop, which winds around the
// torus exactly when pos(u) + delta != pos(v): along x when the x parts
// differ, along y when the y parts differ.  A union hangs one root below the
// other with the displacement that keeps pos(v) = pos(u) + delta.  Positions
// are exact in 32-bit integers: each is a sum of at most N - 1 unit steps
// along the clusters' spanning trees.  The run's wrap flags are sticky, like
// the spanning flag; two clusters cannot wrap along different directions (the
// loops would cross), so "along both" is the conjunction of the two flags.
#include <cstdint>

#include "nz_common.cuh"
#include "nz_internal.cuh"
#include "nz_records.cuh"

namespace nz {

namespace {

__device__ __forceinline__ void add128(uint64_t &lo, uint64_t &hi, uint64_t blo, uint64_t bhi) {
    uint64_t nlo = lo + blo;
    hi += bhi + (nlo < lo ? 1ull : 0ull);
    lo = nlo;
}

constexpr uint32_t kEmpty = kRoot;  // make_root(0, 0): an unoccupied site

// Exact T_k of all clusters and the powers of the largest size.
struct Tally {
    RunState st;
    uint32_t mx;
    uint64_t mx2, mx3, mx4_lo, mx4_hi;

    __device__ void load(const RunState &s) {
        st = s;
        mx = s.max;
        powers();
    }
    __device__ __forceinline__ void powers() {
        mx2 = (uint64_t)mx * mx;
        mx3 = mx2 * mx;
        mx4_lo = mx3 * mx;
        mx4_hi = __umul64hi(mx3, (uint64_t)mx);
    }
    // a new cluster of one site
    __device__ __forceinline__ void add_single() {
        st.t0 += 1u;
        st.t2 += 1u;
        st.t3 += 1u;
        add128(st.t4_lo, st.t4_hi, 1u, 0u);
        if (mx < 1u) { mx = 1u; powers(); }
    }
    // clusters of sizes a and b become one
    __device__ __forceinline__ void merge(uint32_t a, uint32_t b) {
        const uint32_t s = a + b;
        st.t0 -= 1u;
        const uint64_t ab = (uint64_t)a * b;
        st.t2 += 2ull * ab;
        st.t3 += 3ull * ab * s;
        const uint64_t q = 4ull * a * a + 6ull * ab + 4ull * b * b;
        add128(st.t4_lo, st.t4_hi, ab * q, __umul64hi(ab, q));
        if (s > mx) { mx = s; powers(); }
    }
    // row n of the records
    __device__ __forceinline__ void write(const NzRecords &rec, size_t off, bool flag, uint32_t e) const {
        if (rec.max_span) rec.max_span[off] = mx | (flag ? kSpanBit : 0u);
        put_m0_m2(rec, off, st.t0 - (st.t0 ? 1u : 0u), st.t2 - mx2);
        if (rec.m3) rec.m3[off] = st.t3 - mx3;
        const uint64_t m4_lo = st.t4_lo - mx4_lo;
        const uint64_t m4_hi = st.t4_hi - mx4_hi - (st.t4_lo < mx4_lo ? 1ull : 0ull);
        if (rec.m4_lo) rec.m4_lo[off] = m4_lo;
        if (rec.m4_hi) rec.m4_hi[off] = (uint32_t)m4_hi;
        if (rec.edge) rec.edge[off] = e;
    }
};

template <int PERM>
__device__ __forceinline__ uint32_t step_index(const FeistelPerm &fp, const uint32_t *perm, uint32_t idx) {
    return PERM == NZ_PERM_PHILOX ? fp.at(idx) : __ldg(perm + idx);
}

// ------------------------------------------------- grid / chain, site model
// Joins the clusters of u and v (interleaved finds with path splitting, union
// by size); the joined root's side set decides spanning.
template <bool SPAN>
__device__ __forceinline__ void link(uint32_t *node, uint32_t u, uint32_t v, Tally &t) {
    uint32_t xu = u, xv = v;
    uint32_t wu = node[xu], wv = node[xv];
    for (int hops = 0; !(is_root(wu) && is_root(wv)); ++hops) {
        if (hops >= 64) { t.st.flags |= kFlagCorrupt; return; }
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
    if (xu == xv) return;
    const uint32_t a = root_size(wu), b = root_size(wv);
    const uint32_t sides = root_sides(wu) | root_sides(wv);
    uint32_t big = xu, small = xv;
    if (a < b) { big = xv; small = xu; }
    node[small] = big;
    node[big] = make_root(a + b, sides);
    t.merge(a, b);
    if (SPAN && sides == 3u) t.st.flags |= kFlagSpan;
}

// Site kernel at most 56 registers (9 CTAs of 128 per SM), like the bond
// union-find: beside the convolution of the previous window this measured
// 5.84e9 against 5.47e9 site additions/s (L = 256, 100,000 runs).  The torus
// kernel is not capped (72 registers for bonds, 78 for sites; capped, the
// 78-register bond kernel of the time spilled and measured 18 % slower).
#ifndef NZ_SITE_MIN_BLOCKS
#define NZ_SITE_MIN_BLOCKS 9
#endif

template <int KIND, int PERM, bool SPAN>
__global__ void __launch_bounds__(128, NZ_SITE_MIN_BLOCKS) site_window_kernel(UfParams p) {
    const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= p.n_runs) return;
    const GraphDev &g = p.g;
    uint32_t *node = p.nodes + (size_t)r * g.slots;
    Tally t;
    t.load(p.state[r]);
    FeistelPerm fp;
    const uint32_t *perm = nullptr;
    if (PERM == NZ_PERM_PHILOX) fp.init(p.key, p.run0 + (uint64_t)r, g.M);
    else perm = p.perms + (size_t)r * g.M;
    const NzRecords rec = p.rec;
    // the next step's site is computed while this step's first load is in
    // flight (on every path, so that it always advances)
    uint32_t i_next = 0;
    {
        const uint32_t first = p.n_begin > 0 ? p.n_begin - 1u : 0u;
        if (first < g.M) i_next = step_index<PERM>(fp, perm, first);
    }
    for (uint32_t n = p.n_begin; n < p.n_end; ++n) {
        uint32_t i = 0;
        if (n > 0) {
            i = i_next;
            bool advanced = false;
            // a caller-supplied index out of range or repeated occupies nothing
            if (KIND == NZ_GRAPH_GRID2D && i < g.N) {
                // node words in the grid's tiled layout (grid_slot)
                const uint32_t row = i / g.L, col = i - row * g.L;
                auto slot = [&](uint32_t rr, uint32_t cc) {
                    return kGridTiled ? grid_slot(g.tile_cols, rr, cc) : rr * g.L + cc;
                };
                const uint32_t x = slot(row, col);
                const uint32_t wx = node[x];
                if (n < g.M) i_next = step_index<PERM>(fp, perm, n);
                advanced = true;
                if (wx == kEmpty) {
                    const uint32_t sides = node_sides<KIND>(g, i);
                    node[x] = make_root(1u, sides);
                    t.add_single();
                    if (SPAN && sides == 3u) t.st.flags |= kFlagSpan;
                    uint32_t y;
                    if (row > 0 && node[y = slot(row - 1u, col)] != kEmpty) link<SPAN>(node, x, y, t);
                    if (row + 1u < g.L && node[y = slot(row + 1u, col)] != kEmpty) link<SPAN>(node, x, y, t);
                    if (col > 0 && node[y = slot(row, col - 1u)] != kEmpty) link<SPAN>(node, x, y, t);
                    if (col + 1u < g.L && node[y = slot(row, col + 1u)] != kEmpty) link<SPAN>(node, x, y, t);
                }
            } else if (KIND != NZ_GRAPH_GRID2D && i < g.N && node[i] == kEmpty) {
                const uint32_t sides = node_sides<KIND>(g, i);
                node[i] = make_root(1u, sides);
                t.add_single();
                if (SPAN && sides == 3u) t.st.flags |= kFlagSpan;
                if (i > 0 && node[i - 1u] != kEmpty) link<SPAN>(node, i, i - 1u, t);
                if (i + 1u < g.N && node[i + 1u] != kEmpty) link<SPAN>(node, i, i + 1u, t);
            }
            if (!advanced && n < g.M) i_next = step_index<PERM>(fp, perm, n);
        }
        const size_t off = (size_t)(n - p.n_begin) * rec.run_stride + r;
        t.write(rec, off, SPAN && (t.st.flags & kFlagSpan), i);
    }
    t.st.max = t.mx;
    p.state[r] = t.st;
    if (p.errors && (t.st.flags & kFlagCorrupt) && p.n_end == g.M + 1u) atomicAdd(p.errors, 1u);
}

// ------------------------------------------------------ torus with wrapping
// cell: x = union-find word, y = dx, z = dy (two's complement), w unused
__device__ __forceinline__ bool wraps(uint32_t flags, uint32_t crit) {
    const bool x = (flags & kFlagWrapX) != 0, y = (flags & kFlagWrapY) != 0;
    return crit == 0 ? (x || y) : crit == 1 ? x : crit == 2 ? y : (x && y);
}

// Joins u and v = u + (ddx, ddy); interleaved finds with path splitting that
// keep each node's displacement from its parent.
__device__ __forceinline__ void link_torus(uint4 *cell, uint32_t u, uint32_t v, uint4 cu, uint4 cv,
                                           int32_t ddx, int32_t ddy, Tally &t) {
    // cu, cv: the cells of u and v, loaded by the caller
    uint32_t xu = u, xv = v;
    int32_t pux = 0, puy = 0, pvx = 0, pvy = 0;  // positions relative to the current node
    for (int hops = 0; !(is_root(cu.x) && is_root(cv.x)); ++hops) {
        if (hops >= 64) { t.st.flags |= kFlagCorrupt; return; }
        if (!is_root(cu.x)) {
            const uint32_t par = cu.x;
            const uint4 cp = cell[par];
            pux += (int32_t)cu.y;
            puy += (int32_t)cu.z;
            if (!is_root(cp.x)) cell[xu] = make_uint4(cp.x, cu.y + cp.y, cu.z + cp.z, 0u);
            xu = par;
            cu = cp;
        }
        if (!is_root(cv.x)) {
            const uint32_t par = cv.x;
            const uint4 cp = cell[par];
            pvx += (int32_t)cv.y;
            pvy += (int32_t)cv.z;
            if (!is_root(cp.x)) cell[xv] = make_uint4(cp.x, cv.y + cp.y, cv.z + cp.z, 0u);
            xv = par;
            cv = cp;
        }
    }
    // position of v's root as seen from u's root, were v at pos(u) + delta
    const int32_t ox = pux + ddx - pvx, oy = puy + ddy - pvy;
    if (xu == xv) {
        if (ox != 0) t.st.flags |= kFlagWrapX;
        if (oy != 0) t.st.flags |= kFlagWrapY;
        return;
    }
    const uint32_t a = root_size(cu.x), b = root_size(cv.x);
    if (a >= b) {
        cell[xv] = make_uint4(xu, (uint32_t)ox, (uint32_t)oy, 0u);
        cell[xu] = make_uint4(make_root(a + b, 0u), 0u, 0u, 0u);
    } else {
        cell[xu] = make_uint4(xv, (uint32_t)(-ox), (uint32_t)(-oy), 0u);
        cell[xv] = make_uint4(make_root(a + b, 0u), 0u, 0u, 0u);
    }
    t.merge(a, b);
}

template <bool SITE, int PERM, bool SPAN>
__global__ void __launch_bounds__(256) torus_window_kernel(UfParams p) {
    const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= p.n_runs) return;
    const GraphDev &g = p.g;
    uint4 *cell = reinterpret_cast<uint4 *>(p.nodes) + (size_t)r * g.N;
    Tally t;
    t.load(p.state[r]);
    FeistelPerm fp;
    const uint32_t *perm = nullptr;
    if (PERM == NZ_PERM_PHILOX) fp.init(p.key, p.run0 + (uint64_t)r, g.M);
    else perm = p.perms + (size_t)r * g.M;
    const NzRecords rec = p.rec;
    const uint32_t L = g.L;
    // bond model: the next step's index is computed while this step's first
    // loads are in flight (7.3e9 against 7.0e9 bond additions/s at L = 256);
    // the site model measured 2 % slower that way and computes it in place
    uint32_t e_next = 0;
    if (!SITE) {
        const uint32_t first = p.n_begin > 0 ? p.n_begin - 1u : 0u;
        if (first < g.M) e_next = step_index<PERM>(fp, perm, first);
    }
    for (uint32_t n = p.n_begin; n < p.n_end; ++n) {
        uint32_t e = 0;
        if (n > 0) {
            bool advanced = false;
            if (SITE) {
                e = step_index<PERM>(fp, perm, n - 1u);
                if (e < g.N) {
                    const uint4 ce = cell[e];
                    if (ce.x == kEmpty) {
                        const uint4 occupied = make_uint4(make_root(1u, 0u), 0u, 0u, 0u);
                        cell[e] = occupied;
                        t.add_single();
                        const uint32_t row = e / L, col = e - row * L;
                        const uint32_t right = row * L + (col + 1u == L ? 0u : col + 1u);
                        const uint32_t left = row * L + (col == 0u ? L - 1u : col - 1u);
                        const uint32_t down = (row + 1u == L ? 0u : row + 1u) * L + col;
                        const uint32_t up = (row == 0u ? L - 1u : row - 1u) * L + col;
                        // this site's cell is re-read for every link: an earlier link
                        // may have hung it below another root
                        if (cell[right].x != kEmpty) link_torus(cell, e, right, cell[e], cell[right], 1, 0, t);
                        if (cell[left].x != kEmpty) link_torus(cell, e, left, cell[e], cell[left], -1, 0, t);
                        if (cell[down].x != kEmpty) link_torus(cell, e, down, cell[e], cell[down], 0, 1, t);
                        if (cell[up].x != kEmpty) link_torus(cell, e, up, cell[e], cell[up], 0, -1, t);
                    }
                }
            } else if ((e = e_next) < g.M) {
                const bool vertical = e >= g.N;
                const uint32_t u = vertical ? e - g.N : e;
                const uint32_t row = u / L, col = u - row * L;
                const uint32_t v = vertical ? (row + 1u == L ? 0u : row + 1u) * L + col
                                            : row * L + (col + 1u == L ? 0u : col + 1u);
                const uint4 cu = cell[u], cv = cell[v];
                if (n < g.M) e_next = step_index<PERM>(fp, perm, n);
                advanced = true;
                link_torus(cell, u, v, cu, cv, vertical ? 0 : 1, vertical ? 1 : 0, t);
            }
            if (!SITE && !advanced && n < g.M) e_next = step_index<PERM>(fp, perm, n);
        }
        const size_t off = (size_t)(n - p.n_begin) * rec.run_stride + r;
        t.write(rec, off, SPAN && wraps(t.st.flags, g.wrap), e);
    }
    t.st.max = t.mx;
    p.state[r] = t.st;
    if (p.errors && (t.st.flags & kFlagCorrupt) && p.n_end == g.M + 1u) atomicAdd(p.errors, 1u);
}

// ------------------------------------------------------------ initialisers
__global__ void init_site_nodes_kernel(uint64_t total, uint32_t *nodes) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x)
        nodes[i] = kEmpty;
}

__global__ void init_torus_cells_kernel(uint64_t total, uint32_t word, uint4 *cells) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x)
        cells[i] = make_uint4(word, 0u, 0u, 0u);
}

// bond model: N clusters of one node; site model: nothing occupied
__global__ void init_lattice_state_kernel(int32_t n_runs, uint32_t N, uint32_t site, RunState *state) {
    const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_runs) return;
    RunState s;
    const uint32_t c = site ? 0u : N;
    s.t2 = c; s.t3 = c; s.t4_lo = c; s.t4_hi = 0;
    s.t0 = c; s.max = site ? 0u : 1u; s.flags = 0u; s.pad = 0;
    state[r] = s;
}

unsigned grid_for(uint64_t total) {
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152ull * 64) blocks = 152ull * 64;
    return (unsigned)(blocks ? blocks : 1);
}

template <int KIND, int PERM>
void launch_site_k(const UfParams &p, bool span, int block, cudaStream_t s) {
    dim3 grid((p.n_runs + block - 1) / block);
    if (span) site_window_kernel<KIND, PERM, true><<<grid, block, 0, s>>>(p);
    else site_window_kernel<KIND, PERM, false><<<grid, block, 0, s>>>(p);
}

template <bool SITE, int PERM>
void launch_torus_k(const UfParams &p, bool span, int block, cudaStream_t s) {
    dim3 grid((p.n_runs + block - 1) / block);
    if (span) torus_window_kernel<SITE, PERM, true><<<grid, block, 0, s>>>(p);
    else torus_window_kernel<SITE, PERM, false><<<grid, block, 0, s>>>(p);
}

template <int PERM>
void launch_lattice_perm(const UfParams &p, bool span, int block, cudaStream_t s) {
    if (p.g.kind == NZ_GRAPH_TORUS2D) {
        if (p.g.site) launch_torus_k<true, PERM>(p, span, block, s);
        else launch_torus_k<false, PERM>(p, span, block, s);
    } else if (p.g.kind == NZ_GRAPH_GRID2D) {
        launch_site_k<NZ_GRAPH_GRID2D, PERM>(p, span, block, s);
    } else {
        launch_site_k<NZ_GRAPH_CHAIN1D, PERM>(p, span, block, s);
    }
}

}  // namespace

bool lattice_extension(const GraphDev &g) { return g.site || g.kind == NZ_GRAPH_TORUS2D; }

void launch_init_lattice_runs(const GraphDev &g, int32_t n_runs, uint32_t *nodes, RunState *state,
                              cudaStream_t s) {
    // every word of the runs' node arrays (the grid's layout has padding slots)
    const uint64_t total = (uint64_t)n_runs * (g.kind == NZ_GRAPH_TORUS2D ? g.N : g.slots);
    if (g.kind == NZ_GRAPH_TORUS2D)
        init_torus_cells_kernel<<<grid_for(total), 256, 0, s>>>(total, g.site ? kEmpty : make_root(1u, 0u),
                                                                 reinterpret_cast<uint4 *>(nodes));
    else
        init_site_nodes_kernel<<<grid_for(total), 256, 0, s>>>(total, nodes);
    init_lattice_state_kernel<<<(n_runs + 255) / 256, 256, 0, s>>>(n_runs, g.N, g.site, state);
}

void launch_lattice_window(const UfParams &p, int perm_mode, bool span, int block, cudaStream_t s) {
    if (perm_mode == NZ_PERM_PHILOX) launch_lattice_perm<NZ_PERM_PHILOX>(p, span, block, s);
    else launch_lattice_perm<NZ_PERM_GIVEN>(p, span, block, s);
}

}  // namespace nz
