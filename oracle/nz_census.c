/*
 * nz_census.c -- brute-force cluster census (TEST INFRASTRUCTURE ONLY).
 *
 * Checks the lattice extensions of the GPU library -- site percolation and
 * wrapping on the periodic square lattice, which the reference lists as to-do
 * (percolate/__init__.py:68-78) and does not implement -- by a method that
 * shares nothing with the union-find it checks: after every step the clusters
 * of the current configuration are found from scratch by breadth-first search
 * over occupied sites and open bonds, and the statistics are read off them.
 * O(N + M) per step, so test sizes only.
 *
 * The same census run on the bond model of spanning_2d_grid / spanning_1d_chain
 * reproduces nzo_sample_states (the restatement of percolate/hpc.py:195-307
 * pinned to the reference's own outputs), which pins the method itself.
 *
 * Lattices (node = row * L + col):
 *   kind 0 grid  : L x L open square lattice, edges numbered as networkx lists
 *                  spanning_2d_grid(L).edges() (percolate/percolate.py:931-965);
 *                  side 1 = row 0, side 2 = row L-1
 *   kind 1 chain : path 0 .. L-1, edge e = (e, e+1); side 1 = node 0, side 2 = node L-1
 *   kind 3 torus : L x L periodic; edge e < L*L = (e, right neighbour), else
 *                  (e - L*L, neighbour below)
 * Site model: step n occupies site perm[n-1]; the open bonds are all lattice
 * bonds between occupied sites.  Bond model: step n opens edge perm[n-1].
 *
 * Spanning (grid, chain): a cluster holds a side-1 node and a side-2 node.
 * Wrapping (torus): every BFS visit records the node's unwrapped position;
 * an open bond that reaches a visited node at another position closes a loop
 * that winds around the torus (along x if the x parts differ, y if the y
 * parts do).  crit: 0 either, 1 x, 2 y, 3 both.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

static int neighbours(int kind, uint32_t L, uint32_t i, uint32_t *nb, int32_t *dx, int32_t *dy)
{
    int k = 0;
    if (kind == 1) {
        if (i > 0) { nb[k] = i - 1; dx[k] = -1; dy[k] = 0; ++k; }
        if (i + 1 < L) { nb[k] = i + 1; dx[k] = 1; dy[k] = 0; ++k; }
        return k;
    }
    uint32_t r = i / L, c = i % L;
    if (kind == 0) {
        if (c + 1 < L) { nb[k] = i + 1; dx[k] = 1; dy[k] = 0; ++k; }
        if (c > 0) { nb[k] = i - 1; dx[k] = -1; dy[k] = 0; ++k; }
        if (r + 1 < L) { nb[k] = i + L; dx[k] = 0; dy[k] = 1; ++k; }
        if (r > 0) { nb[k] = i - L; dx[k] = 0; dy[k] = -1; ++k; }
        return k;
    }
    nb[k] = r * L + (c + 1) % L; dx[k] = 1; dy[k] = 0; ++k;
    nb[k] = r * L + (c + L - 1) % L; dx[k] = -1; dy[k] = 0; ++k;
    nb[k] = ((r + 1) % L) * L + c; dx[k] = 0; dy[k] = 1; ++k;
    nb[k] = ((r + L - 1) % L) * L + c; dx[k] = 0; dy[k] = -1; ++k;
    return k;
}

/* bond e of the lattice as (u, v, step from u to v) */
static void edge_nodes(int kind, uint32_t L, uint32_t e, uint32_t *u, uint32_t *v, int32_t *dx, int32_t *dy)
{
    if (kind == 1) { *u = e; *v = e + 1; *dx = 1; *dy = 0; return; }
    if (kind == 0) {
        uint32_t row_edges = (L - 1) * (2 * L - 1);
        if (e < row_edges) {
            uint32_t r = e / (2 * L - 1), w = e % (2 * L - 1);
            *u = r * L + w / 2;
            if (w & 1) { *v = *u + 1; *dx = 1; *dy = 0; }
            else { *v = *u + L; *dx = 0; *dy = 1; }
        } else {
            *u = (L - 1) * L + (e - row_edges);
            *v = *u + 1; *dx = 1; *dy = 0;
        }
        return;
    }
    uint32_t N = L * L;
    if (e < N) { *u = e; *v = (e / L) * L + (e % L + 1) % L; *dx = 1; *dy = 0; }
    else { *u = e - N; *v = (((e - N) / L + 1) % L) * L + (e - N) % L; *dx = 0; *dy = 1; }
}

static uint32_t sides_of(int kind, uint32_t L, uint32_t i)
{
    if (kind == 1) return (i == 0 ? 1u : 0u) | (i == L - 1 ? 2u : 0u);
    if (kind == 0) return (i / L == 0 ? 1u : 0u) | (i / L == L - 1 ? 2u : 0u);
    return 0u;
}

/* Rows n = 0 .. steps of one run; steps = N (site) or M (bond).  Returns 0,
 * or -1 for an unknown lattice / allocation failure. */
int nzo_lattice_census(int kind, uint32_t L, int site, int crit, const uint32_t *perm,
                       uint32_t *max_span, uint32_t *m0, uint64_t *m2, uint64_t *m3,
                       uint64_t *m4_lo, uint32_t *m4_hi)
{
    if ((kind != 0 && kind != 1 && kind != 3) || L == 0) return -1;
    const uint32_t N = kind == 1 ? L : L * L;
    const uint32_t M = kind == 1 ? L - 1 : (kind == 0 ? 2 * L * (L - 1) : 2 * L * L);
    const uint32_t steps = site ? N : M;
    uint8_t *occ = calloc(N, 1), *open = calloc(M ? M : 1, 1);
    int32_t *px = malloc(sizeof(int32_t) * N), *py = malloc(sizeof(int32_t) * N);
    uint32_t *queue = malloc(sizeof(uint32_t) * N);
    uint8_t *seen = malloc(N);
    /* adjacency by bond index for the bond model */
    uint32_t *adj_off = calloc(N + 1, sizeof(uint32_t)), *adj = malloc(sizeof(uint32_t) * 2 * (M ? M : 1));
    if (!occ || !open || !px || !py || !queue || !seen || !adj_off || !adj) return -1;
    for (uint32_t e = 0; e < M; ++e) {
        uint32_t u, v; int32_t dx, dy;
        edge_nodes(kind, L, e, &u, &v, &dx, &dy);
        adj_off[u + 1]++; adj_off[v + 1]++;
    }
    for (uint32_t i = 0; i < N; ++i) adj_off[i + 1] += adj_off[i];
    uint32_t *fill = calloc(N, sizeof(uint32_t));
    for (uint32_t e = 0; e < M; ++e) {
        uint32_t u, v; int32_t dx, dy;
        edge_nodes(kind, L, e, &u, &v, &dx, &dy);
        adj[adj_off[u] + fill[u]++] = e;
        adj[adj_off[v] + fill[v]++] = e;
    }
    free(fill);
    if (!site) memset(occ, 1, N);
    for (uint32_t n = 0; n <= steps; ++n) {
        if (n > 0) {
            uint32_t x = perm[n - 1];
            if (site) { if (x < N) occ[x] = 1; }
            else if (x < M) open[x] = 1;
        }
        memset(seen, 0, N);
        uint64_t clusters = 0;
        uint32_t mx = 0;
        u128 t2 = 0, t3 = 0, t4 = 0;
        int span = 0, wx = 0, wy = 0;
        for (uint32_t s = 0; s < N; ++s) {
            if (!occ[s] || seen[s]) continue;
            uint32_t head = 0, tail = 0, size = 0, sides = 0;
            queue[tail++] = s; seen[s] = 1; px[s] = 0; py[s] = 0;
            while (head < tail) {
                uint32_t a = queue[head++];
                ++size;
                sides |= sides_of(kind, L, a);
                uint32_t nb[4]; int32_t ddx[4], ddy[4];
                int k = 0;
                if (site) {
                    k = neighbours(kind, L, a, nb, ddx, ddy);
                } else {
                    for (uint32_t j = adj_off[a]; j < adj_off[a + 1]; ++j) {
                        uint32_t e = adj[j];
                        if (!open[e]) continue;
                        uint32_t u, v; int32_t dx, dy;
                        edge_nodes(kind, L, e, &u, &v, &dx, &dy);
                        if (u == a && v == a) {  /* L = 1 torus: a self-loop, which winds */
                            if (dx) wx = 1;
                            if (dy) wy = 1;
                            continue;
                        }
                        /* (on the L = 2 torus two bonds join the same pair of
                         * nodes; each is its own adjacency entry) */
                        uint32_t other = u == a ? v : u;
                        int32_t sx = u == a ? dx : -dx, sy = u == a ? dy : -dy;
                        if (!seen[other]) {
                            seen[other] = 1; px[other] = px[a] + sx; py[other] = py[a] + sy;
                            queue[tail++] = other;
                        } else {
                            if (px[other] != px[a] + sx) wx = 1;
                            if (py[other] != py[a] + sy) wy = 1;
                        }
                    }
                    continue;
                }
                for (int j = 0; j < k; ++j) {
                    uint32_t b = nb[j];
                    if (!occ[b]) continue;
                    if (b == a) {  /* L = 1 torus: a site is its own neighbour */
                        if (ddx[j]) wx = 1;
                        if (ddy[j]) wy = 1;
                        continue;
                    }
                    if (!seen[b]) {
                        seen[b] = 1; px[b] = px[a] + ddx[j]; py[b] = py[a] + ddy[j];
                        queue[tail++] = b;
                    } else {
                        if (px[b] != px[a] + ddx[j]) wx = 1;
                        if (py[b] != py[a] + ddy[j]) wy = 1;
                    }
                }
            }
            ++clusters;
            if (size > mx) mx = size;
            u128 s2 = (u128)size * size;
            t2 += s2; t3 += s2 * size; t4 += s2 * s2;
            if (sides == 3u) span = 1;
        }
        if (kind == 3) {
            span = crit == 0 ? (wx || wy) : crit == 1 ? wx : crit == 2 ? wy : (wx && wy);
        }
        u128 mx2 = (u128)mx * mx;
        u128 r4 = t4 - mx2 * mx2;
        max_span[n] = mx | (span ? 0x80000000u : 0u);
        m0[n] = (uint32_t)(clusters ? clusters - 1 : 0);
        m2[n] = (uint64_t)(t2 - mx2);
        m3[n] = (uint64_t)(t3 - mx2 * mx);
        m4_lo[n] = (uint64_t)r4;
        m4_hi[n] = (uint32_t)(r4 >> 64);
    }
    free(occ); free(open); free(px); free(py); free(queue); free(seen); free(adj_off); free(adj);
    return 0;
}
