/*
 * nz_oracle.c -- CPU oracle for the Newman-Ziff bond-percolation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA path is
 * compared against; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline / reference arm load it.  The product library never links it.
 *
 * It restates, in plain C with exact integers, the reference algorithm of
 * andsor/pypercolate 0.4.6:
 *
 *   percolate/hpc.py:73-307    bond_sample_states (the Newman-Ziff loop)
 *   percolate/hpc.py:310-404   bond_microcanonical_statistics (M+1 rows)
 *   percolate/hpc.py:443-515   bond_canonical_statistics (FP64 dot products)
 *   percolate/hpc.py:638-702   bond_reduce (pairwise mean/M2 merge)
 *   percolate/percolate.py:931-965 / 899-928  spanning_2d_grid / spanning_1d_chain
 *
 * Moments are kept as exact unsigned 128-bit integers.  The reference stores
 * them as uint64 (hpc.py:68) and its arithmetic wraps modulo 2^64; the low
 * 64 bits of the exact value are what the reference reports.
 *
 * Random permutations (three sources, all restated from published methods):
 *   - Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
 *     as easy as 1, 2, 3", SC'11) keys an alternating Feistel bijection
 *     with cycle walking: the project's permutation of [0, M).
 *   - MT19937 (Matsumoto & Nishimura, ACM TOMACS 8(1), 1998) with the
 *     authors' init_genrand / init_by_array seeding, followed by the
 *     Fisher-Yates shuffle with masked rejection sampling that numpy's legacy
 *     RandomState.permutation uses.  This reproduces
 *     np.random.RandomState(seed).permutation(M) (hpc.py:195,206).
 *   - a caller-supplied permutation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* Philox-4x32-10                                                      */
/* ------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void nzo_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                       uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ------------------------------------------------------------------ */
/* Philox-keyed Feistel permutation of [0, M)                          */
/* ------------------------------------------------------------------ */
/* Alternating Feistel network on b = bits(M-1) bits: left part floor(b/2)
 * bits, right part the rest; even rounds xor the left part with a keyed hash
 * of the right part, odd rounds the other way round; 8 rounds; the hash of a
 * value v to o bits is the top o bits of lowbias32(v ^ k).  Values >= M are
 * re-encrypted (cycle walking), which keeps the map a bijection on [0, M). */
#define NZ_FEISTEL_ROUNDS 8
#define NZ_PERM_TAG 0x5045524Du /* "PERM" */

typedef struct {
    uint32_t M, hl, hr, maskL, maskR;
    uint32_t k[NZ_FEISTEL_ROUNDS];
} nzo_perm_t;

void nzo_perm_init(nzo_perm_t *st, uint64_t key, uint64_t run_id, uint32_t M)
{
    uint32_t bits = 0;
    if (M > 1) {
        uint32_t x = M - 1;
        while (x) { ++bits; x >>= 1; }
    }
    st->M = M;
    st->hl = bits / 2;
    st->hr = bits - st->hl;
    st->maskL = (1u << st->hl) - 1u;
    st->maskR = (1u << st->hr) - 1u;
    uint32_t kk[2] = {(uint32_t)key, (uint32_t)(key >> 32)};
    for (uint32_t half = 0; half < 2; ++half) {
        uint32_t ctr[4] = {(uint32_t)run_id, (uint32_t)(run_id >> 32), half,
                           NZ_PERM_TAG};
        nzo_philox4x32_10(ctr, kk, &st->k[4 * half]);
    }
}

/* lowbias32: C. Wellons' xorshift-multiply integer hash (hash-prospector) */
static inline uint32_t nzo_lowbias32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

static inline uint32_t nzo_feistel_f(uint32_t v, uint32_t obits, uint32_t k)
{
    return obits ? (nzo_lowbias32(v ^ k) >> (32u - obits)) : 0u;
}

static inline uint32_t nzo_feistel(const nzo_perm_t *st, uint32_t x)
{
    uint32_t L = x >> st->hr, R = x & st->maskR;
    for (int i = 0; i < NZ_FEISTEL_ROUNDS; i += 2) {
        L ^= nzo_feistel_f(R, st->hl, st->k[i]) & st->maskL;
        R ^= nzo_feistel_f(L, st->hr, st->k[i + 1]) & st->maskR;
    }
    return (L << st->hr) | R;
}

uint32_t nzo_perm_at(const nzo_perm_t *st, uint32_t n)
{
    uint32_t x = n;
    do {
        x = nzo_feistel(st, x);
    } while (x >= st->M);
    return x;
}

void nzo_philox_permutation(uint64_t key, uint64_t run_id, uint32_t M,
                            uint32_t *out)
{
    nzo_perm_t st;
    nzo_perm_init(&st, key, run_id, M);
    for (uint32_t n = 0; n < M; ++n) out[n] = nzo_perm_at(&st, n);
}

/* ------------------------------------------------------------------ */
/* MT19937 + numpy legacy permutation                                   */
/* ------------------------------------------------------------------ */
#define MT_N 624
#define MT_M 397

typedef struct {
    uint32_t mt[MT_N];
    int mti;
} nzo_mt_t;

static void mt_init_genrand(nzo_mt_t *s, uint32_t seed)
{
    s->mt[0] = seed;
    for (int i = 1; i < MT_N; ++i)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->mti = MT_N;
}

static void mt_init_by_array(nzo_mt_t *s, const uint32_t *key, int len)
{
    mt_init_genrand(s, 19650218u);
    int i = 1, j = 0;
    int k = (MT_N > len) ? MT_N : len;
    for (; k; --k) {
        s->mt[i] = (s->mt[i] ^ ((s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) * 1664525u))
                   + key[j] + (uint32_t)j;
        ++i; ++j;
        if (i >= MT_N) { s->mt[0] = s->mt[MT_N - 1]; i = 1; }
        if (j >= len) j = 0;
    }
    for (k = MT_N - 1; k; --k) {
        s->mt[i] = (s->mt[i] ^ ((s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) * 1566083941u))
                   - (uint32_t)i;
        ++i;
        if (i >= MT_N) { s->mt[0] = s->mt[MT_N - 1]; i = 1; }
    }
    s->mt[0] = 0x80000000u;
    s->mti = MT_N;
}

static uint32_t mt_next(nzo_mt_t *s)
{
    if (s->mti >= MT_N) {
        for (int kk = 0; kk < MT_N; ++kk) {
            uint32_t y = (s->mt[kk] & 0x80000000u) |
                         (s->mt[(kk + 1) % MT_N] & 0x7fffffffu);
            s->mt[kk] = s->mt[(kk + MT_M) % MT_N] ^ (y >> 1) ^
                        ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        s->mti = 0;
    }
    uint32_t y = s->mt[s->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

/* n_words == 0: scalar seed seed_words[0] -> init_genrand;
 * n_words >= 1: array seed -> init_by_array (numpy's legacy seeding). */
void nzo_mt_permutation(const uint32_t *seed_words, int n_words, uint32_t M,
                        uint32_t *out)
{
    nzo_mt_t s;
    if (n_words == 0) mt_init_genrand(&s, seed_words[0]);
    else mt_init_by_array(&s, seed_words, n_words);
    for (uint32_t i = 0; i < M; ++i) out[i] = i;
    for (int64_t i = (int64_t)M - 1; i >= 1; --i) {
        uint32_t max = (uint32_t)i, mask = max;
        mask |= mask >> 1; mask |= mask >> 2; mask |= mask >> 4;
        mask |= mask >> 8; mask |= mask >> 16;
        uint32_t j;
        while ((j = (mt_next(&s) & mask)) > max) {}
        uint32_t t = out[i]; out[i] = out[j]; out[j] = t;
    }
}

/* ------------------------------------------------------------------ */
/* Substrate lattices (implicit edge numbering)                        */
/* ------------------------------------------------------------------ */
/* kind 0: spanning_2d_grid(L)  (percolate/percolate.py:931-965)
 *   perc node (i, j), i = 1..L, j = 0..L-1  ->  index (i-1)*L + j.
 *   Edge order is that of networkx >= 2 for perc_graph.edges(): node-major,
 *   for each node first the edge to (i+1, j), then the edge to (i, j+1).
 *   Side 0 = perc row 1, side 1 = perc row L.  N = L^2, M = 2L(L-1).
 * kind 1: spanning_1d_chain(l)  (percolate/percolate.py:899-928)
 *   perc node k = 1..l -> index k-1; edge e joins e and e+1.
 *   Side 0 = node 0, side 1 = node l-1.  N = l, M = l-1. */
int nzo_lattice_size(int kind, uint32_t L, uint32_t *N, uint32_t *M)
{
    if (L == 0) return 1;
    if (kind == 0) { *N = L * L; *M = 2u * L * (L - 1u); return 0; }
    if (kind == 1) { *N = L; *M = L - 1u; return 0; }
    return 1;
}

int nzo_lattice_graph(int kind, uint32_t L, uint32_t *eu, uint32_t *ev,
                      uint8_t *side)
{
    uint32_t N, M;
    if (nzo_lattice_size(kind, L, &N, &M)) return 1;
    if (kind == 0) {
        uint32_t e = 0;
        for (uint32_t r = 0; r < L; ++r)
            for (uint32_t c = 0; c < L; ++c) {
                uint32_t k = r * L + c;
                if (r + 1 < L) { eu[e] = k; ev[e] = k + L; ++e; }
                if (c + 1 < L) { eu[e] = k; ev[e] = k + 1; ++e; }
            }
        for (uint32_t k = 0; k < N; ++k) {
            uint32_t r = k / L;
            side[k] = (uint8_t)((r == 0 ? 1u : 0u) | (r == L - 1 ? 2u : 0u));
        }
    } else {
        for (uint32_t e = 0; e < M; ++e) { eu[e] = e; ev[e] = e + 1; }
        for (uint32_t k = 0; k < N; ++k)
            side[k] = (uint8_t)((k == 0 ? 1u : 0u) | (k == L - 1 ? 2u : 0u));
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Union-find (weighted by size, full path compression)                */
/* ------------------------------------------------------------------ */
static uint32_t uf_find(uint32_t *parent, uint32_t x)
{
    uint32_t r = x;
    while (parent[r] != r) r = parent[r];
    while (parent[x] != r) { uint32_t nx = parent[x]; parent[x] = r; x = nx; }
    return r;
}

/* ------------------------------------------------------------------ */
/* bond_sample_states restated (percolate/hpc.py:195-307)               */
/* ------------------------------------------------------------------ */
/* Outputs, one entry per n = 0..M (arrays of length M+1; any may be NULL):
 *   edge[n], max_size[n], span[n] (0/1), mom_lo[5*n+k] (low 64 bits),
 *   mom_hi[5*n+k] (high 64 bits of the exact moment).
 * Returns 0, or 2 when spanning is requested but no node touches one of the
 * two sides (the reference raises ValueError for != 2 sides). */
int nzo_sample_states(uint32_t N, uint32_t M, const uint32_t *eu,
                      const uint32_t *ev, const uint8_t *side, int spanning,
                      const uint32_t *perm, uint32_t *edge_out,
                      uint32_t *max_out, uint8_t *span_out, uint64_t *mom_lo,
                      uint64_t *mom_hi)
{
    if (N == 0) return 1;
    uint32_t *parent = (uint32_t *)malloc(sizeof(uint32_t) * N);
    uint32_t *weight = (uint32_t *)malloc(sizeof(uint32_t) * N);
    uint32_t *sp = NULL; /* spanning UF over N perc nodes + 2 side nodes */
    uint32_t *sw = NULL;
    if (!parent || !weight) { free(parent); free(weight); return 3; }
    for (uint32_t i = 0; i < N; ++i) { parent[i] = i; weight[i] = 1; }

    u128 moments[5];
    for (int k = 0; k < 5; ++k) moments[k] = (u128)(N - 1);
    uint32_t max_size = 1;
    int has_span = 0;

    /* n == 0 row (hpc.py:209-221); edge is undefined there, reported as 0 */
#define EMIT(n, e)                                                         \
    do {                                                                   \
        if (edge_out) edge_out[n] = (e);                                   \
        if (max_out) max_out[n] = max_size;                                \
        if (span_out) span_out[n] = (uint8_t)has_span;                     \
        for (int k_ = 0; k_ < 5; ++k_) {                                   \
            if (mom_lo) mom_lo[5 * (size_t)(n) + k_] = (uint64_t)moments[k_]; \
            if (mom_hi) mom_hi[5 * (size_t)(n) + k_] =                     \
                (uint64_t)(moments[k_] >> 64);                             \
        }                                                                  \
    } while (0)

    if (spanning) {
        int s0 = 0, s1 = 0;
        for (uint32_t i = 0; i < N; ++i) { s0 |= side[i] & 1; s1 |= (side[i] >> 1) & 1; }
        if (!(s0 && s1)) { free(parent); free(weight); return 2; }
        sp = (uint32_t *)malloc(sizeof(uint32_t) * (N + 2));
        sw = (uint32_t *)malloc(sizeof(uint32_t) * (N + 2));
        for (uint32_t i = 0; i < N + 2; ++i) { sp[i] = i; sw[i] = 1; }
        /* hpc.py:230-239: every boundary node joins its side's set */
        for (uint32_t i = 0; i < N; ++i)
            for (uint32_t s = 0; s < 2; ++s)
                if (side[i] & (1u << s)) {
                    uint32_t a = uf_find(sp, i), b = uf_find(sp, N + s);
                    if (a != b) {
                        if (sw[a] < sw[b]) { uint32_t t = a; a = b; b = t; }
                        sp[b] = a; sw[a] += sw[b];
                    }
                }
    }
    EMIT(0, 0u);

    uint32_t max_root = 0; /* hpc.py:246: the first perc node */
    for (uint32_t n = 0; n < M; ++n) {
        uint32_t e = perm[n];
        uint32_t r0 = uf_find(parent, eu[e]), r1 = uf_find(parent, ev[e]);
        uint32_t w0 = weight[r0], w1 = weight[r1];
        if (r0 != r1) {
            /* weighted union: the heavier root survives */
            uint32_t big = r0, small = r1;
            if (w0 < w1) { big = r1; small = r0; }
            parent[small] = big;
            weight[big] = w0 + w1;
            if (spanning) {
                uint32_t a = uf_find(sp, r0), b = uf_find(sp, r1);
                if (a != b) {
                    if (sw[a] < sw[b]) { uint32_t t = a; a = b; b = t; }
                    sp[b] = a; sw[a] += sw[b];
                }
                has_span = uf_find(sp, N) == uf_find(sp, N + 1);
            }
            uint32_t root = big;
            uint32_t w = w0 + w1;
            /* hpc.py:283-286: deduct the merged non-maximum clusters */
            uint32_t ws[2] = {w0, w1};
            uint32_t rs[2] = {r0, r1};
            for (int i = 0; i < 2; ++i) {
                if (rs[i] == max_root) continue;
                u128 p = 1;
                for (int k = 0; k < 5; ++k) { moments[k] -= p; p *= ws[i]; }
            }
            if (r0 == max_root || r1 == max_root) {
                max_root = root; /* hpc.py:288-291 */
                max_size = w;
            } else if (max_size >= w) {
                u128 p = 1; /* hpc.py:294-297 */
                for (int k = 0; k < 5; ++k) { moments[k] += p; p *= w; }
            } else {
                max_root = root; /* hpc.py:298-305 */
                u128 p = 1;
                for (int k = 0; k < 5; ++k) { moments[k] += p; p *= max_size; }
                max_size = w;
            }
        }
        EMIT(n + 1, e);
    }
#undef EMIT
    free(parent); free(weight); free(sp); free(sw);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Canonical weights (FP64) and convolution                             */
/* ------------------------------------------------------------------ */
/* Log binomial pmf log B(M, n, p) from lgamma.  The reference builds the pmf
 * by the Newman-Ziff recursion (percolate/percolate.py:1092-1109) and
 * normalises by the sum; the normalised weights agree to rounding. */
static double log_binom(uint32_t M, uint32_t n, double p)
{
    double lp = (n == 0) ? 0.0 : (double)n * log(p);
    double lq = (n == M) ? 0.0 : (double)(M - n) * log1p(-p);
    return lgamma((double)M + 1.0) - lgamma((double)n + 1.0) -
           lgamma((double)(M - n) + 1.0) + lp + lq;
}

/* Normalised weights over the band where log B >= log B(mode) - cutoff.
 * Writes band [lo, lo+len) and w[0..len).  cap = capacity of w. */
int nzo_binomial_band(uint32_t M, double p, double cutoff, uint32_t cap,
                      uint32_t *lo_out, uint32_t *len_out, double *w)
{
    if (p <= 0.0) { *lo_out = 0; *len_out = 1; if (cap < 1) return 1; w[0] = 1.0; return 0; }
    if (p >= 1.0) { *lo_out = M; *len_out = 1; if (cap < 1) return 1; w[0] = 1.0; return 0; }
    uint32_t mode = (uint32_t)floor((double)(M + 1) * p);
    if (mode > M) mode = M;
    double lm = log_binom(M, mode, p);
    uint32_t lo = mode, hi = mode;
    while (lo > 0 && log_binom(M, lo - 1, p) >= lm - cutoff) --lo;
    while (hi < M && log_binom(M, hi + 1, p) >= lm - cutoff) ++hi;
    uint32_t len = hi - lo + 1;
    if (len > cap) return 1;
    double s = 0.0;
    for (uint32_t i = 0; i < len; ++i) { w[i] = exp(log_binom(M, lo + i, p) - lm); s += w[i]; }
    for (uint32_t i = 0; i < len; ++i) w[i] /= s;
    *lo_out = lo; *len_out = len;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Ensemble pipeline on the host cores (CPU baseline)                   */
/* ------------------------------------------------------------------ */
/* For each run: Philox-Feistel permutation -> sample states -> for each p
 * the 7 canonical statistics (hpc.py:495-512) over the weight band -> a
 * pairwise mean/M2 merge across runs (hpc.py:638-702).  Runs are split over
 * n_threads POSIX threads; per-thread partials are merged at the end.
 * Output: mean[P*7], m2[P*7] with statistic order
 *   (spanning, max, m0, m1, m2, m3, m4). */
typedef struct {
    int kind; uint32_t L; uint64_t key; uint64_t run0; uint32_t n_runs;
    uint32_t P; const uint32_t *band_lo; const uint32_t *band_len;
    const double *w; uint32_t wcap;
    double *mean; double *m2; uint64_t count;
    int status;
} nzo_ens_job;

static void *ens_worker(void *arg)
{
    nzo_ens_job *job = (nzo_ens_job *)arg;
    uint32_t N, M;
    nzo_lattice_size(job->kind, job->L, &N, &M);
    uint32_t *eu = malloc(sizeof(uint32_t) * (M ? M : 1));
    uint32_t *ev = malloc(sizeof(uint32_t) * (M ? M : 1));
    uint8_t *side = malloc(N);
    uint32_t *perm = malloc(sizeof(uint32_t) * (M ? M : 1));
    uint32_t *mx = malloc(sizeof(uint32_t) * (M + 1));
    uint8_t *sp = malloc(M + 1);
    uint64_t *lo = malloc(sizeof(uint64_t) * 5 * (M + 1));
    uint64_t *hi = malloc(sizeof(uint64_t) * 5 * (M + 1));
    double *q = malloc(sizeof(double) * 7 * (M + 1));
    nzo_lattice_graph(job->kind, job->L, eu, ev, side);
    job->count = 0;
    for (uint32_t i = 0; i < job->P * 7; ++i) { job->mean[i] = 0; job->m2[i] = 0; }
    for (uint32_t r = 0; r < job->n_runs; ++r) {
        nzo_philox_permutation(job->key, job->run0 + r, M, perm);
        int st = nzo_sample_states(N, M, eu, ev, side, 1, perm, NULL, mx, sp, lo, hi);
        if (st) { job->status = st; break; }
        for (uint32_t n = 0; n <= M; ++n) {
            double *qn = q + 7 * (size_t)n;
            qn[0] = sp[n];
            qn[1] = mx[n];
            for (int k = 0; k < 5; ++k)
                qn[2 + k] = ldexp((double)hi[5 * (size_t)n + k], 64) + (double)lo[5 * (size_t)n + k];
        }
        double cnt = (double)(job->count + 1);
        for (uint32_t p = 0; p < job->P; ++p) {
            double acc[7] = {0, 0, 0, 0, 0, 0, 0};
            const double *w = job->w + (size_t)p * job->wcap;
            uint32_t b0 = job->band_lo[p], bl = job->band_len[p];
            for (uint32_t i = 0; i < bl; ++i) {
                const double *qn = q + 7 * (size_t)(b0 + i);
                for (int s = 0; s < 7; ++s) acc[s] += w[i] * qn[s];
            }
            for (int s = 0; s < 7; ++s) { /* Welford step == merge with (1, x, 0) */
                double *mu = &job->mean[p * 7 + s], *mm = &job->m2[p * 7 + s];
                double d = acc[s] - *mu;
                *mu += d / cnt;
                *mm += d * (acc[s] - *mu);
            }
        }
        job->count += 1;
    }
    free(eu); free(ev); free(side); free(perm); free(mx); free(sp);
    free(lo); free(hi); free(q);
    return NULL;
}

int nzo_ensemble_canonical(int kind, uint32_t L, uint64_t key, uint64_t run0,
                           uint32_t n_runs, uint32_t P, const uint32_t *band_lo,
                           const uint32_t *band_len, const double *w,
                           uint32_t wcap, int n_threads, double *mean_out,
                           double *m2_out)
{
    uint32_t N, M;
    if (nzo_lattice_size(kind, L, &N, &M)) return 1;
    if (n_threads < 1) n_threads = 1;
    if ((uint32_t)n_threads > n_runs) n_threads = (int)(n_runs ? n_runs : 1);
    nzo_ens_job *jobs = calloc((size_t)n_threads, sizeof(nzo_ens_job));
    pthread_t *th = calloc((size_t)n_threads, sizeof(pthread_t));
    uint32_t base = 0;
    for (int t = 0; t < n_threads; ++t) {
        uint32_t cnt = n_runs / (uint32_t)n_threads + ((uint32_t)t < n_runs % (uint32_t)n_threads ? 1u : 0u);
        jobs[t] = (nzo_ens_job){kind, L, key, run0 + base, cnt, P, band_lo, band_len, w, wcap,
                                malloc(sizeof(double) * P * 7), malloc(sizeof(double) * P * 7), 0, 0};
        base += cnt;
        pthread_create(&th[t], NULL, ens_worker, &jobs[t]);
    }
    int status = 0;
    double tot = 0;
    for (uint32_t i = 0; i < P * 7; ++i) { mean_out[i] = 0; m2_out[i] = 0; }
    for (int t = 0; t < n_threads; ++t) {
        pthread_join(th[t], NULL);
        if (jobs[t].status) status = jobs[t].status;
        double nb = (double)jobs[t].count;
        if (nb > 0) { /* pairwise merge (Chan, Golub, LeVeque 1979) */
            double n = tot + nb;
            for (uint32_t i = 0; i < P * 7; ++i) {
                double d = jobs[t].mean[i] - mean_out[i];
                mean_out[i] += d * nb / n;
                m2_out[i] += jobs[t].m2[i] + d * d * tot * nb / n;
            }
            tot = n;
        }
        free(jobs[t].mean); free(jobs[t].m2);
    }
    free(jobs); free(th);
    return status;
}

/* Union-find-only throughput probe: runs n_runs runs (sample states with no
 * per-step output kept beyond a rolling checksum).  Returns a checksum of the
 * final-step statistics so the work cannot be elided. */
typedef struct { int kind; uint32_t L; uint64_t key; uint64_t run0; uint32_t n; uint64_t sum; } nzo_uf_job;

static void *uf_worker(void *arg)
{
    nzo_uf_job *j = (nzo_uf_job *)arg;
    uint32_t N, M;
    nzo_lattice_size(j->kind, j->L, &N, &M);
    uint32_t *eu = malloc(4 * (size_t)(M ? M : 1)), *ev = malloc(4 * (size_t)(M ? M : 1));
    uint8_t *side = malloc(N);
    uint32_t *perm = malloc(4 * (size_t)(M ? M : 1));
    uint32_t *mx = malloc(4 * (size_t)(M + 1));
    nzo_lattice_graph(j->kind, j->L, eu, ev, side);
    j->sum = 0;
    for (uint32_t r = 0; r < j->n; ++r) {
        nzo_philox_permutation(j->key, j->run0 + r, M, perm);
        nzo_sample_states(N, M, eu, ev, side, 1, perm, NULL, mx, NULL, NULL, NULL);
        j->sum += mx[M / 2];
    }
    free(eu); free(ev); free(side); free(perm); free(mx);
    return NULL;
}

uint64_t nzo_ensemble_uf(int kind, uint32_t L, uint64_t key, uint64_t run0,
                         uint32_t n_runs, int n_threads)
{
    if (n_threads < 1) n_threads = 1;
    nzo_uf_job *jobs = calloc((size_t)n_threads, sizeof(nzo_uf_job));
    pthread_t *th = calloc((size_t)n_threads, sizeof(pthread_t));
    uint32_t base = 0;
    for (int t = 0; t < n_threads; ++t) {
        uint32_t cnt = n_runs / (uint32_t)n_threads + ((uint32_t)t < n_runs % (uint32_t)n_threads ? 1u : 0u);
        jobs[t] = (nzo_uf_job){kind, L, key, run0 + base, cnt, 0};
        base += cnt;
        pthread_create(&th[t], NULL, uf_worker, &jobs[t]);
    }
    uint64_t s = 0;
    for (int t = 0; t < n_threads; ++t) { pthread_join(th[t], NULL); s += jobs[t].sum; }
    free(jobs); free(th);
    return s;
}
