/*
 * nz_gb300.h -- C ABI of the GB300 Newman-Ziff bond-percolation library
 * (libnzgb300.so, sources in pypercolate_gb300/csrc/).
 *
 * The library replaces the `percolate.hpc` path of andsor/pypercolate 0.4.6.
 * Every entry point:
 *   - takes plain pointers and sizes (device pointers unless a name says
 *     "host"), never throws, and returns an NZ_* status code;
 *   - is stream-ordered on the `stream` argument (a cudaStream_t, NULL = the
 *     legacy default stream) and does not synchronise unless stated;
 *   - allocates no device memory: the caller owns every buffer, including
 *     scratch, whose size the *_workspace_bytes functions report (nz_ensemble
 *     keeps CUDA stream and event handles of its own, see there).
 * Calls on one stream are serialised by the stream; concurrent calls on
 * different streams must not share output or workspace buffers.
 *
 * Statistic order used by all canonical entry points (7 per p):
 *   0 percolation_probability (spanning), 1 max_cluster_size,
 *   2..6 moments k = 0..4 (largest cluster excluded).
 */
#ifndef NZ_GB300_H
#define NZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------- */
#define NZ_OK 0
#define NZ_ERR_INVALID 1        /* invalid argument (Python: ValueError)       */
#define NZ_ERR_SPANNING_SIDES 2 /* spanning requested, graph lacks two sides
                                   (percolate/hpc.py:197-202: ValueError);
                                   reserved: the sides are graph attributes,
                                   checked by the host layer before a call   */
#define NZ_ERR_TOO_LARGE 3      /* beyond a documented size limit              */
#define NZ_ERR_CUDA 4           /* a CUDA runtime call failed                  */
#define NZ_ERR_WORKSPACE 5      /* workspace smaller than required             */

/* ---- graph kinds ---------------------------------------------------- */
#define NZ_GRAPH_GRID2D 0  /* spanning_2d_grid(L), percolate/percolate.py:931-965 */
#define NZ_GRAPH_CHAIN1D 1 /* spanning_1d_chain(l), percolate/percolate.py:899-928 */
#define NZ_GRAPH_EDGES 2   /* explicit edge list (any perc_graph)              */
#define NZ_GRAPH_TORUS2D 3 /* L x L periodic square lattice: bond e < L*L joins
                              node e = row*L + col to (row, col+1 mod L), bond
                              e >= L*L joins node e - L*L to (row+1 mod L, col);
                              N = L^2, M = 2 L^2.  The "spanning" flag of its
                              records means that a cluster wraps around the
                              torus (criterion: NZ_WRAP_*).  No counterpart in
                              the reference.                                */
#define NZ_KIND_MASK 0xFF

/* Flags or'ed into NzGraph.kind: extensions that the reference lists as
 * to-do (percolate/__init__.py:68-78; percolate/percolate.py:210-211 rejects
 * any model but 'bond').
 * NZ_MODEL_SITE: site percolation on GRID2D, CHAIN1D or TORUS2D -- step n
 *   occupies the n-th site of a permutation of the N sites and joins it to
 *   its occupied neighbours; the number of steps M is then N (nz_graph_size
 *   reports it as num_edges, and every "M" below means the number of steps),
 *   statistics count occupied sites only, and records carry `site` = 1.
 * NZ_WRAP_*: TORUS2D only -- which wrapping sets the flag: a cluster that
 *   wraps along x or y (EITHER, the default), along x (X), along y (Y), or
 *   along both (BOTH), as in Newman & Ziff, Phys. Rev. E 64, 016706 (2001). */
#define NZ_MODEL_SITE 0x100
#define NZ_WRAP_EITHER 0x000
#define NZ_WRAP_X 0x200
#define NZ_WRAP_Y 0x400
#define NZ_WRAP_BOTH 0x600

/* ---- permutation sources -------------------------------------------- */
#define NZ_PERM_PHILOX 0  /* Philox-4x32-10-keyed Feistel bijection: run r uses
                             key `key`, counter run_id = run0 + r             */
#define NZ_PERM_GIVEN 1   /* caller-supplied perms[r * M + n]                 */
#define NZ_PERM_MT19937 2 /* np.random.RandomState(seed).permutation(M),
                             percolate/hpc.py:195,206                         */

/* Size limits (checked; NZ_ERR_TOO_LARGE beyond them). */
#define NZ_MAX_NODES (1u << 21)   /* node ids and exact u64 sums of s^3 */
#define NZ_MAX_RUNS (1u << 24)

/* Graph descriptor.  For NZ_GRAPH_GRID2D / NZ_GRAPH_CHAIN1D only `kind` and
 * `length` are read (N and M are derived); the edge numbering equals the
 * order of networkx's perc_graph.edges() for the reference's builders. */
typedef struct NzGraph {
    int32_t kind;
    uint32_t length;          /* L (grid) or l (chain)                        */
    uint32_t num_nodes;       /* N, NZ_GRAPH_EDGES only                       */
    uint32_t num_edges;       /* M, NZ_GRAPH_EDGES only                       */
    const uint32_t *edge_u;   /* device [M], NZ_GRAPH_EDGES only              */
    const uint32_t *edge_v;   /* device [M]                                   */
    const uint8_t *node_side; /* device [N]: bit 0 touches side 0, bit 1 side 1 */
} NzGraph;

/* Per-step records of one window of steps for a batch of runs.  Each plane
 * is n-major with the run index fastest: element (n, r) is at
 * plane[(n - n_base) * run_stride + r].  Any plane may be NULL. */
typedef struct NzRecords {
    uint32_t *max_span; /* bits 0..30 max cluster size, bit 31 has_spanning   */
    uint32_t *m0;       /* number of clusters - 1                             */
    uint64_t *m2;       /* sum' s^2  (sum over clusters, largest excluded)    */
    uint64_t *m3;       /* sum' s^3                                           */
    uint64_t *m4_lo;    /* sum' s^4, low 64 bits (the reference's uint64)     */
    uint32_t *m4_hi;    /* sum' s^4, bits 64..95                              */
    uint32_t *edge;     /* edge index added at step n (0 at n = 0); site
                           index for site percolation                       */
    int64_t run_stride;
    int32_t site;       /* 0: bond records (m1 = N - max); 1: site records
                           (m1 = n - max: only occupied sites count)         */
    int32_t narrow;     /* 0 in every record set a caller passes.  nz_ensemble
                           sets 1 in its own windows for N <= 65,536, where
                           m0 (< 2^16) is stored as uint16 and m2 (<= N^2/4
                           < 2^31) as uint32 behind the same pointers       */
} NzRecords;

/* ---- library -------------------------------------------------------- */
const char *nz_version(void);
const char *nz_status_string(int status);
/* Fills N and M for a descriptor (host call, no device work). */
int nz_graph_size(const NzGraph *graph, uint32_t *num_nodes, uint32_t *num_edges);

/* ---- microcanonical statistics -------------------------------------- */
/* Replaces percolate/hpc.py:310-404 bond_microcanonical_statistics (and the
 * generator percolate/hpc.py:73-307 bond_sample_states, whose rows are the
 * same) for n_runs independent runs at once.  Writes rows n = 0..M.
 *   spanning      : detect a spanning cluster (needs two sides).
 *   perm_mode     : NZ_PERM_*.
 *   key, run0     : Philox key and first run id (NZ_PERM_PHILOX).
 *   perms         : device [n_runs * M] (NZ_PERM_GIVEN).
 *   mt_seed_words : device [n_runs * mt_words_stride] seed words and
 *   mt_seed_len   : device [n_runs]; len 0 = scalar seed word[0]
 *                   (init_genrand), len k >= 1 = array seed (init_by_array).
 *   workspace     : device scratch of nz_microcanonical_workspace_bytes().
 */
size_t nz_microcanonical_workspace_bytes(const NzGraph *graph, int32_t n_runs,
                                         int32_t perm_mode);
int nz_microcanonical(const NzGraph *graph, int32_t spanning, int32_t n_runs,
                      int32_t perm_mode, uint64_t key, uint64_t run0,
                      const uint32_t *perms, const uint32_t *mt_seed_words,
                      const int32_t *mt_seed_len, int32_t mt_words_stride,
                      void *workspace, size_t workspace_bytes,
                      const NzRecords *out, void *stream);

/* Same computation as nz_microcanonical, for callers that cannot allocate
 * device memory (a host framework that owns the whole device pool, or a
 * foreign-language binding that can only pass buffers it already holds).
 * The scratch nz_microcanonical takes as `workspace` lives instead in a
 * fixed 64 MiB array inside the library (nz_static_scratch_bytes()), which
 * every GPU that loads the library reserves until the process exits; calls
 * needing more (nz_microcanonical_workspace_bytes() > 64 MiB, e.g. more than
 * 255 runs of spanning_2d_grid(256)) return NZ_ERR_TOO_LARGE.  No cudaMalloc,
 * cudaFree or allocating library routine is called (keep the nz_profile_*
 * instrumentation off on this path: when on, it creates CUDA event objects).
 * The array's device address is per CUDA context: the first call in each
 * context (the device's primary context, a context the caller made current,
 * or the new primary context after a cudaDeviceReset) looks it up
 * (cudaGetSymbolAddress) with that context current and caches it under the
 * context's unique ID; make that first call before any stream capture.
 * Every call shares the one array, which keeps the previous call's contents:
 * calls whose execution overlaps on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.
 * (No counterpart in the reference.) */
int nz_microcanonical_noalloc(const NzGraph *graph, int32_t spanning,
                              int32_t n_runs, int32_t perm_mode, uint64_t key,
                              uint64_t run0, const uint32_t *perms,
                              const uint32_t *mt_seed_words,
                              const int32_t *mt_seed_len,
                              int32_t mt_words_stride, const NzRecords *out,
                              void *stream);
size_t nz_static_scratch_bytes(void);

/* Writes the permutations the runs would use (for checking and for
 * NZ_PERM_GIVEN replays): out[r * M + n]. */
int nz_permutations(uint32_t num_edges, int32_t n_runs, int32_t perm_mode,
                    uint64_t key, uint64_t run0, const uint32_t *mt_seed_words,
                    const int32_t *mt_seed_len, int32_t mt_words_stride,
                    uint32_t *out, void *stream);

/* Packs run `run` of a record set into the reference's structured rows
 * (percolate/hpc.py:34-70 microcanonical_statistics_dtype, packed, 53 bytes
 * with the spanning field, 52 without): rows[n * row_bytes ...]. */
int nz_pack_microcanonical_rows(const NzRecords *rec, int32_t run,
                                uint32_t num_nodes, uint32_t num_edges,
                                int32_t spanning, uint8_t *rows, void *stream);

/* ---- canonical statistics ------------------------------------------- */
/* Banded normalised binomial weights B(M, n, p) (percolate/percolate.py:
 * 1067-1109 _binomial_pmf) in FP64 from log-binomials, for P values of p.
 * Band of p_i: n in [band_lo[i], band_lo[i] + band_len[i]), the n where
 * log B >= log B(mode) - cutoff; weights[i * cap + j] for j < band_len[i]
 * (zero-filled to cap).  A band longer than cap is truncated to cap (no
 * error: that would need a host synchronisation); nz_binomial_band_cap()
 * returns a cap no band of (M, cutoff) exceeds. */
int32_t nz_binomial_band_cap(uint32_t num_edges, double cutoff);
int nz_binomial_weights(uint32_t num_edges, const double *ps, int32_t P,
                        double cutoff, int32_t cap, uint32_t *band_lo,
                        uint32_t *band_len, double *weights, void *stream);

/* Full-length FP64 pmf vectors: out[i * (M + 1) + n] (the reference's own
 * convolution_factors layout). */
int nz_binomial_pmf(uint32_t num_edges, const double *ps, int32_t P,
                    double *out, void *stream);

/* Replaces the sums of percolate/percolate.py:1171-1221 (canonical_averages:
 * binomial pmf times every microcanonical average array, confidence bounds
 * included): out[i * cols + c] = sum_j weights[i * cap + j] *
 * values[(band_lo[i] + j) * cols + c] over the band of p_i (rows of the band
 * at or beyond `rows` are skipped), FP64.  values: rows x cols, row-major
 * (one row per n); bands and weights as nz_binomial_weights() writes them
 * (the reference's full-length pmf is zero, in FP64, outside the band of
 * cutoff 745). */
int nz_band_dot(const uint32_t *band_lo, const uint32_t *band_len,
                const double *weights, int32_t cap, int32_t P,
                const double *values, uint32_t rows, int32_t cols,
                double *out, void *stream);

/* Replaces percolate/hpc.py:443-515 bond_canonical_statistics on rows in the
 * reference's packed layout: out[i * 7 + s] = sum_n f_i[n] * Q_s[n] for
 * n_factor_sets full-length factor vectors (factors[i * (M + 1) + n]), FP64. */
int nz_canonical_statistics_rows(const uint8_t *rows, uint32_t num_edges,
                                 int32_t spanning, const double *factors,
                                 int32_t n_factor_sets, double *out,
                                 void *stream);

/* Canonical statistics of records (runs r < n_runs, all n = 0..M), FP64,
 * banded weights: out[(r * P + i) * 7 + s]. */
int nz_canonical_statistics_records(const NzRecords *rec, uint32_t num_nodes,
                                    uint32_t num_edges, int32_t n_runs,
                                    int32_t spanning, const uint32_t *band_lo,
                                    const uint32_t *band_len,
                                    const double *weights, int32_t cap,
                                    int32_t P, double *out, void *stream);

/* ---- averages (n, mean, M2) ------------------------------------------ */
/* Canonical-averages rows use the layout of percolate/hpc.py:518-558
 * (number_of_runs u32, then per statistic mean f8, m2 f8; packed).
 * These entry points work on that byte layout directly. */

/* percolate/hpc.py:561-635 bond_initialize_canonical_averages: packed
 * canonical_statistics rows (hpc.py:407-440) -> canonical_averages rows. */
int nz_initialize_canonical_averages(const uint8_t *canonical_rows, int32_t P,
                                     int32_t spanning, uint8_t *out_rows,
                                     void *stream);
/* percolate/hpc.py:638-702 bond_reduce: pairwise merge of two row sets. */
int nz_bond_reduce(const uint8_t *rows_a, const uint8_t *rows_b, int32_t P,
                   int32_t spanning, uint8_t *out_rows, void *stream);
/* percolate/hpc.py:752-834 finalize_canonical_averages: mean (/N),
 * std = sqrt(M2/(n-1)) (/N), Student-t interval at 1 - alpha; NaN where the
 * reference's scipy call yields NaN. */
int nz_finalize_canonical_averages(const uint8_t *avg_rows, int32_t P,
                                   int32_t spanning, double number_of_nodes,
                                   const double *ps, double alpha,
                                   uint8_t *out_rows, void *stream);

/* Student-t quantile t_{q}(df) for each element (device math, FP64). */
int nz_student_t_quantile(const double *q, const double *df, int32_t count,
                          double *out, void *stream);

/* ---- ensemble (batched fast path) ------------------------------------ */
/* Microcanonical run-reduction accumulators for one lattice size, per
 * n = 0..M (percolate/percolate.py:450-705 semantics): exact integer sums
 * and FP64 sums of squared deviations (pairwise-merged). */
typedef struct NzMicroAccum {
    uint64_t *count;     /* [1] runs accumulated                            */
    uint64_t *span_count;/* [M+1] runs with a spanning cluster               */
    uint64_t *sum_lo;    /* [6][M+1] exact sums of max, m0..m4, low words    */
    uint64_t *sum_hi;    /* [6][M+1] high words                              */
    double *m2;          /* [6][M+1] sums of squared deviations from the mean */
} NzMicroAccum;

/* Microcanonical averages (percolate/percolate.py:450-705 and 968-1064
 * microcanonical_averages / microcanonical_averages_arrays) from the
 * accumulators: out[n * 21 + j], n = 0..M, j = spanning (mean, lo, hi) --
 * Bayesian (k+1)/(R+2) with Beta quantiles --, then max, m0..m4 (mean, lo,
 * hi) divided by num_nodes, Student-t intervals ((mean, mean) if std == 0). */
int nz_microcanonical_finalize(const NzMicroAccum *acc, uint32_t num_nodes,
                               uint32_t num_edges, int32_t spanning,
                               double alpha, int32_t normalize, double *out,
                               void *stream);
/* (normalize bit 0 = 0: absolute units as microcanonical_averages yields
 * them, percolate/percolate.py:708-896; 1: divided by N as in the arrays.
 * With NZ_MICRO_FIELD_MAJOR or-ed in, out is field-major instead:
 * out[j * (M + 1) + n], each value's M + 1 rows contiguous.) */
#define NZ_MICRO_FIELD_MAJOR 2

/* Adds the runs of a record set (rows n_begin..n_end-1 of all its runs; the
 * records' row 0 is n_begin) to the accumulators: the run-reductions of
 * percolate/percolate.py:450-705 at every n. */
int nz_microcanonical_reduce(const NzRecords *rec, uint32_t num_nodes,
                             uint32_t num_edges, int32_t n_runs,
                             uint32_t n_begin, uint32_t n_end,
                             const NzMicroAccum *acc, void *stream);

/* Merges two running states of independent run sets: dst <- dst (+) src.
 * nz_canonical_merge: cols columns of (count, mean, M2) sharing one count per
 * side -- the pairwise update that bond_reduce applies to two
 * canonical_averages rows (percolate/hpc.py:638-702), here on the device
 * arrays of nz_ensemble.  nz_micro_merge: the accumulators of two
 * NzMicroAccum over num_edges + 1 rows (exact sums and spanning counts add,
 * M2 merges pairwise).  Used to combine the shards of several GPUs or
 * processes and checkpointed partial ensembles; dst and src must not alias.
 * The reference merges such partial results through its task store
 * (percolate/share/jugfile.py:240-244) with bond_reduce. */
int nz_canonical_merge(uint64_t *dst_count, double *dst_mean, double *dst_m2,
                       const uint64_t *src_count, const double *src_mean,
                       const double *src_m2, int32_t cols, void *stream);
int nz_micro_merge(const NzMicroAccum *dst, const NzMicroAccum *src,
                   uint32_t num_edges, void *stream);

/* Continues numpy's global MT19937 stream: state_in = 624 key words + the
 * position (np.random.get_state()); draws n_runs permutations of range(M) in
 * order, as the classic API's runs draw np.random.permutation(M)
 * (percolate/percolate.py:270); writes the advanced state to state_out. */
int nz_mt_stream_permutations(const uint32_t *state_in, uint32_t num_edges,
                              int32_t n_runs, uint32_t *out,
                              uint32_t *state_out, void *stream);

/* The whole per-lattice pipeline for n_runs Philox runs:
 * permutation -> union-find -> (optional) fused microcanonical reductions
 * -> banded canonical convolution at P probabilities -> pairwise merge.
 * Results are merged into (acc_count, acc_mean[P*7], acc_m2[P*7]) and, if
 * micro != NULL, into *micro.  conv_precision: 0 = FP64 over each band
 * of `cutoff` (log B >= log B(mode) - cutoff); 1 = FP32 products summed in
 * FP32 over 128-row chunks and carried as FP32 (sum, compensation) pairs,
 * over the rows of the band whose weights are >= e^-30 x the mode's (the
 * weights left out sum to < 1e-13); 2 = the same rows on the tensor cores
 * (tcgen05 kind::tf32, three split products per term).  In 1 and 2 the m2
 * statistic (the susceptibility) runs on a compensated FP32 kernel (FP32 hi +
 * lo weights, exact two-part values, error-free products and sums over the
 * band's core), ~2^-44 relative per run, so that its curve stays within
 * 1e-6 absolute of FP64 where it reaches ~1e4.  A convolution wait that gives
 * up is counted with nz_ensemble_errors.  The union-find runs on `stream`; the reductions
 * and the convolution of each window of records run on a second stream of
 * the library's (one per concurrent call and device, created on first use
 * and kept), overlapping the union-find of the next window, and are joined
 * back into `stream` before the call returns: work enqueued on `stream`
 * afterwards sees the results.  Make a first call before capturing `stream`
 * into a CUDA graph. */
size_t nz_ensemble_workspace_bytes(const NzGraph *graph, int32_t n_runs,
                                   int32_t P, int32_t window);
/* Runs of the last nz_ensemble call on `workspace` (same graph, n_runs, P,
 * window) whose union-find state came out corrupt -- a find that exceeded
 * the depth bound, which union by size makes impossible for valid state --
 * copied to the device word *errors on `stream`.  0 in every valid use.  No
 * counterpart in the reference (its union-find is networkx's). */
int nz_ensemble_errors(const NzGraph *graph, int32_t n_runs, int32_t P,
                       int32_t window, const void *workspace,
                       size_t workspace_bytes, uint32_t *errors, void *stream);
int nz_ensemble(const NzGraph *graph, int32_t spanning, int32_t n_runs,
                uint64_t key, uint64_t run0, const double *ps, int32_t P,
                double cutoff, int32_t window, int32_t conv_precision,
                void *workspace, size_t workspace_bytes, uint64_t *acc_count,
                double *acc_mean, double *acc_m2, const NzMicroAccum *micro,
                void *stream);

/* Launch shapes of the ensemble pipeline, chosen by an autotuner (the Python
 * package's autotune.tune_ensemble) rather than fixed; a field of 0 takes the
 * default.  uf_block: runs per CTA of the union-find (32, 64 or 128; 128);
 * m2_tile: probabilities per CTA of the compensated m2 convolution (8 or 16;
 * 8); reduce_slices: slices of runs of the canonical run reduction (1 ..
 * 256; 1, 16 or 64 by run count); conv_tile: probabilities per CTA of the
 * FP32 convolution kernel of m0, m3 and m4 (8 or 16; 8); taper: 1 =
 * the first and the last record window a quarter window long (the first
 * window's union-find and the last window's reductions run alone), 0 = all
 * windows full (0).  The record window is nz_ensemble's `window`.  No
 * counterpart in the reference (its runs are Python calls). */
typedef struct NzTuning {
    int32_t uf_block;
    int32_t m2_tile;
    int32_t reduce_slices;
    int32_t conv_tile;
    int32_t taper;
} NzTuning;
/* nz_ensemble with explicit launch shapes (tuning may be NULL: defaults);
 * results do not depend on them beyond the order of FP64 additions in the
 * run reduction. */
int nz_ensemble_tuned(const NzGraph *graph, int32_t spanning,
                      int32_t n_runs, uint64_t key, uint64_t run0,
                      const double *ps, int32_t P, double cutoff,
                      int32_t window, int32_t conv_precision,
                      const NzTuning *tuning, void *workspace,
                      size_t workspace_bytes, uint64_t *acc_count,
                      double *acc_mean, double *acc_m2,
                      const NzMicroAccum *micro, void *stream);

/* ---- batched uneven ensembles (one persistent launch) ------------------ */
/* Run r draws its substrate from Philox-4x32-10 (key, counter r): a chain
 * with probability chain_share / 2^32, else a square lattice; the length L
 * (or l) is the largest grid_min + i (chain_min + i) with thr[i] <= u, u a
 * uniform 32-bit word, thr[0] = 0.  For a log-uniform length rounded to the
 * nearest integer, thr[i] = ceil(2^32 ln((len - 1/2) / min) / ln(max / min)).
 * Runs of every lattice (kind, length) = "class" are reduced at `checkpoints`
 * occupation numbers n_j = floor(j M / (checkpoints - 1)), j = 0..F-1, to
 * exact integer sums and exact-numerator M2 of max, m0, m1, m2, m3, m4 and
 * spanning counts (percolate/percolate.py:450-705 statistics at those n).
 * `reduction` picks how (identical results): NZ_MIX_REDUCE_RECORDS -- each
 * run writes its checkpoint statistics, a second kernel reduces them per
 * class; NZ_MIX_REDUCE_FUSED -- the union-find threads add each run's
 * statistics and squares into its class's sums themselves (exact integer
 * atomics), and a per-cell kernel only forms the outputs.  The fused form
 * needs no per-run records and is faster where lattices have many runs each;
 * the records form where they have few (the autotuner measures both). */
#define NZ_MIX_REDUCE_RECORDS 0
#define NZ_MIX_REDUCE_FUSED 1
typedef struct NzMixSpec {
    uint32_t grid_min, grid_max;   /* spanning_2d_grid lengths (inclusive)   */
    uint32_t chain_min, chain_max; /* spanning_1d_chain lengths (inclusive)  */
    uint32_t chain_share;          /* P(chain) * 2^32                         */
    int32_t checkpoints;           /* F >= 2                                  */
    int32_t reduction;             /* NZ_MIX_REDUCE_RECORDS or _FUSED        */
} NzMixSpec;

/* Per class c (grid classes first: c = L - grid_min; then chains:
 * c = n_grid + l - chain_min) and checkpoint j; arrays over [class][F],
 * sums/m2 over [6][class][F] with statistic order max, m0, m1, m2, m3, m4. */
typedef struct NzMixAccum {
    uint32_t *count;   /* [classes] runs in the class                        */
    uint32_t *span;    /* [classes][F] runs with a spanning cluster          */
    uint64_t *sum_lo;  /* [6][classes][F] exact sums, low words              */
    uint64_t *sum_hi;  /* high words                                         */
    double *m2;        /* [6][classes][F] sums of squared deviations         */
    uint32_t *errors;  /* [1] runs skipped by a failed internal check (0)    */
} NzMixAccum;

/* Workspace for n_runs runs and `threads` persistent threads; each thread's
 * node slot is sized for the largest lattice of the spec.  Beside the node
 * slots: per-run checkpoint records (36 B per run and checkpoint) for
 * NZ_MIX_REDUCE_RECORDS, per-class sums (216 B per class and checkpoint)
 * for NZ_MIX_REDUCE_FUSED. */
size_t nz_mix_workspace_bytes(const NzMixSpec *spec, int32_t n_runs,
                              int32_t threads);
/* key_dev: device pointer to the Philox key (read by the kernels, so a
 * captured CUDA graph of this call can be replayed with another key).
 * threads: persistent threads; block: threads per CTA; smem_words: per-thread
 * shared-memory node slot (0 = none) -- runs with N <= smem_words use it.
 * Output arrays are overwritten (not accumulated). */
int nz_mix(const NzMixSpec *spec, const uint32_t *thr_grid,
           const uint32_t *thr_chain, const uint64_t *key_dev, int32_t n_runs,
           int32_t threads, int32_t block, uint32_t smem_words,
           void *workspace, size_t workspace_bytes, const NzMixAccum *out,
           void *stream);

/* ---- MLP surrogate of the canonical curves ---------------------------- */
/* (No counterpart in the reference.)  Fully connected, GELU hidden layers,
 * linear output; widths[0..n_layers] (host array).  GEMM operands are
 * BF16 (activations and gradients rounded to nearest-even where they enter
 * a product), accumulation FP32.  params: flat FP32, per layer W [in][out]
 * row-major then b [out]; params_bf16: its BF16 mirror (2 bytes each). */
int64_t nz_mlp_param_count(const int32_t *widths, int32_t n_layers);
/* floats of z (pre-activations) and of h (activations) for a batch */
int64_t nz_mlp_activation_count(const int32_t *widths, int32_t n_layers,
                                int32_t batch);
int nz_mlp_params_to_bf16(const float *params, int64_t count,
                          void *params_bf16, void *stream);
int nz_mlp_forward(const int32_t *widths, int32_t n_layers, int32_t batch,
                   const float *x, const float *params,
                   const void *params_bf16, float *z, float *h, float *y,
                   void *stream);
/* weighted squared error over [batch][n_out]: loss_parts[i] partial sums of
 * sum w (y - t)^2 / batch (add them up), dy = 2 w (y - t) / batch */
int nz_mlp_loss(const float *y, const float *target, const float *weight,
                int32_t batch, int32_t n_out, float *dy, float *loss_parts,
                int32_t n_parts, void *stream);
/* scratch: 2 * batch * max(widths) floats */
int nz_mlp_backward(const int32_t *widths, int32_t n_layers, int32_t batch,
                    const float *x, const void *params_bf16, const float *z,
                    const float *h, const float *dy, float *grads,
                    float *scratch, void *stream);
/* The GEMMs of nz_mlp_forward / nz_mlp_backward run on the tensor cores
 * (tcgen05, BF16 operands, FP32 accumulation); a tile whose tensor-core
 * waits gave up (after 1 s) is written as NaN and counted.  Reads the count
 * since the last call and resets it (synchronous). */
int nz_mlp_take_errors(uint32_t *count);
/* Adam step (step >= 1); also refreshes params_bf16 */
int nz_mlp_adam(float *params, const float *grads, float *m, float *v,
                void *params_bf16, int64_t count, float lr, float beta1,
                float beta2, float eps, int32_t step, void *stream);

/* ---- memory-system hint ------------------------------------------------ */
/* L2 fetch granularity of the calling CUDA context (cudaLimitMaxL2FetchGranularity:
 * 0, 32, 64 or 128 bytes).  The union-find reads scattered 4-byte node words;
 * 32-byte fetches avoid pulling a second, unused sector from HBM per miss.
 * The limit belongs to the caller's context (it ends with the process) and
 * applies to every kernel of that context, so the library never sets it on
 * its own.  (No counterpart in the reference.) */
int nz_set_l2_fetch_granularity(int32_t bytes);
int nz_get_l2_fetch_granularity(int32_t *bytes);

/* ---- measurement ------------------------------------------------------ */
/* When enabled, every launch sequence of a category below is bracketed by
 * CUDA events recorded on the caller's stream.  nz_profile_read waits for
 * the recorded events, returns per category the number of bracketed
 * sequences and their summed elapsed milliseconds, and clears the record.
 * (The project's own instrumentation; no counterpart in the reference.) */
#define NZ_PROF_SETUP 0      /* weights, run initialisation                 */
#define NZ_PROF_UNION_FIND 1 /* uf_window_kernel                            */
#define NZ_PROF_MICRO 2      /* fused microcanonical reductions             */
#define NZ_PROF_CONV 3       /* banded canonical convolution                */
#define NZ_PROF_REDUCE 4     /* merge over runs                             */
#define NZ_PROF_CATEGORIES 5
void nz_profile_enable(int32_t enabled);
int nz_profile_read(int32_t n_categories, int64_t *launches, double *total_ms);

#ifdef __cplusplus
}
#endif
#endif /* NZ_GB300_H */
