// nz_internal.cuh -- kernel parameter blocks and launcher declarations shared
// between the translation units of libnzgb300.so (not part of the C ABI).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "nz_common.cuh"

namespace nz {

struct UfParams {
    GraphDev g;
    int32_t n_runs;
    uint32_t *nodes;        // [n_runs][g.slots]
    RunState *state;        // [n_runs]
    uint32_t n_begin;       // rows emitted: [n_begin, n_end)
    uint32_t n_end;
    uint64_t key, run0;     // NZ_PERM_PHILOX
    const uint32_t *perms;  // [n_runs][M] otherwise
    NzRecords rec;          // row n of run r at plane[(n - n_begin) * run_stride + r]
    uint32_t *errors;       // if set: +1 per run whose state is corrupt after its last row
};

// nz_uf.cu
void launch_init_runs(const GraphDev &g, int32_t n_runs, uint32_t *nodes, RunState *state,
                      uint32_t *flag_scratch, cudaStream_t s);
void launch_uf_window(const UfParams &p, int perm_mode, bool span, int block, cudaStream_t s);
void launch_philox_perms(uint32_t M, int32_t n_runs, uint64_t key, uint64_t run0, uint32_t *out,
                         cudaStream_t s);
void launch_mt_perms(uint32_t M, int32_t n_runs, const uint32_t *seed_words, const int32_t *seed_len,
                     int32_t stride, uint32_t *out, cudaStream_t s);
void launch_mt_stream_perms(const uint32_t *state_in, uint32_t M, int32_t n_runs, uint32_t *out,
                            uint32_t *state_out, cudaStream_t s);
void launch_pack_rows(const NzRecords &rec, int32_t run, uint32_t N, uint32_t M, int32_t spanning,
                      uint8_t *rows, cudaStream_t s);

// nz_lattice.cu: site percolation and the torus (dispatched from nz_uf.cu)
bool lattice_extension(const GraphDev &g);
void launch_init_lattice_runs(const GraphDev &g, int32_t n_runs, uint32_t *nodes, RunState *state,
                              cudaStream_t s);
void launch_lattice_window(const UfParams &p, int perm_mode, bool span, int block, cudaStream_t s);

// nz_canonical.cu
void launch_binomial_weights(uint32_t M, const double *ps, int32_t P, double cutoff, int32_t cap,
                             uint32_t *band_lo, uint32_t *band_len, double *w, int32_t *overflow,
                             cudaStream_t s);
void launch_binomial_pmf(uint32_t M, const double *ps, int32_t P, double cutoff, double *out, cudaStream_t s);
// out[i * cols + c] = sum over the band of p_i of w[i][j] V[(lo_i + j) * cols + c] (FP64)
void launch_band_dot(const uint32_t *band_lo, const uint32_t *band_len, const double *w, int32_t cap, int32_t P,
                     const double *V, uint32_t rows, int32_t cols, double *out, cudaStream_t s);
void launch_canonical_rows(const uint8_t *rows, uint32_t M, int32_t spanning, const double *factors,
                           int32_t n_sets, double *out, cudaStream_t s);

struct ConvParams {
    NzRecords rec;           // window records, row n at (n - n_begin)
    uint32_t n_begin, n_end; // window rows
    uint32_t N;
    int32_t n_runs;
    int32_t spanning;
    int32_t P, cap;
    const uint32_t *band_lo, *band_len;  // rows of w64, or of w32 on the FP32 path
    const double *w64;       // [P][cap]
    const float *w32;        // [P][cap] (FP32 path, its own narrower bands)
    const float *w32lo;      // [P][cap] w64 - w32 as FP32 (the compensated m2 products)
    const uint32_t *core_lo, *core_len;  // rows whose weight is >= e^-8 of the mode (m2 compensated)
    int32_t m2_tile;         // probabilities per CTA of the compensated m2 kernel (8 or 16)
    int32_t conv_tile;       // probabilities per CTA of the FP32 window kernels (8 or 16)
    double *acc;             // [n_runs][P][7], accumulated (+=)
    uint32_t *errors;        // tensor-core path: counts CTAs whose waits gave up (or null)
};
bool conv_grid_fits(int32_t n_runs, int32_t P);  // grid of launch_conv_window within CUDA's limits
void launch_conv_window(const ConvParams &p, int precision, cudaStream_t s);
// 3xTF32 tensor-core convolution (tcgen05) of the FP32 bands; 0 or -1 (launch error)
bool conv_tc_grid_fits(int32_t n_runs, int32_t P);
int launch_conv_window_tc(const ConvParams &p, cudaStream_t s);
// FP32 weights of the rows where each band's weight is >= rel x its largest,
// re-based at lo32 (the convolution's FP32 band)
// (and their FP32 remainders w64 - w32 in w32lo), and the core rows whose
// weight is >= rel_core x the largest
void launch_narrow_weights_f32(const double *w64, const uint32_t *band_lo, const uint32_t *band_len, int32_t P,
                               int32_t cap, double rel, double rel_core, float *w32, float *w32lo, uint32_t *lo32,
                               uint32_t *len32, uint32_t *core_lo, uint32_t *core_len, cudaStream_t s);
// m2 (statistic 4) of the FP32 paths with compensated products and sums
void launch_conv_m2_comp(const ConvParams &p, cudaStream_t s);
// part: scratch [slices][P*7][3] doubles
void launch_reduce_runs(const double *stats, int32_t n_runs, int32_t P, uint64_t *acc_count,
                        double *acc_mean, double *acc_m2, double *part, int32_t slices, cudaStream_t s);

struct MicroParams {
    NzRecords rec;
    uint32_t n_begin, n_end;
    uint32_t N;
    int32_t n_runs;
    NzMicroAccum acc;
    uint32_t M;
    const uint64_t *count_before;  // device: runs already in acc
};
void launch_micro_window(const MicroParams &p, cudaStream_t s);
void launch_micro_count(uint64_t *count, int32_t n_runs, cudaStream_t s);
void launch_canonical_merge(uint64_t *dst_count, double *dst_mean, double *dst_m2, const uint64_t *src_count,
                            const double *src_mean, const double *src_m2, int32_t cols, cudaStream_t s);
void launch_micro_merge(const NzMicroAccum &dst, const NzMicroAccum &src, uint32_t rows, cudaStream_t s);

void launch_init_avg(const uint8_t *canon_rows, int32_t P, int32_t spanning, uint8_t *out, cudaStream_t s);
void launch_bond_reduce(const uint8_t *a, const uint8_t *b, int32_t P, int32_t spanning, uint8_t *out,
                        cudaStream_t s);
void launch_finalize(const uint8_t *avg, int32_t P, int32_t spanning, double N, const double *ps,
                     double alpha, uint8_t *out, cudaStream_t s);
void launch_micro_finalize(const NzMicroAccum &acc, uint32_t N, uint32_t M, int32_t spanning, double alpha,
                           int32_t normalize, double *out, cudaStream_t s);
void launch_t_quantile(const double *q, const double *df, int32_t count, double *out, cudaStream_t s);

// nz_mix.cu (batched uneven ensembles)
struct MixDev {
    const uint64_t *key_ptr;
    int32_t n_runs;
    uint32_t chain_share;
    uint32_t grid_min, grid_max, chain_min, chain_max;
    uint32_t n_grid, n_chain;
    const uint32_t *thr_grid;
    const uint32_t *thr_chain;
    int32_t F;
};
struct MixRec {
    uint32_t *max_span;
    uint32_t *m0;
    uint64_t *m2, *m3, *m4_lo;
    uint32_t *m4_hi;
};
// Fused reduction: exact per-(class, checkpoint) sums that the union-find
// threads accumulate themselves, kMixCellWords uint64 words per cell, each
// the sum of one 32-bit limb of a statistic (or of its square) over the
// class's runs.
constexpr int kMixCellWords = 27;
struct MixAccum {
    uint32_t *count;
    uint32_t *span;
    uint64_t *sum_lo;
    uint64_t *sum_hi;
    double *m2;
    uint32_t *errors;
};
struct MixLaunch {
    MixDev m;
    uint32_t *cls, *counts, *order, *offsets, *cursor, *queue, *head;
    uint64_t *slot_off;
    uint32_t *nodes;
    int32_t T, block;
    uint32_t smem_words;
    bool fused;       // NZ_MIX_REDUCE_FUSED: cells, else records + mix_reduce_kernel
    MixRec rec;       // [n_runs][F] per plane (records only)
    uint64_t *cells;  // [classes][F][kMixCellWords] (fused only)
    MixAccum acc;
};
int launch_mix(const MixLaunch &p, cudaStream_t s);

}  // namespace nz
