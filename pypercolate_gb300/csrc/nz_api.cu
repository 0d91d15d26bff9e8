// nz_api.cu -- the extern "C" entry points of libnzgb300.so (include/nz_gb300.h).
//
// Host-side orchestration: argument validation, workspace carving, launch
// sequencing on the caller's stream.  Nothing here allocates device memory.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <vector>

#include "nz_common.cuh"
#include "nz_internal.cuh"

using namespace nz;

namespace {

constexpr size_t kAlign = 256;

inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct Carver {
    uint8_t *base;
    size_t used;
    size_t cap;
    template <class T>
    T *take(size_t count) {
        size_t off = align_up(used);
        used = off + count * sizeof(T);
        return base ? reinterpret_cast<T *>(base + off) : nullptr;
    }
    bool ok() const { return used <= cap; }
};

inline int check_launch() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- optional per-kernel timing (CUDA events on the launching stream) ----
struct ProfState {
    std::mutex mu;
    bool enabled = false;
    std::vector<cudaEvent_t> pool;
    struct Rec { int cat; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
};
ProfState g_prof;

struct ProfScope {
    int cat;
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(int c, cudaStream_t st) : cat(c), s(st) {
        if (!g_prof.enabled) return;
        std::lock_guard<std::mutex> lk(g_prof.mu);
        a = g_prof.get();
        b = g_prof.get();
        cudaEventRecord(a, s);
    }
    ~ProfScope() {
        if (!a) return;
        cudaEventRecord(b, s);
        std::lock_guard<std::mutex> lk(g_prof.mu);
        g_prof.recs.push_back({cat, a, b});
    }
};

constexpr uint32_t kRecordBytes = 4 + 4 + 8 + 8 + 8 + 4;  // planes without edge (wide layout)
constexpr uint32_t kNarrowRecordNodes = 65536;  // narrow records (m0 uint16, m2 uint32) up to this N


// Workspace of the microcanonical entry point.
size_t micro_layout(Carver &c, const GraphDev &g, int32_t n_runs, int32_t perm_mode, uint32_t **nodes,
                    RunState **state, uint32_t **flag, uint32_t **perms) {
    *nodes = c.take<uint32_t>((size_t)n_runs * g.slots);
    *state = c.take<RunState>((size_t)n_runs);
    *flag = c.take<uint32_t>(4);
    *perms = perm_mode == NZ_PERM_MT19937 ? c.take<uint32_t>((size_t)n_runs * (g.M ? g.M : 1)) : nullptr;
    return c.used;
}

// A caller's record layout: wide, or narrow (m0 as uint16, m2 as uint32),
// which holds every value only up to N = 65,536 nodes.
bool records_layout_ok(const NzRecords &rec, uint32_t N) {
    return rec.narrow == 0 || (rec.narrow == 1 && N <= kNarrowRecordNodes);
}

}  // namespace

extern "C" {

const char *nz_version(void) { return "pypercolate-gb300 0.1.0 (sm_103a)"; }

const char *nz_status_string(int status) {
    switch (status) {
        case NZ_OK: return "ok";
        case NZ_ERR_INVALID: return "invalid argument";
        case NZ_ERR_SPANNING_SIDES:
            return "Spanning cluster is to be detected, but auxiliary nodes of less or more than 2 types (sides) given.";
        case NZ_ERR_TOO_LARGE: return "size beyond the library's limits";
        case NZ_ERR_CUDA: return "CUDA runtime error";
        case NZ_ERR_WORKSPACE: return "workspace too small";
        default: return "unknown status";
    }
}

int nz_graph_size(const NzGraph *graph, uint32_t *num_nodes, uint32_t *num_edges) {
    if (!graph || !num_nodes || !num_edges) return NZ_ERR_INVALID;
    return graph_size(*graph, *num_nodes, *num_edges);
}

size_t nz_microcanonical_workspace_bytes(const NzGraph *graph, int32_t n_runs, int32_t perm_mode) {
    uint32_t N, M;
    if (!graph || graph_size(*graph, N, M) != NZ_OK || n_runs <= 0) return 0;
    GraphDev g = make_graph_dev(*graph, N, M);
    Carver c{nullptr, 0, 0};
    uint32_t *a, *f, *p;
    RunState *st;
    return align_up(micro_layout(c, g, n_runs, perm_mode, &a, &st, &f, &p));
}

int nz_microcanonical(const NzGraph *graph, int32_t spanning, int32_t n_runs, int32_t perm_mode, uint64_t key,
                      uint64_t run0, const uint32_t *perms, const uint32_t *mt_seed_words,
                      const int32_t *mt_seed_len, int32_t mt_words_stride, void *workspace,
                      size_t workspace_bytes, const NzRecords *out, void *stream) {
    if (!graph || !out || n_runs <= 0) return NZ_ERR_INVALID;
    if ((uint32_t)n_runs > NZ_MAX_RUNS) return NZ_ERR_TOO_LARGE;
    uint32_t N, M;
    int st = graph_size(*graph, N, M);
    if (st) return st;
    if (perm_mode == NZ_PERM_GIVEN && M > 0 && !perms) return NZ_ERR_INVALID;
    if (perm_mode == NZ_PERM_MT19937 && (!mt_seed_words || !mt_seed_len)) return NZ_ERR_INVALID;
    if (perm_mode < 0 || perm_mode > 2) return NZ_ERR_INVALID;
    if (!out->max_span || !out->m0 || !out->m2 || !out->m3 || !out->m4_lo || out->run_stride < n_runs ||
        !records_layout_ok(*out, N))
        return NZ_ERR_INVALID;
    GraphDev g = make_graph_dev(*graph, N, M);
    Carver c{static_cast<uint8_t *>(workspace), 0, workspace_bytes};
    uint32_t *nodes, *flag, *mt_perms;
    RunState *state;
    micro_layout(c, g, n_runs, perm_mode, &nodes, &state, &flag, &mt_perms);
    if (!workspace || !c.ok()) return NZ_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    launch_init_runs(g, n_runs, nodes, state, flag, s);
    const uint32_t *perm_src = perms;
    int mode = perm_mode;
    if (perm_mode == NZ_PERM_MT19937) {
        launch_mt_perms(M, n_runs, mt_seed_words, mt_seed_len, mt_words_stride, mt_perms, s);
        perm_src = mt_perms;
        mode = NZ_PERM_GIVEN;
    }
    UfParams p;
    p.g = g;
    p.n_runs = n_runs;
    p.nodes = nodes;
    p.state = state;
    p.n_begin = 0;
    p.n_end = M + 1;
    p.key = key;
    p.run0 = run0;
    p.perms = perm_src;
    p.rec = *out;
    p.errors = nullptr;
    {
        ProfScope prof(NZ_PROF_UNION_FIND, s);
        launch_uf_window(p, mode, spanning != 0, n_runs >= 128 ? 128 : 32, s);
    }
    return check_launch();
}

int nz_set_l2_fetch_granularity(int32_t bytes) {
    if (bytes != 0 && bytes != 32 && bytes != 64 && bytes != 128) return NZ_ERR_INVALID;
    return cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes) == cudaSuccess ? NZ_OK : NZ_ERR_CUDA;
}

int nz_get_l2_fetch_granularity(int32_t *bytes) {
    if (!bytes) return NZ_ERR_INVALID;
    size_t v = 0;
    if (cudaDeviceGetLimit(&v, cudaLimitMaxL2FetchGranularity) != cudaSuccess) return NZ_ERR_CUDA;
    *bytes = (int32_t)v;
    return NZ_OK;
}

void nz_profile_enable(int32_t enabled) {
    std::lock_guard<std::mutex> lk(g_prof.mu);
    g_prof.enabled = enabled != 0;
}

int nz_profile_read(int32_t n_categories, int64_t *launches, double *total_ms) {
    if (n_categories <= 0 || !launches || !total_ms) return NZ_ERR_INVALID;
    for (int i = 0; i < n_categories; ++i) { launches[i] = 0; total_ms[i] = 0.0; }
    std::lock_guard<std::mutex> lk(g_prof.mu);
    int status = NZ_OK;
    for (auto &r : g_prof.recs) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess)
            status = NZ_ERR_CUDA;
        if (r.cat >= 0 && r.cat < n_categories) { launches[r.cat] += 1; total_ms[r.cat] += ms; }
        g_prof.pool.push_back(r.a);
        g_prof.pool.push_back(r.b);
    }
    g_prof.recs.clear();
    return status;
}

int nz_permutations(uint32_t num_edges, int32_t n_runs, int32_t perm_mode, uint64_t key, uint64_t run0,
                    const uint32_t *mt_seed_words, const int32_t *mt_seed_len, int32_t mt_words_stride,
                    uint32_t *out, void *stream) {
    if (n_runs <= 0 || !out) return NZ_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    if (perm_mode == NZ_PERM_PHILOX) launch_philox_perms(num_edges, n_runs, key, run0, out, s);
    else if (perm_mode == NZ_PERM_MT19937) {
        if (!mt_seed_words || !mt_seed_len) return NZ_ERR_INVALID;
        launch_mt_perms(num_edges, n_runs, mt_seed_words, mt_seed_len, mt_words_stride, out, s);
    } else return NZ_ERR_INVALID;
    return check_launch();
}

int nz_pack_microcanonical_rows(const NzRecords *rec, int32_t run, uint32_t num_nodes, uint32_t num_edges,
                                int32_t spanning, uint8_t *rows, void *stream) {
    if (!rec || !rows || run < 0 || !rec->max_span || !rec->m0 || !rec->m2 || !rec->m3 || !rec->m4_lo ||
        !records_layout_ok(*rec, num_nodes))
        return NZ_ERR_INVALID;
    launch_pack_rows(*rec, run, num_nodes, num_edges, spanning, rows, as_stream(stream));
    return check_launch();
}

int32_t nz_binomial_band_cap(uint32_t num_edges, double cutoff) {
    // Gaussian band half-width sqrt(2 cutoff) sigma with sigma <= sqrt(M)/2,
    // widened by 25 % plus a margin for the skewed tails near p = 0, 1.
    const double sigma = 0.5 * sqrt((double)num_edges);
    double w = 2.0 * 1.25 * sqrt(2.0 * (cutoff > 0 ? cutoff : 0.0)) * sigma + 2.0 * cutoff + 64.0;
    if (w > (double)num_edges + 1.0) w = (double)num_edges + 1.0;
    return (int32_t)ceil(w);
}

int nz_binomial_weights(uint32_t num_edges, const double *ps, int32_t P, double cutoff, int32_t cap,
                        uint32_t *band_lo, uint32_t *band_len, double *weights, void *stream) {
    if (P <= 0 || !ps || !band_lo || !band_len || !weights || cap <= 0 || !(cutoff > 0)) return NZ_ERR_INVALID;
    launch_binomial_weights(num_edges, ps, P, cutoff, cap, band_lo, band_len, weights, nullptr,
                            as_stream(stream));
    return check_launch();
}

int nz_binomial_pmf(uint32_t num_edges, const double *ps, int32_t P, double *out, void *stream) {
    if (P <= 0 || !ps || !out) return NZ_ERR_INVALID;
    launch_binomial_pmf(num_edges, ps, P, 745.0 /* FP64 underflow: the reference's own range */, out,
                        as_stream(stream));
    return check_launch();
}

int nz_band_dot(const uint32_t *band_lo, const uint32_t *band_len, const double *weights, int32_t cap, int32_t P,
                const double *values, uint32_t rows, int32_t cols, double *out, void *stream) {
    if (!band_lo || !band_len || !weights || !values || !out || cap <= 0 || P <= 0 || cols <= 0 || rows == 0)
        return NZ_ERR_INVALID;
    if ((cols + 31) / 32 > 65535) return NZ_ERR_TOO_LARGE;
    launch_band_dot(band_lo, band_len, weights, cap, P, values, rows, cols, out, as_stream(stream));
    return check_launch();
}

int nz_canonical_statistics_rows(const uint8_t *rows, uint32_t num_edges, int32_t spanning, const double *factors,
                                 int32_t n_factor_sets, double *out, void *stream) {
    if (!rows || !factors || !out || n_factor_sets <= 0) return NZ_ERR_INVALID;
    launch_canonical_rows(rows, num_edges, spanning, factors, n_factor_sets, out, as_stream(stream));
    return check_launch();
}

int nz_canonical_statistics_records(const NzRecords *rec, uint32_t num_nodes, uint32_t num_edges, int32_t n_runs,
                                    int32_t spanning, const uint32_t *band_lo, const uint32_t *band_len,
                                    const double *weights, int32_t cap, int32_t P, double *out, void *stream) {
    if (!rec || !band_lo || !band_len || !weights || !out || n_runs <= 0 || P <= 0) return NZ_ERR_INVALID;
    if (!records_layout_ok(*rec, num_nodes)) return NZ_ERR_INVALID;
    if (!conv_grid_fits(n_runs, P)) return NZ_ERR_TOO_LARGE;
    cudaStream_t s = as_stream(stream);
    if (cudaMemsetAsync(out, 0, sizeof(double) * (size_t)n_runs * P * 7, s) != cudaSuccess) return NZ_ERR_CUDA;
    ConvParams p;
    p.rec = *rec;
    p.n_begin = 0;
    p.n_end = num_edges + 1;
    p.N = num_nodes;
    p.n_runs = n_runs;
    p.spanning = spanning;
    p.P = P;
    p.cap = cap;
    p.band_lo = band_lo;
    p.band_len = band_len;
    p.w64 = weights;
    p.w32 = nullptr;
    p.w32lo = nullptr;
    p.core_lo = p.core_len = nullptr;
    p.m2_tile = 8;
    p.conv_tile = 8;
    p.acc = out;
    p.errors = nullptr;
    launch_conv_window(p, 0, s);
    return check_launch();
}

int nz_initialize_canonical_averages(const uint8_t *canonical_rows, int32_t P, int32_t spanning, uint8_t *out_rows,
                                     void *stream) {
    if (!canonical_rows || !out_rows || P < 0) return NZ_ERR_INVALID;
    launch_init_avg(canonical_rows, P, spanning, out_rows, as_stream(stream));
    return check_launch();
}

int nz_bond_reduce(const uint8_t *rows_a, const uint8_t *rows_b, int32_t P, int32_t spanning, uint8_t *out_rows,
                   void *stream) {
    if (!rows_a || !rows_b || !out_rows || P < 0) return NZ_ERR_INVALID;
    launch_bond_reduce(rows_a, rows_b, P, spanning, out_rows, as_stream(stream));
    return check_launch();
}

int nz_finalize_canonical_averages(const uint8_t *avg_rows, int32_t P, int32_t spanning, double number_of_nodes,
                                   const double *ps, double alpha, uint8_t *out_rows, void *stream) {
    if (!avg_rows || !out_rows || !ps || P < 0) return NZ_ERR_INVALID;
    launch_finalize(avg_rows, P, spanning, number_of_nodes, ps, alpha, out_rows, as_stream(stream));
    return check_launch();
}

int nz_microcanonical_finalize(const NzMicroAccum *acc, uint32_t num_nodes, uint32_t num_edges, int32_t spanning,
                               double alpha, int32_t normalize, double *out, void *stream) {
    if (!acc || !out || !acc->count || !acc->span_count || !acc->sum_lo || !acc->sum_hi || !acc->m2)
        return NZ_ERR_INVALID;
    if (!(alpha > 0.0 && alpha < 1.0)) return NZ_ERR_INVALID;
    launch_micro_finalize(*acc, num_nodes, num_edges, spanning, alpha, normalize, out, as_stream(stream));
    return check_launch();
}

int nz_microcanonical_reduce(const NzRecords *rec, uint32_t num_nodes, uint32_t num_edges, int32_t n_runs,
                             uint32_t n_begin, uint32_t n_end, const NzMicroAccum *acc, void *stream) {
    if (!rec || !acc || n_runs <= 0 || n_end <= n_begin || n_end > num_edges + 1) return NZ_ERR_INVALID;
    if (!rec->max_span || !rec->m0 || !rec->m2 || !rec->m3 || !rec->m4_lo || !rec->m4_hi ||
        rec->run_stride < n_runs || !records_layout_ok(*rec, num_nodes))
        return NZ_ERR_INVALID;
    if (!acc->count || !acc->span_count || !acc->sum_lo || !acc->sum_hi || !acc->m2) return NZ_ERR_INVALID;
    MicroParams mp;
    mp.rec = *rec;
    mp.n_begin = n_begin;
    mp.n_end = n_end;
    mp.N = num_nodes;
    mp.n_runs = n_runs;
    mp.acc = *acc;
    mp.M = num_edges;
    mp.count_before = acc->count;
    cudaStream_t s = as_stream(stream);
    launch_micro_window(mp, s);
    launch_micro_count(acc->count, n_runs, s);
    return check_launch();
}

int nz_canonical_merge(uint64_t *dst_count, double *dst_mean, double *dst_m2, const uint64_t *src_count,
                       const double *src_mean, const double *src_m2, int32_t cols, void *stream) {
    if (!dst_count || !src_count || cols < 0 || (cols > 0 && (!dst_mean || !dst_m2 || !src_mean || !src_m2)))
        return NZ_ERR_INVALID;
    if (dst_count == src_count) return NZ_ERR_INVALID;  // merging a state into itself
    launch_canonical_merge(dst_count, dst_mean, dst_m2, src_count, src_mean, src_m2, cols, as_stream(stream));
    return check_launch();
}

int nz_micro_merge(const NzMicroAccum *dst, const NzMicroAccum *src, uint32_t num_edges, void *stream) {
    if (!dst || !src || num_edges >= 0xFFFFFFFFu) return NZ_ERR_INVALID;
    if (!dst->count || !dst->span_count || !dst->sum_lo || !dst->sum_hi || !dst->m2) return NZ_ERR_INVALID;
    if (!src->count || !src->span_count || !src->sum_lo || !src->sum_hi || !src->m2) return NZ_ERR_INVALID;
    if (dst->count == src->count) return NZ_ERR_INVALID;
    launch_micro_merge(*dst, *src, num_edges + 1u, as_stream(stream));
    return check_launch();
}

int nz_mt_stream_permutations(const uint32_t *state_in, uint32_t num_edges, int32_t n_runs, uint32_t *out,
                              uint32_t *state_out, void *stream) {
    if (!state_in || !state_out || n_runs <= 0 || (num_edges > 0 && !out)) return NZ_ERR_INVALID;
    launch_mt_stream_perms(state_in, num_edges, n_runs, out, state_out, as_stream(stream));
    return check_launch();
}

int nz_student_t_quantile(const double *q, const double *df, int32_t count, double *out, void *stream) {
    if (!q || !df || !out || count < 0) return NZ_ERR_INVALID;
    launch_t_quantile(q, df, count, out, as_stream(stream));
    return check_launch();
}

// ------------------------------------------------------------- ensemble
namespace {

struct EnsembleLayout {
    uint32_t *nodes;
    RunState *state;
    uint32_t *flag;
    NzRecords rec[2];  // double-buffered record windows
    uint32_t *band_lo, *band_len;
    uint32_t *band_lo32, *band_len32;  // the FP32 convolution's bands
    uint32_t *core_lo32, *core_len32;  // their cores (compensated m2 rows)
    double *w64;
    float *w32, *w32lo;  // FP32 weights and their remainders
    double *stats;
    double *part;
    int32_t slices;
    int32_t cap;
    int32_t window;
};

constexpr double kDefaultCutoff = 80.0;
// the FP32 convolution uses the rows whose weights are >= e^-30 x the mode's
// (the rest sum to < 1e-13)
constexpr double kConvF32Cutoff = 30.0;
// m2's compensated products cover the rows whose weights are >= e^-8 x the
// mode's (+-4 standard deviations); the rest of the band holds < 1e-4 of the
// weight and is summed in plain FP32
constexpr double kConvCoreCutoff = 8.0;
constexpr int32_t kMaxSlices = 256;  // slices of runs of the canonical run reduction, at most
constexpr uint64_t kM4HighFreeNodes = 115001;  // max_s s^3 (N - s) < 2^64 for N <= 115,000

// Two streams per device on which nz_ensemble runs its record windows: the
// union-find on s1, at the device's greatest stream priority, and the
// consumers of each window (micro reductions, convolution, final reduction)
// on s2, with the events that order them; both fork from and join back into
// the caller's stream.  With the union-find's blocks dispatched first, a
// 100,000-run L = 256 step took 1187.2 against 1197.1 ms on the caller's
// (default-priority) stream, same box: the union-find 1038 against 1082 ms,
// the consumers beside it slower.  Slots are created on first use and kept
// for the life of the process; a call holds one for as long as it enqueues
// work, so concurrent calls never share events.
struct AuxSlot {
    int device;
    cudaStream_t s1, s2;
    cudaEvent_t fork, join1, join, produced[2], consumed[2];
    bool busy;
};

struct AuxPool {
    std::mutex mu;
    std::vector<AuxSlot *> slots;
};
AuxPool g_aux;

AuxSlot *aux_checkout() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_aux.mu);
    for (AuxSlot *a : g_aux.slots)
        if (!a->busy && a->device == dev) { a->busy = true; return a; }
    AuxSlot *a = new AuxSlot();
    a->device = dev;
    int least = 0, greatest = 0;
    bool ok = cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess &&
              cudaStreamCreateWithPriority(&a->s1, cudaStreamNonBlocking, greatest) == cudaSuccess &&
              cudaStreamCreateWithFlags(&a->s2, cudaStreamNonBlocking) == cudaSuccess;
    cudaEvent_t *evs[7] = {&a->fork,        &a->join1,       &a->join,       &a->produced[0],
                           &a->produced[1], &a->consumed[0], &a->consumed[1]};
    for (cudaEvent_t *e : evs) ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) { delete a; return nullptr; }  // (a failed creation leaks at most the handles made)
    a->busy = true;
    g_aux.slots.push_back(a);
    return a;
}

struct AuxGuard {
    AuxSlot *a;
    ~AuxGuard() {
        if (!a) return;
        std::lock_guard<std::mutex> lk(g_aux.mu);
        a->busy = false;
    }
};

// Joins the consumer stream back into the caller's stream on every way out
// of nz_ensemble once the fork is enqueued, so that nothing the caller
// enqueues afterwards (or a freed workspace) can race the consumers.
struct JoinGuard {
    cudaStream_t s, s2;
    cudaEvent_t join;
    bool armed;
    int join_now() {
        armed = false;
        return cudaEventRecord(join, s2) == cudaSuccess && cudaStreamWaitEvent(s, join, 0) == cudaSuccess
                   ? NZ_OK : NZ_ERR_CUDA;
    }
    ~JoinGuard() {
        if (armed) join_now();
    }
};

int32_t pick_window(uint32_t M, int32_t n_runs, int32_t window) {
    if (window > 0) return window > (int32_t)(M + 1) ? (int32_t)(M + 1) : window;
    // records of one window at most ~32 GiB (two windows in flight): at
    // 100,000 runs windows of ~9,500 rows measured 0.8 % faster than ~4,800
    // (16 GiB; 1.4 % faster than ~2,700) and ~19,000 no faster again
    double w = 32.0 * (1ull << 30) / ((double)n_runs * kRecordBytes);
    if (w < 256) w = 256;
    if (w > M + 1) w = M + 1;
    return (int32_t)w;
}

size_t ensemble_layout(Carver &c, const GraphDev &g, int32_t n_runs, int32_t P, double cutoff, int32_t window,
                       EnsembleLayout &L) {
    L.window = pick_window(g.M, n_runs, window);
    L.cap = nz_binomial_band_cap(g.M, cutoff);
    L.nodes = c.take<uint32_t>((size_t)n_runs * g.slots);
    L.state = c.take<RunState>((size_t)n_runs);
    L.flag = c.take<uint32_t>(4);
    const size_t plane = (size_t)L.window * n_runs;
    for (int b = 0; b < 2; ++b) {
        NzRecords &r = L.rec[b];
        // up to N = 65,536 nodes m0 (< 2^16) and m2 (<= N^2/4) are stored in
        // 16 and 32 bits: 26 instead of 32 B per record
        r.narrow = g.N <= kNarrowRecordNodes ? 1 : 0;
        r.max_span = c.take<uint32_t>(plane);
        if (r.narrow) {
            r.m0 = reinterpret_cast<uint32_t *>(c.take<uint16_t>(plane));
            r.m2 = reinterpret_cast<uint64_t *>(c.take<uint32_t>(plane));
        } else {
            r.m0 = c.take<uint32_t>(plane);
            r.m2 = c.take<uint64_t>(plane);
        }
        r.m3 = c.take<uint64_t>(plane);
        r.m4_lo = c.take<uint64_t>(plane);
        // sum' s^4 <= s_max^3 (N - s_max) <= max_s s^3 (N - s) < 2^64 for
        // N <= 115,000 sites (L <= 339): the high words are zero, the plane
        // is left out
        r.m4_hi = (uint64_t)g.N < kM4HighFreeNodes ? nullptr : c.take<uint32_t>(plane);
        r.edge = nullptr;
        r.run_stride = n_runs;
        r.site = (int32_t)g.site;
    }
    L.band_lo = c.take<uint32_t>(P);
    L.band_len = c.take<uint32_t>(P);
    L.w64 = c.take<double>((size_t)P * L.cap);
    L.w32 = c.take<float>((size_t)P * L.cap);
    L.w32lo = c.take<float>((size_t)P * L.cap);
    L.band_lo32 = c.take<uint32_t>(P);
    L.band_len32 = c.take<uint32_t>(P);
    L.core_lo32 = c.take<uint32_t>(P);
    L.core_len32 = c.take<uint32_t>(P);
    L.stats = c.take<double>((size_t)n_runs * P * 7);
    L.slices = n_runs < 1024 ? 1 : (n_runs < 65536 ? 16 : 64);
    // room for the largest tuned slice count
    L.part = c.take<double>((size_t)kMaxSlices * P * 7 * 3);
    return c.used;
}

}  // namespace

size_t nz_ensemble_workspace_bytes(const NzGraph *graph, int32_t n_runs, int32_t P, int32_t window) {
    uint32_t N, M;
    if (!graph || graph_size(*graph, N, M) != NZ_OK || n_runs <= 0 || P <= 0) return 0;
    GraphDev g = make_graph_dev(*graph, N, M);
    Carver c{nullptr, 0, 0};
    EnsembleLayout L;
    return align_up(ensemble_layout(c, g, n_runs, P, kDefaultCutoff, window, L));
}

int nz_ensemble(const NzGraph *graph, int32_t spanning, int32_t n_runs, uint64_t key, uint64_t run0,
                const double *ps, int32_t P, double cutoff, int32_t window, int32_t conv_precision,
                void *workspace, size_t workspace_bytes, uint64_t *acc_count, double *acc_mean, double *acc_m2,
                const NzMicroAccum *micro, void *stream) {
    return nz_ensemble_tuned(graph, spanning, n_runs, key, run0, ps, P, cutoff, window, conv_precision, nullptr,
                             workspace, workspace_bytes, acc_count, acc_mean, acc_m2, micro, stream);
}

int nz_ensemble_tuned(const NzGraph *graph, int32_t spanning, int32_t n_runs, uint64_t key, uint64_t run0,
                      const double *ps, int32_t P, double cutoff, int32_t window, int32_t conv_precision,
                      const NzTuning *tuning, void *workspace, size_t workspace_bytes, uint64_t *acc_count,
                      double *acc_mean, double *acc_m2, const NzMicroAccum *micro, void *stream) {
    if (!graph || n_runs <= 0 || P <= 0 || !ps || !acc_count || !acc_mean || !acc_m2) return NZ_ERR_INVALID;
    int32_t uf_block = 128, m2_tile = 8, slices = 0, conv_tile = 8, taper = 0;
    if (tuning) {
        if (tuning->uf_block) uf_block = tuning->uf_block;
        if (tuning->m2_tile) m2_tile = tuning->m2_tile;
        if (tuning->conv_tile) conv_tile = tuning->conv_tile;
        slices = tuning->reduce_slices;
        taper = tuning->taper != 0;
    }
    if ((uf_block != 32 && uf_block != 64 && uf_block != 128) || (m2_tile != 8 && m2_tile != 16) ||
        (conv_tile != 8 && conv_tile != 16) || slices < 0 || slices > kMaxSlices)
        return NZ_ERR_INVALID;
    if ((uint32_t)n_runs > NZ_MAX_RUNS) return NZ_ERR_TOO_LARGE;
    if (!(cutoff > 0)) cutoff = kDefaultCutoff;
    if (cutoff > kDefaultCutoff) return NZ_ERR_INVALID;  // workspace is sized for the default band
    if (conv_precision < 0 || conv_precision > 2) return NZ_ERR_INVALID;
    uint32_t N, M;
    int st = graph_size(*graph, N, M);
    if (st) return st;
    if (graph->kind == NZ_GRAPH_EDGES) return NZ_ERR_INVALID;  // lattices only on the fast path
    if (!conv_grid_fits(n_runs, P) || !conv_tc_grid_fits(n_runs, P)) return NZ_ERR_TOO_LARGE;
    if (micro && (!micro->count || !micro->span_count || !micro->sum_lo || !micro->sum_hi || !micro->m2))
        return NZ_ERR_INVALID;
    GraphDev g = make_graph_dev(*graph, N, M);
    Carver c{static_cast<uint8_t *>(workspace), 0, workspace_bytes};
    EnsembleLayout L;
    ensemble_layout(c, g, n_runs, P, kDefaultCutoff, window, L);
    if (!workspace || !c.ok()) return NZ_ERR_WORKSPACE;
    if (slices > 0) L.slices = slices < n_runs ? slices : n_runs;
    cudaStream_t s = as_stream(stream);

    {
        ProfScope prof(NZ_PROF_SETUP, s);
        launch_binomial_weights(M, ps, P, cutoff, L.cap, L.band_lo, L.band_len, L.w64, nullptr, s);
        if (conv_precision != 0)
            launch_narrow_weights_f32(L.w64, L.band_lo, L.band_len, P, L.cap, exp(-fmin(cutoff, kConvF32Cutoff)),
                                      exp(-kConvCoreCutoff), L.w32, L.w32lo, L.band_lo32, L.band_len32,
                                      L.core_lo32, L.core_len32, s);
        if (cudaMemsetAsync(L.flag, 0, 4 * sizeof(uint32_t), s) != cudaSuccess) return NZ_ERR_CUDA;
        launch_init_runs(g, n_runs, L.nodes, L.state, L.flag, s);
        if (cudaMemsetAsync(L.stats, 0, sizeof(double) * (size_t)n_runs * P * 7, s) != cudaSuccess)
            return NZ_ERR_CUDA;
    }

    AuxGuard aux{aux_checkout()};
    if (!aux.a) return NZ_ERR_CUDA;
    cudaStream_t s1 = aux.a->s1, s2 = aux.a->s2;
    // fork: the union-find and the consumer streams start after the set-up
    // above on the caller's stream `s`
    if (cudaEventRecord(aux.a->fork, s) != cudaSuccess || cudaStreamWaitEvent(s1, aux.a->fork, 0) != cudaSuccess ||
        cudaStreamWaitEvent(s2, aux.a->fork, 0) != cudaSuccess)
        return NZ_ERR_CUDA;
    JoinGuard joiner1{s, s1, aux.a->join1, true};
    JoinGuard joiner{s, s2, aux.a->join, true};

    UfParams up;
    up.g = g;
    up.n_runs = n_runs;
    up.nodes = L.nodes;
    up.state = L.state;
    up.key = key;
    up.run0 = run0;
    up.perms = nullptr;
    up.errors = L.flag + 1;  // zeroed in the set-up; read by nz_ensemble_errors
    ConvParams cp;
    cp.N = N;
    cp.n_runs = n_runs;
    cp.spanning = spanning;
    cp.P = P;
    cp.cap = L.cap;
    cp.band_lo = conv_precision != 0 ? L.band_lo32 : L.band_lo;
    cp.band_len = conv_precision != 0 ? L.band_len32 : L.band_len;
    cp.w64 = L.w64;
    cp.w32 = L.w32;
    cp.w32lo = L.w32lo;
    cp.core_lo = L.core_lo32;
    cp.core_len = L.core_len32;
    cp.m2_tile = m2_tile;
    cp.conv_tile = conv_tile;
    cp.acc = L.stats;
    cp.errors = L.flag + 1;  // with the union-find's corruption count
    MicroParams mp;
    if (micro) {
        mp.N = N;
        mp.n_runs = n_runs;
        mp.acc = *micro;
        mp.M = M;
        mp.count_before = micro->count;
    }
    // Window k: the union-find fills record buffer k % 2 on s1 while the
    // micro reductions and the convolution of window k - 1 read the other
    // buffer on s2.  The union-find of window k waits until the consumers of
    // window k - 2 (same buffer) are done; the consumers of window k wait for
    // its union-find.  Node words and run state live on s1 only, the
    // accumulators on s2 only.
    int k = 0;
    // Window schedule.  Only the first window's union-find runs with no
    // consumer beside it, and only the last window's consumers with no
    // union-find: with `taper` those two windows are a quarter window long
    // (at least 256 rows), the rest full.
    const uint32_t W = (uint32_t)L.window;
    const uint32_t q = taper ? (W / 4 > 256u ? W / 4 : (W < 256u ? W : 256u)) : W;
    auto window_end = [&](uint32_t w0, int kk) -> uint32_t {
        uint32_t len = W;
        if (taper) {
            const uint32_t rem = M + 1 - w0;
            if (kk == 0) len = q;
            else if (rem > W && rem < W + q) len = rem - q;  // leave a short last window
        }
        return (w0 + len > M + 1) ? M + 1 : w0 + len;
    };
    for (uint32_t w0 = 0, w1 = 0; w0 <= M; w0 = w1, ++k) {
        w1 = window_end(w0, k);
        const int b = k & 1;
        if (k >= 2 && cudaStreamWaitEvent(s1, aux.a->consumed[b], 0) != cudaSuccess) return NZ_ERR_CUDA;
        up.rec = L.rec[b];
        up.n_begin = w0; up.n_end = w1;
        {
            ProfScope prof(NZ_PROF_UNION_FIND, s1);
            launch_uf_window(up, NZ_PERM_PHILOX, spanning != 0, uf_block, s1);
        }
        if (cudaEventRecord(aux.a->produced[b], s1) != cudaSuccess ||
            cudaStreamWaitEvent(s2, aux.a->produced[b], 0) != cudaSuccess)
            return NZ_ERR_CUDA;
        if (micro) {
            ProfScope prof(NZ_PROF_MICRO, s2);
            mp.rec = L.rec[b];
            mp.n_begin = w0; mp.n_end = w1;
            launch_micro_window(mp, s2);
        }
        {
            ProfScope prof(NZ_PROF_CONV, s2);
            cp.rec = L.rec[b];
            cp.n_begin = w0; cp.n_end = w1;
            if (conv_precision == 2) {
                if (launch_conv_window_tc(cp, s2) != 0) return NZ_ERR_CUDA;
            } else {
                launch_conv_window(cp, conv_precision, s2);
            }
        }
        if (cudaEventRecord(aux.a->consumed[b], s2) != cudaSuccess) return NZ_ERR_CUDA;
    }
    {
        ProfScope prof(NZ_PROF_REDUCE, s2);
        if (micro) launch_micro_count(micro->count, n_runs, s2);
        launch_reduce_runs(L.stats, n_runs, P, acc_count, acc_mean, acc_m2, L.part, L.slices, s2);
    }
    // join: `s` continues after everything on s1 and s2
    if (joiner1.join_now() != NZ_OK || joiner.join_now() != NZ_OK) return NZ_ERR_CUDA;
    return check_launch();
}

int nz_ensemble_errors(const NzGraph *graph, int32_t n_runs, int32_t P, int32_t window, const void *workspace,
                       size_t workspace_bytes, uint32_t *errors, void *stream) {
    uint32_t N, M;
    if (!graph || !workspace || !errors || n_runs <= 0 || P <= 0) return NZ_ERR_INVALID;
    int st = graph_size(*graph, N, M);
    if (st) return st;
    GraphDev g = make_graph_dev(*graph, N, M);
    Carver c{static_cast<uint8_t *>(const_cast<void *>(workspace)), 0, workspace_bytes};
    EnsembleLayout L;
    ensemble_layout(c, g, n_runs, P, kDefaultCutoff, window, L);
    if (!c.ok()) return NZ_ERR_WORKSPACE;
    return cudaMemcpyAsync(errors, L.flag + 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice, as_stream(stream)) ==
                   cudaSuccess
               ? NZ_OK
               : NZ_ERR_CUDA;
}

// --------------------------------------------------------- batched uneven
namespace {

int mix_validate(const NzMixSpec *spec, int32_t n_runs, int32_t threads) {
    if (!spec || n_runs <= 0 || threads <= 0) return NZ_ERR_INVALID;
    if ((uint32_t)n_runs > NZ_MAX_RUNS) return NZ_ERR_TOO_LARGE;
    if (spec->grid_min < 1 || spec->grid_max < spec->grid_min || spec->chain_min < 1 ||
        spec->chain_max < spec->chain_min || spec->checkpoints < 2 ||
        (spec->reduction != NZ_MIX_REDUCE_RECORDS && spec->reduction != NZ_MIX_REDUCE_FUSED))
        return NZ_ERR_INVALID;
    if ((uint64_t)spec->grid_max * spec->grid_max > NZ_MAX_NODES || spec->chain_max > NZ_MAX_NODES)
        return NZ_ERR_TOO_LARGE;
    return NZ_OK;
}

size_t mix_layout(Carver &c, const NzMixSpec &sp, int32_t n_runs, int32_t T, MixLaunch &L) {
    const uint32_t n_classes = (sp.grid_max - sp.grid_min + 1) + (sp.chain_max - sp.chain_min + 1);
    const uint64_t nmax = std::max<uint64_t>(grid_slots(sp.grid_max), sp.chain_max);  // node words
    const size_t F = (size_t)sp.checkpoints;
    L.cls = c.take<uint32_t>(n_runs);
    L.counts = c.take<uint32_t>(n_classes);
    L.order = c.take<uint32_t>(n_classes);
    L.offsets = c.take<uint32_t>(n_classes);
    L.cursor = c.take<uint32_t>(n_classes);
    L.queue = c.take<uint32_t>(n_runs);
    L.head = c.take<uint32_t>(1);
    L.slot_off = c.take<uint64_t>((size_t)T + 1);
    L.nodes = c.take<uint32_t>((size_t)T * nmax);
    L.fused = sp.reduction == NZ_MIX_REDUCE_FUSED;
    L.rec = MixRec{};
    L.cells = nullptr;
    if (L.fused) {
        L.cells = c.take<uint64_t>((size_t)n_classes * F * kMixCellWords);
    } else {
        L.rec.max_span = c.take<uint32_t>((size_t)n_runs * F);
        L.rec.m0 = c.take<uint32_t>((size_t)n_runs * F);
        L.rec.m2 = c.take<uint64_t>((size_t)n_runs * F);
        L.rec.m3 = c.take<uint64_t>((size_t)n_runs * F);
        L.rec.m4_lo = c.take<uint64_t>((size_t)n_runs * F);
        L.rec.m4_hi = c.take<uint32_t>((size_t)n_runs * F);
    }
    return c.used;
}

}  // namespace

size_t nz_mix_workspace_bytes(const NzMixSpec *spec, int32_t n_runs, int32_t threads) {
    if (mix_validate(spec, n_runs, threads) != NZ_OK) return 0;
    Carver c{nullptr, 0, 0};
    MixLaunch L;
    return align_up(mix_layout(c, *spec, n_runs, threads, L));
}

int nz_mix(const NzMixSpec *spec, const uint32_t *thr_grid, const uint32_t *thr_chain, const uint64_t *key_dev,
           int32_t n_runs, int32_t threads, int32_t block, uint32_t smem_words, void *workspace,
           size_t workspace_bytes, const NzMixAccum *out, void *stream) {
    int st = mix_validate(spec, n_runs, threads);
    if (st) return st;
    if (!thr_grid || !thr_chain || !key_dev || !out || !out->count || !out->span || !out->sum_lo ||
        !out->sum_hi || !out->m2 || !out->errors)
        return NZ_ERR_INVALID;
    if (block <= 0 || block > 256 || (block & 31)) return NZ_ERR_INVALID;
    if ((size_t)smem_words * 4u * (size_t)block > 227u * 1024u) return NZ_ERR_INVALID;
    Carver c{static_cast<uint8_t *>(workspace), 0, workspace_bytes};
    MixLaunch L;
    mix_layout(c, *spec, n_runs, threads, L);
    if (!workspace || !c.ok()) return NZ_ERR_WORKSPACE;
    L.m.key_ptr = key_dev;
    L.m.n_runs = n_runs;
    L.m.chain_share = spec->chain_share;
    L.m.grid_min = spec->grid_min;
    L.m.grid_max = spec->grid_max;
    L.m.chain_min = spec->chain_min;
    L.m.chain_max = spec->chain_max;
    L.m.n_grid = spec->grid_max - spec->grid_min + 1;
    L.m.n_chain = spec->chain_max - spec->chain_min + 1;
    L.m.thr_grid = thr_grid;
    L.m.thr_chain = thr_chain;
    L.m.F = spec->checkpoints;
    L.T = threads;
    L.block = block;
    L.smem_words = smem_words;
    L.acc.count = out->count;
    L.acc.span = out->span;
    L.acc.sum_lo = out->sum_lo;
    L.acc.sum_hi = out->sum_hi;
    L.acc.m2 = out->m2;
    L.acc.errors = out->errors;
    ProfScope prof(NZ_PROF_UNION_FIND, as_stream(stream));
    return launch_mix(L, as_stream(stream));
}

}  // extern "C"
