// nz_noalloc.cu -- microcanonical statistics with no device allocation at all.
//
// Some callers cannot allocate device memory: a host framework or plugin
// runtime that owns the whole device memory pool and hands out only the
// buffers it manages, or a foreign-language binding that can pass pointers
// to buffers it already holds but has no way to obtain new ones.  For them
// this file keeps the union-find scratch of nz_microcanonical (node words,
// per-run state, MT19937 permutations) in a fixed array that is part of the
// library image: every GPU that loads the library reserves it until the
// process exits.  The caller still supplies inputs and the output records.
#include <cuda.h>  // CUcontext / CUresult types; the driver calls are fetched at run time
#include <cstdint>
#include <mutex>

#include "nz_common.cuh"
#include "nz_internal.cuh"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB

__device__ __align__(256) unsigned char g_nz_static_scratch[kStaticScratchBytes];

// The array's device address belongs to a CUDA context, not to a device: a
// cudaDeviceReset, or a caller that makes its own (non-primary) context
// current, gives the same device another context in which the array sits
// elsewhere.  Addresses are therefore cached per context, keyed by the
// context's ID (cuCtxGetId: unique for the life of the process, so a context
// created after a reset never matches an entry of the one it replaced).  The
// two driver calls are looked up through the runtime so that the library
// does not link libcuda itself.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

struct ScratchEntry {
    unsigned long long ctx_id;
    void *addr;
};
constexpr int kMaxContexts = 64;
std::mutex g_scratch_mu;
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_n = 0;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

bool resolve_driver_calls() {  // with g_scratch_mu held
    if (g_ctx_get_current && g_ctx_get_id) return true;
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
        qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
        return false;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(a);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(b);
    return true;
}

// Device address of the scratch array in the current context.  Host code
// only sees a host-side stand-in under the array's name, so the address is
// taken (cudaGetSymbolAddress) the first time a context calls, with that
// context current, and cached under the context's ID.
int scratch_for_current_context(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NZ_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!resolve_driver_calls()) return NZ_ERR_CUDA;
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return NZ_ERR_CUDA;
    if (!ctx) {
        // nothing current yet: make the device's primary context current
        // (cudaSetDevice initialises it; it allocates nothing)
        if (cudaSetDevice(dev) != cudaSuccess || g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
            return NZ_ERR_CUDA;
    }
    unsigned long long id = 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return NZ_ERR_CUDA;
    for (int i = 0; i < g_scratch_n; ++i)
        if (g_scratch[i].ctx_id == id) { *out = g_scratch[i].addr; return NZ_OK; }
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_nz_static_scratch) != cudaSuccess || !p) return NZ_ERR_CUDA;
    // a full table drops its oldest entry (a context that called long ago
    // looks its address up again)
    if (g_scratch_n == kMaxContexts) {
        for (int i = 1; i < kMaxContexts; ++i) g_scratch[i - 1] = g_scratch[i];
        --g_scratch_n;
    }
    g_scratch[g_scratch_n++] = {id, p};
    *out = p;
    return NZ_OK;
}

}  // namespace

extern "C" {

size_t nz_static_scratch_bytes(void) { return kStaticScratchBytes; }

int nz_microcanonical_noalloc(const NzGraph *graph, int32_t spanning, int32_t n_runs, int32_t perm_mode,
                              uint64_t key, uint64_t run0, const uint32_t *perms,
                              const uint32_t *mt_seed_words, const int32_t *mt_seed_len,
                              int32_t mt_words_stride, const NzRecords *out, void *stream) {
    if (!graph || !out || n_runs <= 0) return NZ_ERR_INVALID;
    const size_t need = nz_microcanonical_workspace_bytes(graph, n_runs, perm_mode);
    if (need == 0) return NZ_ERR_INVALID;
    if (need > kStaticScratchBytes) return NZ_ERR_TOO_LARGE;
    void *scratch = nullptr;
    const int st = scratch_for_current_context(&scratch);
    if (st) return st;
    // The kernels overwrite every node word and run state before reading it;
    // the one flag that must start at zero is cleared by a stream-ordered
    // memset inside nz_microcanonical.
    return nz_microcanonical(graph, spanning, n_runs, perm_mode, key, run0, perms, mt_seed_words, mt_seed_len,
                             mt_words_stride, scratch, kStaticScratchBytes, out, stream);
}

}  // extern "C"
