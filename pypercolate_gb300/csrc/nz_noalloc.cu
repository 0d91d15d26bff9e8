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
#include <cstdint>
#include <mutex>

#include "nz_common.cuh"
#include "nz_internal.cuh"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB

__device__ __align__(256) unsigned char g_nz_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  Host code only
// sees a host-side stand-in under the array's name, so the address is taken
// once per device (with that device current) and cached.
int scratch_for_current_device(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NZ_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return NZ_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_nz_static_scratch) != cudaSuccess || !p) return NZ_ERR_CUDA;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
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
    const int st = scratch_for_current_device(&scratch);
    if (st) return st;
    // The kernels overwrite every node word and run state before reading it;
    // the one flag that must start at zero is cleared by a stream-ordered
    // memset inside nz_microcanonical.
    return nz_microcanonical(graph, spanning, n_runs, perm_mode, key, run0, perms, mt_seed_words, mt_seed_len,
                             mt_words_stride, scratch, kStaticScratchBytes, out, stream);
}

}  // extern "C"
