// Values of one statistic of the per-step records, as the canonical
// convolutions read them.
#pragma once
#include <cstdint>

#include "nz_common.cuh"

namespace nz {

// Statistic S of the record at `off` (S = 0 spanning, 1 max, 2 m0, 3 m1,
// 4 m2, 5 m3, 6 m4; 7 = m4 of records without the m4_hi plane, whose high
// word is zero).  The FP32 loader splits 64-bit words into 32-bit halves so
// that every conversion stays on the FP32 pipe.
template <int S>
__device__ __forceinline__ double record_value(const NzRecords &rec, size_t off, uint32_t N) {
    if (S == 0) return (rec.max_span[off] & kSpanBit) ? 1.0 : 0.0;
    if (S == 1) return (double)(rec.max_span[off] & ~kSpanBit);
    if (S == 2) return (double)rec.m0[off];
    if (S == 3) return (double)(N - (rec.max_span[off] & ~kSpanBit));
    if (S == 4) return (double)rec.m2[off];
    if (S == 5) return (double)rec.m3[off];
    if (S == 7) return (double)rec.m4_lo[off];
    return fma((double)rec.m4_hi[off], 18446744073709551616.0, (double)rec.m4_lo[off]);
}

__device__ __forceinline__ float u64_to_f32(uint64_t x) {
    return fmaf((float)(uint32_t)(x >> 32), 4294967296.0f, (float)(uint32_t)x);
}

template <int S>
__device__ __forceinline__ float record_value_f(const NzRecords &rec, size_t off, uint32_t N) {
    if (S == 0) return (rec.max_span[off] & kSpanBit) ? 1.0f : 0.0f;
    if (S == 1) return (float)(rec.max_span[off] & ~kSpanBit);
    if (S == 2) return (float)rec.m0[off];
    if (S == 3) return (float)(N - (rec.max_span[off] & ~kSpanBit));
    if (S == 4) return u64_to_f32(rec.m2[off]);
    if (S == 5) return u64_to_f32(rec.m3[off]);
    if (S == 7) return u64_to_f32(rec.m4_lo[off]);
    return fmaf((float)rec.m4_hi[off], 18446744073709551616.0f, u64_to_f32(rec.m4_lo[off]));
}

}  // namespace nz
