// Values of one statistic of the per-step records, as the canonical
// convolutions read them.
#pragma once
#include <cstdint>

#include "nz_common.cuh"

namespace nz {

// Statistic S of the record at `off` (S = 0 spanning, 1 max, 2 m0, 3 m1,
// 4 m2, 5 m3, 6 m4; 7 = m4 of records without the m4_hi plane, whose high
// word is zero; 8 = m0 and 9 = m2 of narrow records, stored as uint16 and
// uint32).  The FP32 loader splits 64-bit words into 32-bit halves so
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
    if (S == 8) return (double)reinterpret_cast<const uint16_t *>(rec.m0)[off];
    if (S == 9) return (double)reinterpret_cast<const uint32_t *>(rec.m2)[off];
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
    if (S == 8) return (float)reinterpret_cast<const uint16_t *>(rec.m0)[off];
    if (S == 9) return (float)reinterpret_cast<const uint32_t *>(rec.m2)[off];
    return fmaf((float)rec.m4_hi[off], 18446744073709551616.0f, u64_to_f32(rec.m4_lo[off]));
}

// m0 and m2 of a record in either layout (narrow: uint16 / uint32)
__device__ __forceinline__ uint32_t record_m0(const NzRecords &rec, size_t off) {
    return rec.narrow ? (uint32_t)reinterpret_cast<const uint16_t *>(rec.m0)[off] : rec.m0[off];
}
__device__ __forceinline__ uint64_t record_m2(const NzRecords &rec, size_t off) {
    return rec.narrow ? (uint64_t)reinterpret_cast<const uint32_t *>(rec.m2)[off] : rec.m2[off];
}

// writes m0 and m2 of a record in either layout
__device__ __forceinline__ void put_m0_m2(const NzRecords &rec, size_t off, uint32_t m0, uint64_t m2) {
    if (rec.narrow) {
        if (rec.m0) reinterpret_cast<uint16_t *>(rec.m0)[off] = (uint16_t)m0;
        if (rec.m2) reinterpret_cast<uint32_t *>(rec.m2)[off] = (uint32_t)m2;
    } else {
        if (rec.m0) rec.m0[off] = m0;
        if (rec.m2) rec.m2[off] = m2;
    }
}

}  // namespace nz
