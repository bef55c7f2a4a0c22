// Shared device helpers for libastro_cuda (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/astro_cuda.h"

namespace astro {

constexpr uint32_t kFullMask = 0xFFFFFFFFu;
constexpr float kQuantCells = 2097152.0f;  // 2^21 cells per axis
constexpr uint32_t kQuantMax = 2097151u;

// Spread the low 21 bits of v so that bit i lands on bit 3i (the bit
// placement of interleaveBitsOptimized, MortonCode.metal:7-23), with five
// shift-or-mask steps instead of a 21-iteration loop.
__host__ __device__ __forceinline__ uint64_t spread3_21(uint32_t v) {
    uint64_t x = v & 0x1FFFFFu;
    x = (x | (x << 32)) & 0x001F00000000FFFFull;
    x = (x | (x << 16)) & 0x001F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Inverse of spread3_21: gather bits 0, 3, 6, ... of x into bits 0, 1, 2, ...
__host__ __device__ __forceinline__ uint32_t compact3_21(uint64_t x) {
    x &= 0x1249249249249249ull;
    x = (x ^ (x >> 2)) & 0x10C30C30C30C30C3ull;
    x = (x ^ (x >> 4)) & 0x100F00F00F00F00Full;
    x = (x ^ (x >> 8)) & 0x001F0000FF0000FFull;
    x = (x ^ (x >> 16)) & 0x001F00000000FFFFull;
    x = (x ^ (x >> 32)) & 0x00000000001FFFFFull;
    return (uint32_t)x;
}

__host__ __device__ __forceinline__ uint64_t interleave3(uint32_t x, uint32_t y, uint32_t z) {
    return spread3_21(x) | (spread3_21(y) << 1) | (spread3_21(z) << 2);
}

// Order-preserving maps of floats to unsigned integers, so that bounding
// boxes can be reduced with integer atomicMin/atomicMax.
__device__ __forceinline__ uint32_t f32_to_ordered(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_f32(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
__device__ __forceinline__ unsigned long long f64_to_ordered(double f) {
    unsigned long long u = (unsigned long long)__double_as_longlong(f);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ordered_to_f64(unsigned long long u) {
    return __longlong_as_double(
        (long long)((u & 0x8000000000000000ull) ? (u & 0x7FFFFFFFFFFFFFFFull) : ~u));
}

// Exact 2^e for the exponents used by the cell sizes (|e| <= 21).
__device__ __forceinline__ float exp2_exact(int e) { return __int_as_float((127 + e) << 23); }

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Device-side error word bits, read back by the host after a stream sync.
enum DeviceError : uint32_t {
    kErrLookbackTimeout = 1u << 0,  // a decoupled look-back wait gave up
    kErrStackOverflow = 1u << 1,    // a traversal stack bound was hit
    kErrBadLayer = 1u << 2,
    kErrFrontier = 1u << 3,         // a group walk's frontier or list pool was too small
};

// Bounded spin for decoupled look-back: after this many polls the waiting
// thread records kErrLookbackTimeout and carries on with what it has.
constexpr uint32_t kSpinLimit = 1u << 22;

// Decoupled look-back status words: 2 status bits over a 30-bit count.
constexpr uint32_t kLbAggregate = 1u << 30;
constexpr uint32_t kLbInclusive = 2u << 30;
constexpr uint32_t kLbCountMask = (1u << 30) - 1;

// Spin on the status word of an earlier tile until it is published, then
// return it. After `limit` polls it sets the error bit and returns an
// inclusive zero, so the caller's prefix only misses counts (its stores stay
// below their true positions, inside the output).
__device__ __forceinline__ uint32_t lookback_wait(const uint32_t* word, uint32_t* err,
                                                  uint32_t limit = kSpinLimit) {
    uint32_t v = ld_relaxed_u32(word);
    uint32_t polls = 0;
    while ((v >> 30) == 0) {
        if (++polls > limit) {
            atomicOr(err, kErrLookbackTimeout);
            return kLbInclusive;  // treat as an inclusive zero so the caller stops
        }
        if (polls > 64) __nanosleep(32);
        v = ld_relaxed_u32(word);
    }
    return v;
}

// Decoupled look-back for the status word of column `col` (`stride` words
// per tile) of tiles before `tile`: reads kLbWindow predecessors per
// round so that one memory latency covers several tiles, adds their counts
// back to the first inclusive one, and re-polls (bounded) a word that is not
// published yet. Returns the exclusive prefix of tile `tile`.
constexpr int kLbWindow = 8;
__device__ __forceinline__ uint32_t lookback_window(const uint32_t* words, uint32_t tile,
                                                    uint32_t col, uint32_t* err,
                                                    uint32_t stride = 256,
                                                    uint32_t limit = kSpinLimit) {
    uint32_t prefix = 0;
    int64_t j = (int64_t)tile - 1;
    while (j >= 0) {
        uint32_t v[kLbWindow];
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k)
            v[k] = (j - k >= 0) ? ld_relaxed_u32(words + (size_t)(j - k) * stride + col) : kLbInclusive;
        int k = 0;
        for (; k < kLbWindow; ++k) {
            if ((v[k] >> 30) == 0) break;  // not published yet: wait on it below
            prefix += v[k] & kLbCountMask;
            if ((v[k] & kLbInclusive) != 0) return prefix;
        }
        j -= k;
        if (k < kLbWindow) {
            const uint32_t w = lookback_wait(words + (size_t)j * stride + col, err, limit);
            prefix += w & kLbCountMask;
            if ((w & kLbInclusive) != 0) return prefix;
            --j;
        }
    }
    return prefix;
}

}  // namespace astro
