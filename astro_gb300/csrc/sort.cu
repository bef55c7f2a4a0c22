// Onesweep LSD radix sort of (uint64 key, uint32 value) pairs for sm_103a.
//
// Replaces MetalKernelsRadixSort.sort (Astro/RadixSort.swift:98-185), whose
// 64 one-bit split passes (split_prep / prefixSum / prefixFixup /
// split_scatter, Astro/RadixSort.metal:30-131) each move the whole key and
// index arrays. Here the key is consumed 8 bits per pass:
//   1. one histogram kernel reads the keys once and counts every digit of
//      every pass (warp-ballot peer groups, shared-memory histograms); its
//      last block turns the counts into exclusive digit offsets;
//   2. one kernel per pass: each block takes the next tile (atomic ticket),
//      ranks its keys stably with warp-ballot peer masks and per-warp digit
//      counters in shared memory, publishes its digit counts, stages the
//      tile in sorted order in shared memory, obtains the counts of all
//      earlier tiles by decoupled look-back (bounded waits), and writes each
//      digit's run of the tile with contiguous stores.
// A stable LSD sort yields the one stable permutation, so the result equals
// the reference's bit by bit, including the order of equal keys.
#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace astro {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;
constexpr int kHistBlocksPerSm = 8;

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFullMask, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kWarps; o <<= 1) {
            uint32_t y = __shfl_up_sync(kFullMask, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        if (lane < kWarps) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t r = (warp ? s_warp[warp - 1] : 0u) + x - v;
    __syncthreads();
    return r;
}

// Lanes of the warp whose digit equals this lane's digit, among `valid`.
__device__ __forceinline__ uint32_t peer_mask(uint32_t digit, uint32_t bits, uint32_t valid) {
    uint32_t peers = valid;
    for (uint32_t b = 0; b < bits; ++b) {
        uint32_t bit = (digit >> b) & 1u;
        uint32_t ballot = __ballot_sync(kFullMask, bit);
        peers &= bit ? ballot : ~ballot;
    }
    return peers;
}

// All digit histograms in one read of the keys. Each warp counts into its own
// shared-memory copy with atomics; a warp whose 32 keys share a digit (the
// usual case for the high digits of Morton keys of a Morton-ordered state)
// adds 32 with a single atomic.
__global__ __launch_bounds__(kThreads) void sort_histogram_kernel(
    const uint64_t* __restrict__ keys, const uint32_t* __restrict__ d_count, uint32_t n_est,
    uint32_t key_bits, uint32_t passes, uint32_t* __restrict__ hist, uint32_t* __restrict__ excl,
    uint32_t* __restrict__ done) {
    extern __shared__ uint32_t s_hist[];  // [kWarps][passes][kRadix]
    __shared__ uint32_t s_warp[kWarps];
    __shared__ bool s_last;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = d_count ? min(*d_count, n_est) : n_est;
    const uint32_t per_warp = passes * kRadix;
    for (uint32_t i = tid; i < kWarps * per_warp; i += kThreads) s_hist[i] = 0;
    __syncthreads();
    uint32_t* my_hist = s_hist + warp * per_warp;
    // Each thread takes kHistKeys keys per round (independent loads in flight).
    constexpr int kHistKeys = 4;
    const uint64_t stride = (uint64_t)gridDim.x * kThreads * kHistKeys;
    for (uint64_t base = (uint64_t)blockIdx.x * kThreads * kHistKeys; base < n; base += stride) {
        uint64_t key[kHistKeys];
        bool valid[kHistKeys];
#pragma unroll
        for (int k = 0; k < kHistKeys; ++k) {
            const uint64_t i = base + (uint64_t)k * kThreads + tid;
            valid[k] = i < n;
            key[k] = valid[k] ? __ldcs(keys + i) : 0ull;
        }
#pragma unroll
        for (int k = 0; k < kHistKeys; ++k) {
            const bool full = __all_sync(kFullMask, valid[k]);
            for (uint32_t p = 0; p < passes; ++p) {
                const uint32_t shift = 8u * p;
                const uint32_t bits = min(8u, key_bits - shift);
                const uint32_t digit = (uint32_t)(key[k] >> shift) & ((1u << bits) - 1u);
                const bool same =
                    full && __all_sync(kFullMask, digit == __shfl_sync(kFullMask, digit, 0));
                if (same) {
                    if (lane == 0) atomicAdd(&my_hist[p * kRadix + digit], 32u);
                } else if (valid[k]) {
                    atomicAdd(&my_hist[p * kRadix + digit], 1u);
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t i = tid; i < per_warp; i += kThreads) {
        uint32_t c = 0;
        for (int w = 0; w < kWarps; ++w) c += s_hist[w * per_warp + i];
        if (c) atomicAdd(&hist[i], c);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (uint32_t p = 0; p < passes; ++p) {
        uint32_t c = __ldcg(&hist[p * kRadix + tid]);
        excl[p * kRadix + tid] = block_exclusive_scan(c, s_warp);
    }
}

// The tile in sorted order for the scatter: keys with their values, or
// (lean passes) keys with the tile-local index of their value.
template <int kItems, bool kLean>
struct StageArrays {
    uint64_t keys[kThreads * kItems];
    uint32_t vals[kThreads * kItems];
};
template <int kItems>
struct StageArrays<kItems, true> {
    uint64_t keys[kThreads * kItems];
    uint16_t src[kThreads * kItems];
};

template <int kItems, bool kLean = false>
struct PassSmem {
    static constexpr int kTile = kThreads * kItems;
    union {
        uint32_t warp_hist[kWarps][kRadix];  // ranking: per-warp digit counters
        StageArrays<kItems, kLean> stage;    // scatter: the tile in sorted order
    } u;
    uint32_t tile_start[kRadix];   // first slot of each digit inside the tile
    uint32_t global_base[kRadix];  // first output slot of each digit of this tile
    uint32_t scan_tmp[kWarps];
    uint32_t tile_id;
};

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// One onesweep pass. kItems pairs per thread; kMatch ranks with
// __match_any_sync and one shared atomic per distinct digit, otherwise with
// per-bit ballots and per-warp counters. kLean keeps no value in registers:
// the tile's values are prefetched into L2 when the keys are loaded and
// gathered by their tile-local index (staged as 16 bits beside the key) in
// the scatter, so fewer registers and less shared memory let more blocks
// share an SM.
template <int kItems, int kMinBlocks, bool kMatch, bool kLean = false>
__global__ __launch_bounds__(kThreads, kMinBlocks) void sort_pass_kernel(
    const uint64_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
    const uint32_t* __restrict__ d_count, uint32_t n_est, const uint32_t* __restrict__ excl,
    uint32_t* __restrict__ lookback, uint32_t* __restrict__ tile_counter, uint32_t shift,
    uint32_t digit_bits, uint32_t* __restrict__ err, uint32_t spin_limit) {
    using Smem = PassSmem<kItems, kLean>;
    constexpr int kTile = Smem::kTile;
    static_assert(kTile <= 65536, "tile-local indices fit 16 bits");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = d_count ? min(*d_count, n_est) : n_est;
    if (tid == 0) sm.tile_id = atomicAdd(tile_counter, 1u);
    for (uint32_t i = tid; i < kWarps * kRadix; i += kThreads) (&sm.u.warp_hist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = sm.tile_id;
    const uint64_t tile_base = (uint64_t)tile * kTile;
    if (tile_base >= n) return;
    const uint32_t dmask = (1u << digit_bits) - 1u;
    const uint32_t lt = lanemask_lt();

    // Warp-striped load: warp w owns a contiguous 32*kItems slice, item k of
    // lane j sits at slice + 32k + j, so processing k in order keeps the
    // ranking stable.
    uint64_t key[kItems];
    uint32_t val[kLean ? 1 : kItems], pos[kItems];
    const uint64_t warp_base = tile_base + (uint64_t)warp * 32 * kItems;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t i = warp_base + 32ull * k + lane;
        const bool valid = i < n;
        key[k] = valid ? __ldcs(keys_in + i) : ~0ull;
        if constexpr (kLean) {
            // One prefetch per 32 values (a 128-byte line) of this item.
            if (vals_in && lane == 0 && valid) prefetch_l2(vals_in + i);
        } else {
            val[k] = valid ? (vals_in ? __ldcs(vals_in + i) : (uint32_t)i) : 0u;
        }
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t i = warp_base + 32ull * k + lane;
        const bool valid = i < n;
        const uint32_t digit = (uint32_t)(key[k] >> shift) & dmask;
        if (kMatch) {
            const uint32_t peers = __match_any_sync(kFullMask, valid ? digit : (256u + lane));
            const uint32_t leader = 31u - __clz(peers);
            uint32_t old = 0;
            if (valid && lane == leader) old = atomicAdd(&sm.u.warp_hist[warp][digit], __popc(peers));
            old = __shfl_sync(kFullMask, old, leader);
            pos[k] = old + __popc(peers & lt);
        } else {
            const uint32_t peers = peer_mask(digit, digit_bits, __ballot_sync(kFullMask, valid));
            const uint32_t lower = __popc(peers & lt), cnt = __popc(peers);
            uint32_t old = 0;
            if (valid) old = sm.u.warp_hist[warp][digit];
            __syncwarp();
            if (valid && lower + 1 == cnt) sm.u.warp_hist[warp][digit] = old + cnt;
            __syncwarp();
            pos[k] = old + lower;
        }
    }
    __syncthreads();

    // Thread d owns digit d: per-warp exclusive offsets and the tile count.
    uint32_t tile_cnt = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        uint32_t c = sm.u.warp_hist[w][tid];
        sm.u.warp_hist[w][tid] = tile_cnt;
        tile_cnt += c;
    }
    uint32_t* my_word = lookback + (size_t)tile * kRadix + tid;
    st_relaxed_u32(my_word, (tile == 0 ? kLbInclusive : kLbAggregate) | tile_cnt);
    const uint32_t tile_start = block_exclusive_scan(tile_cnt, sm.scan_tmp);
    sm.tile_start[tid] = tile_start;
    __syncthreads();

    // The tile is staged in sorted order before the look-back: staging needs
    // only tile-local offsets, and the time it takes is slack in which the
    // earlier tiles publish their counts.
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint32_t digit = (uint32_t)(key[k] >> shift) & dmask;
        pos[k] += sm.tile_start[digit] + sm.u.warp_hist[warp][digit];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t i = warp_base + 32ull * k + lane;
        if (i < n) {
            sm.u.stage.keys[pos[k]] = key[k];
            if constexpr (kLean)
                sm.u.stage.src[pos[k]] = (uint16_t)(warp * 32u * kItems + 32u * k + lane);
            else
                sm.u.stage.vals[pos[k]] = val[k];
        }
    }
    uint32_t prefix = 0;
    if (tile > 0) {
        prefix = lookback_window(lookback, tile, tid, err, kRadix, spin_limit);
        st_relaxed_u32(my_word, kLbInclusive | (prefix + tile_cnt));
    }
    sm.global_base[tid] = excl[tid] + prefix;
    __syncthreads();
    const uint32_t tile_n = (uint32_t)min((uint64_t)kTile, (uint64_t)n - tile_base);
    if constexpr (kLean) {
        // Gather every value of this thread's slots first (independent
        // loads in flight), then store.
        uint32_t v[kItems];
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t i = tid + (uint32_t)k * kThreads;
            const uint32_t sidx = i < tile_n ? (uint32_t)sm.u.stage.src[i] : 0u;
            v[k] = i < tile_n ? (vals_in ? __ldcs(vals_in + tile_base + sidx) : (uint32_t)(tile_base + sidx))
                              : 0u;
        }
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t i = tid + (uint32_t)k * kThreads;
            if (i < tile_n) {
                const uint64_t key_i = sm.u.stage.keys[i];
                const uint32_t digit = (uint32_t)(key_i >> shift) & dmask;
                const uint32_t o = sm.global_base[digit] + (i - sm.tile_start[digit]);
                keys_out[o] = key_i;
                vals_out[o] = v[k];
            }
        }
    } else {
        for (uint32_t i = tid; i < tile_n; i += kThreads) {
            const uint64_t k = sm.u.stage.keys[i];
            const uint32_t digit = (uint32_t)(k >> shift) & dmask;
            const uint32_t o = sm.global_base[digit] + (i - sm.tile_start[digit]);
            keys_out[o] = k;
            vals_out[o] = sm.u.stage.vals[i];
        }
    }
}

// ------------------------------------------------------ pipelined pass ----
// Persistent blocks. Each block takes the ticket of its next tile before it
// ranks the current one and has that tile's keys (and values) brought into
// shared memory by bulk asynchronous copies (cp.async.bulk completing on an
// mbarrier), so the load of tile t+1 overlaps the ranking, look-back and
// scatter of tile t. Only whole tiles whose source addresses are 16-byte
// aligned are copied this way; the last, partial tile is read directly.
// Tickets keep their order, so a tile's look-back only waits on tiles that
// running blocks hold and finish first. Every wait is bounded.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for the phase of the given parity; false (and the error bit)
// after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* err,
                                          uint32_t limit) {
    for (uint32_t polls = 0; polls < limit; ++polls) {
        if (mbar_test(bar, parity)) return true;
        if (polls > 64) __nanosleep(32);
    }
    atomicOr(err, kErrLookbackTimeout);
    return false;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

template <int kItems>
struct PipeSmem {
    static constexpr int kTile = kThreads * kItems;
    uint64_t keys[2][kTile];  // tile buffers; the current one is reused as the scatter stage
    uint32_t vals[2][kTile];
    uint32_t warp_hist[kWarps][kRadix];
    uint32_t tile_start[kRadix];
    uint32_t global_base[kRadix];
    uint32_t scan_tmp[kWarps];
    uint32_t tile_next;
    uint32_t pad;
    uint64_t bar[2];
};

template <int kItems, int kMinBlocks>
__global__ __launch_bounds__(kThreads, kMinBlocks) void sort_pass_pipelined_kernel(
    const uint64_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
    const uint32_t* __restrict__ d_count, uint32_t n_est, const uint32_t* __restrict__ excl,
    uint32_t* __restrict__ lookback, uint32_t* __restrict__ tile_counter, uint32_t shift,
    uint32_t digit_bits, uint32_t* __restrict__ err, uint32_t spin_limit) {
    using Smem = PipeSmem<kItems>;
    constexpr int kTile = Smem::kTile;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = d_count ? min(*d_count, n_est) : n_est;
    const uint32_t ntiles = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);
    const uint32_t nfull = n / kTile;  // tiles fetched by bulk copies
    const uint32_t dmask = (1u << digit_bits) - 1u;
    const uint32_t lt = lanemask_lt();
    const uint32_t tx_bytes = kTile * 8u + (vals_in ? kTile * 4u : 0u);

    if (tid == 0) {
        mbar_init(&sm.bar[0]);
        mbar_init(&sm.bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sm.tile_next = atomicAdd(tile_counter, 1u);
    }
    __syncthreads();
    uint32_t cur = sm.tile_next;
    if (cur >= ntiles) return;
    // Thread 0 issues the copies; phase and pending bits are kept by every
    // thread (all of them wait).
    auto issue = [&](uint32_t t, uint32_t buf) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&sm.bar[buf], tx_bytes);
        bulk_load(sm.keys[buf], keys_in + (size_t)t * kTile, kTile * 8u, &sm.bar[buf]);
        if (vals_in) bulk_load(sm.vals[buf], vals_in + (size_t)t * kTile, kTile * 4u, &sm.bar[buf]);
    };
    // Per-buffer bits: the mbarrier phase parity to wait for, and whether a
    // copy into the buffer is in flight.
    uint32_t phase = 0u, pending = 0u;
    uint32_t b = 0;
    if (cur < nfull) {
        if (tid == 0) issue(cur, 0);
        pending |= 1u;
    }
    while (true) {
        if (tid == 0) sm.tile_next = atomicAdd(tile_counter, 1u);
        for (uint32_t i = tid; i < kWarps * kRadix; i += kThreads) (&sm.warp_hist[0][0])[i] = 0;
        __syncthreads();
        const uint32_t next = sm.tile_next;
        if (next < nfull) {
            if (tid == 0) issue(next, b ^ 1u);
            pending |= 1u << (b ^ 1u);
        }
        const uint64_t tile_base = (uint64_t)cur * kTile;
        const uint32_t warp_off = warp * 32u * kItems;
        uint64_t key[kItems];
        uint32_t val[kItems], pos[kItems];
        if ((pending >> b) & 1u) {
            mbar_wait(&sm.bar[b], (phase >> b) & 1u, err, spin_limit);
            phase ^= 1u << b;
            pending &= ~(1u << b);
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                const uint32_t li = warp_off + 32u * k + lane;
                key[k] = sm.keys[b][li];
                val[k] = vals_in ? sm.vals[b][li] : (uint32_t)(tile_base + li);
            }
        } else {
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                const uint64_t i = tile_base + warp_off + 32ull * k + lane;
                const bool valid = i < n;
                key[k] = valid ? __ldcs(keys_in + i) : ~0ull;
                val[k] = valid ? (vals_in ? __ldcs(vals_in + i) : (uint32_t)i) : 0u;
            }
        }
        // Ranking with per-bit ballots, in item order (stable).
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint64_t i = tile_base + warp_off + 32ull * k + lane;
            const bool valid = i < n;
            const uint32_t digit = (uint32_t)(key[k] >> shift) & dmask;
            const uint32_t peers = peer_mask(digit, digit_bits, __ballot_sync(kFullMask, valid));
            const uint32_t lower = __popc(peers & lt), cnt = __popc(peers);
            uint32_t old = 0;
            if (valid) old = sm.warp_hist[warp][digit];
            __syncwarp();
            if (valid && lower + 1 == cnt) sm.warp_hist[warp][digit] = old + cnt;
            __syncwarp();
            pos[k] = old + lower;
        }
        __syncthreads();
        uint32_t tile_cnt = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = sm.warp_hist[w][tid];
            sm.warp_hist[w][tid] = tile_cnt;
            tile_cnt += c;
        }
        uint32_t* my_word = lookback + (size_t)cur * kRadix + tid;
        st_relaxed_u32(my_word, (cur == 0 ? kLbInclusive : kLbAggregate) | tile_cnt);
        const uint32_t tile_start = block_exclusive_scan(tile_cnt, sm.scan_tmp);
        sm.tile_start[tid] = tile_start;
        uint32_t prefix = 0;
        if (cur > 0) {
            prefix = lookback_window(lookback, cur, tid, err, kRadix, spin_limit);
            st_relaxed_u32(my_word, kLbInclusive | (prefix + tile_cnt));
        }
        sm.global_base[tid] = excl[tid] + prefix;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t digit = (uint32_t)(key[k] >> shift) & dmask;
            pos[k] += sm.tile_start[digit] + sm.warp_hist[warp][digit];
        }
        // The current buffer is free (its contents are in registers): stage
        // the tile there in sorted order.
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint64_t i = tile_base + warp_off + 32ull * k + lane;
            if (i < n) {
                sm.keys[b][pos[k]] = key[k];
                sm.vals[b][pos[k]] = val[k];
            }
        }
        __syncthreads();
        const uint32_t tile_n = (uint32_t)min((uint64_t)kTile, (uint64_t)n - tile_base);
        for (uint32_t i = tid; i < tile_n; i += kThreads) {
            const uint64_t kk = sm.keys[b][i];
            const uint32_t digit = (uint32_t)(kk >> shift) & dmask;
            const uint32_t o = sm.global_base[digit] + (i - sm.tile_start[digit]);
            keys_out[o] = kk;
            vals_out[o] = sm.vals[b][i];
        }
        __syncthreads();
        if (next >= ntiles) break;
        cur = next;
        b ^= 1u;
    }
    // A copy is only left in flight if a wait gave up; wait for it (bounded)
    // before the block's shared memory is released.
    for (uint32_t k = 0; k < 2; ++k)
        if ((pending >> k) & 1u) mbar_wait(&sm.bar[k], (phase >> k) & 1u, err, spin_limit);
}

// Pass-kernel variants (items per thread, blocks per SM, ranking; the
// pipelined ones run persistent blocks and need 16-byte aligned inputs).
struct PassVariant {
    int items;
    void (*kernel)(const uint64_t*, const uint32_t*, uint64_t*, uint32_t*, const uint32_t*, uint32_t,
                   const uint32_t*, uint32_t*, uint32_t*, uint32_t, uint32_t, uint32_t*, uint32_t);
    size_t smem;
    bool pipelined;
};
const PassVariant kVariants[] = {
    {16, sort_pass_kernel<16, 2, false>, sizeof(PassSmem<16>), false},
    {16, sort_pass_kernel<16, 2, true>, sizeof(PassSmem<16>), false},
    {12, sort_pass_kernel<12, 3, true>, sizeof(PassSmem<12>), false},
    {8, sort_pass_kernel<8, 4, true>, sizeof(PassSmem<8>), false},
    {20, sort_pass_kernel<20, 2, true>, sizeof(PassSmem<20>), false},
    {12, sort_pass_kernel<12, 3, false>, sizeof(PassSmem<12>), false},
    {8, sort_pass_kernel<8, 4, false>, sizeof(PassSmem<8>), false},
    {12, sort_pass_pipelined_kernel<12, 2>, sizeof(PipeSmem<12>), true},
    {8, sort_pass_pipelined_kernel<8, 3>, sizeof(PipeSmem<8>), true},
    {12, sort_pass_kernel<12, 4, false, true>, sizeof(PassSmem<12, true>), false},
    {16, sort_pass_kernel<16, 3, false, true>, sizeof(PassSmem<16, true>), false},
    {20, sort_pass_kernel<20, 3, true, true>, sizeof(PassSmem<20, true>), false},
};
constexpr int kFallbackVariant = 5;  // for inputs a pipelined variant cannot copy
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
constexpr int kMinItems = 8;  // sizes the look-back words for every variant
static_assert(kThreads * kMinItems == (int)kSortPlanTile, "look-back sizing");
int g_variant = 5;

// Per-device set-up state: the pass kernels' shared-memory attribute is set
// once on each device that sorts, and the SM count is cached per device.
constexpr int kMaxDevices = 64;
bool g_init_done[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};
std::mutex g_init_mutex;

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
    return dev;
}

int num_sms() {
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(g_init_mutex);
    if (g_num_sms[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_num_sms[dev] = n > 0 ? n : 1;
    }
    return g_num_sms[dev];
}

// Position of the error word inside the scratch (the counters come first,
// so the word sits at the same offset for every length and key width).
constexpr size_t kErrWord = 9;

}  // namespace

// Kernel attributes (the pass kernels' shared memory exceeds the 48 KB
// default), set once per device. Safe to call repeatedly and from several
// threads; called before any stream capture.
cudaError_t sort_init() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_init_mutex);
    if (g_init_done[dev]) return cudaSuccess;
    for (int v = 0; v < kNumVariants; ++v) {
        e = cudaFuncSetAttribute(kVariants[v].kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kVariants[v].smem);
        if (e != cudaSuccess) return e;
    }
    // Tuning knob for benchmarks: ASTRO_SORT_VARIANT selects a pass variant.
    if (const char* env = getenv("ASTRO_SORT_VARIANT")) {
        const int v = atoi(env);
        if (v >= 0 && v < kNumVariants) g_variant = v;
    }
    e = cudaFuncSetAttribute(sort_histogram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kWarps * kMaxPasses * kRadix * sizeof(uint32_t)));
    if (e == cudaSuccess) g_init_done[dev] = true;
    return e;
}

uint32_t sort_variant_count() { return (uint32_t)kNumVariants; }

SortPlan sort_plan(uint32_t max_len, uint32_t key_bits) {
    SortPlan p{};
    p.passes = key_bits == 0 ? 1u : (key_bits + 7u) / 8u;
    p.tile = kSortPlanTile;
    p.ntiles = (uint32_t)(((uint64_t)max_len + p.tile - 1) / p.tile);
    size_t off = 0;
    // Zeroed at the start of every sort: counters ([0..7] tile tickets per
    // pass, [8] histogram blocks done, [9] error word), histograms and
    // look-back words.
    p.zero_begin = off;
    p.counters = off;
    off = align_up(off + 4ull * 16, 256);
    p.hist = off;
    off = align_up(off + 4ull * kMaxPasses * kRadix, 256);
    p.lookback = off;
    off = align_up(off + 4ull * p.passes * (size_t)std::max(p.ntiles, 1u) * kRadix, 256);
    p.zero_end = off;
    p.excl = off;
    off = align_up(off + 4ull * kMaxPasses * kRadix, 256);
    p.keys_tmp = off;
    off = align_up(off + 8ull * max_len, 256);
    p.vals_tmp = off;
    off = align_up(off + 4ull * max_len, 256);
    p.total = off;
    return p;
}

namespace {

// The sort's kernels on the scratch `temp` (laid out by sort_plan). With
// `stall_first_tile` (test hook, one pass only) the first pass hands out
// tickets from 1, so tile 0 is never processed and every later tile's
// look-back waits on a word that nobody publishes until `spin_limit` polls.
cudaError_t sort_launch(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                        uint32_t* vals_out, uint32_t n_est, const uint32_t* d_count,
                        uint32_t key_bits, void* temp, size_t temp_bytes, cudaStream_t st,
                        uint32_t* err, uint32_t variant, uint32_t spin_limit,
                        bool stall_first_tile) {
    if (n_est == 0) return cudaSuccess;
    const SortPlan plan = sort_plan(n_est, key_bits);
    if (temp_bytes < plan.total || key_bits > 64 || variant > (uint32_t)kNumVariants)
        return cudaErrorInvalidValue;
    if (stall_first_tile && plan.passes != 1) return cudaErrorInvalidValue;
    cudaError_t e0 = sort_init();
    if (e0 != cudaSuccess) return e0;
    int vi = variant == 0 ? g_variant : (int)variant - 1;
    // Bulk copies need 16-byte aligned sources; the temporaries always are.
    // The stalled test pass needs one block per tile (no persistent blocks).
    if (kVariants[vi].pipelined &&
        (stall_first_tile ||
         (((uintptr_t)keys_in | (uintptr_t)(vals_in ? vals_in : nullptr)) & 15u) != 0))
        vi = kFallbackVariant;
    const PassVariant& pv = kVariants[vi];
    const uint32_t tile = (uint32_t)(kThreads * pv.items);
    const uint32_t ntiles = (uint32_t)(((uint64_t)n_est + tile - 1) / tile);
    uint32_t grid = ntiles;
    if (pv.pipelined) {
        int per_sm = 0;
        cudaError_t eo = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pv.kernel, kThreads,
                                                                       pv.smem);
        if (eo != cudaSuccess) return eo;
        grid = std::min<uint32_t>(ntiles, (uint32_t)std::max(1, per_sm) * (uint32_t)num_sms());
    }
    char* base = static_cast<char*>(temp);
    uint64_t* keys_tmp = reinterpret_cast<uint64_t*>(base + plan.keys_tmp);
    uint32_t* vals_tmp = reinterpret_cast<uint32_t*>(base + plan.vals_tmp);
    uint32_t* excl = reinterpret_cast<uint32_t*>(base + plan.excl);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + plan.hist);
    uint32_t* counters = reinterpret_cast<uint32_t*>(base + plan.counters);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(base + plan.lookback);
    if (!err) err = counters + kErrWord;
    cudaError_t e = cudaMemsetAsync(base + plan.zero_begin, 0, plan.zero_end - plan.zero_begin, st);
    if (e != cudaSuccess) return e;
    if (stall_first_tile) {
        // Pass 0's ticket counter starts at 1 (its low byte set to 1).
        e = cudaMemsetAsync(counters, 1, 1, st);
        if (e != cudaSuccess) return e;
    }
    const uint32_t hist_blocks = (uint32_t)std::min<uint64_t>(
        ((uint64_t)n_est + 4 * kThreads - 1) / (4 * kThreads), (uint64_t)num_sms() * kHistBlocksPerSm);
    const size_t hist_smem = (size_t)kWarps * plan.passes * kRadix * sizeof(uint32_t);
    sort_histogram_kernel<<<hist_blocks, kThreads, hist_smem, st>>>(keys_in, d_count, n_est, key_bits,
                                                                    plan.passes, hist, excl, counters + 8);
    const uint64_t* kin = keys_in;
    const uint32_t* vin = vals_in;
    for (uint32_t p = 0; p < plan.passes; ++p) {
        const bool to_out = ((plan.passes - 1 - p) % 2) == 0;
        uint64_t* kout = to_out ? keys_out : keys_tmp;
        uint32_t* vout = to_out ? vals_out : vals_tmp;
        const uint32_t shift = 8u * p;
        const uint32_t bits = key_bits == 0 ? 0u : std::min(8u, key_bits - shift);
        pv.kernel<<<grid, kThreads, pv.smem, st>>>(
            kin, vin, kout, vout, d_count, n_est, excl + p * kRadix,
            lookback + (size_t)p * plan.ntiles * kRadix, counters + p, shift, bits, err, spin_limit);
        kin = kout;
        vin = vout;
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t sort_pairs(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                       uint32_t* vals_out, uint32_t n_est, const uint32_t* d_count,
                       uint32_t key_bits, void* temp, size_t temp_bytes, cudaStream_t st,
                       uint32_t* err, uint32_t variant) {
    return sort_launch(keys_in, vals_in, keys_out, vals_out, n_est, d_count, key_bits, temp,
                       temp_bytes, st, err, variant, kSpinLimit, false);
}

cudaError_t sort_pairs_stalled(const uint64_t* keys_in, uint64_t* keys_out, uint32_t* vals_out,
                               uint32_t n, uint32_t key_bits, void* temp, size_t temp_bytes,
                               uint32_t spin_limit, cudaStream_t st) {
    return sort_launch(keys_in, nullptr, keys_out, vals_out, n, nullptr, key_bits, temp, temp_bytes,
                       st, nullptr, 0, spin_limit, true);
}

int sort_status(const void* temp, cudaStream_t st) {
    if (!temp) return ASTRO_ERR_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    uint32_t* word = reinterpret_cast<uint32_t*>(static_cast<char*>(const_cast<void*>(temp)) +
                                                 sort_plan(0, 8).counters) + kErrWord;
    uint32_t v = 0;
    if (cudaMemcpy(&v, word, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    if (v == 0) return ASTRO_OK;
    if (cudaMemset(word, 0, sizeof(uint32_t)) != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    return (v & kErrLookbackTimeout) ? ASTRO_ERR_DEVICE_TIMEOUT : ASTRO_ERR_DEVICE_OVERFLOW;
}

}  // namespace astro

extern "C" int astro_radix_sort_temp_bytes(uint32_t max_length, uint32_t key_bits, size_t* bytes) {
    if (!bytes || key_bits > 64) return ASTRO_ERR_INVALID_ARGUMENT;
    *bytes = astro::sort_plan(max_length, key_bits).total;
    return ASTRO_OK;
}

// MetalKernelsRadixSort.sort (Astro/RadixSort.swift:98-105): input/inputIndices
// are read, output/outputIndices receive the sorted pairs, estimatedLength
// sizes the launch and actualCountBuffer (d_actual_count) holds the count.
// On the NULL stream the call waits for the sort and returns its device
// status; on any other stream astro_radix_sort_status reads it later.
extern "C" int astro_radix_sort(const uint64_t* d_input, const uint32_t* d_input_indices,
                                uint64_t* d_output, uint32_t* d_output_indices,
                                uint32_t estimated_length, const uint32_t* d_actual_count,
                                uint32_t key_bits, void* d_temp, size_t temp_bytes, void* stream) {
    if (estimated_length == 0) return ASTRO_OK;  // RadixSort.swift:106
    if (!d_input || !d_output || !d_output_indices || !d_temp || key_bits > 64)
        return ASTRO_ERR_INVALID_ARGUMENT;
    if ((const void*)d_input == (const void*)d_output ||
        (const void*)d_input_indices == (const void*)d_output_indices)
        return ASTRO_ERR_INVALID_ARGUMENT;
    if (temp_bytes < astro::sort_plan(estimated_length, key_bits).total) return ASTRO_ERR_CAPACITY;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = astro::sort_pairs(d_input, d_input_indices, d_output, d_output_indices,
                                      estimated_length, d_actual_count, key_bits, d_temp,
                                      temp_bytes, st, nullptr);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    return st == nullptr ? astro::sort_status(d_temp, st) : ASTRO_OK;
}

extern "C" int astro_radix_sort_status(const void* d_temp, void* stream) {
    return astro::sort_status(d_temp, static_cast<cudaStream_t>(stream));
}

extern "C" int astro_test_sort_lookback_timeout(const uint64_t* d_input, uint64_t* d_output,
                                                uint32_t* d_output_indices, uint32_t n,
                                                uint32_t key_bits, uint32_t spin_limit,
                                                void* d_temp, size_t temp_bytes, void* stream) {
    if (!d_input || !d_output || !d_output_indices || n == 0 || key_bits == 0 || key_bits > 8 ||
        spin_limit == 0 || spin_limit > astro::kSpinLimit)
        return ASTRO_ERR_INVALID_ARGUMENT;
    if ((const void*)d_input == (const void*)d_output) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!d_temp && astro::noalloc_scratch(&d_temp, &temp_bytes) != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    if (temp_bytes < astro::sort_plan(n, key_bits).total) return ASTRO_ERR_CAPACITY;
    cudaError_t e = astro::sort_pairs_stalled(d_input, d_output, d_output_indices, n, key_bits, d_temp,
                                              temp_bytes, spin_limit, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    return ASTRO_OK;
}
