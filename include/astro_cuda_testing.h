/*
 * astro_cuda_testing.h — test hooks of libastro_cuda (no counterpart in the
 * osbo/astro reference). They exercise failure paths that the normal entry
 * points only reach when the device misbehaves, without faulting, trapping
 * or hanging the GPU: every wait they provoke is bounded.
 */
#ifndef ASTRO_CUDA_TESTING_H
#define ASTRO_CUDA_TESTING_H

#include "astro_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Queue a one-pass pair sort (key_bits in 1..8, keys read from d_input,
 * indices generated) on d_temp in which tile 0 is never processed: the
 * decoupled look-back of every later tile waits on a status word that
 * nobody publishes and gives up after spin_limit polls (1 .. 2^22), so
 * astro_radix_sort_status(d_temp, stream) afterwards returns
 * ASTRO_ERR_DEVICE_TIMEOUT. The outputs receive a wrong permutation, every
 * store inside [0, n). d_temp must hold astro_radix_sort_temp_bytes(n,
 * key_bits) bytes; d_temp NULL runs it on the static array of
 * astro_radix_sort_noalloc (n at most its maximum), whose status
 * astro_radix_sort_noalloc_status then returns. */
int astro_test_sort_lookback_timeout(const uint64_t* d_input, uint64_t* d_output,
                                     uint32_t* d_output_indices, uint32_t n, uint32_t key_bits,
                                     uint32_t spin_limit, void* d_temp, size_t temp_bytes,
                                     void* stream);

/* Group-walk buffer sizes of a PHYSICAL context: set_blocks > 0 replaces
 * the list pool with one of set_blocks 64-word blocks, set_frontier_cap > 0
 * (even, at least 2) gives each walk warp's two frontier buffers that many
 * words,
 * and the size estimate taken from max_n and the group size is no longer
 * applied, so that the next walks run out of room and the recovery (the
 * evaluation skipped, buffers grown from the walk's demand, the steps run
 * again) is exercised. astro_read_walk_buffers reports the sizes. Waits for
 * the context's stream. */
int astro_test_walk_capacity(astro_ctx* ctx, uint64_t set_blocks, uint32_t set_frontier_cap);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* ASTRO_CUDA_TESTING_H */
