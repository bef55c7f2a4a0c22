/*
 * ORACLE — test infrastructure only. A CPU restatement of the osbo/astro
 * Barnes-Hut step, used by tests/ and by bench.py's CPU baseline to check
 * and time the CUDA path. Nothing in the product (astro_gb300/, include/)
 * links, loads or calls this code.
 *
 * Parity status: parity unpinned. The reference publishes no golden
 * vectors, fixtures or kernel tests (its tests are empty Xcode templates),
 * and it cannot run here (Swift + Metal on macOS), so nothing the reference
 * holds or produces checks this restatement. It is checked only against the
 * known-answer tests in tests/test_oracle_kat.py and the fixtures under
 * tests/golden/, derived by hand from the reference source
 * (tests/golden/make_golden.py), and the PHYSICAL preset against an FP64
 * direct sum.
 *
 * Two presets (ASTRO_PRESET_* in include/astro_cuda.h):
 *   REFERENCE — every Metal kernel of the step restated as a loop over gid,
 *               in the reference's dispatch order (Renderer.swift:495-755),
 *               with its 64 one-bit split passes, its Blelloch scan, its
 *               per-layer sorts and run detection, and its quirks.
 *   PHYSICAL  — the same pipeline with physical units (bounding-box
 *               quantiser, geometric cells, G and eps^2, leaf/bucket
 *               particle-particle sums, leapfrog), in plain FP32 or in the
 *               precision form, for one or many systems.
 * All FP32 arithmetic is round-to-nearest with no contraction (built with
 * -ffp-contract=off), which is the arithmetic the CUDA kernels reproduce.
 */
#ifndef ASTRO_ORACLE_H
#define ASTRO_ORACLE_H

#include <stdint.h>
#include "../include/astro_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Outputs of the last force evaluation of a run; every pointer may be NULL. */
typedef struct oracle_outputs {
    uint64_t* codes;          /* [n_tree] unsorted keys by particle */
    uint64_t* sorted_codes;   /* [n_tree] */
    uint32_t* sorted_indices; /* [n_tree] */
    uint32_t* layer_counts;   /* [lbits+1] live nodes per layer */
    uint32_t* layer_sizes;    /* [lbits+1] closed-form capacity */
    uint32_t* layer_offsets;  /* [lbits+1] */
    OctreeNode* nodes;        /* [node capacity] */
    float* acc4;              /* [n*4] force buffer (float3, 16-byte stride) */
    uint64_t interactions;    /* filled by PHYSICAL runs */
    uint64_t node_visits;
    uint64_t far_nodes;        /* group walk: expansions formed (group x far node) */
    uint64_t far_interactions; /* accepted nodes evaluated through them, per particle */
    const uint64_t* nodes_index; /* PHYSICAL: nodes holds only these nodes_count slots, */
    uint64_t nodes_count;        /* in this order (NULL: every slot) */
} oracle_outputs;

/* Number of OpenMP threads used by the oracle (<=0: all). Returns the count in effect. */
int oracle_set_threads(int n);

/* -- REFERENCE stage restatements (exported for the known-answer tests) -- */
uint64_t oracle_interleave_bits(uint32_t x, uint32_t y, uint32_t z);
void oracle_generate_morton_codes(const PositionMass* pos, uint64_t* codes, uint64_t* unsorted,
                                  uint32_t count, uint32_t lbits, float offset);
/* ScanKernel.encodeScanTo: exclusive scan of len values (limit lifted). */
void oracle_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t len);
/* MetalKernelsRadixSort.sort: stable sort of count (key, index) pairs with
 * npasses one-bit split passes starting at bit 0. */
void oracle_split_sort(const uint64_t* in_keys, const uint32_t* in_idx, uint64_t* out_keys,
                       uint32_t* out_idx, uint32_t count, uint32_t npasses);
/* Node capacity and closed-form layers (Renderer.swift:373-386) for count
 * tree bodies in nsys systems. Returns the total slot count. */
uint64_t oracle_layer_layout(uint32_t count, uint32_t nsys, uint32_t lbits,
                             uint32_t* sizes, uint32_t* offsets);

/* Run nsteps REFERENCE steps (Renderer.draw compute section) in place.
 * split_passes: 64 reproduces the reference; 3*lbits gives the same result faster. */
int oracle_ref_run(const astro_params* p, PositionMass* pm, VelocityRadius* vr,
                   const ColorType* ct, uint32_t n, uint32_t n_tree, float dt,
                   uint32_t nsteps, uint32_t split_passes, oracle_outputs* out);

/* Run nsteps PHYSICAL steps (one extra force evaluation first) in place over
 * nsys systems of sizes sys_sizes (NULL => one system of n). In the
 * precision form pos64 (3 doubles per particle, may be NULL) receives the
 * FP64 positions. */
int oracle_phys_run(const astro_params* p, PositionMass* pm, VelocityRadius* vr, uint32_t n,
                    const uint32_t* sys_sizes, uint32_t nsys, float dt, uint32_t nsteps,
                    uint32_t split_passes, double* pos64, oracle_outputs* out);

/* lightingPass (BarnesHut.metal:103-167) in place on ct: planets (type 1) and
 * dust (type 2) take the light of the first min(num_stars, 5) particles,
 * whose positions and colours are read before any colour is written. */
void oracle_lighting(const PositionMass* pm, ColorType* ct, uint32_t n, uint32_t num_stars);

/* Headless splat (astro_splat's definition) drawn sequentially: rgba
 * (width * height * 4) and depth (width * height) receive the image. */
void oracle_splat(const PositionMass* pm, const VelocityRadius* vr, const ColorType* ct, uint32_t n,
                  const float* view, const float* proj, const float* cam, uint32_t width,
                  uint32_t height, const float* clear, float* rgba, float* depth);

/* The group walk's far-node expansion: coefficients (a, J, H; 19 floats) of
 * a node of centre of mass and mass cm4 and quadrupole q5 {Qxx, Qyy, Qxy,
 * Qxz, Qyz} about gc3, and the expansion times G at offset rho3 (either
 * output may be NULL). G and eps from p. */
void oracle_far_expand(const astro_params* p, const float* cm4, const float* q5, const float* gc3,
                       const float* rho3, float* coefs19, float* acc3);

/* FP64 softened direct sum for sampled particles against their own system. */
void oracle_direct_accel_f64(const PositionMass* pm, const double* pos64, uint32_t n,
                             const uint32_t* sys_sizes, uint32_t nsys,
                             const uint32_t* sample_idx, uint32_t n_sample, double g,
                             double eps, double* acc3);

#ifdef __cplusplus
}
#endif

#endif
