/*
 * astro_cuda.h — C ABI of libastro_cuda, the sm_103a Barnes-Hut step.
 *
 * This header replaces three things in the osbo/astro reference:
 *   1. the shared layouts of Astro/bridge.h (PositionMass, VelocityRadius,
 *      ColorType, OctreeNode, INVALID_MORTON_CODE) — same byte layouts;
 *   2. the Metal kernel entry points of the per-frame compute section of
 *      Renderer.draw (Astro/Renderer.swift:495-542) — generateMortonCodes,
 *      the radix sort, the layered octree build, barnesHut and updateSpheres;
 *   3. the sort library MetalKernelsRadixSort.sort (Astro/RadixSort.swift:98-105).
 *
 * Conventions:
 *   - Every function returns int: ASTRO_OK (0) or a negative astro_status.
 *     Nothing aborts; the message of the last failure on a context is
 *     available from astro_last_error().
 *   - A context owns all of its device buffers and one CUDA stream. All work
 *     is ordered on that stream. Only astro_download, astro_read_* and
 *     astro_synchronize wait for the device.
 *   - A context is not thread-safe; separate contexts are independent.
 *   - Pointers named d_* are device pointers; all others are host pointers.
 */
#ifndef ASTRO_CUDA_H
#define ASTRO_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASTRO_ABI_VERSION 1

/* bridge.h:91-94 */
#define ASTRO_INVALID_MORTON_CODE 0xFFFFFFFFFFFFFFFFull
/* Octree.metal:10, BarnesHut.metal:7 */
#define ASTRO_INVALID_CHILD 0xFFFFFFFFu
/* 21 bits per axis fit a 63-bit key (MortonCode.metal:7-23). */
#define ASTRO_MAX_LBITS 21
#define ASTRO_MAX_LAYERS (ASTRO_MAX_LBITS + 1)
/* Largest number of independent systems in one batched context. */
#define ASTRO_MAX_SYSTEMS 65536

#if defined(__GNUC__) || defined(__clang__)
#define ASTRO_ALIGN16 __attribute__((aligned(16)))
#else
#define ASTRO_ALIGN16
#endif

/* ---------------------------------------------------------------------------
 * Shared layouts. Metal's float3 is 16 bytes with 16-byte alignment, so every
 * float3 below is three floats plus one pad float.
 * ------------------------------------------------------------------------- */

/* bridge.h:17-24 — 32-byte stride: position @0, mass @16. */
typedef struct ASTRO_ALIGN16 PositionMass {
    float position[3];
    float _pad0;
    float mass;
    float _pad1[3];
} PositionMass;

/* bridge.h:26-33 — 32-byte stride: velocity @0, radius @16. */
typedef struct ASTRO_ALIGN16 VelocityRadius {
    float velocity[3];
    float _pad0;
    float radius;
    float _pad1[3];
} VelocityRadius;

/* bridge.h:35-43 — 32-byte stride: color @0, type @16.
 * type 0 = star, 1 = planet, 2 = dust (Renderer.swift:448-472). */
typedef struct ASTRO_ALIGN16 ColorType {
    float color[4];
    uint32_t type;
    uint32_t _pad[3];
} ColorType;

/* bridge.h:47-65 — 128-byte node. emittedColor / emittedColorCenter: in the
 * REFERENCE preset the stars' (type 0) colours summed and their positions
 * averaged, leaf by leaf, then over children with emitted alpha > 0
 * (Octree.metal:75-106,147-187); zero in the PHYSICAL preset. */
typedef struct ASTRO_ALIGN16 OctreeNode {
    uint64_t mortonCode;        /* @0   */
    uint64_t _pad0;             /* @8   */
    float centerOfMass[3];      /* @16  */
    float _pad1;                /* @28  */
    float totalMass;            /* @32  */
    float _pad2[3];             /* @36  */
    float emittedColor[4];      /* @48  */
    float emittedColorCenter[3];/* @64  */
    float _pad3;                /* @76  */
    uint32_t children[8];       /* @80  */
    uint32_t layer;             /* @112 */
    uint32_t _pad4[3];          /* @116 */
} OctreeNode;

/* ---------------------------------------------------------------------------
 * Status codes.
 * ------------------------------------------------------------------------- */
typedef enum astro_status {
    ASTRO_OK = 0,
    ASTRO_ERR_INVALID_ARGUMENT = -1,
    ASTRO_ERR_CAPACITY = -2,      /* n or the number of systems exceeds the context */
    ASTRO_ERR_CUDA = -3,          /* a CUDA runtime call failed */
    ASTRO_ERR_OUT_OF_MEMORY = -4,
    ASTRO_ERR_STATE = -5,         /* call order violated (e.g. step before upload) */
    ASTRO_ERR_DEVICE_TIMEOUT = -6,/* a bounded device-side wait gave up */
    ASTRO_ERR_NOT_SUPPORTED = -7,
    ASTRO_ERR_DEVICE_OVERFLOW = -8/* a device-side bound (stack depth) was hit */
} astro_status;

/* ---------------------------------------------------------------------------
 * Parameters. Every constant the reference hard-codes is a field here.
 * ------------------------------------------------------------------------- */
typedef enum astro_preset {
    /* The reference's literal semantics: (u32)(p + 1e6) quantiser,
     * node size 2^(21+layer), monopole leaves with the self-leaf skip and the
     * r^2 > 50 cut, g = 1e11, softening added to r^2, damped kick-drift with
     * per-type multipliers, and the last-leaf range of aggregateLeafNodes. */
    ASTRO_PRESET_REFERENCE = 0,
    /* Physical units: bounding-box quantiser, geometric cell size, G and
     * Plummer softening eps^2, particle-particle interaction inside opened
     * leaves and buckets, and updateSpheres' kick-drift without damping
     * (leapfrog with velocities at half steps). Defaults add the quadrupole
     * term and the delta-corrected opening radius, and walk the tree once per
     * group of <= 32 particles (ASTRO_FLAG_PER_PARTICLE restores per-particle
     * decisions). */
    ASTRO_PRESET_PHYSICAL = 1
} astro_preset;

typedef enum astro_form {
    ASTRO_FORM_PLAIN = 0,     /* FP32 throughout */
    ASTRO_FORM_PRECISION = 1  /* FP64 positions and build reductions, FP32
                                 traversal with compensated sums relative to a
                                 per-system origin (PHYSICAL preset only) */
} astro_form;

/* Bit flags for astro_params.flags. */
#define ASTRO_FLAG_IEEE_EXACT 0x1u  /* traversal uses correctly rounded
                                       div/sqrt and no contraction (slower;
                                       reproduces the CPU restatement bit for bit) */
#define ASTRO_FLAG_NO_GRAPH   0x2u  /* astro_step launches kernels directly
                                       instead of replaying a CUDA graph */
#define ASTRO_FLAG_PERSISTENT 0x4u  /* per-particle traversal runs as a persistent
                                       kernel with a work-stealing chunk queue */
#define ASTRO_FLAG_OPEN_DELTA 0x8u  /* PHYSICAL: open a node unless the distance
                                       exceeds size/theta + |com - cell centre| */
#define ASTRO_FLAG_QUADRUPOLE 0x10u /* PHYSICAL: accepted nodes add their
                                       traceless quadrupole term */
#define ASTRO_FLAG_PER_PARTICLE 0x20u /* PHYSICAL: decide node by node for each
                                       particle (the reference's walk) instead of
                                       the group walk over <= 32-particle groups */

typedef struct astro_params {
    uint32_t preset;          /* astro_preset */
    uint32_t form;            /* astro_form */
    uint32_t lbits;           /* bits per axis kept in the key, 1..21; 6 in the
                                 reference (MortonCode.metal:47-50) => 7 layers */
    uint32_t flags;           /* ASTRO_FLAG_* */
    float theta;              /* opening angle (Renderer.swift:864: 0.7) */
    float g;                  /* gravitational constant (BarnesHut.metal:39: 1e11) */
    float softening;          /* REFERENCE: added to r^2 (BarnesHut.metal:40: 0.01);
                                 PHYSICAL: Plummer eps, eps^2 added to r^2 */
    float leaf_min_dist2;     /* REFERENCE: leaf counted only if r^2 > this
                                 (BarnesHut.metal:70: 50) */
    float force_clamp;        /* per-component clamp (BarnesHut.metal:100: 1e5) */
    float quant_offset;       /* REFERENCE quantiser offset (MortonCode.metal:35-37: 1e6) */
    float damping;            /* REFERENCE velocity damping (BarnesHut.metal:189: 0.9995) */
    float type_accel_scale[3];/* REFERENCE per-type multiplier (BarnesHut.metal:181-187: 5,5,1) */
    uint32_t bucket;          /* PHYSICAL: an opened node holding <= bucket
                                 particles is summed particle by particle
                                 (0 = only at layer 0) */
    uint32_t block_warps;     /* traversal: warps per block (0 = autotuned/default) */
    uint32_t group_size;      /* PHYSICAL group walk: at most this many consecutive
                                 particles share one tree walk (one warp; two
                                 particles per lane above 32), 1..64; 0 = 32 */
    uint32_t sort_variant;    /* radix sort pass kernel (items per thread / blocks
                                 per SM / ranking): 0 = library default,
                                 1 = 16/2/ballot, 2 = 16/2/match, 3 = 12/3/match,
                                 4 = 8/4/match, 5 = 20/2/match, 6 = 12/3/ballot,
                                 7 = 8/4/ballot; 8 = 12/2 and 9 = 8/3 ballot with
                                 persistent blocks that bulk-copy the next tile
                                 while ranking the current one (16-byte aligned
                                 inputs; others use 6); lean passes that keep no
                                 value in registers (values prefetched to L2 and
                                 gathered by a staged 16-bit index): 10 =
                                 12/4/ballot, 11 = 16/3/ballot, 12 = 20/3/match */
    uint32_t light_sources;   /* REFERENCE: astro_step runs the lighting pass
                                 with the first light_sources particles (at most
                                 5) as lights (Renderer.swift:539; numStars = 5);
                                 0 = no lighting pass */
    float open_delta_weight;  /* PHYSICAL with ASTRO_FLAG_OPEN_DELTA: a node opens
                                 unless the distance exceeds
                                 size/theta + w |com - cell centre| (default 1;
                                 0 = size/theta) */
    float far_ratio;          /* PHYSICAL group walk: an accepted node whose centre
                                 of mass lies further than r_g / far_ratio from
                                 the centre of the group's box (r_g: the box's
                                 half diagonal) is summed through one
                                 second-order expansion of its field about that
                                 centre, evaluated at each particle of the
                                 group, instead of term by term; 0 = every
                                 accepted node term by term; 0..0.5 */
    uint32_t walk_frontier;   /* PHYSICAL group walk, the frontier's form: 0 = runs
                                 of consecutive child nodes (one per opened
                                 node), 1 = a list of node indices; same walk,
                                 same results, different speed per workload */
} astro_params;

/* Fill *out with the defaults of a preset. */
int astro_params_default(uint32_t preset, astro_params* out);

/* ---------------------------------------------------------------------------
 * Context: the Renderer's buffers (Renderer.swift:336-391) and its per-frame
 * compute section (Renderer.swift:495-542).
 * ------------------------------------------------------------------------- */
typedef struct astro_ctx astro_ctx;

/* Allocate a context for up to max_n particles in up to max_systems systems.
 * Replaces Renderer.makeBuffers (Renderer.swift:336-391). */
int astro_create(const astro_params* params, uint32_t max_n, uint32_t max_systems,
                 astro_ctx** out);
int astro_destroy(astro_ctx* ctx);
int astro_set_params(astro_ctx* ctx, const astro_params* params);
int astro_get_params(const astro_ctx* ctx, astro_params* out);

/* Upload one system. The first n_tree particles are inserted in the tree
 * (Renderer.swift:36 octreeCount); all n feel the force. ct may be NULL:
 * particles below n_tree are then type 1, the rest type 2.
 * PHYSICAL requires n_tree == n. Replaces Renderer.makeSpheres' buffer copy
 * (Renderer.swift:490-492). */
int astro_upload(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                 const ColorType* ct, uint32_t n, uint32_t n_tree);

/* Upload nsys independent systems laid out back to back (PHYSICAL only).
 * Each system gets its own tree; keys carry the system id in their high bits. */
int astro_upload_systems(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                         const uint32_t* sys_sizes, uint32_t nsys);

/* Copy the particle state back (waits for the stream). */
int astro_download(astro_ctx* ctx, PositionMass* pm, VelocityRadius* vr, uint32_t n);

/* Pipelined transfers for a stream of independent inputs: neither call
 * waits. astro_upload_async replaces the state with n new particles in the
 * layout of the last astro_upload / astro_upload_systems (same n, same
 * systems, the same particle types and colours in the REFERENCE preset),
 * taking effect in stream order after the steps already queued;
 * its host-to-device copy runs on a copy stream of its own, so it overlaps
 * those steps. astro_download_async delivers the state as it is after the
 * steps queued before it; its device-to-host copy also runs on its own
 * stream and overlaps the steps queued after it. Two staging slots each way
 * let one transfer per direction be in flight while the next is queued.
 * The host buffers must stay valid, and the downloaded ones unread, until
 * astro_synchronize returns; pinned (page-locked) host memory is needed for
 * the copies to overlap. If a group walk outgrew its buffers during steps
 * whose state such a transfer replaced or read, those steps cannot be run
 * again: the next astro_synchronize grows the buffers and returns
 * ASTRO_ERR_DEVICE_OVERFLOW, and the batch should be run again. */
int astro_upload_async(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                       uint32_t n);
int astro_download_async(astro_ctx* ctx, PositionMass* pm, VelocityRadius* vr, uint32_t n);

/* Stage calls, in step order. Each is stream-ordered and does not wait. */
int astro_encode(astro_ctx* ctx);    /* generateMortonCodes + fillIndices (MortonCode.metal:26-52, Octree.metal:39-51) */
int astro_sort(astro_ctx* ctx);      /* radixSorter.sort at layer 0 (Renderer.swift:522-528) */
int astro_build(astro_ctx* ctx);     /* countUniqueMortonCodes + aggregateLeafNodes + buildInternalNodes (Renderer.swift:529-533,714-755) */
int astro_traverse(astro_ctx* ctx);  /* barnesHut (BarnesHut.metal:22-101) */
int astro_integrate(astro_ctx* ctx, float dt); /* updateSpheres (BarnesHut.metal:169-196) */

/* nsteps full steps: encode, sort, build, traverse, integrate (v += a dt,
 * x += v dt). PHYSICAL fuses the integration into the traversal and keeps
 * the particle state in Morton order between steps. The step is captured in
 * a CUDA graph once per upload/params/dt and replayed (ASTRO_FLAG_NO_GRAPH
 * launches it directly). */
int astro_step(astro_ctx* ctx, float dt, uint32_t nsteps);
/* astro_step for a batch of independent systems: sys_sizes must equal the
 * systems given to astro_upload_systems (ASTRO_ERR_INVALID_ARGUMENT
 * otherwise); all systems advance together in one step graph. */
int astro_step_batched(astro_ctx* ctx, const uint32_t* sys_sizes, uint32_t nsys, float dt,
                       uint32_t nsteps);
int astro_synchronize(astro_ctx* ctx);

/* Readbacks (wait for the stream). */
int astro_read_keys(astro_ctx* ctx, uint64_t* codes, uint64_t* sorted_codes,
                    uint32_t* sorted_indices, uint32_t n);
/* layer_sizes/offsets: closed-form capacity (Renderer.swift:373-386);
 * layer_counts: live nodes per layer (the reference's parentCount per layer). */
int astro_read_tree_info(astro_ctx* ctx, uint32_t* n_layers, uint32_t* layer_sizes,
                         uint32_t* layer_offsets, uint32_t* layer_counts,
                         uint32_t max_layers);
/* AoS nodes [first, first+count) in the reference layout; slots past a
 * layer's live count read as the cleared node of clearOctreeNodeBuffer
 * (Octree.metal:253-269). */
int astro_read_nodes(astro_ctx* ctx, OctreeNode* nodes, uint64_t first, uint64_t count);
/* Accelerations (the reference's forceBuffer, float3 with 16-byte stride). */
int astro_read_accel(astro_ctx* ctx, float* acc4, uint32_t n);
/* Traversal statistics of the last traversal, summed over particles: all
 * interactions (cell + particle-particle), nodes tested, and the cell
 * (accepted node) interactions among them. */
int astro_read_stats(astro_ctx* ctx, uint64_t* interactions, uint64_t* node_visits,
                     uint64_t* cell_interactions);

/* Far-node statistics of the last group walk (params.far_ratio > 0): the
 * expansions formed (one per walk and far node; the chunks of a leaf larger
 * than a group share one walk) and, summed over
 * particles, the accepted nodes evaluated through them (a part of
 * cell_interactions above). */
int astro_read_far_stats(astro_ctx* ctx, uint64_t* far_nodes, uint64_t* far_interactions);

/* Device times of the last group-walk traversal made by a stage call
 * (astro_traverse; graph-replayed steps are not timed): the walk that
 * builds the interaction lists, and the evaluation that sums them
 * (including the per-walk far-node sums for groups of more than 32)
 * (CUDA events on the context's stream; waits for them). */
int astro_read_traverse_times(astro_ctx* ctx, float* walk_ms, float* eval_ms);

/* Group-walk buffers (PHYSICAL, group walk). The walk writes each group's
 * interaction lists into a pool of 64-word blocks and walks the tree level
 * by level through two frontier buffers per walk warp. A walk that needs
 * more room than they have (small theta, large buckets) writes nothing past
 * them and counts what it needs; its evaluation is skipped, leaving forces
 * and particles as they were, and at the next check of the device
 * (astro_synchronize, a readback) the buffers grow to the counted need and
 * the skipped steps run again, so the results equal those of buffers large
 * enough from the start. Every call that reads or replaces the state
 * (readbacks, uploads, stage calls, parameter changes, saving) first waits
 * for the steps launched since the last check, so none sees a state whose
 * steps may still run again; astro_step and astro_step_batched themselves
 * do not wait. Stage calls (astro_traverse) rerun their own traversal
 * before returning. Reports the pool size in blocks, the frontier buffer size in
 * words and the steps and traversals run again since astro_create (any
 * pointer may be NULL). Waits for the context's stream. */
int astro_read_walk_buffers(astro_ctx* ctx, uint64_t* list_blocks, uint32_t* frontier_cap,
                            uint64_t* reruns);

/* FP64 direct-sum accelerations (G, eps as the context's PHYSICAL params) of
 * the sampled particles against all particles of their own system, computed
 * on the device from the current positions. acc3 holds 3 doubles per sample. */
int astro_direct_accel_f64(astro_ctx* ctx, const uint32_t* sample_idx, uint32_t n_sample,
                           double* acc3);

/* Lighting pass (BarnesHut.metal:103-167), REFERENCE preset: every planet
 * (type 1) and dust particle (type 2) takes the light of the first
 * min(num_stars, 5) particles,
 *   rgb = sum_s rgb_s / max(|x_s - x| / 4e5, 1e-9)^2   (bridge.h:98),
 *   alpha = 1 for planets, min(max(r, g, b), 0.25) for dust;
 * stars keep their colour. The lights' positions and colours are taken before
 * the pass writes any colour. Colours are the ColorType values of the upload
 * (zero when none were given). */
int astro_lighting(astro_ctx* ctx, uint32_t num_stars);
/* ColorType of every particle (colour after the last lighting pass, type) in
 * upload order. */
int astro_read_colors(astro_ctx* ctx, ColorType* ct, uint32_t n);

/* ---------------------------------------------------------------------------
 * Headless splat: the scene pass of the reference's renderer
 * (Spheres.metal:23-64, Renderer.swift:780-830) into an image, REFERENCE
 * preset. Each particle is projected as clip = P * (V * (x - camera, 1)).
 * Stars and planets (types 0, 1) are drawn as opaque discs of their sphere's
 * projected radius (the unit-extent sphere mesh scaled by the radius) at the
 * centre's depth; dust (type 2) as blended point sprites of `radius` pixels.
 * Draw order is particle order, the depth test is "less" with depth writes,
 * and every colour write is rounded to half precision (rgba16Float).
 * ------------------------------------------------------------------------- */
typedef struct astro_camera {
    float view[16];           /* column-major (simd_float4x4 columns): viewMatrix */
    float projection[16];     /* column-major: projectionMatrix */
    float position[3];        /* cameraPosition */
    float _pad;
} astro_camera;

/* rgba: width * height * 4 floats, row 0 at the top; depth: width * height
 * floats or NULL (host buffers). clear: RGBA clear colour, NULL for the
 * reference's background (0, 0, 1/255, 1); depth clears to 1. */
int astro_splat(astro_ctx* ctx, const astro_camera* camera, uint32_t width, uint32_t height,
                const float* clear, float* rgba, float* depth);

/* ---------------------------------------------------------------------------
 * State files: the role of makeSpheres / resetSimulation
 * (Renderer.swift:148-152,441-493) for a headless step loop, which the
 * reference rebuilds from an unseeded generator on every reset.
 *
 * A state file (little-endian) is an astro_state_header followed by
 *   uint32_t       sys_sizes[nsys]
 *   PositionMass   pm[n]      particles in the context's current slot order
 *   VelocityRadius vr[n]
 *   uint32_t       ids[n]     upload index of each slot
 *   uint32_t       types[n]   if contents & ASTRO_STATE_TYPES (REFERENCE preset)
 *   double         pos64[3n]  if contents & ASTRO_STATE_POS64 (precision form;
 *                             x, y, z per particle)
 * Loading restores the slot order, so a loaded context's next steps are
 * bit-identical to the saved context's. Colours are not state (only the type
 * is): a loaded REFERENCE context has type-only ColorType values.
 * ------------------------------------------------------------------------- */
#define ASTRO_STATE_MAGIC "ASTROST1"
#define ASTRO_STATE_VERSION 1u
#define ASTRO_STATE_TYPES 0x1u
#define ASTRO_STATE_POS64 0x2u

typedef struct astro_state_header {
    char magic[8];            /* ASTRO_STATE_MAGIC, not NUL-terminated */
    uint32_t version;         /* ASTRO_STATE_VERSION */
    uint32_t header_bytes;    /* sizeof(astro_state_header) */
    astro_params params;
    uint64_t step;            /* caller's step counter */
    double time;              /* caller's simulated time */
    uint32_t n;
    uint32_t n_tree;
    uint32_t nsys;
    uint32_t contents;        /* ASTRO_STATE_* */
} astro_state_header;

/* Write the context's state (between steps) with the caller's step count and
 * time. */
int astro_save_state(astro_ctx* ctx, const char* path, uint64_t step, double time);
/* Create a context for at least max_n particles (0: exactly the file's) from
 * a state file and restore its state; *step and *time (may be NULL) receive
 * the saved counters. */
int astro_load_state(const char* path, uint32_t max_n, astro_ctx** out, uint64_t* step,
                     double* time);

/* Device pointer access for callers that own their own kernels. */
int astro_get_stream(astro_ctx* ctx, void** stream);

/* Autotune the knobs of a PHYSICAL context on its current particles: the
 * launch knobs (lbits, bucket, group_size, block_warps, sort_variant), kept
 * within a median relative acceleration error of max(target, 1.02 x the
 * starting error) against the FP64 direct sum on sampled particles, and
 * the accuracy knobs (open_delta_weight, far_ratio) within max(0.8 x
 * target, 1.02 x the starting error). Steps are timed with dt = 0, so the
 * particles are unchanged. The best setting is applied to the context and,
 * when path is not NULL, written there as JSON (knobs, step time, error,
 * every trial); on failure the context keeps its parameters and particles.
 * astro_autotune: target 1e-3, 1,024 samples. */
int astro_autotune(astro_ctx* ctx, const char* path);
int astro_autotune_ex(astro_ctx* ctx, const char* path, float target, uint32_t samples);
/* astro_autotune_ex holding the knobs of `keep` (ASTRO_TUNE_KEEP_* bits) at
 * the context's values, e.g. the tree depth a workload is quoted at. */
#define ASTRO_TUNE_KEEP_LBITS 0x1u
#define ASTRO_TUNE_KEEP_GROUP_SIZE 0x2u
#define ASTRO_TUNE_KEEP_ACCURACY 0x4u  /* open_delta_weight and far_ratio */
int astro_autotune_keep(astro_ctx* ctx, const char* path, float target, uint32_t samples,
                        uint32_t keep);

const char* astro_last_error(const astro_ctx* ctx);
const char* astro_version(void);
const char* astro_status_string(int status);

/* ---------------------------------------------------------------------------
 * Stand-alone sort: MetalKernelsRadixSort.sort (Astro/RadixSort.swift:98-185).
 * Stable ascending sort of (uint64 key, uint32 index) pairs. The element
 * count is read on the device from d_actual_count (NULL => estimated_length);
 * the launch is sized by estimated_length. d_input_indices NULL => 0..n-1.
 * Inputs are not modified. Only the low key_bits bits of each key take part
 * (key_bits = 64 reproduces the reference's 64 one-bit passes exactly;
 * fewer bits give the same permutation when the high bits are zero).
 * Temporary device memory is supplied by the caller.
 *
 * Device status: the sort's look-back waits are bounded; a wait that gives
 * up (ASTRO_ERR_DEVICE_TIMEOUT) leaves a wrong permutation, written inside
 * the output. On the NULL stream astro_radix_sort waits for the sort and
 * returns that status. On any other stream it returns once the sort is
 * queued; astro_radix_sort_status then waits for the stream and returns the
 * status of the last sort that used d_temp (and clears it).
 * ------------------------------------------------------------------------- */
int astro_radix_sort_temp_bytes(uint32_t max_length, uint32_t key_bits, size_t* bytes);
int astro_radix_sort(const uint64_t* d_input, const uint32_t* d_input_indices,
                     uint64_t* d_output, uint32_t* d_output_indices,
                     uint32_t estimated_length, const uint32_t* d_actual_count,
                     uint32_t key_bits, void* d_temp, size_t temp_bytes,
                     void* stream);
/* No counterpart in the reference (its sort reports nothing): ASTRO_OK or
 * ASTRO_ERR_DEVICE_TIMEOUT for the last sort made with d_temp, after
 * waiting for stream. */
int astro_radix_sort_status(const void* d_temp, void* stream);

/* ---------------------------------------------------------------------------
 * The same sort for callers that cannot allocate device memory (no
 * counterpart in the reference). Hosts whose device memory belongs to another
 * allocator, frame loops with a fixed preallocated budget, and embedders that
 * forbid allocation after start-up cannot supply or create a temporary
 * buffer; this entry point uses a static device array of the library instead
 * and allocates nothing. It sorts at most ASTRO_RADIX_SORT_NOALLOC_MAX_LENGTH
 * pairs (larger estimated_length returns ASTRO_ERR_CAPACITY); every GPU that
 * loads the library holds the array (about 16 MiB) until exit. All calls on a
 * device share the array: calls that overlap on the GPU race, so serialise
 * them. The first call on a device resolves the array's address there; make
 * it before any stream capture begins. Device status as astro_radix_sort:
 * returned by the call itself on the NULL stream, otherwise by
 * astro_radix_sort_noalloc_status (the last no-alloc sort on the current
 * device, after waiting for stream).
 * ------------------------------------------------------------------------- */
#define ASTRO_RADIX_SORT_NOALLOC_MAX_LENGTH 1048576u
int astro_radix_sort_noalloc(const uint64_t* d_input, const uint32_t* d_input_indices,
                             uint64_t* d_output, uint32_t* d_output_indices,
                             uint32_t estimated_length, const uint32_t* d_actual_count,
                             uint32_t key_bits, void* stream);
int astro_radix_sort_noalloc_status(void* stream);

/* ---------------------------------------------------------------------------
 * Seeded initial conditions (host side, FP64 then cast). Counter-based
 * Philox4x32-10 streams keyed by (seed, system, particle), so any host
 * produces identical sets. Replaces Renderer.makeSpheres (Renderer.swift:441-493).
 * ------------------------------------------------------------------------- */
typedef enum astro_ic_kind {
    ASTRO_IC_PLUMMER = 0,      /* scale a = p0, mass M = p1, equilibrium velocities */
    ASTRO_IC_DISK_BULGE = 1,   /* exponential disk R_d = 1, z_d = 0.1 (80%) + Hernquist bulge (20%), M = 1 */
    ASTRO_IC_TWO_PLUMMER = 2,  /* two Plummer spheres a = 1, M = 0.5 each, separation p0 on a parabolic approach */
    ASTRO_IC_UNIFORM_CUBE = 3, /* unit cube, Gaussian velocities sigma = p0, log-normal masses sigma = p1, total 1 */
    ASTRO_IC_REFERENCE_SCENE = 4 /* the reference's scene: p0 stars, p1 planets, rest dust (Renderer.swift:25-46,441-493) */
} astro_ic_kind;

int astro_generate_ic(uint32_t kind, uint64_t seed, uint32_t system, uint32_t n,
                      double p0, double p1, PositionMass* pm, VelocityRadius* vr,
                      ColorType* ct /* may be NULL */);
/* nsys sizes drawn log-uniformly in [n_min, n_max] and, when scales is not
 * NULL, one scale radius per system uniform in [a_min, a_max]. */
int astro_generate_system_sizes(uint64_t seed, uint32_t nsys, uint32_t n_min, uint32_t n_max,
                                double a_min, double a_max, uint32_t* sizes, double* scales);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* ASTRO_CUDA_H */
