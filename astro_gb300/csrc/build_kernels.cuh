// Argument blocks and launchers of the pipeline kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace astro {

struct TopoArgs {
    const uint64_t* keys;
    uint32_t n;
    uint32_t lbits;
    uint32_t ntiles;
    uint32_t offset[ASTRO_MAX_LAYERS];
    uint32_t* pbeg;
    uint32_t* cbeg;
    uint32_t* parent;    // per node: the node one layer up holding it (kNoParent at the top)
    uint64_t* node_key;  // per node: its first particle's key >> 3 * layer
    uint32_t* layer_count;
    uint32_t* lookback;  // [ntiles][32] status words
    uint32_t* tile_counter;
    uint32_t* err;
};

struct AggArgs {
    const uint32_t* perm;      // REFERENCE: sorted slot -> upload index
    const float4* pos;         // REFERENCE: upload order; PHYSICAL: sorted order (the
                               // precision form's FP32 frame relative to the origin)
    const SysInfo* sys;
    const uint32_t* pbeg;
    const uint32_t* node_cbeg;
    const uint32_t* parent;    // per node: its parent (kNoParent at the top layer)
    uint32_t* arrive;          // per internal node: children aggregated so far (zeroed per build)
    const uint32_t* layer_count;
    uint32_t offset[ASTRO_MAX_LAYERS];  // first node of each layer
    float4* node_cm;
    uint4* node_rng;
    uint64_t* node_key;
    void* node_sum;
    // PHYSICAL extras: quadrupole moments, per-node opening radius, groups.
    float* node_crit2;
    float4* node_q;        // Qxx, Qyy, Qxy, Qxz
    float* node_qyz;       // Qyz
    // Groups of the group walk, one record each: (first particle, end
    // particle, walk end, chunk index). A leaf holding more particles than
    // a group is cut into consecutive chunks that share one walk against the
    // whole leaf's box: chunk k's walk starts at its first chunk (record
    // index - k), whose walk range is [first, walk end) = the leaf. Every
    // other group walks its own range (walk end = end, chunk index 0).
    uint4* groups;
    uint32_t* group_count;
    // REFERENCE: star colours (ColorType colour of type-0 particles) summed
    // into each node's emittedColor and averaged into emittedColorCenter
    // (Octree.metal:75-106,147-187); NULL node_ecol = not computed.
    const float4* colors;  // upload order
    const uint32_t* types; // upload order
    float4* node_ecol;     // emittedColor
    float4* node_ecen;     // emittedColorCenter (w unused)
    uint32_t n;
    uint32_t lbits;
    uint32_t want_quad;
    uint32_t want_delta;
    float theta;
    float delta_weight;    // w of the opening radius size/theta + w delta
    uint32_t group_size;   // particles per group walk, 1..kGroupSize
    uint32_t* err;         // device error word (kErrBadLayer: a node with > 8 children)
};

constexpr uint32_t kGroupSize = 64;     // largest group of the group walk (two particles per lane)
constexpr uint32_t kDefaultGroupSize = 32;  // group_size 0
constexpr uint32_t kNoParent = 0xFFFFFFFFu;

struct DirectArgs {
    const float4* pos;
    const double* x64;
    const uint32_t* slot;       // state slot of each sample
    const uint32_t* sys_begin;  // its system's slot range
    const uint32_t* sys_end;
    double* out;
    uint32_t n;
    uint32_t n_sample;
    double g;
    double eps2;
};

// The lists of one group of the group walk, written by the walk kernel and
// read by the evaluation kernel. Each list is a chain of blocks of
// kListBlockWords words of the list pool (block b at lists[b * kListBlockWords],
// the next block of the chain in list_next[b]): accepted node ids (cells,
// far nodes) one word each, leaf particle ranges two words each. Also the
// centre of the group's bounding box (the far nodes' expansion point).
constexpr uint32_t kListBlockWords = 64;
struct GroupDesc {
    uint32_t leaf_first, n_leaf;
    uint32_t cell_first, n_cell;
    uint32_t far_first, n_far;
    float gcx, gcy, gcz;
    uint32_t pad[3];
    float far_co[20];  // the far nodes' summed expansion coefficients (19 used)
};

struct TraverseArgs {
    const float4* node_cm;
    const uint4* node_rng;
    const uint64_t* node_key;
    const SysInfo* sys;
    const float4* pos;          // positions the forces are evaluated at
    const uint64_t* sorted_keys;
    float4* acc;
    // PHYSICAL epilogue: kick-drift from the B buffers into the A buffers.
    const float4* vel_in;
    float4* vel_out;
    float4* pos_out;
    const uint32_t* id_in;
    uint32_t* id_out;
    const double* x64_in;
    double* x64_out;
    // REFERENCE: own key for the self-leaf test, particle types.
    const uint64_t* codes;
    const uint32_t* types;
    uint32_t n_tree;
    uint32_t n;
    uint32_t lbits;
    uint32_t root;
    uint32_t bucket;
    float g;
    float eps2;          // PHYSICAL eps^2; REFERENCE softening added to r^2
    float clampv;
    float dt;
    float theta;
    float leaf_min_dist2;
    uint32_t* err;
    unsigned long long* stats;
    uint32_t* queue;
    // PHYSICAL opening radius / quadrupole / group walk.
    uint32_t delta;
    uint32_t quad;
    const float* node_crit2;
    const float4* node_q;
    const float* node_qyz;
    const uint4* groups;      // group walk: (first, end, walk end, chunk index), see AggArgs
    const uint32_t* group_count;
    uint32_t* frontier;       // group walk: per-warp frontier ping-pong buffers,
                              // 2 * frontier_cap words each
    uint32_t frontier_cap;
    GroupDesc* desc;          // group walk: per group, its lists in the pool and centre
    uint32_t* lists;          // group walk: list pool, lists_blocks blocks
    uint32_t* list_next;      // group walk: next block of each block's chain
    uint32_t lists_blocks;    // pool size in blocks
    uint32_t* lists_used;     // pool bump counter (blocks handed out, past the end
                              // when the pool is too small: the demand)
    uint32_t* eval_queue;     // queue of the group evaluation kernel
    uint32_t* frontier_need;  // group walk: largest frontier (words) a walk wanted
                              // past frontier_cap (atomicMax)
    uint32_t* evals_done;     // group walk: evaluations that ran (one per launch)
    uint32_t nsys;
    float far2;               // group walk: far_ratio^2 (0: no far nodes)
    uint32_t group_chunk;     // group walk: groups visited in scrambled chunks of this
                              // many (0: in queue order)
    uint32_t walk_runs;       // group walk: frontier of runs (1) or of node indices (0)
};

cudaError_t launch_encode_ref(const float4* pos, uint64_t* codes, uint32_t n_tree, uint32_t lbits,
                              float offset, cudaStream_t st);
cudaError_t launch_encode_phys(bool prec, const Chunk* chunks, uint32_t nchunks, const SysInfo* sys,
                               float4* pos, const double* x64, uint64_t* codes, uint32_t n,
                               uint32_t lbits, cudaStream_t st);
cudaError_t launch_bbox(bool prec, const Chunk* chunks, uint32_t nchunks, const float4* pos,
                        const double* x64, uint32_t n, uint32_t* bb32, unsigned long long* bb64,
                        cudaStream_t st);
cudaError_t launch_setup(bool prec, SysInfo* sys, uint32_t nsys, uint32_t* bb32,
                         unsigned long long* bb64, uint32_t lbits, float theta, uint32_t root_offset,
                         cudaStream_t st);
cudaError_t launch_reorder(bool prec, const uint32_t* perm, const float4* pos_a, const float4* vel_a,
                           const uint32_t* id_a, const double* x_a, float4* pos_b, float4* vel_b,
                           uint32_t* id_b, double* x_b, uint32_t n, cudaStream_t st);
uint32_t topology_tiles(uint32_t n);
cudaError_t launch_topology(const TopoArgs& a, cudaStream_t st);
// First layer the bottom-up aggregation climbs from (below it: one launch per layer).
uint32_t climb_first_layer(const LayerTable& t);
cudaError_t launch_aggregate(int mode, const AggArgs& a, const LayerTable& t, cudaStream_t st);
cudaError_t launch_integrate_ref(float4* pos, float4* vel, const float4* acc, const uint32_t* types,
                                 uint32_t n, float dt, const astro_params& p, cudaStream_t st);
cudaError_t launch_upload_convert(bool prec, const PositionMass* pm, const VelocityRadius* vr,
                                  const ColorType* ct, float4* pos, float4* vel, uint32_t* ids,
                                  uint32_t* types, double* x64, uint32_t n, uint32_t n_tree,
                                  cudaStream_t st);
// With inv_scratch (n words) the state is gathered into upload order
// through the inverse of ids; without, scattered through ids.
cudaError_t launch_download_convert(bool prec, const float4* pos, const float4* vel,
                                    const uint32_t* ids, const double* x64, PositionMass* pm,
                                    VelocityRadius* vr, uint32_t n, cudaStream_t st,
                                    uint32_t* inv_scratch = nullptr);
cudaError_t launch_scatter_u64(const uint64_t* src, const uint32_t* ids, uint64_t* dst, uint32_t n,
                               cudaStream_t st);
cudaError_t launch_scatter_f4(const float4* src, const uint32_t* ids, float4* dst, uint32_t n,
                              cudaStream_t st);
// ecol/ecen: emitted colours and their centres (NULL: zero, as in the
// PHYSICAL preset).
cudaError_t launch_readback_nodes(const float4* cm, const uint4* rng, const uint64_t* key,
                                  const float4* ecol, const float4* ecen,
                                  const uint32_t* layer_count, uint32_t l, uint32_t layer_offset,
                                  uint32_t first_in_layer, uint32_t count, OctreeNode* out,
                                  cudaStream_t st);
cudaError_t launch_direct_sum(const DirectArgs& a, cudaStream_t st);
cudaError_t launch_inverse_ids(const uint32_t* ids, uint32_t* inv, uint32_t n, cudaStream_t st);
cudaError_t launch_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t* dst, uint32_t n,
                              cudaStream_t st);
cudaError_t launch_types_from_colors(const ColorType* ct, uint32_t* types, float4* colors, uint32_t n,
                                     cudaStream_t st);
// Lighting pass; lights: 10 float4 of scratch (positions, colours).
cudaError_t launch_lighting(const float4* pos, const uint32_t* types, float4* colors, float4* lights,
                            uint32_t n, uint32_t num_stars, cudaStream_t st);
cudaError_t launch_colors_out(const float4* colors, const uint32_t* types, ColorType* out, uint32_t n,
                              cudaStream_t st);
cudaError_t launch_kick_drift(bool prec, float4* pos, float4* vel, double* x64, const float4* acc,
                              uint32_t n, float dt, cudaStream_t st);

// Headless splat (splat.cu).
struct SplatArgs {
    const float4* pos;       // REFERENCE state, upload order
    const float4* vel;       // w = radius
    const float4* colors;
    const uint32_t* types;
    uint32_t n;
    float view[16];          // column-major
    float proj[16];          // column-major
    float cam[3];
    uint32_t width, height;
    float clear[4];
    float clear_depth;
    float4* prim;            // per particle: window x, y, depth, size / radius (pixels)
    uint32_t* kind;          // 0 culled, 1 disc, 2 point
    uint64_t* keys;          // fragments (pixel << 32 | particle)
    uint32_t cap;
    uint32_t* cursor;
    float4* image;           // width * height, row 0 = top
    float* depth;
};
cudaError_t launch_splat_project(const SplatArgs& a, cudaStream_t st);
cudaError_t launch_splat_emit(const SplatArgs& a, cudaStream_t st);
cudaError_t launch_splat_clear(const SplatArgs& a, cudaStream_t st);
cudaError_t launch_splat_fold(const SplatArgs& a, const uint64_t* keys, uint32_t count,
                              cudaStream_t st);

// Traversal (traverse.cu).
struct TraverseConfig {
    bool exact;       // correctly rounded arithmetic (reproduces the CPU restatement)
    bool precision;   // compensated sums, FP64 drift
    bool batched;     // several systems: per-lane system and root
    bool persistent;  // persistent blocks with a work-stealing chunk queue
    int warps;        // warps per block (2, 4 or 8)
    bool quad;        // quadrupole terms (group walk template switch)
    bool far_pre;     // group walk: far-node sums once per walk in group_far_kernel
                      // (groups of more than 32), else in each group's evaluation
};
cudaError_t launch_traverse_ref(const TraverseArgs& a, cudaStream_t st);
cudaError_t launch_traverse_phys(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st);
// Group walk: warps of the persistent walk launch (each owns two frontier
// buffers of frontier_cap words), the list pool size in blocks for n
// particles in groups of at most group_size, and the two launches (walk,
// then evaluation).
uint32_t group_walk_warps();
size_t group_list_blocks(uint32_t n, uint32_t group_size);
// ev (optional, three events): recorded before the walk, between the walk
// and the evaluation, and after it.
cudaError_t launch_traverse_groups(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st,
                                   cudaEvent_t* ev = nullptr);

}  // namespace astro
