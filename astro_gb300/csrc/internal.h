// Internal declarations shared by the translation units of libastro_cuda.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/astro_cuda.h"

namespace astro {

// Per-system quantiser, frame and opening thresholds, rebuilt every step by
// the setup kernel from the bounding box of the current positions.
struct SysInfo {
    float lo[3];       // lower corner of the box, in the system's FP32 frame
    float scale;       // 2^21 / extent
    float ext;         // box extent (largest axis)
    uint32_t root;     // node index of the system's root
    uint32_t begin;    // particle range (the same in upload and Morton order)
    uint32_t end;
    double origin[3];  // precision form: FP64 origin of the FP32 frame
    double _pad0;
    float crit2[ASTRO_MAX_LAYERS];  // (cell size / theta)^2 per layer
    uint32_t _pad1[2];
};

// Contiguous particle range inside one system, processed by one block of the
// per-particle kernels that need to know the system (bbox, encode).
struct Chunk {
    uint32_t sys, begin, end, _pad;
};
constexpr uint32_t kChunkParticles = 4096;

struct LayerTable {
    uint32_t n_layers;
    uint32_t offset[ASTRO_MAX_LAYERS];
    uint32_t size[ASTRO_MAX_LAYERS];
};

// ---------------------------------------------------------------- sort ----
struct SortPlan {
    size_t keys_tmp, vals_tmp, excl, zero_begin, hist, counters, lookback, zero_end, total;
    uint32_t passes, ntiles, tile;
};
// Pairs per tile assumed when sizing the look-back words (the smallest tile
// of any pass variant, 256 threads x 8 pairs).
constexpr uint32_t kSortPlanTile = 2048;
SortPlan sort_plan(uint32_t max_len, uint32_t key_bits);
cudaError_t sort_init();
// Stable sort of n_est (key, value) pairs (count read from d_count when not
// NULL). vals_in NULL => values are 0..n-1. err (device word) collects
// look-back timeouts; NULL => the error word inside temp (sort_status).
// variant: 0 = the library default, 1..sort_variant_count() = a pass kernel
// of the astro_params.sort_variant table.
cudaError_t sort_pairs(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                       uint32_t* vals_out, uint32_t n_est, const uint32_t* d_count,
                       uint32_t key_bits, void* temp, size_t temp_bytes, cudaStream_t st,
                       uint32_t* err, uint32_t variant = 0);
uint32_t sort_variant_count();
// Test hook: a one-pass sort (key_bits <= 8) whose tile 0 is never
// processed, so the look-back waits of the later tiles give up after
// spin_limit polls and set the error word of `temp`.
cudaError_t sort_pairs_stalled(const uint64_t* keys_in, uint64_t* keys_out, uint32_t* vals_out,
                               uint32_t n, uint32_t key_bits, void* temp, size_t temp_bytes,
                               uint32_t spin_limit, cudaStream_t st);
// Waits for st, then reads and clears the error word of a sort scratch:
// ASTRO_OK, ASTRO_ERR_DEVICE_TIMEOUT (a look-back wait gave up) or ASTRO_ERR_CUDA.
int sort_status(const void* temp, cudaStream_t st);
// The no-alloc sort's static scratch on the current device (sort_noalloc.cu).
cudaError_t noalloc_scratch(void** ptr, size_t* bytes);

// ------------------------------------------------------------ pipeline ----
struct DeviceState;  // defined in context.cu
struct GroupDesc;    // build_kernels.cuh

}  // namespace astro

// The opaque context of the C ABI.
struct astro_ctx {
    astro_params p{};
    uint32_t max_n = 0, max_sys = 0;
    int device = 0;
    cudaStream_t stream = nullptr;

    // Current upload.
    bool uploaded = false;
    uint32_t n = 0, n_tree = 0, nsys = 0;
    uint32_t lbits = 6, sysbits = 0, key_bits = 18;
    astro::LayerTable layers{};
    uint64_t capacity = 0;
    uint32_t nchunks = 0;
    bool tree_valid = false;
    bool state_in_b = false;          // PHYSICAL: current state in the B buffers
    std::vector<uint32_t> sys_sizes;

    // Particle state. PHYSICAL keeps it in Morton order (buffer A holds the
    // current state between steps; B is the permuted copy within a step).
    float4* pos[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    uint32_t* ids[2] = {nullptr, nullptr};
    double* x64[2] = {nullptr, nullptr};  // SoA x | y | z, precision form
    float4* acc = nullptr;
    float4* colors = nullptr;         // REFERENCE: ColorType colours (lighting pass)
    float4* lights = nullptr;         // REFERENCE: lighting pass light snapshot
    // Headless splat (allocated on first use).
    float4* splat_prim = nullptr;
    uint32_t* splat_kind = nullptr;
    float4* splat_image = nullptr;
    float* splat_depth = nullptr;
    uint64_t splat_pixels = 0;
    uint64_t* frag_keys = nullptr;
    uint64_t* frag_sorted = nullptr;
    uint32_t* frag_vals = nullptr;
    void* frag_temp = nullptr;
    size_t frag_temp_bytes = 0;
    uint32_t frag_cap = 0;
    uint32_t* types = nullptr;
    uint64_t* codes = nullptr;        // keys in the state order before sorting
    uint64_t* sorted_keys = nullptr;
    uint32_t* perm = nullptr;
    void* staging = nullptr;          // upload/download, 64 B per particle
    size_t staging_bytes = 0;
    // Asynchronous upload/download (created on first use): a copy stream
    // each way, two staging slots each way (64 B per particle each), and the
    // events that order copies, conversions and the step stream.
    cudaStream_t h2d_stream = nullptr;
    cudaStream_t d2h_stream = nullptr;
    void* stage_in[2] = {nullptr, nullptr};
    void* stage_out[2] = {nullptr, nullptr};
    cudaEvent_t ev_in_copied[2] = {nullptr, nullptr};   // host -> slot copy done
    cudaEvent_t ev_in_used[2] = {nullptr, nullptr};     // slot converted into the state
    cudaEvent_t ev_out_ready[2] = {nullptr, nullptr};   // state converted into the slot
    cudaEvent_t ev_out_copied[2] = {nullptr, nullptr};  // slot -> host copy done
    uint32_t in_slot = 0, out_slot = 0;
    uint32_t* dl_inv = nullptr;       // downloads: inverse of the ids (upload order -> slot)
    bool steps_unrerunnable = false;  // an async transfer touched the state of unchecked steps

    // Tree.
    uint64_t tree_capacity = 0;       // allocated node slots
    float4* node_cm = nullptr;        // centre of mass, mass
    uint4* node_rng = nullptr;        // first child, end child, first particle, end particle
    uint64_t* node_key = nullptr;
    void* node_sum = nullptr;         // float4 or double4 raw sums (S, M)
    uint32_t* node_pbeg = nullptr;
    uint32_t* node_cbeg = nullptr;
    uint32_t* node_parent = nullptr;
    uint32_t* node_arrive = nullptr;
    float* node_crit2 = nullptr;      // opening radius^2 per node
    float4* node_ecol = nullptr;      // REFERENCE: emittedColor per node
    float4* node_ecen = nullptr;      // REFERENCE: emittedColorCenter per node
    float4* node_q = nullptr;         // quadrupole Qxx, Qyy, Qxy, Qxz
    float* node_qyz = nullptr;        // quadrupole Qyz
    uint4* groups = nullptr;          // group-walk records (<= n)
    uint32_t* frontier = nullptr;     // group-walk per-warp frontier buffers
    size_t frontier_words = 0;
    uint32_t frontier_cap = 16384;   // words per frontier buffer (set by astro_create)
    astro::GroupDesc* group_desc = nullptr;  // group walk: per-group lists (<= max_n groups)
    uint32_t* lists = nullptr;        // group walk: list pool
    uint32_t* list_next = nullptr;    // group walk: block chain links
    size_t lists_blocks = 0;
    size_t lists_blocks_want = 0;     // group walk: pool size a walk asked for
    bool walk_estimate_off = false;   // group walk: size the pool by demand only (test hook)
    uint64_t walk_reruns = 0;         // steps / traversals run again after a walk overflow
    uint32_t pending_steps = 0;       // steps launched since the last device check
    float pending_dt = 0.f;           // their time step
    uint32_t* layer_count = nullptr;  // device [ASTRO_MAX_LAYERS]

    // Systems.
    astro::SysInfo* sys = nullptr;
    uint32_t* bbox32 = nullptr;               // 6 per system
    unsigned long long* bbox64 = nullptr;     // 6 per system
    astro::Chunk* chunks = nullptr;
    uint32_t chunk_capacity = 0;

    // Scratch.
    void* sort_temp = nullptr;
    size_t sort_temp_bytes = 0;
    uint32_t* topo_lookback = nullptr;
    size_t topo_lookback_words = 0;
    uint32_t* counters = nullptr;             // [0] topology tiles, [1] traversal queue, [2] groups
    uint32_t* err = nullptr;                  // device error word
    cudaEvent_t trav_ev[3] = {nullptr, nullptr, nullptr};  // traversal stage call: before,
                                              // between walk and evaluation, after
    bool trav_timed = false;                  // the last traversal stage call recorded them
    unsigned long long* stats = nullptr;      // interactions, node visits, cell
                                              // interactions, far nodes, far interactions
    void* readback = nullptr;
    size_t readback_bytes = 0;

    // Graph of one step.
    cudaGraphExec_t graph = nullptr;
    float graph_dt = 0.0f;
    bool graph_valid = false;

    std::string last_error;
};
