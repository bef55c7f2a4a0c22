// libastro_cuda context and C ABI (include/astro_cuda.h).
//
// The context plays the role of the reference Renderer's compute state
// (Astro/Renderer.swift:56-70,336-391) and its per-frame compute section
// (Renderer.draw, Renderer.swift:495-542), on one CUDA stream:
//
// REFERENCE step: encode (codes by particle) -> sort -> topology ->
//   aggregate (perm gathers) -> traverse (per particle) -> integrate.
// PHYSICAL step: bbox -> setup -> encode -> sort -> reorder the state into
//   Morton order -> topology -> aggregate -> traverse with the kick-drift
//   fused into its epilogue. The state stays in Morton order between steps
//   (buffer A); ids map it back to upload order for downloads and readbacks.
//   astro_step replays the step as a CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "build_kernels.cuh"
#include "common.cuh"
#include "internal.h"
#include "../../include/astro_cuda_testing.h"

using astro::Chunk;
using astro::LayerTable;
using astro::SysInfo;

namespace {

constexpr const char* kVersion = "astro_gb300 1.0 (sm_103a)";
// Traversal counters: interactions, node visits, cell interactions, far
// nodes, far interactions.
constexpr int kNumStats = 5;

int fail(astro_ctx* ctx, int code, const char* what) {
    if (ctx) ctx->last_error = what;
    return code;
}

int cuda_fail(astro_ctx* ctx, cudaError_t e, const char* where) {
    if (ctx) {
        ctx->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    }
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? ASTRO_ERR_OUT_OF_MEMORY : ASTRO_ERR_CUDA;
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

template <typename T>
cudaError_t dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

template <typename T>
void dev_free(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

bool is_phys(const astro_ctx* ctx) { return ctx->p.preset == ASTRO_PRESET_PHYSICAL; }
bool is_prec(const astro_ctx* ctx) { return is_phys(ctx) && ctx->p.form == ASTRO_FORM_PRECISION; }

uint32_t bits_for(uint32_t nsys) {
    uint32_t b = 0;
    while ((1ull << b) < nsys) ++b;
    return b;
}

int validate_params(const astro_params* p, const char** why) {
    if (!p) return (*why = "params is NULL", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->preset > ASTRO_PRESET_PHYSICAL) return (*why = "unknown preset", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->form > ASTRO_FORM_PRECISION) return (*why = "unknown form", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->form == ASTRO_FORM_PRECISION && p->preset != ASTRO_PRESET_PHYSICAL)
        return (*why = "the precision form needs the PHYSICAL preset", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->lbits < 1 || p->lbits > ASTRO_MAX_LBITS)
        return (*why = "lbits must be in [1, 21]", ASTRO_ERR_INVALID_ARGUMENT);
    if (!(p->theta > 0.0f) || !std::isfinite(p->theta))
        return (*why = "theta must be positive", ASTRO_ERR_INVALID_ARGUMENT);
    if (!std::isfinite(p->g) || !std::isfinite(p->softening) || p->softening < 0.0f)
        return (*why = "g and softening must be finite, softening >= 0", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->block_warps != 0 && p->block_warps != 2 && p->block_warps != 4 && p->block_warps != 8)
        return (*why = "block_warps must be 0, 2, 4 or 8", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->group_size > astro::kGroupSize)
        return (*why = "group_size must be in [0, 64]", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->sort_variant > astro::sort_variant_count())
        return (*why = "unknown sort_variant", ASTRO_ERR_INVALID_ARGUMENT);
    if (!(p->open_delta_weight >= 0.0f) || !std::isfinite(p->open_delta_weight))
        return (*why = "open_delta_weight must be finite and >= 0", ASTRO_ERR_INVALID_ARGUMENT);
    if (!(p->far_ratio >= 0.0f && p->far_ratio <= 0.5f))
        return (*why = "far_ratio must be in [0, 0.5]", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->walk_frontier > 1)
        return (*why = "walk_frontier must be 0 (runs) or 1 (node list)", ASTRO_ERR_INVALID_ARGUMENT);
    if (p->light_sources > 0 && p->preset != ASTRO_PRESET_REFERENCE)
        return (*why = "the lighting pass needs the REFERENCE preset", ASTRO_ERR_INVALID_ARGUMENT);
    return ASTRO_OK;
}

// Closed-form layer capacity (Renderer.swift:373-386) summed over systems.
void layer_table(const std::vector<uint32_t>& sizes, uint32_t lbits, LayerTable* t,
                 uint64_t* capacity) {
    std::memset(t, 0, sizeof(*t));
    t->n_layers = lbits + 1;
    uint64_t off = 0;
    for (uint32_t l = 0; l <= lbits; ++l) {
        const uint32_t bits = 3u * (lbits - l);
        const uint64_t possible = bits >= 40 ? (1ull << 40) : (1ull << bits);
        uint64_t size = 0;
        for (uint32_t s : sizes) size += std::min<uint64_t>(s, possible);
        t->size[l] = (uint32_t)size;
        t->offset[l] = (uint32_t)off;
        off += size;
    }
    *capacity = off;
}

int ensure_tree(astro_ctx* ctx, uint64_t capacity) {
    if (capacity <= ctx->tree_capacity) return ASTRO_OK;
    if (capacity >= (1ull << 32)) return fail(ctx, ASTRO_ERR_CAPACITY, "node capacity exceeds 2^32");
    dev_free(ctx->node_cm);
    dev_free(ctx->node_rng);
    dev_free(ctx->node_key);
    if (ctx->node_sum) cudaFree(ctx->node_sum);
    ctx->node_sum = nullptr;
    dev_free(ctx->node_pbeg);
    dev_free(ctx->node_cbeg);
    dev_free(ctx->node_parent);
    dev_free(ctx->node_arrive);
    dev_free(ctx->node_crit2);
    dev_free(ctx->node_ecol);
    dev_free(ctx->node_ecen);
    dev_free(ctx->node_q);
    dev_free(ctx->node_qyz);
    ctx->tree_capacity = 0;
    const uint64_t cap = capacity;
    CK(dev_alloc(&ctx->node_crit2, cap));
    if (!is_phys(ctx)) {
        CK(dev_alloc(&ctx->node_ecol, cap));
        CK(dev_alloc(&ctx->node_ecen, cap));
    }
    CK(dev_alloc(&ctx->node_q, cap));
    CK(dev_alloc(&ctx->node_qyz, cap));
    CK(dev_alloc(&ctx->node_cm, cap));
    CK(dev_alloc(&ctx->node_rng, cap));
    CK(dev_alloc(&ctx->node_key, cap));
    CK(cudaMalloc(&ctx->node_sum, cap * 32));  // room for double4 sums
    CK(dev_alloc(&ctx->node_pbeg, cap + 1));
    CK(dev_alloc(&ctx->node_cbeg, cap + 1));
    CK(dev_alloc(&ctx->node_parent, cap));
    CK(dev_alloc(&ctx->node_arrive, cap));
    ctx->tree_capacity = cap;
    return ASTRO_OK;
}

int ensure_x64(astro_ctx* ctx) {
    if (ctx->x64[0]) return ASTRO_OK;
    CK(dev_alloc(&ctx->x64[0], 3ull * ctx->max_n));
    CK(dev_alloc(&ctx->x64[1], 3ull * ctx->max_n));
    return ASTRO_OK;
}

int ensure_frontier(astro_ctx* ctx);
void drop_graph(astro_ctx* ctx);
int launch_steps(astro_ctx* ctx, float dt, uint32_t nsteps);

// After a group walk ran out of frontier or list room (the evaluation then
// skipped, leaving the state as it was): sizes the buffers from what the
// walk asked for (pool blocks handed out, largest frontier wanted; both
// under-counted when the frontier was cut short, hence at least doubled)
// and clears the error word and the counters. The stream is idle.
int grow_walk_buffers(astro_ctx* ctx, uint32_t* evals_done) {
    uint32_t c[3] = {0, 0, 0};  // pool blocks handed out, frontier wanted, evaluations run
    CK(cudaMemcpy(c, ctx->counters + 4, sizeof(c), cudaMemcpyDeviceToHost));
    *evals_done = c[2];
    const size_t slack = (size_t)astro::group_walk_warps() * 16;
    if (c[0] >= ctx->lists_blocks)
        ctx->lists_blocks_want = std::max<size_t>(2 * ctx->lists_blocks, (size_t)c[0] + c[0] / 4 + slack);
    // Frontier sizes stay multiples of 4 words: the run form stores 8-byte
    // runs in both buffers of a warp, the second starting frontier_cap words in.
    const uint64_t fmax = std::max<uint64_t>(64, 2ull * ctx->max_n);
    if (c[1] > ctx->frontier_cap || c[0] < ctx->lists_blocks) {
        const uint64_t want = std::min<uint64_t>(
            fmax, std::max<uint64_t>(2ull * ctx->frontier_cap, (uint64_t)c[1] + c[1] / 4));
        ctx->frontier_cap = (uint32_t)((want + 3) & ~3ull);
    }
    ctx->lists_blocks_want = std::min<size_t>(ctx->lists_blocks_want, 0xFFFFFF00ull);
    drop_graph(ctx);  // the captured step holds the old buffers and sizes
    CK(cudaMemset(ctx->counters + 4, 0, sizeof(c)));
    CK(cudaMemset(ctx->err, 0, sizeof(uint32_t)));
    return ensure_frontier(ctx);
}

// Read and clear the device error word (waits for the stream). Steps whose
// group walk ran out of room were not evaluated; they run again with
// larger buffers, so the state continues exactly as without the overflow.
int check_device(astro_ctx* ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h2d_stream) CK(cudaStreamSynchronize(ctx->h2d_stream));
    if (ctx->d2h_stream) CK(cudaStreamSynchronize(ctx->d2h_stream));
    uint32_t err = 0;
    CK(cudaMemcpy(&err, ctx->err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err == astro::kErrFrontier && ctx->pending_steps > 0 && ctx->steps_unrerunnable) {
        // Asynchronous transfers replaced or delivered the state of steps
        // that were skipped: they cannot be run again here.
        uint32_t done = 0;
        int r = grow_walk_buffers(ctx, &done);
        ctx->pending_steps = 0;
        ctx->steps_unrerunnable = false;
        if (r != ASTRO_OK) return r;
        return fail(ctx, ASTRO_ERR_DEVICE_OVERFLOW,
                    "a group walk outgrew its buffers during steps whose state asynchronous "
                    "transfers replaced or read; the buffers have grown: run those steps again");
    }
    ctx->steps_unrerunnable = false;
    for (int attempt = 0; err == astro::kErrFrontier && ctx->pending_steps > 0 && attempt < 16;
         ++attempt) {
        uint32_t done = 0;
        int r = grow_walk_buffers(ctx, &done);
        if (r != ASTRO_OK) return r;
        const uint32_t left = ctx->pending_steps - std::min(done, ctx->pending_steps);
        ctx->pending_steps = 0;
        ctx->walk_reruns += left;
        drop_graph(ctx);
        if ((r = launch_steps(ctx, ctx->pending_dt, left)) != ASTRO_OK) return r;
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(&err, ctx->err, sizeof(err), cudaMemcpyDeviceToHost));
    }
    if (ctx->pending_steps > 0) {
        ctx->pending_steps = 0;
        CK(cudaMemset(ctx->counters + 6, 0, sizeof(uint32_t)));
    }
    if (err) {
        CK(cudaMemset(ctx->err, 0, sizeof(uint32_t)));
        if (err & astro::kErrLookbackTimeout)
            return fail(ctx, ASTRO_ERR_DEVICE_TIMEOUT, "a decoupled look-back wait gave up");
        if (err & astro::kErrFrontier)
            return fail(ctx, ASTRO_ERR_DEVICE_OVERFLOW,
                        "a group walk buffer (frontier or list pool) overflowed");
        return fail(ctx, ASTRO_ERR_DEVICE_OVERFLOW, "a traversal stack bound was hit");
    }
    return ASTRO_OK;
}

// Buffers holding the current PHYSICAL state: A between steps, B after
// astro_sort until the traversal writes A back.
struct Cur {
    float4* pos;
    float4* vel;
    uint32_t* ids;
    double* x64;
};
Cur current(astro_ctx* ctx) {
    const int b = ctx->state_in_b ? 1 : 0;
    return Cur{ctx->pos[b], ctx->vel[b], is_phys(ctx) ? ctx->ids[b] : nullptr, ctx->x64[b]};
}

astro::TraverseConfig traverse_config(const astro_ctx* ctx) {
    astro::TraverseConfig c;
    c.exact = (ctx->p.flags & ASTRO_FLAG_IEEE_EXACT) != 0;
    c.precision = is_prec(ctx);
    c.batched = ctx->nsys > 1;
    c.persistent = (ctx->p.flags & ASTRO_FLAG_PERSISTENT) != 0;
    c.warps = ctx->p.block_warps ? (int)ctx->p.block_warps : 4;
    c.quad = (ctx->p.flags & ASTRO_FLAG_QUADRUPOLE) != 0;
    // Far-node sums once per walk for groups of more than 32 (measured
    // faster there: the evaluation of two particles per lane holds fewer
    // values, and the chunks of a leaf share the sums); in each group's
    // evaluation otherwise.
    c.far_pre = ctx->p.far_ratio > 0.f && ctx->p.group_size > 32;
    return c;
}

bool group_walk(const astro_ctx* ctx) {
    return is_phys(ctx) && (ctx->p.flags & ASTRO_FLAG_PER_PARTICLE) == 0;
}

// Buffers of the group walk: two frontier buffers of frontier_cap words per
// warp of the persistent walk launch; the list pool (blocks and their chain
// links, sized for max_n); one descriptor per group (at most max_n groups).
int ensure_frontier(astro_ctx* ctx) {
    if (!group_walk(ctx)) return ASTRO_OK;
    const size_t words = (size_t)astro::group_walk_warps() * 2 * ctx->frontier_cap;
    if (words > ctx->frontier_words) {
        drop_graph(ctx);  // a captured step holds the old buffers
        dev_free(ctx->frontier);
        ctx->frontier_words = 0;
        CK(dev_alloc(&ctx->frontier, words));
        ctx->frontier_words = words;
    }
    const size_t estimate =
        ctx->walk_estimate_off
            ? 0
            : astro::group_list_blocks(ctx->max_n, ctx->p.group_size ? ctx->p.group_size
                                                                     : astro::kDefaultGroupSize);
    const size_t blocks = std::max(estimate, ctx->lists_blocks_want);
    if (blocks > ctx->lists_blocks) {
        drop_graph(ctx);
        dev_free(ctx->lists);
        dev_free(ctx->list_next);
        ctx->lists_blocks = 0;
        CK(dev_alloc(&ctx->lists, blocks * astro::kListBlockWords));
        CK(dev_alloc(&ctx->list_next, blocks));
        ctx->lists_blocks = blocks;
    }
    if (!ctx->group_desc) CK(dev_alloc(&ctx->group_desc, ctx->max_n));
    return ASTRO_OK;
}

// --------------------------------------------------------------- stages --

int stage_encode(astro_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    if (!is_phys(ctx)) {
        CK(astro::launch_encode_ref(ctx->pos[0], ctx->codes, ctx->n_tree, ctx->lbits,
                                    ctx->p.quant_offset, st));
        return ASTRO_OK;
    }
    if (ctx->state_in_b) return fail(ctx, ASTRO_ERR_STATE, "encode called between sort and traverse");
    const bool prec = is_prec(ctx);
    CK(astro::launch_bbox(prec, ctx->chunks, ctx->nchunks, ctx->pos[0], ctx->x64[0], ctx->n,
                          ctx->bbox32, ctx->bbox64, st));
    CK(astro::launch_setup(prec, ctx->sys, ctx->nsys, ctx->bbox32, ctx->bbox64, ctx->lbits,
                           ctx->p.theta, ctx->layers.offset[ctx->lbits], st));
    CK(astro::launch_encode_phys(prec, ctx->chunks, ctx->nchunks, ctx->sys, ctx->pos[0],
                                 ctx->x64[0], ctx->codes, ctx->n, ctx->lbits, st));
    return ASTRO_OK;
}

int stage_sort(astro_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    const uint32_t count = is_phys(ctx) ? ctx->n : ctx->n_tree;
    CK(astro::sort_pairs(ctx->codes, nullptr, ctx->sorted_keys, ctx->perm, count, nullptr,
                         ctx->key_bits, ctx->sort_temp, ctx->sort_temp_bytes, st, ctx->err,
                         ctx->p.sort_variant));
    if (is_phys(ctx)) {
        if (ctx->state_in_b) return fail(ctx, ASTRO_ERR_STATE, "sort called twice without traverse");
        CK(astro::launch_reorder(is_prec(ctx), ctx->perm, ctx->pos[0], ctx->vel[0], ctx->ids[0],
                                 ctx->x64[0], ctx->pos[1], ctx->vel[1], ctx->ids[1], ctx->x64[1],
                                 ctx->n, st));
        ctx->state_in_b = true;
    }
    return ASTRO_OK;
}

int stage_build(astro_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    const uint32_t count = is_phys(ctx) ? ctx->n : ctx->n_tree;
    if (count == 0) return ASTRO_OK;
    if (is_phys(ctx) && !ctx->state_in_b) return fail(ctx, ASTRO_ERR_STATE, "build called before sort");
    astro::TopoArgs t{};
    t.keys = ctx->sorted_keys;
    t.n = count;
    t.lbits = ctx->lbits;
    t.ntiles = astro::topology_tiles(count);
    for (uint32_t l = 0; l <= ctx->lbits; ++l) t.offset[l] = ctx->layers.offset[l];
    t.pbeg = ctx->node_pbeg;
    t.cbeg = ctx->node_cbeg;
    t.parent = ctx->node_parent;
    t.node_key = ctx->node_key;
    t.layer_count = ctx->layer_count;
    t.lookback = ctx->topo_lookback;
    t.tile_counter = ctx->counters;
    t.err = ctx->err;
    CK(cudaMemsetAsync(ctx->topo_lookback, 0, (size_t)t.ntiles * 32 * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(ctx->counters, 0, sizeof(uint32_t), st));
    CK(astro::launch_topology(t, st));
    astro::AggArgs a{};
    a.perm = ctx->perm;
    a.pos = is_phys(ctx) ? ctx->pos[1] : ctx->pos[0];
    a.sys = ctx->sys;
    a.pbeg = ctx->node_pbeg;
    a.node_cbeg = ctx->node_cbeg;
    a.parent = ctx->node_parent;
    a.arrive = ctx->node_arrive;
    a.layer_count = ctx->layer_count;
    for (uint32_t l = 0; l <= ctx->lbits; ++l) a.offset[l] = ctx->layers.offset[l];
    a.node_cm = ctx->node_cm;
    a.node_rng = ctx->node_rng;
    a.node_key = ctx->node_key;
    a.node_sum = ctx->node_sum;
    a.node_crit2 = ctx->node_crit2;
    a.node_q = ctx->node_q;
    a.node_qyz = ctx->node_qyz;
    a.groups = ctx->groups;
    a.group_count = ctx->counters + 2;
    if (!is_phys(ctx)) {
        a.colors = ctx->colors;
        a.types = ctx->types;
        a.node_ecol = ctx->node_ecol;
        a.node_ecen = ctx->node_ecen;
    }
    a.n = count;
    a.lbits = ctx->lbits;
    a.want_quad = (ctx->p.flags & ASTRO_FLAG_QUADRUPOLE) ? 1u : 0u;
    a.want_delta = (ctx->p.flags & ASTRO_FLAG_OPEN_DELTA) ? 1u : 0u;
    a.theta = ctx->p.theta;
    a.delta_weight = ctx->p.open_delta_weight;
    a.group_size = ctx->p.group_size ? ctx->p.group_size : astro::kDefaultGroupSize;
    a.err = ctx->err;
    CK(cudaMemsetAsync(ctx->counters + 2, 0, sizeof(uint32_t), st));
    const uint32_t l0 = astro::climb_first_layer(ctx->layers);
    if (l0 < ctx->lbits) {
        // Arrival counters of the layers the aggregation climbs into.
        const uint64_t first = ctx->layers.offset[l0 + 1];
        const uint64_t end = (uint64_t)ctx->layers.offset[ctx->lbits] + ctx->layers.size[ctx->lbits];
        CK(cudaMemsetAsync(ctx->node_arrive + first, 0, (end - first) * sizeof(uint32_t), st));
    }
    const int mode = !is_phys(ctx) ? 0 : (is_prec(ctx) ? 2 : 1);
    CK(astro::launch_aggregate(mode, a, ctx->layers, st));
    ctx->tree_valid = true;
    return ASTRO_OK;
}

astro::TraverseArgs traverse_args(astro_ctx* ctx, float dt, bool integrate) {
    astro::TraverseArgs a{};
    a.node_cm = ctx->node_cm;
    a.node_rng = ctx->node_rng;
    a.node_key = ctx->node_key;
    a.sys = ctx->sys;
    a.sorted_keys = ctx->sorted_keys;
    a.acc = ctx->acc;
    a.n_tree = ctx->n_tree;
    a.n = ctx->n;
    a.lbits = ctx->lbits;
    a.root = ctx->layers.offset[ctx->lbits];
    a.bucket = ctx->p.bucket;
    a.g = ctx->p.g;
    a.clampv = ctx->p.force_clamp;
    a.dt = integrate ? dt : 0.0f;
    a.theta = ctx->p.theta;
    a.leaf_min_dist2 = ctx->p.leaf_min_dist2;
    a.err = ctx->err;
    a.stats = ctx->stats;
    a.queue = ctx->counters + 1;
    a.delta = (ctx->p.flags & ASTRO_FLAG_OPEN_DELTA) ? 1u : 0u;
    a.far2 = ctx->p.far_ratio * ctx->p.far_ratio;
    // Groups are queued system by system; for a batch, visiting them in
    // scrambled chunks of 256 measured 4% faster (a single system: 0-2%
    // slower, so it keeps the Morton order).
    a.group_chunk = ctx->nsys > 1 ? 256u : 0u;
    a.walk_runs = ctx->p.walk_frontier == 0 ? 1u : 0u;
    a.quad = (ctx->p.flags & ASTRO_FLAG_QUADRUPOLE) ? 1u : 0u;
    a.node_crit2 = ctx->node_crit2;
    a.node_q = ctx->node_q;
    a.node_qyz = ctx->node_qyz;
    a.groups = ctx->groups;
    a.group_count = ctx->counters + 2;
    a.frontier = ctx->frontier;
    a.frontier_cap = ctx->frontier_cap;
    a.desc = ctx->group_desc;
    a.lists = ctx->lists;
    a.list_next = ctx->list_next;
    a.lists_blocks = (uint32_t)ctx->lists_blocks;
    a.eval_queue = ctx->counters + 3;
    a.lists_used = ctx->counters + 4;
    a.frontier_need = ctx->counters + 5;
    a.evals_done = ctx->counters + 6;
    a.nsys = ctx->nsys;
    if (is_phys(ctx)) {
        a.eps2 = ctx->p.softening * ctx->p.softening;
        a.pos = ctx->pos[1];
        a.vel_in = ctx->vel[1];
        a.vel_out = ctx->vel[0];
        a.pos_out = ctx->pos[0];
        a.id_in = ctx->ids[1];
        a.id_out = ctx->ids[0];
        a.x64_in = ctx->x64[1];
        a.x64_out = ctx->x64[0];
    } else {
        a.eps2 = ctx->p.softening;
        a.pos = ctx->pos[0];
        a.codes = ctx->codes;
        a.types = ctx->types;
    }
    return a;
}

// PHYSICAL: dt > 0 fuses the kick-drift into the traversal; dt == 0 only
// evaluates forces (the state is copied back to A unchanged).
int stage_traverse(astro_ctx* ctx, float dt, bool integrate) {
    cudaStream_t st = ctx->stream;
    CK(cudaMemsetAsync(ctx->stats, 0, kNumStats * sizeof(unsigned long long), st));
    if (!is_phys(ctx)) {
        if (ctx->n_tree == 0) {
            CK(cudaMemsetAsync(ctx->acc, 0, sizeof(float4) * ctx->n, st));
            return ASTRO_OK;
        }
        if (!ctx->tree_valid) return fail(ctx, ASTRO_ERR_STATE, "traverse called before build");
        CK(astro::launch_traverse_ref(traverse_args(ctx, 0.0f, false), st));
        return ASTRO_OK;
    }
    if (!ctx->state_in_b || !ctx->tree_valid)
        return fail(ctx, ASTRO_ERR_STATE, "traverse called before sort and build");
    if (group_walk(ctx)) {
        int r = ensure_frontier(ctx);
        if (r != ASTRO_OK) return r;
        // Stage calls (outside stream capture) time the walk and the
        // evaluation (with the far-node sums when they run apart).
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(st, &cap));
        const bool timed = cap == cudaStreamCaptureStatusNone;
        CK(astro::launch_traverse_groups(traverse_args(ctx, dt, integrate), traverse_config(ctx), st,
                                         timed ? ctx->trav_ev : nullptr));
        ctx->trav_timed = timed;
    } else {
        CK(astro::launch_traverse_phys(traverse_args(ctx, dt, integrate), traverse_config(ctx), st));
    }
    ctx->state_in_b = false;
    return ASTRO_OK;
}

int stage_integrate(astro_ctx* ctx, float dt) {
    if (!is_phys(ctx)) {
        CK(astro::launch_integrate_ref(ctx->pos[0], ctx->vel[0], ctx->acc, ctx->types, ctx->n, dt,
                                       ctx->p, ctx->stream));
        return ASTRO_OK;
    }
    if (ctx->state_in_b) return fail(ctx, ASTRO_ERR_STATE, "integrate called before traverse");
    CK(astro::launch_kick_drift(is_prec(ctx), ctx->pos[0], ctx->vel[0], ctx->x64[0], ctx->acc,
                                ctx->n, dt, ctx->stream));
    return ASTRO_OK;
}

int run_step(astro_ctx* ctx, float dt) {
    int r;
    if ((r = stage_encode(ctx)) != ASTRO_OK) return r;
    if ((r = stage_sort(ctx)) != ASTRO_OK) return r;
    if ((r = stage_build(ctx)) != ASTRO_OK) return r;
    if (is_phys(ctx)) return stage_traverse(ctx, dt, true);
    if ((r = stage_traverse(ctx, 0.0f, false)) != ASTRO_OK) return r;
    // barnesHut, lightingPass, updateSpheres (Renderer.swift:538-540).
    if (ctx->p.light_sources > 0)
        CK(astro::launch_lighting(ctx->pos[0], ctx->types, ctx->colors, ctx->lights, ctx->n,
                                  ctx->p.light_sources, ctx->stream));
    return stage_integrate(ctx, dt);
}

void drop_graph(astro_ctx* ctx) {
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
    ctx->graph_valid = false;
}

int capture_step(astro_ctx* ctx, float dt) {
    drop_graph(ctx);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int r = run_step(ctx, dt);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (r != ASTRO_OK) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
    ctx->graph_valid = true;
    ctx->graph_dt = dt;
    return ASTRO_OK;
}

// Launches nsteps whole steps (graph replays unless ASTRO_FLAG_NO_GRAPH);
// group-walk steps are counted until the next device check.
int launch_steps(astro_ctx* ctx, float dt, uint32_t nsteps) {
    if (nsteps == 0) return ASTRO_OK;
    if (group_walk(ctx)) {
        ctx->pending_steps += nsteps;
        ctx->pending_dt = dt;
    }
    int r;
    if ((ctx->p.flags & ASTRO_FLAG_NO_GRAPH) != 0) {
        for (uint32_t s = 0; s < nsteps; ++s)
            if ((r = run_step(ctx, dt)) != ASTRO_OK) return r;
        return ASTRO_OK;
    }
    // Walk buffers are sized outside the capture (no allocation inside it);
    // the step is captured once per (upload, params, dt) and replayed.
    if ((r = ensure_frontier(ctx)) != ASTRO_OK) return r;
    if (!(ctx->graph_valid && ctx->graph_dt == dt))
        if ((r = capture_step(ctx, dt)) != ASTRO_OK) return r;
    for (uint32_t s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(ctx->graph, ctx->stream));
    ctx->tree_valid = true;
    return ASTRO_OK;
}

// A stage-call traversal whose walk ran out of room runs again at once with
// larger buffers (the sorted state and the tree are still in place). Other
// device errors stay in the error word for the next check.
int settle_traverse(astro_ctx* ctx) {
    for (int attempt = 0; attempt < 16; ++attempt) {
        CK(cudaStreamSynchronize(ctx->stream));
        uint32_t err = 0;
        CK(cudaMemcpy(&err, ctx->err, sizeof(err), cudaMemcpyDeviceToHost));
        if (err != astro::kErrFrontier) break;
        uint32_t done = 0;
        int r = grow_walk_buffers(ctx, &done);
        if (r != ASTRO_OK) return r;
        ctx->state_in_b = true;
        ++ctx->walk_reruns;
        if ((r = stage_traverse(ctx, 0.0f, false)) != ASTRO_OK) return r;
    }
    CK(cudaMemsetAsync(ctx->counters + 6, 0, sizeof(uint32_t), ctx->stream));
    return ASTRO_OK;
}

}  // namespace

// Steps launched since the last device check are checked (and rerun after
// a group-walk overflow) before any call that reads or replaces the state,
// so no call sees a state whose steps may still be run again.
#define SETTLE()                                                        \
    do {                                                                \
        if (ctx && ctx->pending_steps > 0) {                            \
            const int settle_r_ = check_device(ctx);                    \
            if (settle_r_ != ASTRO_OK) return settle_r_;                \
        }                                                               \
    } while (0)

// ------------------------------------------------------------------ ABI --

extern "C" {

const char* astro_version(void) { return kVersion; }

const char* astro_status_string(int status) {
    switch (status) {
        case ASTRO_OK: return "ok";
        case ASTRO_ERR_INVALID_ARGUMENT: return "invalid argument";
        case ASTRO_ERR_CAPACITY: return "capacity exceeded";
        case ASTRO_ERR_CUDA: return "CUDA error";
        case ASTRO_ERR_OUT_OF_MEMORY: return "out of device memory";
        case ASTRO_ERR_STATE: return "call order violated";
        case ASTRO_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
        case ASTRO_ERR_NOT_SUPPORTED: return "not supported";
        case ASTRO_ERR_DEVICE_OVERFLOW: return "device-side bound exceeded";
        default: return "unknown status";
    }
}

const char* astro_last_error(const astro_ctx* ctx) {
    return ctx ? ctx->last_error.c_str() : "no context";
}

int astro_params_default(uint32_t preset, astro_params* out) {
    if (!out) return ASTRO_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->preset = preset;
    out->form = ASTRO_FORM_PLAIN;
    out->lbits = 6;                 // MortonCode.metal:47-50
    out->theta = 0.7f;              // Renderer.swift:864
    out->open_delta_weight = 1.0f;
    out->force_clamp = 1e5f;        // BarnesHut.metal:100
    if (preset == ASTRO_PRESET_REFERENCE) {
        out->g = 1e11f;             // BarnesHut.metal:39
        out->softening = 0.01f;     // BarnesHut.metal:40
        out->leaf_min_dist2 = 50.0f;// BarnesHut.metal:70
        out->quant_offset = 1e6f;   // MortonCode.metal:35-37
        out->damping = 0.9995f;     // BarnesHut.metal:189
        out->type_accel_scale[0] = 5.0f;  // BarnesHut.metal:181-187
        out->type_accel_scale[1] = 5.0f;
        out->type_accel_scale[2] = 1.0f;
        out->bucket = 0;
        out->light_sources = 5;     // numStars (Renderer.swift:26)
    } else if (preset == ASTRO_PRESET_PHYSICAL) {
        out->g = 1.0f;
        out->softening = 0.01f;
        out->damping = 1.0f;
        out->type_accel_scale[0] = out->type_accel_scale[1] = out->type_accel_scale[2] = 1.0f;
        out->bucket = 16;
        out->flags = ASTRO_FLAG_OPEN_DELTA | ASTRO_FLAG_QUADRUPOLE;
    } else {
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    return ASTRO_OK;
}

int astro_create(const astro_params* params, uint32_t max_n, uint32_t max_systems,
                 astro_ctx** out) {
    if (!out) return ASTRO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const char* why = nullptr;
    int r = validate_params(params, &why);
    if (r != ASTRO_OK) return r;
    if (max_n == 0 || max_n > (1u << 30) || max_systems == 0 || max_systems > ASTRO_MAX_SYSTEMS)
        return ASTRO_ERR_INVALID_ARGUMENT;
    astro_ctx* ctx = new (std::nothrow) astro_ctx();
    if (!ctx) return ASTRO_ERR_OUT_OF_MEMORY;
    ctx->p = *params;
    ctx->max_n = max_n;
    ctx->max_sys = max_systems;
    // A walk frontier holds at most one layer's nodes of one system (node
    // list) or one run per opened node (runs, two words each): 2 max_n words.
    ctx->frontier_cap = (uint32_t)std::min<uint64_t>(16384, std::max<uint64_t>(64, 4ull * ((max_n + 1) / 2)));
    auto cleanup = [&](int code) {
        astro_destroy(ctx);
        return code;
    };
#define CKC(call)                                          \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cleanup(cuda_fail(nullptr, e_, #call)); \
    } while (0)
    CKC(cudaGetDevice(&ctx->device));
    CKC(astro::sort_init());
    CKC(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        CKC(dev_alloc(&ctx->pos[b], max_n));
        CKC(dev_alloc(&ctx->vel[b], max_n));
        CKC(dev_alloc(&ctx->ids[b], max_n));
    }
    CKC(dev_alloc(&ctx->acc, max_n));
    CKC(dev_alloc(&ctx->types, max_n));
    if (params->preset == ASTRO_PRESET_REFERENCE) {
        CKC(dev_alloc(&ctx->colors, max_n));
        CKC(dev_alloc(&ctx->lights, 16));
    }
    CKC(dev_alloc(&ctx->codes, max_n));
    CKC(dev_alloc(&ctx->sorted_keys, max_n));
    CKC(dev_alloc(&ctx->perm, max_n));
    ctx->staging_bytes = 64ull * max_n + 4096;
    CKC(cudaMalloc(&ctx->staging, ctx->staging_bytes));
    ctx->sort_temp_bytes = astro::sort_plan(max_n, 64).total;
    CKC(cudaMalloc(&ctx->sort_temp, ctx->sort_temp_bytes));
    ctx->topo_lookback_words = (size_t)astro::topology_tiles(max_n) * 32 + 32;
    CKC(dev_alloc(&ctx->topo_lookback, ctx->topo_lookback_words));
    CKC(dev_alloc(&ctx->counters, 16));
    CKC(dev_alloc(&ctx->groups, max_n));
    CKC(dev_alloc(&ctx->err, 1));
    CKC(dev_alloc(&ctx->stats, kNumStats));
    for (cudaEvent_t& e : ctx->trav_ev) CKC(cudaEventCreate(&e));
    CKC(dev_alloc(&ctx->layer_count, ASTRO_MAX_LAYERS));
    CKC(dev_alloc(&ctx->sys, max_systems));
    CKC(dev_alloc(&ctx->bbox32, 6ull * max_systems));
    CKC(dev_alloc(&ctx->bbox64, 6ull * max_systems));
    ctx->chunk_capacity = max_n / astro::kChunkParticles + max_systems + 1;
    CKC(dev_alloc(&ctx->chunks, ctx->chunk_capacity));
    CKC(cudaMemset(ctx->err, 0, sizeof(uint32_t)));
    CKC(cudaMemset(ctx->layer_count, 0, sizeof(uint32_t) * ASTRO_MAX_LAYERS));
    CKC(cudaMemset(ctx->stats, 0, kNumStats * sizeof(unsigned long long)));
    if (params->form == ASTRO_FORM_PRECISION && ensure_x64(ctx) != ASTRO_OK)
        return cleanup(ASTRO_ERR_OUT_OF_MEMORY);
#undef CKC
    *out = ctx;
    return ASTRO_OK;
}

int astro_destroy(astro_ctx* ctx) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->h2d_stream) cudaStreamSynchronize(ctx->h2d_stream);
    if (ctx->d2h_stream) cudaStreamSynchronize(ctx->d2h_stream);
    drop_graph(ctx);
    for (int b = 0; b < 2; ++b) {
        dev_free(ctx->pos[b]);
        dev_free(ctx->vel[b]);
        dev_free(ctx->ids[b]);
        dev_free(ctx->x64[b]);
    }
    dev_free(ctx->acc);
    dev_free(ctx->types);
    dev_free(ctx->colors);
    dev_free(ctx->lights);
    dev_free(ctx->splat_prim);
    dev_free(ctx->splat_kind);
    dev_free(ctx->splat_image);
    dev_free(ctx->splat_depth);
    dev_free(ctx->frag_keys);
    dev_free(ctx->frag_sorted);
    dev_free(ctx->frag_vals);
    if (ctx->frag_temp) cudaFree(ctx->frag_temp);
    dev_free(ctx->codes);
    dev_free(ctx->sorted_keys);
    dev_free(ctx->perm);
    if (ctx->staging) cudaFree(ctx->staging);
    dev_free(ctx->dl_inv);
    for (int i = 0; i < 2; ++i) {
        if (ctx->stage_in[i]) cudaFree(ctx->stage_in[i]);
        if (ctx->stage_out[i]) cudaFree(ctx->stage_out[i]);
        for (cudaEvent_t e : {ctx->ev_in_copied[i], ctx->ev_in_used[i], ctx->ev_out_ready[i],
                              ctx->ev_out_copied[i]})
            if (e) cudaEventDestroy(e);
    }
    if (ctx->h2d_stream) cudaStreamDestroy(ctx->h2d_stream);
    if (ctx->d2h_stream) cudaStreamDestroy(ctx->d2h_stream);
    if (ctx->sort_temp) cudaFree(ctx->sort_temp);
    dev_free(ctx->topo_lookback);
    dev_free(ctx->counters);
    dev_free(ctx->err);
    dev_free(ctx->stats);
    dev_free(ctx->layer_count);
    dev_free(ctx->sys);
    dev_free(ctx->bbox32);
    dev_free(ctx->bbox64);
    dev_free(ctx->chunks);
    dev_free(ctx->node_cm);
    dev_free(ctx->node_rng);
    dev_free(ctx->node_key);
    if (ctx->node_sum) cudaFree(ctx->node_sum);
    dev_free(ctx->node_pbeg);
    dev_free(ctx->node_cbeg);
    dev_free(ctx->node_parent);
    dev_free(ctx->node_arrive);
    dev_free(ctx->node_crit2);
    dev_free(ctx->node_ecol);
    dev_free(ctx->node_ecen);
    dev_free(ctx->node_q);
    dev_free(ctx->node_qyz);
    dev_free(ctx->groups);
    dev_free(ctx->frontier);
    dev_free(ctx->lists);
    dev_free(ctx->list_next);
    dev_free(ctx->group_desc);
    if (ctx->readback) cudaFree(ctx->readback);
    for (cudaEvent_t& e : ctx->trav_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return ASTRO_OK;
}

int astro_get_params(const astro_ctx* ctx, astro_params* out) {
    if (!ctx || !out) return ASTRO_ERR_INVALID_ARGUMENT;
    *out = ctx->p;
    return ASTRO_OK;
}

// Changing preset, form or lbits discards the uploaded state (upload again);
// the other fields take effect at the next step.
int astro_set_params(astro_ctx* ctx, const astro_params* params) {
    SETTLE();
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    const char* why = nullptr;
    int r = validate_params(params, &why);
    if (r != ASTRO_OK) return fail(ctx, r, why);
    const bool structural = params->preset != ctx->p.preset || params->form != ctx->p.form ||
                            params->lbits != ctx->p.lbits;
    if (params->form == ASTRO_FORM_PRECISION && (r = ensure_x64(ctx)) != ASTRO_OK) return r;
    if (params->preset == ASTRO_PRESET_REFERENCE && !ctx->colors) {
        if (dev_alloc(&ctx->colors, ctx->max_n) != cudaSuccess ||
            dev_alloc(&ctx->lights, 16) != cudaSuccess) {
            dev_free(ctx->colors);
            dev_free(ctx->lights);
            return fail(ctx, ASTRO_ERR_OUT_OF_MEMORY, "colour buffers");
        }
    }
    ctx->p = *params;
    drop_graph(ctx);
    if ((r = ensure_frontier(ctx)) != ASTRO_OK) return r;
    if (structural) {
        ctx->uploaded = false;
        ctx->tree_valid = false;
        ctx->state_in_b = false;
    }
    return ASTRO_OK;
}

static int upload_particles(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                            const ColorType* ct, uint32_t n, uint32_t n_tree);

static int upload_common(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                         const ColorType* ct, uint32_t n, uint32_t n_tree,
                         const std::vector<uint32_t>& sizes) {
    cudaStream_t st = ctx->stream;
    const bool phys = is_phys(ctx), prec = is_prec(ctx);
    // New particles in the same layout (counts, system sizes, depth) as the
    // last upload: the buffers, the system records' layout fields and the
    // captured step stay valid (every data-dependent field is recomputed by
    // each step), so only the particles are copied in.
    const bool same_layout = ctx->uploaded && n == ctx->n && n_tree == ctx->n_tree &&
                             sizes == ctx->sys_sizes && ctx->lbits == ctx->p.lbits;
    ctx->tree_valid = false;
    ctx->state_in_b = false;
    if (same_layout) return upload_particles(ctx, pm, vr, ct, n, n_tree);
    drop_graph(ctx);
    ctx->uploaded = false;
    ctx->n = n;
    ctx->n_tree = n_tree;
    ctx->nsys = (uint32_t)sizes.size();
    ctx->lbits = ctx->p.lbits;
    ctx->sysbits = ctx->nsys > 1 ? bits_for(ctx->nsys) : 0;
    ctx->key_bits = 3 * ctx->lbits + ctx->sysbits;
    if (ctx->key_bits > 64)
        return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "3*lbits + system bits exceeds 64 key bits");
    layer_table(sizes, ctx->lbits, &ctx->layers, &ctx->capacity);
    int r = ensure_tree(ctx, ctx->capacity);
    if (r != ASTRO_OK) return r;
    if ((r = ensure_frontier(ctx)) != ASTRO_OK) return r;
    if (prec && (r = ensure_x64(ctx)) != ASTRO_OK) return r;
    // Systems and chunks.
    std::vector<SysInfo> sys(ctx->nsys);
    std::vector<Chunk> chunks;
    uint32_t off = 0;
    for (uint32_t s = 0; s < ctx->nsys; ++s) {
        std::memset(&sys[s], 0, sizeof(SysInfo));
        sys[s].begin = off;
        sys[s].end = off + sizes[s];
        sys[s].root = ctx->layers.offset[ctx->lbits] + s;
        for (uint32_t b = off; b < off + sizes[s]; b += astro::kChunkParticles)
            chunks.push_back(Chunk{s, b, std::min(b + astro::kChunkParticles, off + sizes[s]), 0});
        off += sizes[s];
    }
    if (chunks.size() > ctx->chunk_capacity) return fail(ctx, ASTRO_ERR_CAPACITY, "too many chunks");
    ctx->nchunks = (uint32_t)chunks.size();
    ctx->sys_sizes = sizes;
    CK(cudaMemcpyAsync(ctx->sys, sys.data(), sizeof(SysInfo) * sys.size(), cudaMemcpyHostToDevice, st));
    if (!chunks.empty())
        CK(cudaMemcpyAsync(ctx->chunks, chunks.data(), sizeof(Chunk) * chunks.size(),
                           cudaMemcpyHostToDevice, st));
    // Box accumulators start empty.
    CK(cudaMemsetAsync(ctx->bbox32, 0, 6ull * ctx->nsys * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(ctx->bbox64, 0, 6ull * ctx->nsys * sizeof(unsigned long long), st));
    {
        std::vector<uint32_t> lo32(6ull * ctx->nsys, 0);
        std::vector<unsigned long long> lo64(6ull * ctx->nsys, 0);
        for (uint32_t s = 0; s < ctx->nsys; ++s)
            for (int a = 0; a < 3; ++a) {
                lo32[6ull * s + a] = ~0u;
                lo64[6ull * s + a] = ~0ull;
            }
        CK(cudaMemcpyAsync(ctx->bbox32, lo32.data(), lo32.size() * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ctx->bbox64, lo64.data(), lo64.size() * 8, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));  // the host vectors go out of scope
    }
    return upload_particles(ctx, pm, vr, ct, n, n_tree);
}

// Copy streams, staging slots and events of the asynchronous transfers.
static int ensure_async(astro_ctx* ctx) {
    if (ctx->d2h_stream) return ASTRO_OK;
    const size_t bytes = 64ull * ctx->max_n;
    for (int i = 0; i < 2; ++i) {
        if (!ctx->stage_in[i]) CK(cudaMalloc(&ctx->stage_in[i], bytes));
        if (!ctx->stage_out[i]) CK(cudaMalloc(&ctx->stage_out[i], bytes));
        for (cudaEvent_t* e : {&ctx->ev_in_copied[i], &ctx->ev_in_used[i], &ctx->ev_out_ready[i],
                               &ctx->ev_out_copied[i]})
            if (!*e) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    if (!ctx->h2d_stream) CK(cudaStreamCreateWithFlags(&ctx->h2d_stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking));
    return ASTRO_OK;
}

// The particle copy of an upload: host arrays through the staging buffer into
// the state (A) buffers, ids 0..n-1, types and colours.
static int upload_particles(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                            const ColorType* ct, uint32_t n, uint32_t n_tree) {
    cudaStream_t st = ctx->stream;
    const bool phys = is_phys(ctx), prec = is_prec(ctx);
    char* stg = static_cast<char*>(ctx->staging);
    PositionMass* d_pm = reinterpret_cast<PositionMass*>(stg);
    VelocityRadius* d_vr = reinterpret_cast<VelocityRadius*>(stg + 32ull * ctx->max_n);
    CK(cudaMemcpyAsync(d_pm, pm, sizeof(PositionMass) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_vr, vr, sizeof(VelocityRadius) * n, cudaMemcpyHostToDevice, st));
    ColorType* d_ct = nullptr;
    if (ct) {
        // ColorType shares the staging area after the velocities are converted.
        CK(astro::launch_upload_convert(prec, d_pm, d_vr, nullptr, ctx->pos[0], ctx->vel[0],
                                        phys ? ctx->ids[0] : nullptr, nullptr, ctx->x64[0], n,
                                        n_tree, st));
        d_ct = reinterpret_cast<ColorType*>(stg);
        CK(cudaMemcpyAsync(d_ct, ct, sizeof(ColorType) * n, cudaMemcpyHostToDevice, st));
        CK(astro::launch_types_from_colors(d_ct, ctx->types, ctx->colors, n, st));
    } else {
        if (ctx->colors) CK(cudaMemsetAsync(ctx->colors, 0, sizeof(float4) * n, st));
        CK(astro::launch_upload_convert(prec, d_pm, d_vr, nullptr, ctx->pos[0], ctx->vel[0],
                                        phys ? ctx->ids[0] : nullptr, ctx->types, ctx->x64[0], n,
                                        n_tree, st));
    }
    ctx->uploaded = true;
    return ASTRO_OK;
}

int astro_upload(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                 const ColorType* ct, uint32_t n, uint32_t n_tree) {
    SETTLE();
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!pm || !vr || n == 0 || n_tree > n)
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "upload: null pointer, n == 0 or n_tree > n");
    if (n > ctx->max_n) return fail(ctx, ASTRO_ERR_CAPACITY, "upload: n exceeds max_n");
    if (is_phys(ctx) && n_tree != n)
        return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "PHYSICAL preset needs n_tree == n");
    std::vector<uint32_t> sizes(1, n_tree);
    return upload_common(ctx, pm, vr, ct, n, n_tree, sizes);
}

int astro_upload_systems(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                         const uint32_t* sys_sizes, uint32_t nsys) {
    SETTLE();
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!pm || !vr || !sys_sizes || nsys == 0)
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "upload_systems: null pointer or nsys == 0");
    if (!is_phys(ctx)) return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "systems need the PHYSICAL preset");
    if (nsys > ctx->max_sys) return fail(ctx, ASTRO_ERR_CAPACITY, "nsys exceeds max_systems");
    uint64_t total = 0;
    std::vector<uint32_t> sizes(sys_sizes, sys_sizes + nsys);
    for (uint32_t s : sizes) {
        if (s == 0) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "empty system");
        total += s;
    }
    if (total > ctx->max_n) return fail(ctx, ASTRO_ERR_CAPACITY, "total particles exceed max_n");
    return upload_common(ctx, pm, vr, nullptr, (uint32_t)total, (uint32_t)total, sizes);
}

int astro_download(astro_ctx* ctx, PositionMass* pm, VelocityRadius* vr, uint32_t n) {
    SETTLE();
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!ctx->uploaded) return fail(ctx, ASTRO_ERR_STATE, "download before upload");
    if (n != ctx->n || (!pm && !vr)) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "download: n mismatch");
    cudaStream_t st = ctx->stream;
    const Cur c = current(ctx);
    char* stg = static_cast<char*>(ctx->staging);
    PositionMass* d_pm = reinterpret_cast<PositionMass*>(stg);
    VelocityRadius* d_vr = reinterpret_cast<VelocityRadius*>(stg + 32ull * ctx->max_n);
    if (c.ids && !ctx->dl_inv) CK(dev_alloc(&ctx->dl_inv, ctx->max_n));
    CK(astro::launch_download_convert(is_prec(ctx), c.pos, c.vel, c.ids, c.x64, d_pm, d_vr, n, st,
                                      ctx->dl_inv));
    if (pm) CK(cudaMemcpyAsync(pm, d_pm, sizeof(PositionMass) * n, cudaMemcpyDeviceToHost, st));
    if (vr) CK(cudaMemcpyAsync(vr, d_vr, sizeof(VelocityRadius) * n, cudaMemcpyDeviceToHost, st));
    return check_device(ctx);
}

int astro_upload_async(astro_ctx* ctx, const PositionMass* pm, const VelocityRadius* vr,
                       uint32_t n) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!pm || !vr) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "upload_async: null pointer");
    if (!ctx->uploaded)
        return fail(ctx, ASTRO_ERR_STATE, "upload_async: needs an earlier upload (it keeps that layout)");
    if (n != ctx->n) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "upload_async: n differs from the upload's");
    int r = ensure_async(ctx);
    if (r != ASTRO_OK) return r;
    if (ctx->pending_steps > 0) ctx->steps_unrerunnable = true;
    const uint32_t s = ctx->in_slot;
    ctx->in_slot ^= 1u;
    char* stg = static_cast<char*>(ctx->stage_in[s]);
    PositionMass* d_pm = reinterpret_cast<PositionMass*>(stg);
    VelocityRadius* d_vr = reinterpret_cast<VelocityRadius*>(stg + 32ull * ctx->max_n);
    // The slot is free once the conversion that last read it has run; the
    // copy itself overlaps the steps queued before it.
    CK(cudaStreamWaitEvent(ctx->h2d_stream, ctx->ev_in_used[s], 0));
    CK(cudaMemcpyAsync(d_pm, pm, sizeof(PositionMass) * n, cudaMemcpyHostToDevice, ctx->h2d_stream));
    CK(cudaMemcpyAsync(d_vr, vr, sizeof(VelocityRadius) * n, cudaMemcpyHostToDevice, ctx->h2d_stream));
    CK(cudaEventRecord(ctx->ev_in_copied[s], ctx->h2d_stream));
    // The state is replaced in step-stream order, after the queued steps;
    // particle types and colours stay those of the last upload.
    cudaStream_t st = ctx->stream;
    CK(cudaStreamWaitEvent(st, ctx->ev_in_copied[s], 0));
    CK(astro::launch_upload_convert(is_prec(ctx), d_pm, d_vr, nullptr, ctx->pos[0], ctx->vel[0],
                                    is_phys(ctx) ? ctx->ids[0] : nullptr, nullptr, ctx->x64[0], n,
                                    ctx->n_tree, st));
    CK(cudaEventRecord(ctx->ev_in_used[s], st));
    ctx->tree_valid = false;
    ctx->state_in_b = false;
    return ASTRO_OK;
}

int astro_download_async(astro_ctx* ctx, PositionMass* pm, VelocityRadius* vr, uint32_t n) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!ctx->uploaded) return fail(ctx, ASTRO_ERR_STATE, "download before upload");
    if (n != ctx->n || (!pm && !vr))
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "download_async: n mismatch or no output");
    int r = ensure_async(ctx);
    if (r != ASTRO_OK) return r;
    if (ctx->pending_steps > 0) ctx->steps_unrerunnable = true;
    const uint32_t s = ctx->out_slot;
    ctx->out_slot ^= 1u;
    char* stg = static_cast<char*>(ctx->stage_out[s]);
    PositionMass* d_pm = reinterpret_cast<PositionMass*>(stg);
    VelocityRadius* d_vr = reinterpret_cast<VelocityRadius*>(stg + 32ull * ctx->max_n);
    cudaStream_t st = ctx->stream;
    // The slot is free once its last copy to the host has run; the copy of
    // this state overlaps the steps queued after it.
    CK(cudaStreamWaitEvent(st, ctx->ev_out_copied[s], 0));
    const Cur c = current(ctx);
    if (c.ids && !ctx->dl_inv) CK(dev_alloc(&ctx->dl_inv, ctx->max_n));
    CK(astro::launch_download_convert(is_prec(ctx), c.pos, c.vel, c.ids, c.x64, d_pm, d_vr, n, st,
                                      ctx->dl_inv));
    CK(cudaEventRecord(ctx->ev_out_ready[s], st));
    CK(cudaStreamWaitEvent(ctx->d2h_stream, ctx->ev_out_ready[s], 0));
    if (pm) CK(cudaMemcpyAsync(pm, d_pm, sizeof(PositionMass) * n, cudaMemcpyDeviceToHost, ctx->d2h_stream));
    if (vr) CK(cudaMemcpyAsync(vr, d_vr, sizeof(VelocityRadius) * n, cudaMemcpyDeviceToHost, ctx->d2h_stream));
    CK(cudaEventRecord(ctx->ev_out_copied[s], ctx->d2h_stream));
    return ASTRO_OK;
}

#define NEED_UPLOAD()                                                          \
    do {                                                                       \
        if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;                           \
        if (!ctx->uploaded) return fail(ctx, ASTRO_ERR_STATE, "no upload yet"); \
    } while (0)

int astro_encode(astro_ctx* ctx) {
    SETTLE();
    NEED_UPLOAD();
    drop_graph(ctx);
    return stage_encode(ctx);
}
int astro_sort(astro_ctx* ctx) {
    SETTLE();
    NEED_UPLOAD();
    drop_graph(ctx);
    return stage_sort(ctx);
}
int astro_build(astro_ctx* ctx) {
    SETTLE();
    NEED_UPLOAD();
    drop_graph(ctx);
    return stage_build(ctx);
}
int astro_traverse(astro_ctx* ctx) {
    NEED_UPLOAD();
    drop_graph(ctx);
    int r;
    if (ctx->pending_steps > 0 && (r = check_device(ctx)) != ASTRO_OK) return r;
    if ((r = stage_traverse(ctx, 0.0f, false)) != ASTRO_OK) return r;
    return group_walk(ctx) ? settle_traverse(ctx) : ASTRO_OK;
}
int astro_integrate(astro_ctx* ctx, float dt) {
    SETTLE();
    NEED_UPLOAD();
    drop_graph(ctx);
    return stage_integrate(ctx, dt);
}

int astro_step(astro_ctx* ctx, float dt, uint32_t nsteps) {
    NEED_UPLOAD();
    if (!std::isfinite(dt)) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "dt must be finite");
    if (ctx->state_in_b) return fail(ctx, ASTRO_ERR_STATE, "step called between sort and traverse");
    // Steps still unchecked run again at their own dt if they overflowed.
    int r;
    if (ctx->pending_steps > 0 && ctx->pending_dt != dt && (r = check_device(ctx)) != ASTRO_OK)
        return r;
    return launch_steps(ctx, dt, nsteps);
}

int astro_synchronize(astro_ctx* ctx) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    return check_device(ctx);
}

int astro_get_stream(astro_ctx* ctx, void** stream) {
    if (!ctx || !stream) return ASTRO_ERR_INVALID_ARGUMENT;
    *stream = ctx->stream;
    return ASTRO_OK;
}

int astro_read_keys(astro_ctx* ctx, uint64_t* codes, uint64_t* sorted_codes,
                    uint32_t* sorted_indices, uint32_t n) {
    SETTLE();
    NEED_UPLOAD();
    const uint32_t count = is_phys(ctx) ? ctx->n : ctx->n_tree;
    if (n != count) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "read_keys: n must be the tree count");
    cudaStream_t st = ctx->stream;
    const Cur c = current(ctx);
    uint64_t* tmp = static_cast<uint64_t*>(ctx->staging);
    if (codes) {
        if (is_phys(ctx)) {
            CK(astro::launch_scatter_u64(ctx->sorted_keys, c.ids, tmp, n, st));
            CK(cudaMemcpyAsync(codes, tmp, 8ull * n, cudaMemcpyDeviceToHost, st));
        } else {
            CK(cudaMemcpyAsync(codes, ctx->codes, 8ull * n, cudaMemcpyDeviceToHost, st));
        }
    }
    if (sorted_codes)
        CK(cudaMemcpyAsync(sorted_codes, ctx->sorted_keys, 8ull * n, cudaMemcpyDeviceToHost, st));
    if (sorted_indices)
        CK(cudaMemcpyAsync(sorted_indices, is_phys(ctx) ? c.ids : ctx->perm, 4ull * n,
                           cudaMemcpyDeviceToHost, st));
    if (codes) CK(cudaStreamSynchronize(st));
    return check_device(ctx);
}

int astro_read_tree_info(astro_ctx* ctx, uint32_t* n_layers, uint32_t* layer_sizes,
                         uint32_t* layer_offsets, uint32_t* layer_counts, uint32_t max_layers) {
    SETTLE();
    NEED_UPLOAD();
    const uint32_t L = ctx->layers.n_layers;
    if (n_layers) *n_layers = L;
    if ((layer_sizes || layer_offsets || layer_counts) && max_layers < L)
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "read_tree_info: max_layers too small");
    for (uint32_t l = 0; l < L; ++l) {
        if (layer_sizes) layer_sizes[l] = ctx->layers.size[l];
        if (layer_offsets) layer_offsets[l] = ctx->layers.offset[l];
    }
    if (layer_counts) {
        CK(cudaMemcpyAsync(layer_counts, ctx->layer_count, 4ull * L, cudaMemcpyDeviceToHost,
                           ctx->stream));
    }
    return check_device(ctx);
}

int astro_read_nodes(astro_ctx* ctx, OctreeNode* nodes, uint64_t first, uint64_t count) {
    SETTLE();
    NEED_UPLOAD();
    if (!nodes || first + count > ctx->capacity)
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "read_nodes: range outside the node capacity");
    cudaStream_t st = ctx->stream;
    const uint64_t chunk = 1ull << 18;  // nodes per staging round (32 MB)
    if (!ctx->readback) {
        ctx->readback_bytes = chunk * sizeof(OctreeNode);
        CK(cudaMalloc(&ctx->readback, ctx->readback_bytes));
    }
    OctreeNode* d_out = static_cast<OctreeNode*>(ctx->readback);
    uint64_t pos = first;
    while (pos < first + count) {
        // Layer of slot pos.
        uint32_t l = 0;
        while (l + 1 < ctx->layers.n_layers && ctx->layers.offset[l + 1] <= pos) ++l;
        const uint64_t layer_end = (uint64_t)ctx->layers.offset[l] + ctx->layers.size[l];
        const uint64_t m = std::min<uint64_t>({chunk, first + count - pos, layer_end - pos});
        CK(astro::launch_readback_nodes(ctx->node_cm, ctx->node_rng, ctx->node_key,
                                        ctx->node_ecol, ctx->node_ecen,
                                        ctx->layer_count, l, ctx->layers.offset[l],
                                        (uint32_t)(pos - ctx->layers.offset[l]), (uint32_t)m, d_out,
                                        st));
        CK(cudaMemcpyAsync(nodes + (pos - first), d_out, m * sizeof(OctreeNode),
                           cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        pos += m;
    }
    return check_device(ctx);
}

int astro_read_accel(astro_ctx* ctx, float* acc4, uint32_t n) {
    SETTLE();
    NEED_UPLOAD();
    if (!acc4 || n != ctx->n) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "read_accel: n mismatch");
    cudaStream_t st = ctx->stream;
    if (is_phys(ctx)) {
        float4* tmp = static_cast<float4*>(ctx->staging);
        CK(astro::launch_scatter_f4(ctx->acc, current(ctx).ids, tmp, n, st));
        CK(cudaMemcpyAsync(acc4, tmp, 16ull * n, cudaMemcpyDeviceToHost, st));
    } else {
        CK(cudaMemcpyAsync(acc4, ctx->acc, 16ull * n, cudaMemcpyDeviceToHost, st));
    }
    return check_device(ctx);
}

int astro_read_stats(astro_ctx* ctx, uint64_t* interactions, uint64_t* node_visits,
                     uint64_t* cell_interactions) {
    SETTLE();
    NEED_UPLOAD();
    unsigned long long s[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(s, ctx->stats, sizeof(s), cudaMemcpyDeviceToHost, ctx->stream));
    int r = check_device(ctx);
    if (interactions) *interactions = s[0];
    if (node_visits) *node_visits = s[1];
    if (cell_interactions) *cell_interactions = s[2];
    return r;
}

int astro_read_far_stats(astro_ctx* ctx, uint64_t* far_nodes, uint64_t* far_interactions) {
    SETTLE();
    NEED_UPLOAD();
    unsigned long long s[kNumStats] = {0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(s, ctx->stats, sizeof(s), cudaMemcpyDeviceToHost, ctx->stream));
    int r = check_device(ctx);
    if (far_nodes) *far_nodes = s[3];
    if (far_interactions) *far_interactions = s[4];
    return r;
}

int astro_read_traverse_times(astro_ctx* ctx, float* walk_ms, float* eval_ms) {
    SETTLE();
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!ctx->trav_timed) return fail(ctx, ASTRO_ERR_STATE, "no timed group walk stage call yet");
    CK(cudaEventSynchronize(ctx->trav_ev[2]));
    float w = 0.f, e = 0.f;
    CK(cudaEventElapsedTime(&w, ctx->trav_ev[0], ctx->trav_ev[1]));
    CK(cudaEventElapsedTime(&e, ctx->trav_ev[1], ctx->trav_ev[2]));
    if (walk_ms) *walk_ms = w;
    if (eval_ms) *eval_ms = e;
    return ASTRO_OK;
}

int astro_direct_accel_f64(astro_ctx* ctx, const uint32_t* sample_idx, uint32_t n_sample,
                           double* acc3) {
    SETTLE();
    NEED_UPLOAD();
    if (!sample_idx || !acc3 || n_sample == 0 || n_sample > ctx->n)
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "direct_accel: bad samples");
    if (!is_phys(ctx)) return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "direct sum needs the PHYSICAL preset");
    cudaStream_t st = ctx->stream;
    const Cur c = current(ctx);
    // Staging layout: inverse ids | samples | slots | begin | end | out.
    char* stg = static_cast<char*>(ctx->staging);
    uint32_t* inv = reinterpret_cast<uint32_t*>(stg);
    uint32_t* d_samples = inv + ctx->n;
    uint32_t* d_slots = d_samples + n_sample;
    uint32_t* d_begin = d_slots + n_sample;
    uint32_t* d_end = d_begin + n_sample;
    double* d_out = reinterpret_cast<double*>(
        (reinterpret_cast<uintptr_t>(d_end + n_sample) + 15) & ~uintptr_t(15));
    std::vector<uint32_t> begin(n_sample), end(n_sample);
    std::vector<uint32_t> offs(ctx->sys_sizes.size() + 1, 0);
    for (size_t s = 0; s < ctx->sys_sizes.size(); ++s) offs[s + 1] = offs[s] + ctx->sys_sizes[s];
    for (uint32_t k = 0; k < n_sample; ++k) {
        if (sample_idx[k] >= ctx->n) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "sample out of range");
        const size_t s = std::upper_bound(offs.begin(), offs.end(), sample_idx[k]) - offs.begin() - 1;
        begin[k] = offs[s];
        end[k] = offs[s + 1];
    }
    CK(astro::launch_inverse_ids(c.ids, inv, ctx->n, st));
    CK(cudaMemcpyAsync(d_samples, sample_idx, 4ull * n_sample, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_begin, begin.data(), 4ull * n_sample, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_end, end.data(), 4ull * n_sample, cudaMemcpyHostToDevice, st));
    CK(astro::launch_gather_u32(inv, d_samples, d_slots, n_sample, st));
    astro::DirectArgs a{};
    a.pos = c.pos;
    a.x64 = is_prec(ctx) ? c.x64 : nullptr;
    a.slot = d_slots;
    a.sys_begin = d_begin;
    a.sys_end = d_end;
    a.out = d_out;
    a.n = ctx->n;
    a.n_sample = n_sample;
    a.g = ctx->p.g;
    a.eps2 = (double)ctx->p.softening * (double)ctx->p.softening;
    CK(astro::launch_direct_sum(a, st));
    CK(cudaMemcpyAsync(acc3, d_out, 24ull * n_sample, cudaMemcpyDeviceToHost, st));
    return check_device(ctx);
}

int astro_lighting(astro_ctx* ctx, uint32_t num_stars) {
    SETTLE();
    NEED_UPLOAD();
    if (is_phys(ctx)) return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "lighting needs the REFERENCE preset");
    CK(astro::launch_lighting(ctx->pos[0], ctx->types, ctx->colors, ctx->lights, ctx->n, num_stars,
                              ctx->stream));
    return ASTRO_OK;
}

int astro_read_colors(astro_ctx* ctx, ColorType* ct, uint32_t n) {
    SETTLE();
    NEED_UPLOAD();
    if (is_phys(ctx)) return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "colours need the REFERENCE preset");
    if (!ct || n != ctx->n) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "read_colors: n mismatch");
    ColorType* tmp = static_cast<ColorType*>(ctx->staging);
    CK(astro::launch_colors_out(ctx->colors, ctx->types, tmp, n, ctx->stream));
    CK(cudaMemcpyAsync(ct, tmp, sizeof(ColorType) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return check_device(ctx);
}

int astro_splat(astro_ctx* ctx, const astro_camera* camera, uint32_t width, uint32_t height,
                const float* clear, float* rgba, float* depth) {
    SETTLE();
    NEED_UPLOAD();
    if (is_phys(ctx)) return fail(ctx, ASTRO_ERR_NOT_SUPPORTED, "the splat draws the REFERENCE preset");
    if (!camera || !rgba || width == 0 || height == 0)
        return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "splat: bad camera, image or size");
    const uint64_t pixels = (uint64_t)width * height;
    if (pixels > (1ull << 31)) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "splat: image too large");
    cudaStream_t st = ctx->stream;
    if (!ctx->splat_prim) {
        CK(dev_alloc(&ctx->splat_prim, ctx->max_n));
        CK(dev_alloc(&ctx->splat_kind, ctx->max_n + 1));  // + the fragment cursor
    }
    if (pixels > ctx->splat_pixels) {
        dev_free(ctx->splat_image);
        dev_free(ctx->splat_depth);
        ctx->splat_pixels = 0;
        CK(dev_alloc(&ctx->splat_image, pixels));
        CK(dev_alloc(&ctx->splat_depth, pixels));
        ctx->splat_pixels = pixels;
    }
    astro::SplatArgs a{};
    a.pos = ctx->pos[0];
    a.vel = ctx->vel[0];
    a.colors = ctx->colors;
    a.types = ctx->types;
    a.n = ctx->n;
    std::memcpy(a.view, camera->view, sizeof(a.view));
    std::memcpy(a.proj, camera->projection, sizeof(a.proj));
    std::memcpy(a.cam, camera->position, sizeof(a.cam));
    a.width = width;
    a.height = height;
    const float background[4] = {0.0f / 255.0f, 0.0f / 255.0f, 1.0f / 255.0f, 1.0f};  // Renderer.swift:46
    std::memcpy(a.clear, clear ? clear : background, sizeof(a.clear));
    a.clear_depth = 1.0f;  // Renderer.swift:768
    a.prim = ctx->splat_prim;
    a.kind = ctx->splat_kind;
    a.cursor = ctx->splat_kind + ctx->max_n;
    a.image = ctx->splat_image;
    a.depth = ctx->splat_depth;
    CK(astro::launch_splat_project(a, st));
    // Fragments: emit, and emit again into a larger buffer if they overflowed.
    uint32_t count = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
        a.keys = ctx->frag_keys;
        a.cap = ctx->frag_cap;
        CK(cudaMemsetAsync(a.cursor, 0, sizeof(uint32_t), st));
        CK(astro::launch_splat_emit(a, st));
        CK(cudaMemcpyAsync(&count, a.cursor, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (count <= ctx->frag_cap) break;
        dev_free(ctx->frag_keys);
        dev_free(ctx->frag_sorted);
        dev_free(ctx->frag_vals);
        if (ctx->frag_temp) cudaFree(ctx->frag_temp);
        ctx->frag_temp = nullptr;
        ctx->frag_cap = 0;
        const uint32_t cap = (uint32_t)std::min<uint64_t>((uint64_t)count + count / 4 + 1024, 0xFFFFFFFFull);
        const uint32_t key_bits = 64;
        ctx->frag_temp_bytes = astro::sort_plan(cap, key_bits).total;
        CK(dev_alloc(&ctx->frag_keys, cap));
        CK(dev_alloc(&ctx->frag_sorted, cap));
        CK(dev_alloc(&ctx->frag_vals, cap));
        CK(cudaMalloc(&ctx->frag_temp, ctx->frag_temp_bytes));
        ctx->frag_cap = cap;
    }
    if (count > ctx->frag_cap) return fail(ctx, ASTRO_ERR_CAPACITY, "splat: fragment count grew");
    // Sort by (pixel, particle): the per-pixel draw order.
    uint32_t pixel_bits = 0;
    while ((1ull << pixel_bits) < pixels) ++pixel_bits;
    CK(astro::sort_pairs(ctx->frag_keys, nullptr, ctx->frag_sorted, ctx->frag_vals, count, nullptr,
                         32u + pixel_bits, ctx->frag_temp, ctx->frag_temp_bytes, st, ctx->err));
    CK(astro::launch_splat_clear(a, st));
    CK(astro::launch_splat_fold(a, ctx->frag_sorted, count, st));
    CK(cudaMemcpyAsync(rgba, ctx->splat_image, 16ull * pixels, cudaMemcpyDeviceToHost, st));
    if (depth) CK(cudaMemcpyAsync(depth, ctx->splat_depth, 4ull * pixels, cudaMemcpyDeviceToHost, st));
    return check_device(ctx);
}

// ------------------------------------------------------------ state files --

}  // extern "C"

namespace {

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
    bool put(const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }
    bool get(void* p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }
};

}  // namespace

extern "C" {

int astro_save_state(astro_ctx* ctx, const char* path, uint64_t step, double time) {
    SETTLE();
    NEED_UPLOAD();
    if (!path) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "save_state: path is NULL");
    if (ctx->state_in_b) return fail(ctx, ASTRO_ERR_STATE, "save_state in the middle of a step");
    const uint32_t n = ctx->n;
    cudaStream_t st = ctx->stream;
    const Cur c = current(ctx);
    const bool has_types = !is_phys(ctx), has64 = is_prec(ctx);
    std::vector<float4> pos(n), vel(n);
    std::vector<uint32_t> ids(n), types(has_types ? n : 0);
    std::vector<double> soa(has64 ? 3ull * n : 0);
    CK(cudaMemcpyAsync(pos.data(), c.pos, 16ull * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(vel.data(), c.vel, 16ull * n, cudaMemcpyDeviceToHost, st));
    if (c.ids) CK(cudaMemcpyAsync(ids.data(), c.ids, 4ull * n, cudaMemcpyDeviceToHost, st));
    else
        for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    if (has_types) CK(cudaMemcpyAsync(types.data(), ctx->types, 4ull * n, cudaMemcpyDeviceToHost, st));
    if (has64) CK(cudaMemcpyAsync(soa.data(), c.x64, 24ull * n, cudaMemcpyDeviceToHost, st));
    int r = check_device(ctx);
    if (r != ASTRO_OK) return r;
    std::vector<PositionMass> pm(n);
    std::vector<VelocityRadius> vr(n);
    std::vector<double> xyz(has64 ? 3ull * n : 0);
    std::memset(pm.data(), 0, sizeof(PositionMass) * n);
    std::memset(vr.data(), 0, sizeof(VelocityRadius) * n);
    for (uint32_t i = 0; i < n; ++i) {
        pm[i].position[0] = pos[i].x;
        pm[i].position[1] = pos[i].y;
        pm[i].position[2] = pos[i].z;
        pm[i].mass = pos[i].w;
        vr[i].velocity[0] = vel[i].x;
        vr[i].velocity[1] = vel[i].y;
        vr[i].velocity[2] = vel[i].z;
        vr[i].radius = vel[i].w;
        if (has64)
            for (int a = 0; a < 3; ++a) {
                xyz[3ull * i + a] = soa[(size_t)a * n + i];
                pm[i].position[a] = (float)soa[(size_t)a * n + i];
            }
    }
    astro_state_header h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, ASTRO_STATE_MAGIC, 8);
    h.version = ASTRO_STATE_VERSION;
    h.header_bytes = sizeof(h);
    h.params = ctx->p;
    h.step = step;
    h.time = time;
    h.n = n;
    h.n_tree = ctx->n_tree;
    h.nsys = ctx->nsys;
    h.contents = (has_types ? ASTRO_STATE_TYPES : 0u) | (has64 ? ASTRO_STATE_POS64 : 0u);
    File f;
    f.f = std::fopen(path, "wb");
    if (!f.f) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "save_state: cannot open the file");
    bool ok = f.put(&h, sizeof(h)) && f.put(ctx->sys_sizes.data(), 4ull * ctx->nsys) &&
              f.put(pm.data(), sizeof(PositionMass) * n) && f.put(vr.data(), sizeof(VelocityRadius) * n) &&
              f.put(ids.data(), 4ull * n) && f.put(types.data(), 4ull * types.size()) &&
              f.put(xyz.data(), 8ull * xyz.size());
    ok = (std::fclose(f.f) == 0) && ok;
    f.f = nullptr;
    if (!ok) return fail(ctx, ASTRO_ERR_INVALID_ARGUMENT, "save_state: write failed");
    return ASTRO_OK;
}

int astro_load_state(const char* path, uint32_t max_n, astro_ctx** out, uint64_t* step,
                     double* time) {
    if (!path || !out) return ASTRO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    File f;
    f.f = std::fopen(path, "rb");
    if (!f.f) return ASTRO_ERR_INVALID_ARGUMENT;
    astro_state_header h;
    if (!f.get(&h, sizeof(h)) || std::memcmp(h.magic, ASTRO_STATE_MAGIC, 8) != 0 ||
        h.version != ASTRO_STATE_VERSION || h.header_bytes != sizeof(h) || h.n == 0 ||
        h.nsys == 0 || h.n_tree > h.n || (h.contents & ~(ASTRO_STATE_TYPES | ASTRO_STATE_POS64)))
        return ASTRO_ERR_INVALID_ARGUMENT;
    const char* why = nullptr;
    if (validate_params(&h.params, &why) != ASTRO_OK) return ASTRO_ERR_INVALID_ARGUMENT;
    const bool phys = h.params.preset == ASTRO_PRESET_PHYSICAL;
    const bool prec = phys && h.params.form == ASTRO_FORM_PRECISION;
    if (((h.contents & ASTRO_STATE_TYPES) != 0) == phys ||
        ((h.contents & ASTRO_STATE_POS64) != 0) != prec || (!phys && h.nsys != 1))
        return ASTRO_ERR_INVALID_ARGUMENT;
    const uint32_t n = h.n;
    std::vector<uint32_t> sizes(h.nsys), ids(n), types(phys ? 0 : n);
    std::vector<PositionMass> pm(n);
    std::vector<VelocityRadius> vr(n);
    std::vector<double> xyz(prec ? 3ull * n : 0);
    if (!f.get(sizes.data(), 4ull * h.nsys) || !f.get(pm.data(), sizeof(PositionMass) * n) ||
        !f.get(vr.data(), sizeof(VelocityRadius) * n) || !f.get(ids.data(), 4ull * n) ||
        !f.get(types.data(), 4ull * types.size()) || !f.get(xyz.data(), 8ull * xyz.size()))
        return ASTRO_ERR_INVALID_ARGUMENT;
    uint64_t total = 0;
    for (uint32_t s : sizes) total += s;
    if (phys ? total != n : sizes[0] != h.n_tree) return ASTRO_ERR_INVALID_ARGUMENT;
    // ids must be a permutation of 0..n-1.
    {
        std::vector<uint8_t> seen(n, 0);
        for (uint32_t i : ids) {
            if (i >= n || seen[i]) return ASTRO_ERR_INVALID_ARGUMENT;
            seen[i] = 1;
        }
    }
    astro_ctx* ctx = nullptr;
    int r = astro_create(&h.params, std::max(max_n, n), h.nsys, &ctx);
    if (r != ASTRO_OK) return r;
    if (!phys) {
        std::vector<ColorType> ct(n);
        std::memset(ct.data(), 0, sizeof(ColorType) * n);
        for (uint32_t i = 0; i < n; ++i) ct[i].type = types[i];
        r = astro_upload(ctx, pm.data(), vr.data(), ct.data(), n, h.n_tree);
    } else if (h.nsys == 1) {
        r = astro_upload(ctx, pm.data(), vr.data(), nullptr, n, n);
    } else {
        r = astro_upload_systems(ctx, pm.data(), vr.data(), sizes.data(), h.nsys);
    }
    if (r == ASTRO_OK && phys) {
        // The saved slot order and upload indices; the FP64 master positions.
        cudaStream_t st = ctx->stream;
        cudaError_t e = cudaMemcpyAsync(ctx->ids[0], ids.data(), 4ull * n, cudaMemcpyHostToDevice, st);
        std::vector<double> soa(prec ? 3ull * n : 0);
        for (uint32_t i = 0; i < n && prec; ++i)
            for (int a = 0; a < 3; ++a) soa[(size_t)a * n + i] = xyz[3ull * i + a];
        if (e == cudaSuccess && prec)
            e = cudaMemcpyAsync(ctx->x64[0], soa.data(), 24ull * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) r = fail(ctx, ASTRO_ERR_CUDA, cudaGetErrorString(e));
    }
    if (r == ASTRO_OK) r = check_device(ctx);
    if (r != ASTRO_OK) {
        astro_destroy(ctx);
        return r;
    }
    if (step) *step = h.step;
    if (time) *time = h.time;
    *out = ctx;
    return ASTRO_OK;
}

int astro_read_walk_buffers(astro_ctx* ctx, uint64_t* list_blocks, uint32_t* frontier_cap,
                            uint64_t* reruns) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    int r = check_device(ctx);
    if (r != ASTRO_OK) return r;
    if (list_blocks) *list_blocks = ctx->lists_blocks;
    if (frontier_cap) *frontier_cap = ctx->frontier_cap;
    if (reruns) *reruns = ctx->walk_reruns;
    return ASTRO_OK;
}

int astro_test_walk_capacity(astro_ctx* ctx, uint64_t set_blocks, uint32_t set_frontier_cap) {
    if (!ctx || (set_frontier_cap != 0 && (set_frontier_cap < 2 || set_frontier_cap % 2 != 0)) ||
        set_blocks > 0xFFFFFF00ull)
        return ASTRO_ERR_INVALID_ARGUMENT;
    if (!is_phys(ctx)) return fail(ctx, ASTRO_ERR_STATE, "the group walk is PHYSICAL only");
    int r = check_device(ctx);
    if (r != ASTRO_OK) return r;
    drop_graph(ctx);
    ctx->walk_estimate_off = true;
    if (set_blocks) {
        dev_free(ctx->lists);
        dev_free(ctx->list_next);
        ctx->lists_blocks = 0;
        ctx->lists_blocks_want = set_blocks;
    }
    if (set_frontier_cap) {
        dev_free(ctx->frontier);
        ctx->frontier_words = 0;
        ctx->frontier_cap = set_frontier_cap;
    }
    if ((r = ensure_frontier(ctx)) != ASTRO_OK) return r;
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

}  // extern "C"
