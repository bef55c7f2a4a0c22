// Group walk of the PHYSICAL preset: barnesHut (Astro/BarnesHut.metal:22-101)
// with the opening decisions made once per group of consecutive
// Morton-sorted particles, in two kernels (three for groups of more than
// 32 with far nodes).
//
// group_walk_kernel — one warp per group of at most 64 particles (a tree
//   cell or a pack of sibling cells, emitted with the tree); the chunks a
//   leaf larger than a group is cut into share one walk against the whole
//   leaf's box (its particles are in no spatial order inside the leaf, so
//   each chunk's box is nearly the leaf's anyway). The warp walks
//   the tree breadth first from the system's root, testing 32 frontier nodes
//   at a time against the walk's bounding box: an accepted node goes to the
//   cell list, or to the far list when its centre of mass lies further than
//   r_g / far_ratio from the box centre (r_g the box's half diagonal); an
//   opened leaf or bucket goes to the leaf list; any other opened node puts
//   its children in the next frontier. Each list is a chain of 64-word
//   blocks of a shared pool (the warp takes blocks from the pool in batches);
//   a per-walk record holds the chains and the box centre.
// group_far_kernel — the far nodes' second-order field expansion about the
//   walk's box centre, once per walk (groups of more than 32): lane l
//   expands far nodes l, l + 32, ... into its partial of the 19
//   coefficients, the partials are combined by an xor butterfly (16 .. 1)
//   and the sums go into the walk's record. Groups of up to 32 form the
//   same sums in their own evaluation.
// group_eval_kernel — one warp per group: each lane holds one particle (two
//   for groups of 33..64; copies of each particle for groups of at most 16
//   in the fast form). Each particle evaluates the far-node expansion at
//   its offset from the box centre. Cells are
//   gathered into shared memory and summed; the listed leaves' particles are
//   staged 32 at a time and summed. The epilogue clamps, stores the
//   acceleration and performs the kick-drift (v += a dt, x += v dt).
//
// The walk needs few registers and many resident warps (it waits on node
// loads); the evaluation needs registers for its sums. Split, each runs at
// its own occupancy. The fast form evaluates two sources per instruction in
// packed FP32 pairs from arrays staged in shared memory; the exact form
// rounds every operation as the CPU restatement does, in its order.
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "build_kernels.cuh"
#include "common.cuh"
#include "traverse_terms.cuh"

namespace astro {
namespace {

// Walk kernel: warps per block and the resident warps per SM it is sized for.
constexpr int kWalkWarps = 4;
constexpr int kWalkWarpsPerSm = 32;
constexpr uint32_t kNoBlock = 0xFFFFFFFFu;

// Resident warps per SM the evaluation's register allocation is sized for:
// 24 (80 registers, a few spilled), except the plain form's 8-warp blocks
// at 16 (up to 128 registers, none spilled). Measured: the plain C3 and C1
// lines (8-warp blocks) 4.86 -> 4.79 ms and 0.251 -> 0.241 ms at 16; the
// precision form's 8-warp blocks lost at 16 (C5 18.9 -> 19.3 ms, C2 1.40
// -> 1.48 ms); 4-warp blocks at C5 and C4 ran best at 24 (17.32 and 7.33
// ms, against 17.46 and 7.47 at 20 and 17.38 and 7.54 at 28).
#ifndef ASTRO_GROUP_WARPS_PER_SM
#define ASTRO_GROUP_WARPS_PER_SM 24
#endif
#ifndef ASTRO_GROUP_WARPS_PER_SM_8
#define ASTRO_GROUP_WARPS_PER_SM_8 16
#endif

// Cell records staged per warp (the evaluation's shared memory): two list
// blocks of node ids at a time with 4-warp blocks, one with 8 (static
// shared memory stays under 48 KB).
constexpr int cell_cap(int warps) {
    return warps >= 8 ? (int)kListBlockWords : 2 * (int)kListBlockWords;
}

// A staged accepted cell of the exact form: centre of mass and mass, and
// with quadrupoles {Qxx, Qyy, Qxy, Qxz} and {Qyz, Qzz}.
template <bool kQuad>
struct CellSlot {
    float4 cm;
    float4 q;
    float4 q2;
};
template <>
struct CellSlot<false> {
    float4 cm;
};

// Queue ticket -> group index. For a batch the groups are visited in whole
// chunks of consecutive groups in a scrambled chunk order (a bijection:
// 1000003 is prime and larger than the chunk count); the last partial chunk
// keeps its place.
__device__ __forceinline__ uint32_t group_of_ticket(uint32_t gi, uint32_t ngroups, uint32_t chunk) {
    if (chunk > 0) {
        const uint32_t nfull = ngroups / chunk;
        if (gi < nfull * chunk)
            gi = (uint32_t)(((uint64_t)(gi / chunk) * 1000003ull) % nfull) * chunk + gi % chunk;
    }
    return gi;
}

// The tail of one list of the group being walked: its first and current
// blocks, the items in the current block and in the list.
struct ListTail {
    uint32_t first, blk, fill, count;
};

// Blocks of the pool a walk warp holds for its lists: [next, end), taken
// from the pool kBlockBatch at a time (one atomic per batch).
constexpr uint32_t kBlockBatch = 16;
struct BlockCache {
    uint32_t next, end;
};

// Appends the items of the lanes in `mask` (in lane order) to list L, whose
// items are kWords words each (this lane's words w0, w1). A full block is
// chained to a new one. Blocks numbered past the pool's end are not
// written: the walk goes on counting them (the pool counter ends at the
// demand), `failed` marks the group and the error bit makes the evaluation
// skip, so the host can grow the pool and run the traversal again.
// `mask` is warp-uniform.
template <uint32_t kWords>
__device__ __forceinline__ void list_append(const TraverseArgs& a, ListTail& L, BlockCache& bc,
                                            uint32_t mask, uint32_t lane, uint32_t lt, uint32_t w0,
                                            uint32_t w1, bool& failed) {
    constexpr uint32_t kCap = kListBlockWords / kWords;
    const uint32_t cnt = __popc(mask);
    const uint32_t rank = __popc(mask & lt);
    auto alloc = [&]() {
        if (bc.next == bc.end) {
            uint32_t b = 0;
            if (lane == 0) b = atomicAdd(a.lists_used, kBlockBatch);
            b = __shfl_sync(kFullMask, b, 0);
            bc.next = b;
            bc.end = b + kBlockBatch;
        }
        const uint32_t blk = bc.next++;
        if (blk >= a.lists_blocks && !failed) {
            if (lane == 0) atomicOr(a.err, kErrFrontier);
            failed = true;
        }
        return blk;
    };
    if (L.blk == kNoBlock) {
        L.blk = L.first = alloc();
        L.fill = 0;
    }
    uint32_t b = L.blk, slot = L.fill + rank;
    const uint32_t room = kCap - L.fill;
    if (cnt > room) {
        const uint32_t nb = alloc();
        if (lane == 0 && L.blk < a.lists_blocks && nb < a.lists_blocks) a.list_next[L.blk] = nb;
        if (rank >= room) {
            b = nb;
            slot = rank - room;
        }
        L.blk = nb;
        L.fill = cnt - room;
    } else {
        L.fill += cnt;
    }
    L.count += cnt;
    if (((mask >> lane) & 1u) && b < a.lists_blocks) {
        uint32_t* dst = a.lists + (size_t)b * kListBlockWords + slot * kWords;
        if constexpr (kWords == 2) *reinterpret_cast<uint2*>(dst) = make_uint2(w0, w1);
        else *dst = w0;
    }
}

// Reads a list chain block by block.
struct ChainCursor {
    uint32_t blk;
    __device__ __forceinline__ const uint32_t* words(const TraverseArgs& a) const {
        return a.lists + (size_t)blk * kListBlockWords;
    }
    __device__ __forceinline__ void advance(const TraverseArgs& a) { blk = __ldg(&a.list_next[blk]); }
};

}  // namespace

// ------------------------------------------------------------------ walk --

__global__ __launch_bounds__(kWalkWarps * 32, kWalkWarpsPerSm / kWalkWarps) void group_walk_kernel(
    TraverseArgs a) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t gw = blockIdx.x * kWalkWarps + warp;
    uint32_t* const buf0 = a.frontier + (size_t)gw * 2 * a.frontier_cap;
    uint32_t* const buf1 = buf0 + a.frontier_cap;
    const uint32_t ngroups = *a.group_count;
    const bool far_on = a.far2 > 0.f;
    unsigned long long visits = 0, far_nodes = 0;
    BlockCache bcache{0u, 0u};

    while (true) {
        uint32_t gi = 0;
        if (lane == 0) gi = atomicAdd(a.queue, 1u);
        gi = __shfl_sync(kFullMask, gi, 0);
        if (gi >= ngroups) break;
        gi = group_of_ticket(gi, ngroups, a.group_chunk);
        const uint4 gr = a.groups[gi];
        // Later chunks of a leaf use the walk of its first chunk.
        if (gr.w != 0u) continue;
        // The walk's box: the group, or the whole leaf a first chunk stands
        // for (any number of particles, 64 at a time).
        const uint32_t wcount = gr.z - gr.x;
        float lo_x = INFINITY, lo_y = INFINITY, lo_z = INFINITY;
        float hi_x = -INFINITY, hi_y = -INFINITY, hi_z = -INFINITY;
        for (uint32_t b = 0; b < wcount; b += 64u) {
            const bool v0 = b + lane < wcount, v1 = b + 32u + lane < wcount;
            if (v0) {
                const float4 p0 = a.pos[gr.x + b + lane];
                lo_x = fminf(lo_x, p0.x), lo_y = fminf(lo_y, p0.y), lo_z = fminf(lo_z, p0.z);
                hi_x = fmaxf(hi_x, p0.x), hi_y = fmaxf(hi_y, p0.y), hi_z = fmaxf(hi_z, p0.z);
            }
            if (v1) {
                const float4 p1 = a.pos[gr.x + b + 32u + lane];
                lo_x = fminf(lo_x, p1.x), lo_y = fminf(lo_y, p1.y), lo_z = fminf(lo_z, p1.z);
                hi_x = fmaxf(hi_x, p1.x), hi_y = fmaxf(hi_y, p1.y), hi_z = fmaxf(hi_z, p1.z);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo_x = fminf(lo_x, __shfl_xor_sync(kFullMask, lo_x, o));
            lo_y = fminf(lo_y, __shfl_xor_sync(kFullMask, lo_y, o));
            lo_z = fminf(lo_z, __shfl_xor_sync(kFullMask, lo_z, o));
            hi_x = fmaxf(hi_x, __shfl_xor_sync(kFullMask, hi_x, o));
            hi_y = fmaxf(hi_y, __shfl_xor_sync(kFullMask, hi_y, o));
            hi_z = fmaxf(hi_z, __shfl_xor_sync(kFullMask, hi_z, o));
        }
        const float gcx = __fmul_rn(__fadd_rn(lo_x, hi_x), 0.5f);
        const float gcy = __fmul_rn(__fadd_rn(lo_y, hi_y), 0.5f);
        const float gcz = __fmul_rn(__fadd_rn(lo_z, hi_z), 0.5f);
        const float hrx = __fmul_rn(__fsub_rn(hi_x, lo_x), 0.5f);
        const float hry = __fmul_rn(__fsub_rn(hi_y, lo_y), 0.5f);
        const float hrz = __fmul_rn(__fsub_rn(hi_z, lo_z), 0.5f);
        const float rg2 =
            __fadd_rn(__fmul_rn(hrx, hrx), __fadd_rn(__fmul_rn(hry, hry), __fmul_rn(hrz, hrz)));
        const uint32_t sys = a.nsys > 1 ? (uint32_t)(a.sorted_keys[gr.x] >> (3u * a.lbits)) : 0u;
        const float* crit_layer = a.sys[sys].crit2;
        ListTail cells{kNoBlock, kNoBlock, 0u, 0u}, leaves = cells, fars = cells;
        bool failed = false;
        uint32_t tested = 0;

        // One frontier chunk: node nd (when `has`) at `layer`. Appends the
        // accepted, far and opened-leaf nodes to the lists in frontier order
        // and returns the opened node's child range (empty otherwise).
        auto test_nodes = [&](bool has, uint32_t nd, int layer) -> uint2 {
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            uint4 r = make_uint4(0u, 0u, 0u, 0u);
            float crit = 0.f;
            if (has) {
                c = __ldg(&a.node_cm[nd]);
                r = __ldg(&a.node_rng[nd]);
                crit = a.delta ? __ldg(&a.node_crit2[nd]) : __ldg(&crit_layer[layer]);
            }
            const float bx = fmaxf(fmaxf(__fsub_rn(lo_x, c.x), __fsub_rn(c.x, hi_x)), 0.f);
            const float by = fmaxf(fmaxf(__fsub_rn(lo_y, c.y), __fsub_rn(c.y, hi_y)), 0.f);
            const float bz = fmaxf(fmaxf(__fsub_rn(lo_z, c.z), __fsub_rn(c.z, hi_z)), 0.f);
            const float dist2 =
                __fadd_rn(__fadd_rn(__fmul_rn(bx, bx), __fmul_rn(by, by)), __fmul_rn(bz, bz));
            const bool accepted = has && dist2 > crit;
            const bool leaf = has && !accepted && (layer == 0 || r.w - r.z <= a.bucket);
            const bool opn = has && !accepted && !leaf;
            bool far = false;
            if (far_on && accepted) {
                const float Dx = __fsub_rn(c.x, gcx), Dy = __fsub_rn(c.y, gcy), Dz = __fsub_rn(c.z, gcz);
                const float D2 =
                    __fadd_rn(__fmul_rn(Dx, Dx), __fadd_rn(__fmul_rn(Dy, Dy), __fmul_rn(Dz, Dz)));
                far = __fmul_rn(a.far2, D2) > rg2;
            }
            const bool acc = accepted && !far;
            tested += __popc(__ballot_sync(kFullMask, has));
            const uint32_t bfar = __ballot_sync(kFullMask, far);
            if (bfar) list_append<1>(a, fars, bcache, bfar, lane, lt, nd, 0u, failed);
            const uint32_t bacc = __ballot_sync(kFullMask, acc);
            if (bacc) list_append<1>(a, cells, bcache, bacc, lane, lt, nd, 0u, failed);
            const uint32_t bleaf = __ballot_sync(kFullMask, leaf);
            if (bleaf) list_append<2>(a, leaves, bcache, bleaf, lane, lt, r.z, r.w, failed);
            return opn ? make_uint2(r.x, r.y) : make_uint2(0u, 0u);
        };

        if (a.walk_runs) {
            // The frontier holds runs of consecutive node indices (first,
            // count) in walk order: an opened node's children are consecutive,
            // so it adds one run, and a chunk of 32 nodes is found by a shuffle
            // search over 32 runs loaded at once.
            uint2* cur = reinterpret_cast<uint2*>(buf0);
            uint2* nxt = reinterpret_cast<uint2*>(buf1);
            const uint32_t run_cap = a.frontier_cap / 2u;
            if (lane == 0) cur[0] = make_uint2(a.sys[sys].root, 1u);
            uint32_t ncur = 1;
            int layer = (int)a.lbits;
            __syncwarp();
            while (ncur > 0) {
                uint32_t nnext = 0;
                for (uint32_t rb = 0; rb < ncur; rb += 32u) {
                    const uint32_t nrun = min(32u, ncur - rb);
                    const uint2 run = lane < nrun ? cur[rb + lane] : make_uint2(0u, 0u);
                    uint32_t rincl = run.y;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(kFullMask, rincl, o);
                        if (lane >= (uint32_t)o) rincl += y;
                    }
                    const uint32_t rpre = rincl - run.y;
                    const uint32_t rtotal = __shfl_sync(kFullMask, rincl, 31);
                    for (uint32_t t0 = 0; t0 < rtotal; t0 += 32u) {
                        const uint32_t pos = t0 + lane;
                        uint32_t e = 0;
#pragma unroll
                        for (uint32_t step = 16; step > 0; step >>= 1) {
                            const uint32_t cand = e + step;
                            const uint32_t pc = __shfl_sync(kFullMask, rpre, cand & 31u);
                            if (cand < nrun && pc <= pos) e = cand;
                        }
                        const uint32_t first = __shfl_sync(kFullMask, run.x, e);
                        const uint32_t estart = __shfl_sync(kFullMask, rpre, e);
                        const bool has = pos < rtotal;
                        const uint2 ch = test_nodes(has, has ? first + (pos - estart) : 0u, layer);
                        const bool opn = ch.y > ch.x;
                        const uint32_t bopen = __ballot_sync(kFullMask, opn);
                        if (bopen) {
                            if (nnext + __popc(bopen) <= run_cap) {
                                if (opn) nxt[nnext + __popc(bopen & lt)] = make_uint2(ch.x, ch.y - ch.x);
                                nnext += __popc(bopen);
                            } else if (lane == 0) {
                                atomicOr(a.err, kErrFrontier);
                                atomicMax(a.frontier_need, 2u * (nnext + __popc(bopen)));
                            }
                        }
                    }
                }
                __syncwarp();
                uint2* t = cur;
                cur = nxt;
                nxt = t;
                ncur = nnext;
                --layer;
            }
        } else {
            // The frontier holds node indices, each opened node adding its
            // children one by one.
            uint32_t* cur = buf0;
            uint32_t* nxt = buf1;
            if (lane == 0) cur[0] = a.sys[sys].root;
            uint32_t ncur = 1;
            int layer = (int)a.lbits;
            __syncwarp();
            while (ncur > 0) {
                uint32_t nnext = 0;
                for (uint32_t base = 0; base < ncur; base += 32u) {
                    const uint32_t k = base + lane;
                    const bool has = k < ncur;
                    const uint2 ch = test_nodes(has, has ? cur[k] : 0u, layer);
                    const uint32_t cnt = ch.y - ch.x;
                    uint32_t incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
                        if (lane >= (uint32_t)o) incl += y;
                    }
                    const uint32_t total = __shfl_sync(kFullMask, incl, 31);
                    if (nnext + total <= a.frontier_cap) {
                        const uint32_t o0 = nnext + incl - cnt;
                        for (uint32_t j = 0; j < cnt; ++j) nxt[o0 + j] = ch.x + j;
                        nnext += total;
                    } else if (lane == 0) {
                        atomicOr(a.err, kErrFrontier);
                        atomicMax(a.frontier_need, nnext + total);
                    }
                }
                __syncwarp();
                uint32_t* t = cur;
                cur = nxt;
                nxt = t;
                ncur = nnext;
                --layer;
            }
        }

        // The group's descriptor (empty lists if the pool ran out).
        if (failed) leaves.count = cells.count = fars.count = 0;
        if (lane < 12) {
            const uint32_t w[12] = {leaves.first, leaves.count, cells.first, cells.count,
                                    fars.first, fars.count, __float_as_uint(gcx), __float_as_uint(gcy),
                                    __float_as_uint(gcz), 0u, 0u, 0u};
            uint32_t v = w[0];
#pragma unroll
            for (int k = 1; k < 12; ++k)
                if (lane == (uint32_t)k) v = w[k];
            reinterpret_cast<uint32_t*>(a.desc + gi)[lane] = v;
        }
        // Per particle of the walk; one expansion per walk and far node.
        visits += (unsigned long long)wcount * tested;
        far_nodes += fars.count;
    }
    if (lane == 0) {
        atomicAdd(&a.stats[1], visits);
        if (far_nodes) atomicAdd(&a.stats[3], far_nodes);
    }
}

// ------------------------------------------------------------ far nodes --

// The far-node expansion of every walk, once: lane l sums the coefficients
// of far nodes l, l + 32, ... in walk order; the partials are combined
// pairwise (lane l + lane l^o, o = 16 .. 1), leaving the sum in every lane;
// the 19 sums go into the walk's record, where the evaluation of each group
// sharing the walk reads them. One warp per record, records in order.
template <bool kExact, bool kQuad>
__global__ __launch_bounds__(128) void group_far_kernel(TraverseArgs a) {
    const uint32_t lane = threadIdx.x & 31;
    // A walk that ran out of room left incomplete lists: nothing to expand.
    if (*reinterpret_cast<volatile const uint32_t*>(a.err) & kErrFrontier) return;
    const uint32_t ngroups = *a.group_count;
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32u);
    const float eps2 = a.eps2;
    for (uint32_t gi = blockIdx.x * (blockDim.x / 32u) + (threadIdx.x >> 5); gi < ngroups;
         gi += nwarps) {
        if (a.groups[gi].w != 0u) continue;  // a later chunk: no walk of its own
        GroupDesc* const dp = a.desc + gi;
        const uint32_t n_far = dp->n_far;
        if (n_far == 0u) continue;
        const float gcx = dp->gcx, gcy = dp->gcy, gcz = dp->gcz;
        float fc[kFarCoefs];
#pragma unroll
        for (int k = 0; k < kFarCoefs; ++k) fc[k] = 0.f;
        // Far node f sits at position f mod 64 of block f / 64 of the chain.
        // Each lane reads its next node id (f + 32) before it expands node
        // f, so only the node record's load waits at the top of an
        // iteration; the expansions stay in walk order.
        ChainCursor cur{dp->far_first};
        uint32_t nd = lane < n_far ? cur.words(a)[lane] : 0u;
        for (uint32_t f = lane; f < n_far; f += 32u) {
            const float4 c = __ldg(&a.node_cm[nd]);
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            float qyz = 0.f;
            if constexpr (kQuad) {
                q = __ldg(&a.node_q[nd]);
                qyz = __ldg(&a.node_qyz[nd]);
            }
            const uint32_t fn = f + 32u;
            if (fn < n_far) {
                if ((fn % kListBlockWords) < 32u) cur.advance(a);
                nd = cur.words(a)[fn % kListBlockWords];
            }
            if constexpr (kQuad)
                far_coefs<kExact, true>(c, q, qyz, -(q.x + q.y), gcx, gcy, gcz, eps2, fc);
            else
                far_coefs<kExact, false>(c, q, 0.f, 0.f, gcx, gcy, gcz, eps2, fc);
        }
#pragma unroll
        for (int k = 0; k < kFarCoefs; ++k) {
            float v = fc[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v = xadd<kExact>(v, __shfl_xor_sync(kFullMask, v, o));
            fc[k] = v;
        }
        float v = fc[0];
#pragma unroll
        for (int k = 1; k < kFarCoefs; ++k)
            if (lane == (uint32_t)k) v = fc[k];
        if (lane < (uint32_t)kFarCoefs) dp->far_co[lane] = v;
    }
}

// ------------------------------------------------------------ evaluation --

namespace {

// Evaluation of one group whose particles sit kPer per lane (kPer = 2:
// particles lane and lane + 32). Adds this lane's interaction counts.
template <bool kExact, bool kPrec, bool kQuad, int kCellCap, int kPer, bool kPipe, bool kFarPre>
__device__ __forceinline__ void eval_group(const TraverseArgs& a, const uint2 gr, const GroupDesc& d,
                                           const float* __restrict__ far_co,
                                           CellSlot<kQuad>* s_cell, float4* s_tile, uint32_t* s_jdx,
                                           uint32_t lane, uint32_t& inter, uint32_t& cell_inter,
                                           uint32_t& far_inter) {
    constexpr int kCellArrays = kQuad ? 10 : 4;
    static_assert(kCellArrays * 4 <= (int)sizeof(CellSlot<kQuad>) && kCellCap % 4 == 0,
                  "cell arrays fit the cell records");
    const uint32_t gcount = gr.y - gr.x;
    const float g = a.g, eps2 = a.eps2;
    // Fast form with eps^2 a normal float: every r^2 is normal (rsqrt_ftz
    // applies) and a particle's own term is exactly zero (no self test).
    const bool normal_r2 = !kExact && eps2 >= kFltMin;
    constexpr std::true_type kTrue{};
    constexpr std::false_type kFalse{};
    // A group of at most 16 particles runs (fast form, one per lane) as
    // reps = 32 / gcount copies (lane = rep * gcount + particle), each copy
    // summing every reps-th listed source; the copies' partial sums are
    // added at the end. The exact form keeps one copy, for the CPU
    // restatement's order.
    const uint32_t reps = (kExact || kPer == 2) ? 1u : max(1u, 32u / gcount);
    const uint32_t rep = kPer == 2 ? 0u : lane / gcount;
    uint32_t ip[kPer];
    bool valid[kPer];
    float4 me[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const uint32_t slot = kPer == 2 ? lane + 32u * k : lane - rep * gcount;
        valid[k] = kPer == 2 ? slot < gcount : rep < reps;
        ip[k] = gr.x + slot;
        me[k] = valid[k] ? a.pos[ip[k]] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // The copy that writes each particle (counts and epilogue).
    bool owner[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) owner[k] = valid[k] && rep == 0;
    uint32_t owned = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) owned += owner[k] ? 1u : 0u;
    const float gcx = d.gcx, gcy = d.gcy, gcz = d.gcz;

    // Far nodes: lane l sums the coefficients of far nodes l, l + 32, ...
    // in walk order; the partials are combined pairwise (lane l + lane l^o,
    // o = 16 .. 1), leaving the sum in every lane; each particle adds the
    // expansion at its offset.
    float fx[kPer], fy[kPer], fz[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) fx[k] = fy[k] = fz[k] = 0.f;
    if (d.n_far > 0) {
        float fc[kFarCoefs];
        if constexpr (kFarPre) {
            // The walk's summed coefficients (group_far_kernel), the same for
            // every chunk that shares the walk.
            float buf[kFarCoefs + 1];
#pragma unroll
            for (int k = 0; k < (kFarCoefs + 1) / 4; ++k) {
                const float4 v = __ldg(reinterpret_cast<const float4*>(far_co) + k);
                buf[4 * k] = v.x, buf[4 * k + 1] = v.y, buf[4 * k + 2] = v.z, buf[4 * k + 3] = v.w;
            }
#pragma unroll
            for (int k = 0; k < kFarCoefs; ++k) fc[k] = buf[k];
        } else {
#pragma unroll
            for (int k = 0; k < kFarCoefs; ++k) fc[k] = 0.f;
            // Far node f sits at position f mod 64 of block f / 64 of the
            // chain; each lane reads its next node id before expanding node f.
            ChainCursor cur{d.far_first};
            uint32_t nd = lane < d.n_far ? cur.words(a)[lane] : 0u;
            for (uint32_t f = lane; f < d.n_far; f += 32u) {
                const float4 c = __ldg(&a.node_cm[nd]);
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                float qyz = 0.f;
                if constexpr (kQuad) {
                    q = __ldg(&a.node_q[nd]);
                    qyz = __ldg(&a.node_qyz[nd]);
                }
                const uint32_t fn = f + 32u;
                if (fn < d.n_far) {
                    if ((fn % kListBlockWords) < 32u) cur.advance(a);
                    nd = cur.words(a)[fn % kListBlockWords];
                }
                if constexpr (kQuad)
                    far_coefs<kExact, true>(c, q, qyz, -(q.x + q.y), gcx, gcy, gcz, eps2, fc);
                else
                    far_coefs<kExact, false>(c, q, 0.f, 0.f, gcx, gcy, gcz, eps2, fc);
            }
#pragma unroll
            for (int k = 0; k < kFarCoefs; ++k) {
                float v = fc[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v = xadd<kExact>(v, __shfl_xor_sync(kFullMask, v, o));
                fc[k] = v;
            }
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k)
            far_eval<kExact>(fc, xadd<kExact>(me[k].x, -gcx), xadd<kExact>(me[k].y, -gcy),
                             xadd<kExact>(me[k].z, -gcz), fx[k], fy[k], fz[k]);
        inter += owned * d.n_far;
        cell_inter += owned * d.n_far;
        far_inter += owned * d.n_far;
    }

    Accum<kExact, kPrec> cells[kPer], leaves[kPer];
    float* const cell_soa = reinterpret_cast<float*>(s_cell);

    // Cells, kCellCap at a time: gathered into shared memory (the fast form
    // as arrays x, y, z, m and, with quadrupoles, -Qxx, -Qyy, -Qxy, -Qxz,
    // -Qyz, -Qzz, padded with massless cells to a multiple of 4), then summed
    // by every lane against each of its particles. The fast form leaves G
    // out of the terms and applies it once at the end.
    ChainCursor ccur{d.cell_first};
    // Node id j of a chunk of one or two list blocks.
    auto cell_id = [&](uint32_t j, const uint32_t* b0, const uint32_t* b1) {
        return j < kListBlockWords ? b0[j] : b1[j - kListBlockWords];
    };
    for (uint32_t c0 = 0; c0 < d.n_cell; c0 += (uint32_t)kCellCap) {
        const uint32_t m = min((uint32_t)kCellCap, d.n_cell - c0);
        if (c0 > 0) ccur.advance(a);
        const uint32_t* b0 = ccur.words(a);
        const uint32_t* b1 = b0;
        if (kCellCap > (int)kListBlockWords && m > kListBlockWords) {
            ccur.advance(a);
            b1 = ccur.words(a);
        }
        __syncwarp();
        if constexpr (kExact) {
#pragma unroll 4
            for (uint32_t j = lane; j < m; j += 32u) {
                const uint32_t nd = cell_id(j, b0, b1);
                s_cell[j].cm = __ldg(&a.node_cm[nd]);
                if constexpr (kQuad) {
                    const float4 q = __ldg(&a.node_q[nd]);
                    s_cell[j].q = q;
                    s_cell[j].q2 = make_float4(__ldg(&a.node_qyz[nd]), -(q.x + q.y), 0.f, 0.f);
                }
            }
        } else {
            const uint32_t m4 = (m + 3u) & ~3u;
#pragma unroll 4
            for (uint32_t j = lane; j < m4; j += 32u) {
                float v[kCellArrays];
#pragma unroll
                for (int k = 0; k < kCellArrays; ++k) v[k] = 0.f;
                if (j < m) {
                    const uint32_t nd = cell_id(j, b0, b1);
                    const float4 c = __ldg(&a.node_cm[nd]);
                    v[0] = c.x;
                    v[1] = c.y;
                    v[2] = c.z;
                    v[3] = c.w;
                    if constexpr (kQuad) {
                        const float4 q = __ldg(&a.node_q[nd]);
                        const float qyz = __ldg(&a.node_qyz[nd]);
                        v[4] = -q.x;
                        v[5] = -q.y;
                        v[6] = -q.z;
                        v[7] = -q.w;
                        v[8] = -qyz;
                        v[9] = q.x + q.y;
                    }
                }
#pragma unroll
                for (int k = 0; k < kCellArrays; ++k) cell_soa[k * kCellCap + j] = v[k];
            }
        }
        __syncwarp();
        if constexpr (kExact) {
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                if (!valid[k]) continue;
                for (uint32_t e = 0; e < m; ++e) {
                    const CellSlot<kQuad>& cs = s_cell[e];
                    const float4 c = cs.cm;
                    const float dx = __fsub_rn(c.x, me[k].x), dy = __fsub_rn(c.y, me[k].y),
                                dz = __fsub_rn(c.z, me[k].z);
                    const float r2t =
                        __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    float tx, ty, tz;
                    if constexpr (kQuad)
                        cell_term<true>(dx, dy, dz, r2t, c.w, true, cs.q, cs.q2.x, g, eps2, tx, ty, tz);
                    else
                        cell_term<true>(dx, dy, dz, r2t, c.w, false, make_float4(0.f, 0.f, 0.f, 0.f),
                                        0.f, g, eps2, tx, ty, tz);
                    cells[k].push(tx, ty, tz);
                    cells[k].step();
                }
            }
        } else if (normal_r2 && reps == 1) {
            // Two cells per instruction (packed FP32 pairs): even and odd
            // cells summed apart and joined at the end; the precision form
            // Kahan-adds the chunk's partial once.
            const float2* v = reinterpret_cast<const float2*>(cell_soa);
            constexpr int kV = kCellCap / 2;  // float2s per array
            float2 nmx[kPer], nmy[kPer], nmz[kPer], sx[kPer], sy[kPer], sz[kPer];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                nmx[k] = make_float2(-me[k].x, -me[k].x);
                nmy[k] = make_float2(-me[k].y, -me[k].y);
                nmz[k] = make_float2(-me[k].z, -me[k].z);
                sx[k] = sy[k] = sz[k] = make_float2(0.f, 0.f);
            }
            const float2 e2 = make_float2(eps2, eps2);
            const uint32_t n2 = ((m + 3u) & ~3u) >> 1;
#pragma unroll 2
            for (uint32_t j = 0; j < n2; ++j) {
                const float2 X = v[j], Y = v[kV + j], Z = v[2 * kV + j], M = v[3 * kV + j];
                if constexpr (kQuad) {
                    const float2 A = v[4 * kV + j], B = v[5 * kV + j], C = v[6 * kV + j],
                                 D = v[7 * kV + j], E = v[8 * kV + j], F = v[9 * kV + j];
#pragma unroll
                    for (int k = 0; k < kPer; ++k)
                        cell_pair_quad(X, Y, Z, M, A, B, C, D, E, F, nmx[k], nmy[k], nmz[k], e2, sx[k],
                                       sy[k], sz[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < kPer; ++k)
                        mono_pair(X, Y, Z, M, nmx[k], nmy[k], nmz[k], e2, sx[k], sy[k], sz[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const float px = sx[k].x + sx[k].y, py = sy[k].x + sy[k].y, pz = sz[k].x + sz[k].y;
                if (kPrec) {
                    cells[k].add(px, py, pz);
                } else {
                    cells[k].ax += px;
                    cells[k].ay += py;
                    cells[k].az += pz;
                }
            }
        } else {
            // Copies of small groups, or eps^2 below FLT_MIN: one cell at a
            // time, every reps-th one.
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                if (!valid[k]) continue;
                float px = 0.f, py = 0.f, pz = 0.f;
                auto cell = [&](uint32_t e, auto ftz) {
                    const float* cs = cell_soa + e;
                    const float dx = cs[0] - me[k].x, dy = cs[kCellCap] - me[k].y,
                                dz = cs[2 * kCellCap] - me[k].z, mm = cs[3 * kCellCap];
                    const float inv =
                        rsq<decltype(ftz)::value>(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
                    const float u = inv * inv, inv3 = u * inv;
                    if constexpr (kQuad) {
                        // inv^3 (M + 5/2 u^2 d.Qd) d - inv^5 Qd, u = 1/r^2,
                        // with the staged quadrupole negated: qx.. = -(Qd) and
                        // dqd = -d.Qd.
                        const float nxx = cs[4 * kCellCap], nyy = cs[5 * kCellCap],
                                    nxy = cs[6 * kCellCap], nxz = cs[7 * kCellCap],
                                    nyz = cs[8 * kCellCap], nzz = cs[9 * kCellCap];
                        const float qx = fmaf(nxx, dx, fmaf(nxy, dy, nxz * dz));
                        const float qy = fmaf(nxy, dx, fmaf(nyy, dy, nyz * dz));
                        const float qz = fmaf(nxz, dx, fmaf(nyz, dy, nzz * dz));
                        const float dqd = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
                        const float sa = inv3 * fmaf(-2.5f * u * u, dqd, mm);
                        const float sb = inv3 * u;
                        px = fmaf(sb, qx, fmaf(sa, dx, px));
                        py = fmaf(sb, qy, fmaf(sa, dy, py));
                        pz = fmaf(sb, qz, fmaf(sa, dz, pz));
                    } else {
                        const float sa = inv3 * mm;
                        px = fmaf(sa, dx, px);
                        py = fmaf(sa, dy, py);
                        pz = fmaf(sa, dz, pz);
                    }
                };
                if (normal_r2) {
#pragma unroll 2
                    for (uint32_t e = rep; e < m; e += reps) cell(e, kTrue);
                } else {
#pragma unroll 2
                    for (uint32_t e = rep; e < m; e += reps) cell(e, kFalse);
                }
                if (kPrec) {
                    cells[k].add(px, py, pz);
                } else {
                    cells[k].ax += px;
                    cells[k].ay += py;
                    cells[k].az += pz;
                }
            }
        }
        inter += owned * m;
        cell_inter += owned * m;
    }

    // Leaf particles: the listed ranges, 32 at a time (one list block), are
    // concatenated and staged 32 particles at a time (a shuffle binary search
    // over the ranges' prefix sums finds each lane's particle), keeping the
    // walk order. The fast form stages the tile as arrays x[32], y[32],
    // z[32], m[32] with massless (exactly zero) entries past the end.
    float* const tile_soa = reinterpret_cast<float*>(s_tile);
    ChainCursor lcur{d.leaf_first};
    for (uint32_t l0 = 0; l0 < d.n_leaf; l0 += 32u) {
        const uint32_t nl = min(32u, d.n_leaf - l0);
        if (l0 > 0) lcur.advance(a);
        uint32_t rb = 0, rlen = 0;
        if (lane < nl) {
            const uint2 rg = reinterpret_cast<const uint2*>(lcur.words(a))[lane];
            rb = rg.x;
            rlen = rg.y - rg.x;
        }
        uint32_t incl = rlen;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t pre = incl - rlen;
        const uint32_t total = __shfl_sync(kFullMask, incl, 31);
        // Particle index of list position t0 + lane (all lanes take part).
        auto locate = [&](uint32_t t0) -> uint32_t {
            const uint32_t pos = t0 + lane;
            uint32_t e = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
                const uint32_t cand = e + step;
                const uint32_t pc = __shfl_sync(kFullMask, pre, cand & 31u);
                if (cand < nl && pc <= pos) e = cand;
            }
            const uint32_t eb = __shfl_sync(kFullMask, rb, e);
            const uint32_t ep = __shfl_sync(kFullMask, pre, e);
            return eb + (pos - ep);
        };
        // kPipe (fast form): the next tile's particle is loaded while the
        // current tile is summed, its L2 latency hidden behind the tile's work.
        constexpr bool kPipeTile = kPipe && !kExact;
        const float4 kZero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t jn = 0;
        float4 pn = kZero4;
        if (kPipeTile && total > 0u) {
            jn = locate(0u);
            pn = lane < total ? __ldg(&a.pos[jn]) : kZero4;
        }
        for (uint32_t t0 = 0; t0 < total; t0 += 32u) {
            const uint32_t pos = t0 + lane;
            const uint32_t j = kPipeTile ? jn : locate(t0);
            __syncwarp();
            if constexpr (kExact) {
                if (pos < total) {
                    s_tile[lane] = __ldg(&a.pos[j]);
                    s_jdx[lane] = j;
                }
            } else {
                const float4 p = kPipeTile ? pn : (pos < total ? __ldg(&a.pos[j]) : kZero4);
                tile_soa[lane] = p.x;
                tile_soa[32 + lane] = p.y;
                tile_soa[64 + lane] = p.z;
                tile_soa[96 + lane] = p.w;
                s_jdx[lane] = j;
                if (kPipeTile && t0 + 32u < total) {
                    jn = locate(t0 + 32u);
                    pn = pos + 32u < total ? __ldg(&a.pos[jn]) : kZero4;
                }
            }
            __syncwarp();
            const uint32_t cnt = min(32u, total - t0);
            if constexpr (kExact) {
#pragma unroll
                for (int k = 0; k < kPer; ++k) {
                    if (!valid[k]) continue;
                    for (uint32_t q = 0; q < cnt; ++q) {
                        if (s_jdx[q] != ip[k]) {
                            const float4 p = s_tile[q];
                            float tx, ty, tz;
                            particle_term<true>(__fsub_rn(p.x, me[k].x), __fsub_rn(p.y, me[k].y),
                                                __fsub_rn(p.z, me[k].z), p.w, g, eps2, tx, ty, tz);
                            leaves[k].push(tx, ty, tz);
                            ++inter;
                        }
                        leaves[k].step();
                    }
                }
            } else if (normal_r2 && reps == 1) {
                // eps > 0: the self term is exactly zero, so no test is
                // needed. Two sources per instruction (packed FP32 pairs);
                // even and odd sources summed apart and joined after the
                // tile, whose partial the precision form Kahan-adds once.
                const float2* v = reinterpret_cast<const float2*>(tile_soa);
                float2 nmx[kPer], nmy[kPer], nmz[kPer], sx[kPer], sy[kPer], sz[kPer];
#pragma unroll
                for (int k = 0; k < kPer; ++k) {
                    nmx[k] = make_float2(-me[k].x, -me[k].x);
                    nmy[k] = make_float2(-me[k].y, -me[k].y);
                    nmz[k] = make_float2(-me[k].z, -me[k].z);
                    sx[k] = sy[k] = sz[k] = make_float2(0.f, 0.f);
                }
                const float2 e2 = make_float2(eps2, eps2);
                if (cnt == 32u) {
#pragma unroll 8
                    for (uint32_t q = 0; q < 16u; ++q) {
                        const float2 X = v[q], Y = v[16 + q], Z = v[32 + q], M = v[48 + q];
#pragma unroll
                        for (int k = 0; k < kPer; ++k)
                            mono_pair(X, Y, Z, M, nmx[k], nmy[k], nmz[k], e2, sx[k], sy[k], sz[k]);
                    }
                } else {
                    const uint32_t n2 = (cnt + 1u) >> 1;
#pragma unroll 2
                    for (uint32_t q = 0; q < n2; ++q) {
                        const float2 X = v[q], Y = v[16 + q], Z = v[32 + q], M = v[48 + q];
#pragma unroll
                        for (int k = 0; k < kPer; ++k)
                            mono_pair(X, Y, Z, M, nmx[k], nmy[k], nmz[k], e2, sx[k], sy[k], sz[k]);
                    }
                }
#pragma unroll
                for (int k = 0; k < kPer; ++k) {
                    const float px = sx[k].x + sx[k].y, py = sy[k].x + sy[k].y, pz = sz[k].x + sz[k].y;
                    if (kPrec) {
                        leaves[k].add(px, py, pz);
                    } else {
                        leaves[k].ax += px;
                        leaves[k].ay += py;
                        leaves[k].az += pz;
                    }
                }
                inter += owned * cnt;
            } else {
#pragma unroll
                for (int k = 0; k < kPer; ++k) {
                    if (!valid[k]) continue;
                    float px = 0.f, py = 0.f, pz = 0.f;
                    if (normal_r2) {
                        // Copies of small groups: every reps-th source, no self test.
#pragma unroll 4
                        for (uint32_t q = rep; q < cnt; q += reps) {
                            const float dx = tile_soa[q] - me[k].x, dy = tile_soa[32 + q] - me[k].y,
                                        dz = tile_soa[64 + q] - me[k].z;
                            const float inv = rsqrt_ftz(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
                            const float sc = tile_soa[96 + q] * (inv * inv * inv);
                            px = fmaf(dx, sc, px);
                            py = fmaf(dy, sc, py);
                            pz = fmaf(dz, sc, pz);
                        }
                        if (owner[k]) inter += cnt;
                    } else {
                        // eps^2 below FLT_MIN: the particle's own entry is skipped.
                        for (uint32_t q = rep; q < cnt; q += reps) {
                            if (s_jdx[q] == ip[k]) continue;
                            float tx, ty, tz;
                            particle_term<false>(tile_soa[q] - me[k].x, tile_soa[32 + q] - me[k].y,
                                                 tile_soa[64 + q] - me[k].z, tile_soa[96 + q], 1.0f,
                                                 eps2, tx, ty, tz);
                            px += tx;
                            py += ty;
                            pz += tz;
                            ++inter;
                        }
                    }
                    if (kPrec) {
                        leaves[k].add(px, py, pz);
                    } else {
                        leaves[k].ax += px;
                        leaves[k].ay += py;
                        leaves[k].az += pz;
                    }
                }
            }
            __syncwarp();
        }
    }
    // The self-free fast loop counted each particle's own entry once.
    if (normal_r2) inter -= owned;

    // Sums, clamp, acceleration and kick-drift (updateSpheres' v += a dt,
    // x += v dt without damping).
    float sxo[kPer], syo[kPer], szo[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        if (kExact) {
            cells[k].finish();
            leaves[k].finish();
            sxo[k] = __fadd_rn(cells[k].ax, leaves[k].ax);
            syo[k] = __fadd_rn(cells[k].ay, leaves[k].ay);
            szo[k] = __fadd_rn(cells[k].az, leaves[k].az);
            if (d.n_far > 0) {
                sxo[k] = __fadd_rn(sxo[k], __fmul_rn(g, fx[k]));
                syo[k] = __fadd_rn(syo[k], __fmul_rn(g, fy[k]));
                szo[k] = __fadd_rn(szo[k], __fmul_rn(g, fz[k]));
            }
        } else {
            // Compensated sums: the running sum minus its pending correction.
            sxo[k] = (cells[k].ax - cells[k].cx) + (leaves[k].ax - leaves[k].cx);
            syo[k] = (cells[k].ay - cells[k].cy) + (leaves[k].ay - leaves[k].cy);
            szo[k] = (cells[k].az - cells[k].cz) + (leaves[k].az - leaves[k].cz);
        }
    }
    if (!kExact && kPer == 1 && reps > 1) {
        __syncwarp();
        if (valid[0]) s_tile[lane] = make_float4(sxo[0], syo[0], szo[0], 0.f);
        __syncwarp();
        if (owner[0])
            for (uint32_t r = 1; r < reps; ++r) {
                const float4 t = s_tile[lane + r * gcount];
                sxo[0] += t.x;
                syo[0] += t.y;
                szo[0] += t.z;
            }
        __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        if (!kExact) {
            sxo[k] = (sxo[k] + fx[k]) * g;
            syo[k] = (syo[k] + fy[k]) * g;
            szo[k] = (szo[k] + fz[k]) * g;
        }
        if (!owner[k]) continue;
        const uint32_t i = ip[k];
        const float cl = a.clampv, dt = a.dt;
        const float ax = fminf(fmaxf(sxo[k], -cl), cl);
        const float ay = fminf(fmaxf(syo[k], -cl), cl);
        const float az = fminf(fmaxf(szo[k], -cl), cl);
        a.acc[i] = make_float4(ax, ay, az, 0.f);
        float4 v = a.vel_in[i];
        v.x = __fadd_rn(v.x, __fmul_rn(ax, dt));
        v.y = __fadd_rn(v.y, __fmul_rn(ay, dt));
        v.z = __fadd_rn(v.z, __fmul_rn(az, dt));
        a.vel_out[i] = v;
        a.id_out[i] = a.id_in[i];
        if (kPrec) {
            const size_t n = a.n;
            const double ddt = (double)dt;
            a.x64_out[i] = __dadd_rn(a.x64_in[i], __dmul_rn((double)v.x, ddt));
            a.x64_out[n + i] = __dadd_rn(a.x64_in[n + i], __dmul_rn((double)v.y, ddt));
            a.x64_out[2 * n + i] = __dadd_rn(a.x64_in[2 * n + i], __dmul_rn((double)v.z, ddt));
            a.pos_out[i] = me[k];
        } else {
            a.pos_out[i] = make_float4(__fadd_rn(me[k].x, __fmul_rn(v.x, dt)),
                                       __fadd_rn(me[k].y, __fmul_rn(v.y, dt)),
                                       __fadd_rn(me[k].z, __fmul_rn(v.z, dt)), me[k].w);
        }
    }
}

}  // namespace

#if ASTRO_GROUP_WARPS_PER_SM > 0
#define ASTRO_EVAL_BOUNDS(w, prec)                                                            \
    __launch_bounds__((w) * 32,                                                              \
                      ((w) >= 8 && !(prec) ? ASTRO_GROUP_WARPS_PER_SM_8 : ASTRO_GROUP_WARPS_PER_SM) / \
                          (w))
#else
#define ASTRO_EVAL_BOUNDS(w, prec) __launch_bounds__((w) * 32)
#endif

template <bool kExact, bool kPrec, bool kQuad, int kWarps, bool kFarPre>
__global__ ASTRO_EVAL_BOUNDS(kWarps, kPrec) void group_eval_kernel(TraverseArgs a) {
    constexpr int kCellCap = cell_cap(kWarps);
    // Leaf tiles loaded one tile ahead with 4-warp blocks; the 8-warp blocks
    // (half the cell staging per warp) keep the load in line, which measured
    // faster for them (two Plummer spheres, 4,194,304 particles: 5.10 vs
    // 5.18 ms; with 4-warp blocks the look-ahead took 1.8% off the
    // 16,777,216-particle cube and 4% off 256 batched systems).
    constexpr bool kPipe = kWarps < 8;
    __shared__ CellSlot<kQuad> s_cell[kWarps][kCellCap];
    __shared__ float4 s_tile[kWarps][32];
    __shared__ uint32_t s_jdx[kWarps][32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // A walk that ran out of frontier or list room left incomplete lists:
    // nothing is evaluated or integrated (the state stays as it was) and
    // the host runs the traversal again with larger buffers.
    if (*reinterpret_cast<volatile const uint32_t*>(a.err) & kErrFrontier) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.evals_done, 1u);
    const uint32_t ngroups = *a.group_count;
    uint32_t inter = 0, cell_inter = 0, far_inter = 0;
    while (true) {
        uint32_t gi = 0;
        if (lane == 0) gi = atomicAdd(a.eval_queue, 1u);
        gi = __shfl_sync(kFullMask, gi, 0);
        if (gi >= ngroups) break;
        gi = group_of_ticket(gi, ngroups, a.group_chunk);
        const uint4 rec = a.groups[gi];
        const uint2 gr = make_uint2(rec.x, rec.y);
        // The walk of the leaf's first chunk: its lists and centre (the first
        // 48 bytes of the record) and its far-node coefficients.
        const GroupDesc* dp = a.desc + (gi - rec.w);
        GroupDesc d;
        {
            const uint4* w = reinterpret_cast<const uint4*>(dp);
            const uint4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2);
            d.leaf_first = w0.x, d.n_leaf = w0.y, d.cell_first = w0.z, d.n_cell = w0.w;
            d.far_first = w1.x, d.n_far = w1.y, d.gcx = __uint_as_float(w1.z);
            d.gcy = __uint_as_float(w1.w), d.gcz = __uint_as_float(w2.x);
        }
        if (gr.y - gr.x > 32u)
            eval_group<kExact, kPrec, kQuad, kCellCap, 2, kPipe, kFarPre>(a, gr, d, dp->far_co, s_cell[warp], s_tile[warp],
                                                                 s_jdx[warp], lane, inter,
                                                                 cell_inter, far_inter);
        else
            eval_group<kExact, kPrec, kQuad, kCellCap, 1, kPipe, kFarPre>(a, gr, d, dp->far_co, s_cell[warp], s_tile[warp],
                                                                 s_jdx[warp], lane, inter,
                                                                 cell_inter, far_inter);
    }
    unsigned long long i64 = inter, c64 = cell_inter, f64 = far_inter;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        i64 += __shfl_xor_sync(kFullMask, i64, o);
        c64 += __shfl_xor_sync(kFullMask, c64, o);
        f64 += __shfl_xor_sync(kFullMask, f64, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stats[0], i64);
        atomicAdd(&a.stats[2], c64);
        if (f64) atomicAdd(&a.stats[4], f64);
    }
}

// ------------------------------------------------------------- launches --

namespace {

constexpr int kMaxDevices = 64;
int g_sms[kMaxDevices] = {};
int g_walk_per_sm[kMaxDevices] = {};
std::mutex g_mutex;

int device_index() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
    return dev;
}

int sm_count() {
    const int dev = device_index();
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_sms[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms[dev] = n > 0 ? n : 1;
    }
    return g_sms[dev];
}

uint32_t walk_blocks() {
    const int dev = device_index();
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        per_sm = g_walk_per_sm[dev];
    }
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, group_walk_kernel, kWalkWarps * 32, 0);
        per_sm = std::max(1, per_sm);
        std::lock_guard<std::mutex> lock(g_mutex);
        g_walk_per_sm[dev] = per_sm;
    }
    return (uint32_t)per_sm * (uint32_t)sm_count();
}

template <bool kExact, bool kPrec, bool kQuad, int kWarps, bool kFarPre>
cudaError_t launch_eval_t(const TraverseArgs& a, cudaStream_t st) {
    auto kernel = group_eval_kernel<kExact, kPrec, kQuad, kWarps, kFarPre>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarps * 32, 0);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = (uint32_t)std::max(1, per_sm) * (uint32_t)sm_count();
    kernel<<<blocks, kWarps * 32, 0, st>>>(a);
    return cudaGetLastError();
}

template <bool kExact, bool kPrec, bool kQuad, bool kFarPre>
cudaError_t launch_eval_w(const TraverseArgs& a, int warps, cudaStream_t st) {
    return warps == 8 ? launch_eval_t<kExact, kPrec, kQuad, 8, kFarPre>(a, st)
                      : launch_eval_t<kExact, kPrec, kQuad, 4, kFarPre>(a, st);
}

template <bool kExact, bool kPrec>
cudaError_t launch_eval_q(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st) {
    if (c.far_pre)
        return c.quad ? launch_eval_w<kExact, kPrec, true, true>(a, c.warps, st)
                      : launch_eval_w<kExact, kPrec, false, true>(a, c.warps, st);
    return c.quad ? launch_eval_w<kExact, kPrec, true, false>(a, c.warps, st)
                  : launch_eval_w<kExact, kPrec, false, false>(a, c.warps, st);
}

}  // namespace

uint32_t group_walk_warps() { return walk_blocks() * (uint32_t)kWalkWarps; }

size_t group_list_blocks(uint32_t n, uint32_t group_size) {
    // Measured lists run to about 1,800 words per group (a 524,288-body disk
    // with far nodes at ratio 0.15, groups of at most 32), with at most three
    // partly filled blocks per group; groups average at least half the group
    // size. 2,048 words per group of half the group size, plus the batches of
    // blocks the walk warps hold, leaves room.
    const size_t groups = (size_t)n / std::max(1u, group_size / 2u) + 1;
    const size_t words = std::max<size_t>(groups * 2048, (size_t)1 << 22);
    const size_t blocks = words / kListBlockWords + (size_t)group_walk_warps() * kBlockBatch;
    return std::min<size_t>(blocks, 0xFFFFFF00ull);
}

cudaError_t launch_traverse_groups(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st,
                                   cudaEvent_t* ev) {
    if (a.n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    // Evaluation queue and list pool counter (adjacent words).
    e = cudaMemsetAsync(a.eval_queue, 0, 2 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (ev && (e = cudaEventRecord(ev[0], st)) != cudaSuccess) return e;
    group_walk_kernel<<<walk_blocks(), kWalkWarps * 32, 0, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (ev && (e = cudaEventRecord(ev[1], st)) != cudaSuccess) return e;
    if (c.far_pre && a.far2 > 0.f) {
        const uint32_t blocks = walk_blocks();
        if (c.exact)
            c.quad ? group_far_kernel<true, true><<<blocks, 128, 0, st>>>(a)
                   : group_far_kernel<true, false><<<blocks, 128, 0, st>>>(a);
        else
            c.quad ? group_far_kernel<false, true><<<blocks, 128, 0, st>>>(a)
                   : group_far_kernel<false, false><<<blocks, 128, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (c.exact)
        e = c.precision ? launch_eval_q<true, true>(a, c, st) : launch_eval_q<true, false>(a, c, st);
    else
        e = c.precision ? launch_eval_q<false, true>(a, c, st) : launch_eval_q<false, false>(a, c, st);
    if (e != cudaSuccess) return e;
    return ev ? cudaEventRecord(ev[2], st) : cudaSuccess;
}

}  // namespace astro
