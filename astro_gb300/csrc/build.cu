// Encode, bounding box, tree topology and aggregation kernels.
//
// Reference stages replaced here (Astro/Renderer.swift:505-533,714-755):
//   generateMortonCodes + fillIndices (MortonCode.metal:26-52, Octree.metal:39-51)
//   countUniqueMortonCodes per layer: markUniques, the scan, scatterUniques,
//     copyLastScanToParentCount (Octree.metal:282-334)
//   aggregateLeafNodes / aggregateNodes (Octree.metal:53-202)
// The reference finds the runs of every layer with one sort + scan + scatter
// per layer over all N entries. Here a single pass over the sorted keys finds
// the node starts of all layers at once (topology_kernel); the large layers
// are aggregated one launch each and the small top layers in one climbing
// launch (aggregate_tree_kernel).
#include <algorithm>

#include "build_kernels.cuh"
#include "common.cuh"
#include "internal.h"

namespace astro {

// ------------------------------------------------------------- encode ----

// generateMortonCodes with the reference quantiser (u32)(p + 1e6): the
// float-to-uint conversion saturates and rounds toward zero.
__global__ void encode_ref_kernel(const float4* __restrict__ pos, uint64_t* __restrict__ codes,
                                  uint32_t n_tree, uint32_t unused_bits, float offset) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_tree) return;
    const float4 q = pos[i];
    const uint32_t x = __float2uint_rz(__fadd_rn(q.x, offset));
    const uint32_t y = __float2uint_rz(__fadd_rn(q.y, offset));
    const uint32_t z = __float2uint_rz(__fadd_rn(q.z, offset));
    codes[i] = interleave3(x, y, z) >> unused_bits;
}

__device__ __forceinline__ uint32_t quantise(float x, float lo, float scale) {
    return min(__float2uint_rz(__fmul_rn(__fsub_rn(x, lo), scale)), kQuantMax);
}

// Bounding-box quantiser of the PHYSICAL preset, one block per chunk. In the
// precision form the FP32 frame relative to the system origin is written
// to pos here (x64 is the master copy).
template <bool kPrec>
__global__ __launch_bounds__(256) void encode_phys_kernel(const Chunk* __restrict__ chunks,
                                                          const SysInfo* __restrict__ sys,
                                                          float4* __restrict__ pos,
                                                          const double* __restrict__ x64,
                                                          uint64_t* __restrict__ codes, uint32_t n,
                                                          uint32_t lbits) {
    const Chunk c = chunks[blockIdx.x];
    const SysInfo& s = sys[c.sys];
    const float lox = s.lo[0], loy = s.lo[1], loz = s.lo[2], scale = s.scale;
    const uint32_t unused_bits = 63u - 3u * lbits;
    const uint64_t sys_bits = (uint64_t)c.sys << (3u * lbits);
    double ox = 0, oy = 0, oz = 0;
    if (kPrec) {
        ox = s.origin[0];
        oy = s.origin[1];
        oz = s.origin[2];
    }
    for (uint32_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
        float4 q = pos[i];
        if (kPrec) {
            q.x = __double2float_rn(__dsub_rn(x64[i], ox));
            q.y = __double2float_rn(__dsub_rn(x64[(size_t)n + i], oy));
            q.z = __double2float_rn(__dsub_rn(x64[2 * (size_t)n + i], oz));
            pos[i] = q;
        }
        const uint32_t qx = quantise(q.x, lox, scale);
        const uint32_t qy = quantise(q.y, loy, scale);
        const uint32_t qz = quantise(q.z, loz, scale);
        codes[i] = sys_bits | (interleave3(qx, qy, qz) >> unused_bits);
    }
}

// ------------------------------------------------------- bounding box ----

template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(kFullMask, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFullMask, v, o));
    return v;
}

// Block-level min/max of six ordered keys followed by one atomic per value.
template <typename U>
__device__ __forceinline__ void block_bbox_commit(U lo[3], U hi[3], U* acc) {
    __shared__ U s_red[8][6];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = warp_min(lo[a]);
        hi[a] = warp_max(hi[a]);
    }
    if (lane == 0)
        for (int a = 0; a < 3; ++a) {
            s_red[warp][a] = lo[a];
            s_red[warp][3 + a] = hi[a];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        const uint32_t nw = blockDim.x >> 5;
        U v = s_red[0][threadIdx.x];
        for (uint32_t w = 1; w < nw; ++w)
            v = threadIdx.x < 3 ? min(v, s_red[w][threadIdx.x]) : max(v, s_red[w][threadIdx.x]);
        if (threadIdx.x < 3) atomicMin(acc + threadIdx.x, v);
        else atomicMax(acc + threadIdx.x, v);
    }
}

// Bounding box of the current positions, one block per chunk, accumulated
// per system with one atomic per block and value.
template <bool kPrec>
__global__ __launch_bounds__(256) void bbox_kernel(const Chunk* __restrict__ chunks,
                                                   const float4* __restrict__ pos,
                                                   const double* __restrict__ x64, uint32_t n,
                                                   uint32_t* __restrict__ bb32,
                                                   unsigned long long* __restrict__ bb64) {
    const Chunk c = chunks[blockIdx.x];
    if (kPrec) {
        unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
        for (uint32_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x)
            for (int a = 0; a < 3; ++a) {
                unsigned long long o = f64_to_ordered(x64[(size_t)a * n + i]);
                lo[a] = min(lo[a], o);
                hi[a] = max(hi[a], o);
            }
        block_bbox_commit(lo, hi, bb64 + 6ull * c.sys);
    } else {
        uint32_t lo[3] = {~0u, ~0u, ~0u}, hi[3] = {0, 0, 0};
        for (uint32_t i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
            const float4 q = pos[i];
            const float v[3] = {q.x, q.y, q.z};
            for (int a = 0; a < 3; ++a) {
                uint32_t o = f32_to_ordered(v[a]);
                lo[a] = min(lo[a], o);
                hi[a] = max(hi[a], o);
            }
        }
        block_bbox_commit(lo, hi, bb32 + 6ull * c.sys);
    }
}

// Per-system quantiser and opening thresholds from the box accumulators,
// which are then reset for the next accumulation.
template <bool kPrec>
__global__ void setup_kernel(SysInfo* __restrict__ sys, uint32_t nsys,
                             uint32_t* __restrict__ bb32, unsigned long long* __restrict__ bb64,
                             uint32_t lbits, float theta, uint32_t root_offset) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    SysInfo& info = sys[s];
    float lo[3], hi[3];
    if (kPrec) {
        for (int a = 0; a < 3; ++a) {
            const double l = ordered_to_f64(bb64[6ull * s + a]);
            const double h = ordered_to_f64(bb64[6ull * s + 3 + a]);
            const double o = __dmul_rn(__dadd_rn(l, h), 0.5);
            info.origin[a] = o;
            lo[a] = __double2float_rn(__dsub_rn(l, o));
            hi[a] = __double2float_rn(__dsub_rn(h, o));
            bb64[6ull * s + a] = ~0ull;
            bb64[6ull * s + 3 + a] = 0ull;
        }
    } else {
        for (int a = 0; a < 3; ++a) {
            lo[a] = ordered_to_f32(bb32[6ull * s + a]);
            hi[a] = ordered_to_f32(bb32[6ull * s + 3 + a]);
            info.origin[a] = 0.0;
            bb32[6ull * s + a] = ~0u;
            bb32[6ull * s + 3 + a] = 0u;
        }
    }
    float ext = 0.0f;
    for (int a = 0; a < 3; ++a) {
        info.lo[a] = lo[a];
        ext = fmaxf(ext, __fsub_rn(hi[a], lo[a]));
    }
    if (!(ext > 0.0f) || !isfinite(ext)) ext = 1.0f;
    info.ext = ext;
    info.scale = __fdiv_rn(kQuantCells, ext);
    info.root = root_offset + s;
    for (uint32_t l = 0; l <= lbits; ++l) {
        const float c = __fdiv_rn(__fmul_rn(ext, exp2_exact((int)l - (int)lbits)), theta);
        info.crit2[l] = __fmul_rn(c, c);
    }
}

// ------------------------------------------------------------ reorder ----

// Permute the PHYSICAL state into the new Morton order (B <- A[perm]).
template <bool kPrec>
__global__ void reorder_kernel(const uint32_t* __restrict__ perm, const float4* __restrict__ pos_a,
                               const float4* __restrict__ vel_a, const uint32_t* __restrict__ id_a,
                               const double* __restrict__ x_a, float4* __restrict__ pos_b,
                               float4* __restrict__ vel_b, uint32_t* __restrict__ id_b,
                               double* __restrict__ x_b, uint32_t n) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t s = perm[j];
    pos_b[j] = pos_a[s];
    vel_b[j] = vel_a[s];
    id_b[j] = id_a[s];
    if (kPrec) {
        x_b[j] = x_a[s];
        x_b[(size_t)n + j] = x_a[(size_t)n + s];
        x_b[2 * (size_t)n + j] = x_a[2 * (size_t)n + s];
    }
}

// ----------------------------------------------------------- topology ----

constexpr int kTopoThreads = 256;
constexpr int kTopoWarps = kTopoThreads / 32;
constexpr int kTopoItems = 8;
constexpr int kTopoTile = kTopoThreads * kTopoItems;

// One pass over the sorted keys finds the nodes of every layer. Position i
// starts a node at layer l when its key differs from key i-1 above bit 3l,
// i.e. for l <= lev(i) = floor(msb(k[i] ^ k[i-1]) / 3) (capped at lbits;
// lev(0) = lbits). The index of that node inside its layer is the number of
// starts before i, found per layer with warp ballots and a decoupled
// look-back across tiles. Each start writes the node's first particle and,
// above layer 0, its first child (the node starting at i one layer down).
// This yields the runs of markUniques/scatterUniques (Octree.metal:282-318)
// for all layers without re-sorting or re-scanning per layer. Each node
// below the top layer also gets its parent: the node one layer up that
// holds its first particle (the bottom-up aggregation climbs these links).
__global__ __launch_bounds__(kTopoThreads) void topology_kernel(TopoArgs a) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_off[ASTRO_MAX_LAYERS];
    __shared__ uint32_t s_wcnt[kTopoWarps][32];
    __shared__ uint32_t s_prefix[32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int lbits = (int)a.lbits;
    if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
    if (tid < ASTRO_MAX_LAYERS) s_off[tid] = a.offset[tid];
    if (tid < 32)
        for (int w = 0; w < kTopoWarps; ++w) s_wcnt[w][tid] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * kTopoTile;
    if (base >= a.n) return;
    const uint64_t warp_base = base + (uint64_t)warp * 32 * kTopoItems;
    const uint32_t lt = lanemask_lt();

    uint64_t key[kTopoItems];
    int lev[kTopoItems];
    uint64_t carry = (warp_base > 0 && warp_base <= a.n) ? a.keys[warp_base - 1] : 0ull;
#pragma unroll
    for (int k = 0; k < kTopoItems; ++k) {
        const uint64_t i = warp_base + 32ull * k + lane;
        const bool valid = i < a.n;
        key[k] = valid ? a.keys[i] : 0ull;
        uint64_t prev = __shfl_up_sync(kFullMask, key[k], 1);
        if (lane == 0) prev = carry;
        carry = __shfl_sync(kFullMask, key[k], 31);
        int lv = -1;
        if (valid) {
            if (i == 0) lv = lbits;
            else if (key[k] != prev) lv = min(lbits, (63 - __clzll((long long)(key[k] ^ prev))) / 3);
        }
        lev[k] = lv;
    }
    // Starts per layer within this warp (lane l keeps layer l).
    uint32_t my_cnt = 0;
#pragma unroll
    for (int k = 0; k < kTopoItems; ++k)
        for (int l = 0; l <= lbits; ++l) {
            const uint32_t b = __ballot_sync(kFullMask, lev[k] >= l);
            if (b == 0) break;
            if ((int)lane == l) my_cnt += __popc(b);
        }
    if ((int)lane <= lbits) s_wcnt[warp][lane] = my_cnt;
    __syncthreads();
    if ((int)tid <= lbits) {
        uint32_t run = 0;
        for (int w = 0; w < kTopoWarps; ++w) {
            const uint32_t c = s_wcnt[w][tid];
            s_wcnt[w][tid] = run;
            run += c;
        }
        uint32_t* word = a.lookback + (size_t)tile * 32 + tid;
        st_relaxed_u32(word, (tile == 0 ? kLbInclusive : kLbAggregate) | run);
        uint32_t prefix = 0;
        if (tile > 0) {
            prefix = lookback_window(a.lookback, tile, tid, a.err, 32);
            st_relaxed_u32(word, kLbInclusive | (prefix + run));
        }
        s_prefix[tid] = prefix;
        if (tile == a.ntiles - 1) a.layer_count[tid] = prefix + run;
    }
    __syncthreads();
    uint32_t running = (int)lane <= lbits ? s_prefix[lane] + s_wcnt[warp][lane] : 0u;
#pragma unroll
    for (int k = 0; k < kTopoItems; ++k) {
        const uint32_t i = (uint32_t)(warp_base + 32ull * k + lane);
        uint32_t idx_below = 0;
        uint32_t pending = kNoParent;  // this lane's node one layer down, parent not yet written
        for (int l = 0; l <= lbits; ++l) {
            const uint32_t b = __ballot_sync(kFullMask, lev[k] >= l);
            const uint32_t base_l = __shfl_sync(kFullMask, running, l);
            // Starts of layer l before particle i.
            const uint32_t rank = base_l + __popc(b & lt);
            if (pending != kNoParent) {
                // The parent holds i: the layer-l node starting at i, else the
                // last one starting before it.
                a.parent[pending] = s_off[l] + (lev[k] >= l ? rank : rank - 1u);
                pending = kNoParent;
            }
            if (b == 0) break;
            if (lev[k] >= l) {
                const uint32_t node = s_off[l] + rank;
                a.pbeg[node] = i;
                a.node_key[node] = key[k] >> (3u * l);
                if (l > 0) a.cbeg[node] = s_off[l - 1] + idx_below;
                idx_below = rank;
                if (l < lbits) pending = node;
                else a.parent[node] = kNoParent;
            }
            if ((int)lane == l) running += __popc(b);
        }
    }
}

// -------------------------------------------------------- aggregation ----

// Traceless quadrupole accumulation of mass m at offset d from the centre of
// mass: Q += m (3 d d^T - |d|^2 I), components Qxx, Qyy, Qxy, Qxz, Qyz, each
// product and sum rounded separately.
__device__ __forceinline__ void quad_add(float q[5], float m, float dx, float dy, float dz) {
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    const float tx = __fmul_rn(3.0f, dx), ty = __fmul_rn(3.0f, dy);
    q[0] = __fadd_rn(q[0], __fmul_rn(m, __fsub_rn(__fmul_rn(tx, dx), r2)));
    q[1] = __fadd_rn(q[1], __fmul_rn(m, __fsub_rn(__fmul_rn(ty, dy), r2)));
    q[2] = __fadd_rn(q[2], __fmul_rn(m, __fmul_rn(tx, dy)));
    q[3] = __fadd_rn(q[3], __fmul_rn(m, __fmul_rn(tx, dz)));
    q[4] = __fadd_rn(q[4], __fmul_rn(m, __fmul_rn(ty, dz)));
}

// Opening radius^2 of a node: (size / theta + w |com - cell centre|)^2, the
// cell found from the node's key prefix in its system's box.
// Geometric centre (x, y, z) and edge (w) of the layer-l cell of a node;
// node_key = first key >> 3l: the system above bit 3 (lbits - l), the
// cell's code below it (3 (lbits - l) <= 63).
__device__ __forceinline__ float4 cell_box(const AggArgs& a, uint64_t node_key, uint32_t l) {
    const uint32_t below = 3u * (a.lbits - l);
    const uint32_t s = (uint32_t)(node_key >> below);
    const SysInfo& si = a.sys[s];
    const uint64_t code = node_key & ((1ull << below) - 1ull);
    const float size = __fmul_rn(si.ext, exp2_exact((int)l - (int)a.lbits));
    const float half = __fmul_rn(0.5f, size);
    return make_float4(__fadd_rn(si.lo[0], __fmul_rn((float)(2u * compact3_21(code) + 1u), half)),
                       __fadd_rn(si.lo[1], __fmul_rn((float)(2u * compact3_21(code >> 1) + 1u), half)),
                       __fadd_rn(si.lo[2], __fmul_rn((float)(2u * compact3_21(code >> 2) + 1u), half)),
                       size);
}

__device__ __forceinline__ float node_crit2(const AggArgs& a, uint64_t node_key, uint32_t l, float4 cm) {
    const float4 box = cell_box(a, node_key, l);
    const float size = box.w, cx = box.x, cy = box.y, cz = box.z;
    const float dx = __fsub_rn(cm.x, cx), dy = __fsub_rn(cm.y, cy), dz = __fsub_rn(cm.z, cz);
    const float dd = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    const float crit = __fadd_rn(__fdiv_rn(size, a.theta), __fmul_rn(a.delta_weight, __fsqrt_rn(dd)));
    return __fmul_rn(crit, crit);
}

// PHYSICAL centre of mass (and mass) from the raw sums: one reciprocal of
// the mass and three products; zero for a massless node. FP32: a correctly
// rounded reciprocal. Precision form: the FP32 reciprocal refined by one
// FP64 Newton step, r = r0 + r0 (1 - m r0) (about 46 bits, two FMAs instead
// of an FP64 division), then FP64 products rounded to FP32.
__device__ __forceinline__ float4 com_from_sums(float sx, float sy, float sz, float m) {
    if (!(m > 0.f)) return make_float4(0.f, 0.f, 0.f, m);
    const float inv = __fdiv_rn(1.0f, m);
    return make_float4(__fmul_rn(sx, inv), __fmul_rn(sy, inv), __fmul_rn(sz, inv), m);
}
__device__ __forceinline__ float4 com_from_sums(double sx, double sy, double sz, double m) {
    if (!(m > 0.0)) return make_float4(0.f, 0.f, 0.f, __double2float_rn(m));
    const double r0 = (double)__fdiv_rn(1.0f, __double2float_rn(m));
    const double inv = __fma_rn(r0, __fma_rn(-m, r0, 1.0), r0);
    return make_float4(__double2float_rn(__dmul_rn(sx, inv)), __double2float_rn(__dmul_rn(sy, inv)),
                       __double2float_rn(__dmul_rn(sz, inv)), __double2float_rn(m));
}

// Slots for c groups of this thread: the active lanes of the warp add their
// counts and one lane claims them with a single atomic (one atomic per warp
// instead of one per group on the shared counter); lanes take their runs in
// lane order.
__device__ __forceinline__ uint32_t reserve_groups(uint32_t* counter, uint32_t c) {
    const uint32_t mask = __activemask();
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t prefix = 0, total = 0;
    for (uint32_t m = mask; m != 0u; m &= m - 1u) {
        const uint32_t l = (uint32_t)__ffs(m) - 1u;
        const uint32_t cl = __shfl_sync(mask, c, l);
        if (l < lane) prefix += cl;
        total += cl;
    }
    const uint32_t leader = (uint32_t)__ffs(mask) - 1u;
    uint32_t base = 0;
    if (lane == leader && total != 0u) base = atomicAdd(counter, total);
    return __shfl_sync(mask, base, leader) + prefix;
}

// Visits the particles [pb, pe) in order, loading four at a time so that
// four loads are in flight (the sums stay in particle order).
template <typename F>
__device__ __forceinline__ void for_particles(const float4* __restrict__ pos, uint32_t pb,
                                              uint32_t pe, F&& f) {
    uint32_t i = pb;
    for (; i + 4u <= pe; i += 4u) {
        float4 q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = __ldg(&pos[i + u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) f(q[u]);
    }
    for (; i < pe; ++i) f(__ldg(&pos[i]));
}

// Mass moments of a leaf's particles about a point c (the cell's centre):
// first moments D = sum m d and second moments S = sum m d d^T, d = x - c,
// in FP32, each product and sum rounded separately. quadrupole() shifts them
// to the centre of mass e + c (e = com - c): P = S - e D^T - D e^T + M e e^T,
// Q = 3 P - tr(P) I (traceless), components Qxx, Qyy, Qxy, Qxz, Qyz. The
// particles lie inside the cell, so |d| is at most its half diagonal and
// the shift loses little; one read of the particles then gives the sums and
// the quadrupole together (a second pass about the centre of mass re-read
// them from DRAM once the position array had streamed through L2).
struct CellMoments {
    float dx = 0.f, dy = 0.f, dz = 0.f;
    float sxx = 0.f, syy = 0.f, szz = 0.f, sxy = 0.f, sxz = 0.f, syz = 0.f;
    __device__ __forceinline__ void add(float4 q, float4 c) {
        const float ux = __fsub_rn(q.x, c.x), uy = __fsub_rn(q.y, c.y), uz = __fsub_rn(q.z, c.z);
        const float tx = __fmul_rn(q.w, ux), ty = __fmul_rn(q.w, uy), tz = __fmul_rn(q.w, uz);
        dx = __fadd_rn(dx, tx);
        dy = __fadd_rn(dy, ty);
        dz = __fadd_rn(dz, tz);
        sxx = __fadd_rn(sxx, __fmul_rn(tx, ux));
        syy = __fadd_rn(syy, __fmul_rn(ty, uy));
        szz = __fadd_rn(szz, __fmul_rn(tz, uz));
        sxy = __fadd_rn(sxy, __fmul_rn(tx, uy));
        sxz = __fadd_rn(sxz, __fmul_rn(tx, uz));
        syz = __fadd_rn(syz, __fmul_rn(ty, uz));
    }
    // P_ab = ((S_ab - e_a D_b) - e_b D_a) + e_a (M e_b)
    __device__ __forceinline__ static float shifted(float s, float ea, float eb, float da, float db,
                                                    float m) {
        return __fadd_rn(__fsub_rn(__fsub_rn(s, __fmul_rn(ea, db)), __fmul_rn(eb, da)),
                         __fmul_rn(ea, __fmul_rn(m, eb)));
    }
    __device__ __forceinline__ void quadrupole(float4 cm, float4 c, float q[5]) const {
        const float ex = __fsub_rn(cm.x, c.x), ey = __fsub_rn(cm.y, c.y), ez = __fsub_rn(cm.z, c.z);
        const float m = cm.w;
        const float pxx = shifted(sxx, ex, ex, dx, dx, m);
        const float pyy = shifted(syy, ey, ey, dy, dy, m);
        const float pzz = shifted(szz, ez, ez, dz, dz, m);
        const float pxy = shifted(sxy, ex, ey, dx, dy, m);
        const float pxz = shifted(sxz, ex, ez, dx, dz, m);
        const float pyz = shifted(syz, ey, ez, dy, dz, m);
        const float tr = __fadd_rn(__fadd_rn(pxx, pyy), pzz);
        q[0] = __fsub_rn(__fmul_rn(3.0f, pxx), tr);
        q[1] = __fsub_rn(__fmul_rn(3.0f, pyy), tr);
        q[2] = __fmul_rn(3.0f, pxy);
        q[3] = __fmul_rn(3.0f, pxz);
        q[4] = __fmul_rn(3.0f, pyz);
    }
};

// aggregateLeafNodes (Octree.metal:53-117), one thread per leaf.
// kMode 0 (REFERENCE): state in upload order, gathered through perm; FP32
//   sums of m and x*m in sorted order; the last leaf sums [start, numUnique)
//   as the reference does (Octree.metal:71).
// kMode 1 (PHYSICAL plain): state already in sorted order; raw FP32 sums.
// kMode 2 (PHYSICAL precision): FP64 sums of m and m*x over the FP32
//   positions relative to the system origin.
template <int kMode, bool kQuad>
__device__ __forceinline__ void aggregate_leaf_node_q(const AggArgs& a, uint32_t j, uint32_t u0) {
    const uint32_t pb = a.pbeg[j];
    const uint32_t pe = (j + 1 < u0) ? a.pbeg[j + 1] : a.n;
    // PHYSICAL quadrupole in the same read of the particles as the sums:
    // moments about the cell's centre, shifted to the centre of mass after.
    uint64_t node_key = 0;
    float4 box = make_float4(0.f, 0.f, 0.f, 0.f);
    if (kMode != 0 && (kQuad || a.want_delta)) node_key = a.node_key[j];
    if (kQuad) box = cell_box(a, node_key, 0);
    CellMoments mom;
    float4 cm = make_float4(0.f, 0.f, 0.f, 0.f);
    if (kMode == 0) {
        const uint32_t sum_end = (j + 1 < u0) ? pe : u0;
        float m = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
        // Stars (type 0): colours summed, positions averaged (Octree.metal:85-99).
        float4 ec = make_float4(0.f, 0.f, 0.f, 0.f), en = ec;
        uint32_t suns = 0;
        for (uint32_t i = pb; i < sum_end; ++i) {
            const uint32_t pi = a.perm[i];
            const float4 q = a.pos[pi];
            m = __fadd_rn(m, q.w);
            sx = __fadd_rn(sx, __fmul_rn(q.x, q.w));
            sy = __fadd_rn(sy, __fmul_rn(q.y, q.w));
            sz = __fadd_rn(sz, __fmul_rn(q.z, q.w));
            if (a.node_ecol && a.types[pi] == 0u) {
                const float4 c = a.colors[pi];
                ec = make_float4(__fadd_rn(ec.x, c.x), __fadd_rn(ec.y, c.y), __fadd_rn(ec.z, c.z),
                                 __fadd_rn(ec.w, c.w));
                en = make_float4(__fadd_rn(en.x, q.x), __fadd_rn(en.y, q.y), __fadd_rn(en.z, q.z), 0.f);
                ++suns;
            }
        }
        if (m > 0.f) cm = make_float4(__fdiv_rn(sx, m), __fdiv_rn(sy, m), __fdiv_rn(sz, m), m);
        else cm.w = m;
        if (a.node_ecol) {
            const float ns = fmaxf((float)suns, 1e-9f);
            a.node_ecol[j] = ec;
            a.node_ecen[j] = make_float4(__fdiv_rn(en.x, ns), __fdiv_rn(en.y, ns), __fdiv_rn(en.z, ns), 0.f);
        }
    } else if (kMode == 1) {
        float m = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
        for_particles(a.pos, pb, pe, [&](const float4 q) {
            m = __fadd_rn(m, q.w);
            sx = __fadd_rn(sx, __fmul_rn(q.w, q.x));
            sy = __fadd_rn(sy, __fmul_rn(q.w, q.y));
            sz = __fadd_rn(sz, __fmul_rn(q.w, q.z));
            if (kQuad) mom.add(q, box);
        });
        reinterpret_cast<float4*>(a.node_sum)[j] = make_float4(sx, sy, sz, m);
        cm = com_from_sums(sx, sy, sz, m);
    } else {
        // FP64 sums of m * x over the FP32 positions relative to the system
        // origin (written by the encode from the FP64 master copy): the
        // product of two floats is exact in FP64, so each FMA rounds once,
        // exactly as a multiply-then-add would.
        double m = 0, sx = 0, sy = 0, sz = 0;
        for_particles(a.pos, pb, pe, [&](const float4 q) {
            const double mi = (double)q.w;
            m = __dadd_rn(m, mi);
            sx = __fma_rn(mi, (double)q.x, sx);
            sy = __fma_rn(mi, (double)q.y, sy);
            sz = __fma_rn(mi, (double)q.z, sz);
            if (kQuad) mom.add(q, box);
        });
        reinterpret_cast<double4*>(a.node_sum)[j] = make_double4(sx, sy, sz, m);
        if (pe - pb == 1 && m >= 1.17549435e-38) {
            // One particle of normal FP32 mass: the sums are m*x exactly and
            // the reciprocal is within 2^-47 of 1/m, so the FP32 centre of
            // mass is x itself (+0 for -0, as the sums give).
            const float4 q = a.pos[pb];
            cm = make_float4(__fadd_rn(q.x, 0.f), __fadd_rn(q.y, 0.f), __fadd_rn(q.z, 0.f), q.w);
        } else {
            cm = com_from_sums(sx, sy, sz, m);
        }
    }
    a.node_cm[j] = cm;
    a.node_rng[j] = make_uint4(0u, 0u, pb, pe);
    if (kMode != 0) {
        if (kQuad) {
            float q[5];
            mom.quadrupole(cm, box, q);
            a.node_q[j] = make_float4(q[0], q[1], q[2], q[3]);
            a.node_qyz[j] = q[4];
        }
        if (a.want_delta) a.node_crit2[j] = node_crit2(a, node_key, 0, cm);
        // A leaf holding more than one group is cut into group-sized chunks.
        const uint32_t gs = a.group_size;
        const uint32_t c = pe - pb > gs ? (pe - pb + gs - 1u) / gs : 0u;
        const uint32_t slot = reserve_groups(a.group_count, c);
        for (uint32_t i = 0; i < c; ++i)
            a.groups[slot + i] = make_uint4(pb + i * gs, min(pb + (i + 1u) * gs, pe), pe, i);
    }
}

template <int kMode>
__device__ __forceinline__ void aggregate_leaf_node(const AggArgs& a, uint32_t j, uint32_t u0) {
    if (kMode != 0 && a.want_quad) aggregate_leaf_node_q<kMode, true>(a, j, u0);
    else aggregate_leaf_node_q<kMode, false>(a, j, u0);
}

// aggregateNodes (Octree.metal:120-202) for node j of layer l (one thread).
// Children are the contiguous run of layer l-1 nodes sharing code >> 3 (at
// most 8). Each thread first loads all its children's records together
// (one memory latency instead of one per child), then sums them in child
// order with the same roundings as a sequential loop.
// kMode 0 sums child centre of mass times child mass (the reference's
// formula); kModes 1 and 2 add the children's raw sums.
// Children are read through L2 (ld.global.cg): the climbing kernel below
// reads records that other blocks wrote in the same launch.
__device__ __forceinline__ float4 ld_l2(const float4* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_l2(const float* p) { return __ldcg(p); }
__device__ __forceinline__ uint4 ld_l2(const uint4* p) { return __ldcg(p); }
__device__ __forceinline__ double4 ld_l2(const double4* p) {
    const double2 lo = __ldcg(reinterpret_cast<const double2*>(p));
    const double2 hi = __ldcg(reinterpret_cast<const double2*>(p) + 1);
    return make_double4(lo.x, lo.y, hi.x, hi.y);
}

template <int kMode>
__device__ __forceinline__ void aggregate_internal_node(const AggArgs& a, uint32_t l, uint32_t j,
                                                        uint32_t u) {
    const uint32_t off = a.offset[l], off_below = a.offset[l - 1];
    const uint32_t node = off + j;
    const uint32_t cb = a.node_cbeg[node];
    const uint32_t ce = (j + 1 < u) ? a.node_cbeg[node + 1] : off_below + a.layer_count[l - 1];
    const uint32_t pb = a.pbeg[node];
    const uint32_t pe = (j + 1 < u) ? a.pbeg[node + 1] : a.n;
    if (ce - cb > 8u) atomicOr(a.err, kErrBadLayer);
    const uint32_t nch = min(ce - cb, 8u);
    float4 cm = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 ccm[8];  // children's centres of mass (modes 0 and quadrupoles)
    const bool need_ccm = kMode == 0 || (kMode != 0 && a.want_quad);
    if (need_ccm) {
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k)
            ccm[k] = k < nch ? ld_l2(a.node_cm + cb + k) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (kMode == 0) {
        float m = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
            if (k < nch) {
                const float4 q = ccm[k];
                m = __fadd_rn(m, q.w);
                sx = __fadd_rn(sx, __fmul_rn(q.x, q.w));
                sy = __fadd_rn(sy, __fmul_rn(q.y, q.w));
                sz = __fadd_rn(sz, __fmul_rn(q.z, q.w));
            }
        }
        if (m > 0.f) cm = make_float4(__fdiv_rn(sx, m), __fdiv_rn(sy, m), __fdiv_rn(sz, m), m);
        else cm.w = m;
        if (a.node_ecol) {
            // Children whose emitted colour has alpha > 0: colours summed,
            // centres averaged over those children (Octree.metal:155-178).
            float4 ec = make_float4(0.f, 0.f, 0.f, 0.f), en = ec;
            uint32_t suns = 0;
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) {
                if (k < nch) {
                    const float4 c = ld_l2(a.node_ecol + cb + k);
                    if (c.w > 0.f) {
                        const float4 e = ld_l2(a.node_ecen + cb + k);
                        ec = make_float4(__fadd_rn(ec.x, c.x), __fadd_rn(ec.y, c.y),
                                         __fadd_rn(ec.z, c.z), __fadd_rn(ec.w, c.w));
                        en = make_float4(__fadd_rn(en.x, e.x), __fadd_rn(en.y, e.y),
                                         __fadd_rn(en.z, e.z), 0.f);
                        ++suns;
                    }
                }
            }
            if (suns > 0) {
                const float ns = (float)suns;
                en = make_float4(__fdiv_rn(en.x, ns), __fdiv_rn(en.y, ns), __fdiv_rn(en.z, ns), 0.f);
            }
            a.node_ecol[node] = ec;
            a.node_ecen[node] = en;
        }
    } else if (nch == 1) {
        // One child (most nodes of the lower layers): every sum is the
        // child's (0 + s is exact, and no sum is -0 since all start at +0),
        // so the sums, the centre of mass and the moments equal the child's;
        // copying them is what the arithmetic below would produce.
        if (kMode == 1)
            reinterpret_cast<float4*>(a.node_sum)[node] = ld_l2(reinterpret_cast<const float4*>(a.node_sum) + cb);
        else
            reinterpret_cast<double4*>(a.node_sum)[node] = ld_l2(reinterpret_cast<const double4*>(a.node_sum) + cb);
        cm = need_ccm ? ccm[0] : ld_l2(a.node_cm + cb);
    } else if (kMode == 1) {
        const float4* sum = reinterpret_cast<const float4*>(a.node_sum);
        float4 cs[8];
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) cs[k] = k < nch ? ld_l2(sum + cb + k) : make_float4(0.f, 0.f, 0.f, 0.f);
        float m = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
            if (k < nch) {
                sx = __fadd_rn(sx, cs[k].x);
                sy = __fadd_rn(sy, cs[k].y);
                sz = __fadd_rn(sz, cs[k].z);
                m = __fadd_rn(m, cs[k].w);
            }
        }
        reinterpret_cast<float4*>(a.node_sum)[node] = make_float4(sx, sy, sz, m);
        cm = com_from_sums(sx, sy, sz, m);
    } else {
        const double4* sum = reinterpret_cast<const double4*>(a.node_sum);
        double4 cs[8];
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) cs[k] = k < nch ? ld_l2(sum + cb + k) : make_double4(0.0, 0.0, 0.0, 0.0);
        double m = 0, sx = 0, sy = 0, sz = 0;
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) {
            if (k < nch) {
                sx = __dadd_rn(sx, cs[k].x);
                sy = __dadd_rn(sy, cs[k].y);
                sz = __dadd_rn(sz, cs[k].z);
                m = __dadd_rn(m, cs[k].w);
            }
        }
        reinterpret_cast<double4*>(a.node_sum)[node] = make_double4(sx, sy, sz, m);
        cm = com_from_sums(sx, sy, sz, m);
    }
    a.node_cm[node] = cm;
    a.node_rng[node] = make_uint4(cb, ce, pb, pe);
    if (kMode != 0) {
        if (a.want_quad && nch == 1) {
            a.node_q[node] = ld_l2(a.node_q + cb);
            a.node_qyz[node] = ld_l2(a.node_qyz + cb);
        } else if (a.want_quad) {
            float4 qc[8];
            float qyz[8];
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) {
                qc[k] = k < nch ? ld_l2(a.node_q + cb + k) : make_float4(0.f, 0.f, 0.f, 0.f);
                qyz[k] = k < nch ? ld_l2(a.node_qyz + cb + k) : 0.f;
            }
            float q[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) {
                if (k < nch) {
                    const float4 cc = ccm[k];
                    quad_add(q, cc.w, __fsub_rn(cc.x, cm.x), __fsub_rn(cc.y, cm.y), __fsub_rn(cc.z, cm.z));
                    q[0] = __fadd_rn(q[0], qc[k].x);
                    q[1] = __fadd_rn(q[1], qc[k].y);
                    q[2] = __fadd_rn(q[2], qc[k].z);
                    q[3] = __fadd_rn(q[3], qc[k].w);
                    q[4] = __fadd_rn(q[4], qyz[k]);
                }
            }
            a.node_q[node] = make_float4(q[0], q[1], q[2], q[3]);
            a.node_qyz[node] = q[4];
        }
        if (a.want_delta) a.node_crit2[node] = node_crit2(a, a.node_key[node], l, cm);
        // Groups: a node over the group size packs runs of consecutive
        // small children (greedy, in child order); a small top-layer node is
        // a group by itself.
        const uint32_t gs = a.group_size;
        uint2 cr[8];
        const bool split = pe - pb > gs;
        if (split) {
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k) {
                const uint4 rng = k < nch ? ld_l2(a.node_rng + cb + k) : make_uint4(0u, 0u, 0u, 0u);
                cr[k] = make_uint2(rng.z, rng.w);
            }
        }
        // The packing runs twice: to count the groups, then to write them
        // into the slots reserved for this node.
        auto pack = [&](auto&& emit) {
            if (split) {
                uint32_t gb = 0, ge = 0;
#pragma unroll
                for (uint32_t k = 0; k < 8; ++k) {
                    if (k >= nch) break;
                    const uint32_t cc = cr[k].y - cr[k].x;
                    if (cc <= gs) {
                        if (ge == gb) {
                            gb = cr[k].x;
                            ge = cr[k].y;
                        } else if ((ge - gb) + cc <= gs) {
                            ge = cr[k].y;
                        } else {
                            emit(gb, ge);
                            gb = cr[k].x;
                            ge = cr[k].y;
                        }
                    } else if (ge != gb) {
                        emit(gb, ge);
                        gb = ge = 0;
                    }
                }
                if (ge != gb) emit(gb, ge);
            } else if (l == a.lbits) {
                emit(pb, pe);
            }
        };
        uint32_t c = 0;
        pack([&](uint32_t, uint32_t) { ++c; });
        uint32_t slot = reserve_groups(a.group_count, c);
        pack([&](uint32_t b, uint32_t e) { a.groups[slot++] = make_uint4(b, e, e, 0u); });
    }
}

// Bottom-up aggregation. Layers of at least kClimbMinNodes nodes (capacity)
// run one launch each, a thread per node with coalesced records; the rest
// of the tree runs in one launch that climbs: a thread per node of the
// first small layer aggregates its node, then makes the records visible
// (fence) and counts itself in at the parent; the thread that brings the
// parent's count to its number of children aggregates the parent (reading
// the children through L2) and climbs on; the others stop. Every node is
// aggregated once, after all its children, with the arithmetic of the
// per-node functions above; no thread waits on another. The small top
// layers thus cost one launch instead of one each.
constexpr uint32_t kClimbMinNodes = 32768;
template <int kMode>
__global__ __launch_bounds__(128) void aggregate_leaf_kernel(AggArgs a) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t u0 = a.layer_count[0];
    if (j < u0) aggregate_leaf_node<kMode>(a, j, u0);
}

template <int kMode>
__global__ __launch_bounds__(128) void aggregate_internal_kernel(AggArgs a, uint32_t l) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t u = a.layer_count[l];
    if (j < u) aggregate_internal_node<kMode>(a, l, j, u);
}

// Layers l0 and up in one launch: one thread per node of layer l0.
template <int kMode>
__global__ __launch_bounds__(128) void aggregate_tree_kernel(AggArgs a, uint32_t l0) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t u0 = a.layer_count[l0];
    if (j >= u0) return;
    if (l0 == 0) aggregate_leaf_node<kMode>(a, j, u0);
    else aggregate_internal_node<kMode>(a, l0, j, u0);
    uint32_t node = a.offset[l0] + j;
    for (uint32_t l = l0 + 1; l <= a.lbits; ++l) {
        const uint32_t p = a.parent[node];
        if (p == kNoParent) return;
        const uint32_t u = a.layer_count[l];
        const uint32_t jp = p - a.offset[l];
        if (jp >= u) {
            atomicOr(a.err, kErrBadLayer);
            return;
        }
        const uint32_t cb = a.node_cbeg[p];
        const uint32_t ce = (jp + 1 < u) ? a.node_cbeg[p + 1] : a.offset[l - 1] + a.layer_count[l - 1];
        if (ce - cb > 1u) {
            __threadfence();
            if (atomicAdd(&a.arrive[p], 1u) != ce - cb - 1u) return;
            __threadfence();
        }
        aggregate_internal_node<kMode>(a, l, jp, u);
        node = p;
    }
}

// ---------------------------------------------------------- integrate ----

// updateSpheres (BarnesHut.metal:169-196): a = F * scale[type];
// v = v * damping + a * dt; x += v * dt.
__global__ void integrate_ref_kernel(float4* __restrict__ pos, float4* __restrict__ vel,
                                     const float4* __restrict__ acc,
                                     const uint32_t* __restrict__ types, uint32_t n, float dt,
                                     float damping, float s0, float s1, float s2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = acc[i];
    const uint32_t t = types[i];
    if (t <= 2u) {
        const float s = t == 0 ? s0 : (t == 1 ? s1 : s2);
        a.x = __fmul_rn(a.x, s);
        a.y = __fmul_rn(a.y, s);
        a.z = __fmul_rn(a.z, s);
    }
    float4 v = vel[i];
    v.x = __fadd_rn(__fmul_rn(v.x, damping), __fmul_rn(a.x, dt));
    v.y = __fadd_rn(__fmul_rn(v.y, damping), __fmul_rn(a.y, dt));
    v.z = __fadd_rn(__fmul_rn(v.z, damping), __fmul_rn(a.z, dt));
    vel[i] = v;
    float4 p = pos[i];
    p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
    p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
    p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
    pos[i] = p;
}

// ------------------------------------------------- upload / download -----

template <bool kPrec>
__global__ void upload_convert_kernel(const PositionMass* __restrict__ pm,
                                      const VelocityRadius* __restrict__ vr,
                                      const ColorType* __restrict__ ct, float4* __restrict__ pos,
                                      float4* __restrict__ vel, uint32_t* __restrict__ ids,
                                      uint32_t* __restrict__ types, double* __restrict__ x64,
                                      uint32_t n, uint32_t n_tree) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p0 = *reinterpret_cast<const float4*>(&pm[i].position[0]);
    const float m = pm[i].mass;
    const float4 v0 = *reinterpret_cast<const float4*>(&vr[i].velocity[0]);
    pos[i] = make_float4(p0.x, p0.y, p0.z, m);
    vel[i] = make_float4(v0.x, v0.y, v0.z, vr[i].radius);
    if (ids) ids[i] = i;
    if (types) types[i] = ct ? ct[i].type : (i < n_tree ? 1u : 2u);
    if (kPrec) {
        x64[i] = (double)p0.x;
        x64[(size_t)n + i] = (double)p0.y;
        x64[2 * (size_t)n + i] = (double)p0.z;
    }
}

template <bool kPrec>
__global__ void download_convert_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                        const uint32_t* __restrict__ ids,
                                        const double* __restrict__ x64, PositionMass* __restrict__ pm,
                                        VelocityRadius* __restrict__ vr, uint32_t n) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t i = ids ? ids[j] : j;
    const float4 p = pos[j], v = vel[j];
    float4 out_p = make_float4(p.x, p.y, p.z, 0.f);
    if (kPrec)
        out_p = make_float4(__double2float_rn(x64[j]), __double2float_rn(x64[(size_t)n + j]),
                            __double2float_rn(x64[2 * (size_t)n + j]), 0.f);
    *reinterpret_cast<float4*>(&pm[i].position[0]) = out_p;
    *reinterpret_cast<float4*>(&pm[i].mass) = make_float4(p.w, 0.f, 0.f, 0.f);
    *reinterpret_cast<float4*>(&vr[i].velocity[0]) = make_float4(v.x, v.y, v.z, 0.f);
    *reinterpret_cast<float4*>(&vr[i].radius) = make_float4(v.w, 0.f, 0.f, 0.f);
}

// The same conversion as a gather: output slot o (upload order) reads state
// slot inv[o] (inv = the inverse of ids), so the 64 bytes written per
// particle are contiguous across a warp and only the reads are scattered.
template <bool kPrec>
__global__ void download_gather_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                       const uint32_t* __restrict__ inv,
                                       const double* __restrict__ x64, PositionMass* __restrict__ pm,
                                       VelocityRadius* __restrict__ vr, uint32_t n) {
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const uint32_t j = inv ? __ldg(&inv[o]) : o;
    const float4 p = __ldg(&pos[j]), v = __ldg(&vel[j]);
    float4 out_p = make_float4(p.x, p.y, p.z, 0.f);
    if (kPrec)
        out_p = make_float4(__double2float_rn(x64[j]), __double2float_rn(x64[(size_t)n + j]),
                            __double2float_rn(x64[2 * (size_t)n + j]), 0.f);
    *reinterpret_cast<float4*>(&pm[o].position[0]) = out_p;
    *reinterpret_cast<float4*>(&pm[o].mass) = make_float4(p.w, 0.f, 0.f, 0.f);
    *reinterpret_cast<float4*>(&vr[o].velocity[0]) = make_float4(v.x, v.y, v.z, 0.f);
    *reinterpret_cast<float4*>(&vr[o].radius) = make_float4(v.w, 0.f, 0.f, 0.f);
}

// Scatter a per-state-slot array back to upload order through ids.
template <typename T>
__global__ void scatter_by_id_kernel(const T* __restrict__ src, const uint32_t* __restrict__ ids,
                                     T* __restrict__ dst, uint32_t n) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    dst[ids ? ids[j] : j] = src[j];
}

// AoS OctreeNode (bridge.h:47-65) for the slots [first, first+count) of
// layer l; slots past the live count read as the cleared node
// (clearOctreeNodeBuffer, Octree.metal:253-269).
__global__ void readback_nodes_kernel(const float4* __restrict__ node_cm,
                                      const uint4* __restrict__ node_rng,
                                      const uint64_t* __restrict__ node_key,
                                      const float4* __restrict__ node_ecol,
                                      const float4* __restrict__ node_ecen,
                                      const uint32_t* __restrict__ layer_count, uint32_t l,
                                      uint32_t layer_offset, uint32_t first_in_layer,
                                      uint32_t count, OctreeNode* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t j = first_in_layer + k;
    OctreeNode o;
    uint32_t* w = reinterpret_cast<uint32_t*>(&o);
    for (int q = 0; q < 32; ++q) w[q] = 0;
    o.mortonCode = ASTRO_INVALID_MORTON_CODE;
    for (int c = 0; c < 8; ++c) o.children[c] = ASTRO_INVALID_CHILD;
    if (j < layer_count[l]) {
        const uint32_t node = layer_offset + j;
        const float4 cm = node_cm[node];
        o.mortonCode = node_key[node];
        o.centerOfMass[0] = cm.x;
        o.centerOfMass[1] = cm.y;
        o.centerOfMass[2] = cm.z;
        o.totalMass = cm.w;
        o.layer = l;
        if (node_ecol) {
            const float4 ec = node_ecol[node], en = node_ecen[node];
            o.emittedColor[0] = ec.x;
            o.emittedColor[1] = ec.y;
            o.emittedColor[2] = ec.z;
            o.emittedColor[3] = ec.w;
            o.emittedColorCenter[0] = en.x;
            o.emittedColorCenter[1] = en.y;
            o.emittedColorCenter[2] = en.z;
        }
        if (l > 0) {
            const uint4 r = node_rng[node];
            for (uint32_t c = 0; c < 8 && r.x + c < r.y; ++c) o.children[c] = r.x + c;
        }
    }
    out[k] = o;
}

// ------------------------------------------------ FP64 direct sum --------

constexpr int kDirectSamples = 8;

// Softened FP64 direct sum for sampled particles (error reference). Each
// block takes kDirectSamples samples and one slice of their particles
// (threads stride over it) and adds its partial sums to the output.
__global__ __launch_bounds__(256) void direct_sum_f64_kernel(DirectArgs a) {
    __shared__ double s_red[8][kDirectSamples][3];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t first = blockIdx.x * kDirectSamples;
    double xi[kDirectSamples][3], acc[kDirectSamples][3];
    uint32_t self[kDirectSamples], lo[kDirectSamples], hi[kDirectSamples];
    uint32_t glo = 0xFFFFFFFFu, ghi = 0;
    for (int s = 0; s < kDirectSamples; ++s) {
        const uint32_t k = first + s;
        const bool ok = k < a.n_sample;
        const uint32_t slot = ok ? a.slot[k] : 0u;
        self[s] = ok ? slot : 0xFFFFFFFFu;
        lo[s] = ok ? a.sys_begin[k] : 1u;
        hi[s] = ok ? a.sys_end[k] : 0u;
        if (ok) {
            glo = min(glo, lo[s]);
            ghi = max(ghi, hi[s]);
        }
        for (int c = 0; c < 3; ++c) {
            xi[s][c] = ok ? (a.x64 ? a.x64[(size_t)c * a.n + slot]
                                   : (double)(&a.pos[slot].x)[c])
                          : 0.0;
            acc[s][c] = 0.0;
        }
    }
    // blockIdx.y takes one of gridDim.y slices of the samples' particle range.
    const uint32_t span = ghi > glo ? ghi - glo : 0u;
    const uint32_t per = (span + gridDim.y - 1) / gridDim.y;
    const uint32_t jb = glo + blockIdx.y * per, je = min(ghi, jb + per);
    for (uint32_t j = jb + tid; j < je; j += blockDim.x) {
        const float4 q = a.pos[j];
        double xj[3];
        for (int c = 0; c < 3; ++c)
            xj[c] = a.x64 ? a.x64[(size_t)c * a.n + j] : (double)(&q.x)[c];
        const double gm = a.g * (double)q.w;
        for (int s = 0; s < kDirectSamples; ++s) {
            if (j < lo[s] || j >= hi[s] || j == self[s]) continue;
            const double dx = xj[0] - xi[s][0], dy = xj[1] - xi[s][1], dz = xj[2] - xi[s][2];
            const double r2 = dx * dx + dy * dy + dz * dz + a.eps2;
            const double inv = 1.0 / sqrt(r2);
            const double w = gm * inv * inv * inv;
            acc[s][0] += w * dx;
            acc[s][1] += w * dy;
            acc[s][2] += w * dz;
        }
    }
    for (int s = 0; s < kDirectSamples; ++s)
        for (int c = 0; c < 3; ++c) {
            double v = acc[s][c];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
            if (lane == 0) s_red[warp][s][c] = v;
        }
    __syncthreads();
    if (tid < kDirectSamples * 3) {
        const int s = tid / 3, c = tid % 3;
        double v = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) v += s_red[w][s][c];
        if (first + s < a.n_sample) atomicAdd(&a.out[3ull * (first + s) + c], v);
    }
}

__global__ void gather_u32_kernel(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx,
                                  uint32_t* __restrict__ dst, uint32_t n) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[idx[k]];
}

__global__ void types_from_colors_kernel(const ColorType* __restrict__ ct, uint32_t* __restrict__ types,
                                         float4* __restrict__ colors, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    types[i] = ct[i].type;
    if (colors) colors[i] = *reinterpret_cast<const float4*>(&ct[i].color[0]);
}

// lightingPass (BarnesHut.metal:103-167) for the particles in upload order:
// the lights' positions and colours (lights[0..nl) and lights[kMaxLights..])
// were copied before the pass, so no light reads a colour written here.
constexpr uint32_t kMaxLights = 5;
constexpr float kLightAttenuation = 4e5f;  // LIGHT_ATTENUATION_DISTANCE, bridge.h:98

__global__ void lights_snapshot_kernel(const float4* __restrict__ pos,
                                       const float4* __restrict__ colors, float4* __restrict__ lights,
                                       uint32_t nl) {
    const uint32_t s = threadIdx.x;
    if (s < nl) {
        lights[s] = pos[s];
        lights[kMaxLights + s] = colors[s];
    }
}

__global__ void lighting_kernel(const float4* __restrict__ pos, const uint32_t* __restrict__ types,
                                const float4* __restrict__ lights, float4* __restrict__ colors,
                                uint32_t n, uint32_t nl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t type = types[i];
    if (type != 1u && type != 2u) return;
    const float4 p = pos[i];
    float lr = 0.f, lg = 0.f, lb = 0.f;
    for (uint32_t s = 0; s < nl; ++s) {
        const float4 q = lights[s], c = lights[kMaxLights + s];
        const float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
        const float dist =
            __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        const float dn = fmaxf(__fdiv_rn(dist, kLightAttenuation), 1e-9f);
        const float att = __fdiv_rn(1.0f, __fmul_rn(dn, dn));
        lr = __fadd_rn(lr, __fmul_rn(c.x, att));
        lg = __fadd_rn(lg, __fmul_rn(c.y, att));
        lb = __fadd_rn(lb, __fmul_rn(c.z, att));
    }
    const float a = type == 2u ? fminf(fmaxf(lr, fmaxf(lg, lb)), 0.25f) : 1.0f;
    colors[i] = make_float4(lr, lg, lb, a);
}

// ColorType in upload order from colours and types.
__global__ void colors_out_kernel(const float4* __restrict__ colors, const uint32_t* __restrict__ types,
                                  ColorType* __restrict__ out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    *reinterpret_cast<float4*>(&out[i].color[0]) = colors[i];
    *reinterpret_cast<uint4*>(&out[i].type) = make_uint4(types[i], 0u, 0u, 0u);
}

// Stand-alone PHYSICAL kick-drift (the same arithmetic as the traversal
// epilogue): v += a dt, x += v dt, x in FP64 in the precision form.
template <bool kPrec>
__global__ void kick_drift_kernel(float4* __restrict__ pos, float4* __restrict__ vel,
                                  double* __restrict__ x64, const float4* __restrict__ acc,
                                  uint32_t n, float dt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = acc[i];
    float4 v = vel[i];
    v.x = __fadd_rn(v.x, __fmul_rn(a.x, dt));
    v.y = __fadd_rn(v.y, __fmul_rn(a.y, dt));
    v.z = __fadd_rn(v.z, __fmul_rn(a.z, dt));
    vel[i] = v;
    if (kPrec) {
        const double ddt = (double)dt;
        x64[i] = __dadd_rn(x64[i], __dmul_rn((double)v.x, ddt));
        x64[(size_t)n + i] = __dadd_rn(x64[(size_t)n + i], __dmul_rn((double)v.y, ddt));
        x64[2 * (size_t)n + i] = __dadd_rn(x64[2 * (size_t)n + i], __dmul_rn((double)v.z, ddt));
    } else {
        float4 p = pos[i];
        p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
        p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
        p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
        pos[i] = p;
    }
}

__global__ void inverse_ids_kernel(const uint32_t* __restrict__ ids, uint32_t* __restrict__ inv,
                                   uint32_t n) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) inv[ids[j]] = j;
}

// ------------------------------------------------------------ launchers --

namespace {
inline uint32_t blocks_for(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }
}  // namespace

cudaError_t launch_encode_ref(const float4* pos, uint64_t* codes, uint32_t n_tree, uint32_t lbits,
                              float offset, cudaStream_t st) {
    if (n_tree == 0) return cudaSuccess;
    encode_ref_kernel<<<blocks_for(n_tree, 256), 256, 0, st>>>(pos, codes, n_tree, 63u - 3u * lbits,
                                                               offset);
    return cudaGetLastError();
}

cudaError_t launch_encode_phys(bool prec, const Chunk* chunks, uint32_t nchunks, const SysInfo* sys,
                               float4* pos, const double* x64, uint64_t* codes, uint32_t n,
                               uint32_t lbits, cudaStream_t st) {
    if (prec)
        encode_phys_kernel<true><<<nchunks, 256, 0, st>>>(chunks, sys, pos, x64, codes, n, lbits);
    else
        encode_phys_kernel<false><<<nchunks, 256, 0, st>>>(chunks, sys, pos, x64, codes, n, lbits);
    return cudaGetLastError();
}

cudaError_t launch_bbox(bool prec, const Chunk* chunks, uint32_t nchunks, const float4* pos,
                        const double* x64, uint32_t n, uint32_t* bb32, unsigned long long* bb64,
                        cudaStream_t st) {
    if (prec) bbox_kernel<true><<<nchunks, 256, 0, st>>>(chunks, pos, x64, n, bb32, bb64);
    else bbox_kernel<false><<<nchunks, 256, 0, st>>>(chunks, pos, x64, n, bb32, bb64);
    return cudaGetLastError();
}

cudaError_t launch_setup(bool prec, SysInfo* sys, uint32_t nsys, uint32_t* bb32,
                         unsigned long long* bb64, uint32_t lbits, float theta, uint32_t root_offset,
                         cudaStream_t st) {
    if (prec)
        setup_kernel<true><<<blocks_for(nsys, 128), 128, 0, st>>>(sys, nsys, bb32, bb64, lbits,
                                                                  theta, root_offset);
    else
        setup_kernel<false><<<blocks_for(nsys, 128), 128, 0, st>>>(sys, nsys, bb32, bb64, lbits,
                                                                   theta, root_offset);
    return cudaGetLastError();
}

cudaError_t launch_reorder(bool prec, const uint32_t* perm, const float4* pos_a, const float4* vel_a,
                           const uint32_t* id_a, const double* x_a, float4* pos_b, float4* vel_b,
                           uint32_t* id_b, double* x_b, uint32_t n, cudaStream_t st) {
    if (prec)
        reorder_kernel<true><<<blocks_for(n, 256), 256, 0, st>>>(perm, pos_a, vel_a, id_a, x_a,
                                                                 pos_b, vel_b, id_b, x_b, n);
    else
        reorder_kernel<false><<<blocks_for(n, 256), 256, 0, st>>>(perm, pos_a, vel_a, id_a, x_a,
                                                                  pos_b, vel_b, id_b, x_b, n);
    return cudaGetLastError();
}

uint32_t topology_tiles(uint32_t n) { return blocks_for(n, kTopoTile); }

cudaError_t launch_topology(const TopoArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    topology_kernel<<<a.ntiles, kTopoThreads, 0, st>>>(a);
    return cudaGetLastError();
}

uint32_t climb_first_layer(const LayerTable& t) {
    uint32_t l0 = 0;
    while (l0 + 1 < t.n_layers && t.size[l0] >= kClimbMinNodes) ++l0;
    return l0;
}

cudaError_t launch_aggregate(int mode, const AggArgs& a, const LayerTable& t, cudaStream_t st) {
    const uint32_t t0 = 128;
    const uint32_t l0 = climb_first_layer(t);
    for (uint32_t l = 0; l < l0; ++l) {
        const uint32_t g = blocks_for(t.size[l], t0);
        if (l == 0) {
            if (mode == 0) aggregate_leaf_kernel<0><<<g, t0, 0, st>>>(a);
            else if (mode == 1) aggregate_leaf_kernel<1><<<g, t0, 0, st>>>(a);
            else aggregate_leaf_kernel<2><<<g, t0, 0, st>>>(a);
        } else {
            if (mode == 0) aggregate_internal_kernel<0><<<g, t0, 0, st>>>(a, l);
            else if (mode == 1) aggregate_internal_kernel<1><<<g, t0, 0, st>>>(a, l);
            else aggregate_internal_kernel<2><<<g, t0, 0, st>>>(a, l);
        }
    }
    const uint32_t g = blocks_for(t.size[l0], t0);
    if (mode == 0) aggregate_tree_kernel<0><<<g, t0, 0, st>>>(a, l0);
    else if (mode == 1) aggregate_tree_kernel<1><<<g, t0, 0, st>>>(a, l0);
    else aggregate_tree_kernel<2><<<g, t0, 0, st>>>(a, l0);
    return cudaGetLastError();
}

cudaError_t launch_integrate_ref(float4* pos, float4* vel, const float4* acc, const uint32_t* types,
                                 uint32_t n, float dt, const astro_params& p, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    integrate_ref_kernel<<<blocks_for(n, 256), 256, 0, st>>>(
        pos, vel, acc, types, n, dt, p.damping, p.type_accel_scale[0], p.type_accel_scale[1],
        p.type_accel_scale[2]);
    return cudaGetLastError();
}

cudaError_t launch_upload_convert(bool prec, const PositionMass* pm, const VelocityRadius* vr,
                                  const ColorType* ct, float4* pos, float4* vel, uint32_t* ids,
                                  uint32_t* types, double* x64, uint32_t n, uint32_t n_tree,
                                  cudaStream_t st) {
    if (prec)
        upload_convert_kernel<true><<<blocks_for(n, 256), 256, 0, st>>>(pm, vr, ct, pos, vel, ids,
                                                                        types, x64, n, n_tree);
    else
        upload_convert_kernel<false><<<blocks_for(n, 256), 256, 0, st>>>(pm, vr, ct, pos, vel, ids,
                                                                         types, x64, n, n_tree);
    return cudaGetLastError();
}

cudaError_t launch_download_convert(bool prec, const float4* pos, const float4* vel,
                                    const uint32_t* ids, const double* x64, PositionMass* pm,
                                    VelocityRadius* vr, uint32_t n, cudaStream_t st,
                                    uint32_t* inv_scratch) {
    if (inv_scratch || !ids) {
        // The inverse permutation (a 4-byte scatter), then a gather with
        // contiguous 64-byte writes.
        if (ids) inverse_ids_kernel<<<blocks_for(n, 256), 256, 0, st>>>(ids, inv_scratch, n);
        const uint32_t* inv = ids ? inv_scratch : nullptr;
        if (prec)
            download_gather_kernel<true><<<blocks_for(n, 256), 256, 0, st>>>(pos, vel, inv, x64, pm,
                                                                             vr, n);
        else
            download_gather_kernel<false><<<blocks_for(n, 256), 256, 0, st>>>(pos, vel, inv, x64, pm,
                                                                              vr, n);
        return cudaGetLastError();
    }
    if (prec)
        download_convert_kernel<true><<<blocks_for(n, 256), 256, 0, st>>>(pos, vel, ids, x64, pm,
                                                                          vr, n);
    else
        download_convert_kernel<false><<<blocks_for(n, 256), 256, 0, st>>>(pos, vel, ids, x64, pm,
                                                                           vr, n);
    return cudaGetLastError();
}

cudaError_t launch_scatter_u64(const uint64_t* src, const uint32_t* ids, uint64_t* dst, uint32_t n,
                               cudaStream_t st) {
    scatter_by_id_kernel<uint64_t><<<blocks_for(n, 256), 256, 0, st>>>(src, ids, dst, n);
    return cudaGetLastError();
}
cudaError_t launch_scatter_f4(const float4* src, const uint32_t* ids, float4* dst, uint32_t n,
                              cudaStream_t st) {
    scatter_by_id_kernel<float4><<<blocks_for(n, 256), 256, 0, st>>>(src, ids, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_readback_nodes(const float4* cm, const uint4* rng, const uint64_t* key,
                                  const float4* ecol, const float4* ecen,
                                  const uint32_t* layer_count, uint32_t l, uint32_t layer_offset,
                                  uint32_t first_in_layer, uint32_t count, OctreeNode* out,
                                  cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    readback_nodes_kernel<<<blocks_for(count, 128), 128, 0, st>>>(
        cm, rng, key, ecol, ecen, layer_count, l, layer_offset, first_in_layer, count, out);
    return cudaGetLastError();
}

cudaError_t launch_direct_sum(const DirectArgs& a, cudaStream_t st) {
    if (a.n_sample == 0) return cudaSuccess;
    // Sample blocks times slices of the particle range (each slice adds its
    // partial sums), about 1,024 blocks in all, slices of at least 8,192.
    const uint32_t xb = blocks_for(a.n_sample, kDirectSamples);
    const uint32_t ys = std::max(1u, std::min((1024u + xb - 1) / xb, (a.n + 8191u) / 8192u));
    cudaError_t e = cudaMemsetAsync(a.out, 0, 24ull * a.n_sample, st);
    if (e != cudaSuccess) return e;
    direct_sum_f64_kernel<<<dim3(xb, ys), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_inverse_ids(const uint32_t* ids, uint32_t* inv, uint32_t n, cudaStream_t st) {
    inverse_ids_kernel<<<blocks_for(n, 256), 256, 0, st>>>(ids, inv, n);
    return cudaGetLastError();
}

cudaError_t launch_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t* dst, uint32_t n,
                              cudaStream_t st) {
    gather_u32_kernel<<<blocks_for(n, 256), 256, 0, st>>>(src, idx, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_types_from_colors(const ColorType* ct, uint32_t* types, float4* colors, uint32_t n,
                                     cudaStream_t st) {
    types_from_colors_kernel<<<blocks_for(n, 256), 256, 0, st>>>(ct, types, colors, n);
    return cudaGetLastError();
}

cudaError_t launch_lighting(const float4* pos, const uint32_t* types, float4* colors, float4* lights,
                            uint32_t n, uint32_t num_stars, cudaStream_t st) {
    const uint32_t nl = std::min(std::min(num_stars, kMaxLights), n);
    if (n == 0) return cudaSuccess;
    if (nl > 0) lights_snapshot_kernel<<<1, 32, 0, st>>>(pos, colors, lights, nl);
    lighting_kernel<<<blocks_for(n, 256), 256, 0, st>>>(pos, types, lights, colors, n, nl);
    return cudaGetLastError();
}

cudaError_t launch_colors_out(const float4* colors, const uint32_t* types, ColorType* out, uint32_t n,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    colors_out_kernel<<<blocks_for(n, 256), 256, 0, st>>>(colors, types, out, n);
    return cudaGetLastError();
}

cudaError_t launch_kick_drift(bool prec, float4* pos, float4* vel, double* x64, const float4* acc,
                              uint32_t n, float dt, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (prec) kick_drift_kernel<true><<<blocks_for(n, 256), 256, 0, st>>>(pos, vel, x64, acc, n, dt);
    else kick_drift_kernel<false><<<blocks_for(n, 256), 256, 0, st>>>(pos, vel, x64, acc, n, dt);
    return cudaGetLastError();
}

}  // namespace astro
