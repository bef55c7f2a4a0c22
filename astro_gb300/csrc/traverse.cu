// Barnes-Hut force traversal: barnesHut (Astro/BarnesHut.metal:22-101).
//
// traverse_ref_kernel — the REFERENCE preset: one thread per particle in
//   upload order, a private stack, node size 2^(21+layer), monopole leaves
//   with the self-leaf skip and the r^2 > leaf_min cut, softening added to
//   r^2, clamp; correctly rounded FP32 operations in the reference's order.
//
// traverse_phys_kernel — the PHYSICAL preset: one warp per 32 consecutive
//   Morton-ordered particles. The warp walks the tree once for all its
//   lanes with a shared stack of child ranges {begin, end, layer, lane mask};
//   a lane only evaluates nodes whose mask holds its bit, and a node is
//   opened for the lanes that reject it, so every lane makes exactly the
//   decisions of its own depth-first walk, in the same order (children are
//   taken last first, as the reference's LIFO stack pops them). Node
//   records (SoA float4 centre of mass/mass + uint4 ranges) are read through
//   the read-only path as warp-broadcast loads. Opened leaves and buckets are
//   staged 32 particles at a time in shared memory and summed particle by
//   particle. The epilogue clamps, stores the acceleration and performs the
//   kick-drift (v += a dt, x += v dt).
#include <algorithm>

#include "build_kernels.cuh"
#include "common.cuh"
#include "traverse_terms.cuh"

namespace astro {

constexpr int kRefStack = 160;   // >= 7 * 21 + 1 entries (8 children per opened node)
constexpr int kPhysStack = 64;   // >= 32 roots + 22 layers of ranges

__global__ __launch_bounds__(128) void traverse_ref_kernel(TraverseArgs a) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= a.n) return;
    uint32_t st_node[kRefStack];
    uint8_t st_layer[kRefStack];
    uint32_t sp = 0;
    st_node[sp] = a.root;
    st_layer[sp] = (uint8_t)a.lbits;
    ++sp;
    const float4 me = a.pos[gid];
    const uint32_t type = a.types[gid];
    const uint64_t my_code =
        (type != 2u && gid < a.n_tree) ? a.codes[gid] : ASTRO_INVALID_MORTON_CODE;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    uint32_t inter = 0, visits = 0;
    while (sp > 0) {
        --sp;
        const uint32_t nd = st_node[sp];
        const uint32_t layer = st_layer[sp];
        ++visits;
        const float4 c = __ldg(&a.node_cm[nd]);
        const float dx = __fsub_rn(c.x, me.x), dy = __fsub_rn(c.y, me.y), dz = __fsub_rn(c.z, me.z);
        float dist_sqr = __fadd_rn(
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)), a.eps2);
        dist_sqr = fmaxf(dist_sqr, 1e-6f);
        float dist = __fsqrt_rn(dist_sqr);
        dist = fmaxf(dist, 1e-6f);
        const bool is_leaf = layer == 0;
        bool add = false;
        if (is_leaf) {
            const bool is_self = type != 2u && my_code == __ldg(&a.node_key[nd]);
            add = !is_self && dist_sqr > a.leaf_min_dist2;
        } else if (__fdiv_rn(exp2_exact(21 + (int)layer), dist) < a.theta) {
            add = true;
        } else {
            const uint4 r = __ldg(&a.node_rng[nd]);
            for (uint32_t ch = r.x; ch < r.y; ++ch) {
                if (sp < kRefStack) {
                    st_node[sp] = ch;
                    st_layer[sp] = (uint8_t)(layer - 1);
                    ++sp;
                } else {
                    atomicOr(a.err, kErrStackOverflow);
                }
            }
        }
        if (add) {
            const float gm = __fmul_rn(a.g, c.w), den = __fmul_rn(dist_sqr, dist);
            fx = __fadd_rn(fx, __fdiv_rn(__fmul_rn(gm, dx), den));
            fy = __fadd_rn(fy, __fdiv_rn(__fmul_rn(gm, dy), den));
            fz = __fadd_rn(fz, __fdiv_rn(__fmul_rn(gm, dz), den));
            ++inter;
        }
    }
    const float cl = a.clampv;
    a.acc[gid] = make_float4(fminf(fmaxf(fx, -cl), cl), fminf(fmaxf(fy, -cl), cl),
                             fminf(fmaxf(fz, -cl), cl), 0.f);
    atomicAdd(&a.stats[0], (unsigned long long)inter);
    atomicAdd(&a.stats[1], (unsigned long long)visits);
    atomicAdd(&a.stats[2], (unsigned long long)inter);
}

template <bool kExact, bool kPrec, bool kBatched, bool kPersistent, int kWarps>
__global__ __launch_bounds__(kWarps * 32) void traverse_phys_kernel(TraverseArgs a) {
    __shared__ uint4 s_stack[kWarps][kPhysStack];
    __shared__ float4 s_tile[kWarps][32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t nchunks = (a.n + 31u) / 32u;
    const float g = a.g, eps2 = a.eps2;
    uint32_t inter = 0, visits = 0, cell_inter = 0;
    uint32_t chunk = blockIdx.x * kWarps + warp;
    while (true) {
        if (kPersistent) {
            uint32_t c = 0;
            if (lane == 0) c = atomicAdd(a.queue, 1u);
            chunk = __shfl_sync(kFullMask, c, 0);
        }
        if (chunk >= nchunks) break;
        const uint32_t ip = chunk * 32u + lane;
        const bool valid = ip < a.n;
        const float4 me = valid ? a.pos[ip] : make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t sys = 0;
        if (kBatched) sys = valid ? (uint32_t)(a.sorted_keys[ip] >> (3u * a.lbits)) : 0u;
        const float* crit2 = a.sys[sys].crit2;
        const uint32_t valid_mask = __ballot_sync(kFullMask, valid);

        // The current range lives in registers (the same in every lane); the
        // ranges below it wait in the warp's shared-memory stack.
        uint32_t sp = 0;
        uint4 cur;
        if (kBatched) {
            // One root range per system present in the warp.
            uint32_t rem = valid_mask;
            bool first = true;
            while (rem) {
                const uint32_t leader = __ffs(rem) - 1;
                const uint32_t s = __shfl_sync(kFullMask, sys, leader);
                const uint32_t grp = __ballot_sync(kFullMask, valid && sys == s);
                const uint32_t root = a.sys[s].root;
                const uint4 e = make_uint4(root, root + 1, a.lbits, grp);
                if (first) {
                    cur = e;
                    first = false;
                } else {
                    if (lane == 0) s_stack[warp][sp] = e;
                    ++sp;
                }
                rem &= ~grp;
            }
        } else {
            cur = make_uint4(a.root, a.root + 1, a.lbits, valid_mask);
        }
        __syncwarp();

        Accum<kExact, kPrec> acc;
        bool more = valid_mask != 0;
        while (more) {
            const uint32_t nd = cur.y - 1;
            cur.y = nd;
            const bool exhausted = cur.y == cur.x;
            const uint32_t layer = cur.z;
            const bool active = (cur.w >> lane) & 1u;
            const float4 c = __ldg(&a.node_cm[nd]);
            const float dx = __fsub_rn(c.x, me.x), dy = __fsub_rn(c.y, me.y),
                        dz = __fsub_rn(c.z, me.z);
            const float r2t =
                __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const float crit = a.delta ? __ldg(&a.node_crit2[nd]) : __ldg(&crit2[layer]);
            const bool accept = active && r2t > crit;
            if (accept) {
                float tx, ty, tz;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                float qyz = 0.f;
                if (a.quad) {
                    q = __ldg(&a.node_q[nd]);
                    qyz = __ldg(&a.node_qyz[nd]);
                }
                cell_term<kExact>(dx, dy, dz, r2t, c.w, a.quad != 0, q, qyz, g, eps2, tx, ty, tz);
                acc.add(tx, ty, tz);
                ++inter;
                ++cell_inter;
            }
            visits += active ? 1u : 0u;
            const uint32_t open_mask = __ballot_sync(kFullMask, active && !accept);
            if (open_mask != 0) {
                const uint4 r = __ldg(&a.node_rng[nd]);
                if (layer != 0 && r.w - r.z > a.bucket) {
                    // Open: descend into the children, keep the rest of this range.
                    if (!exhausted) {
                        if (sp < (uint32_t)kPhysStack) {
                            if (lane == 0) s_stack[warp][sp] = cur;
                            ++sp;
                        } else if (lane == 0) {
                            atomicOr(a.err, kErrStackOverflow);
                        }
                    }
                    cur = make_uint4(r.x, r.y, layer - 1, open_mask);
                    continue;
                }
                // Leaf or bucket: particle-particle sums over 32-particle tiles.
                const bool open = (open_mask >> lane) & 1u;
                for (uint32_t t = r.z; t < r.w; t += 32u) {
                    const uint32_t j = t + lane;
                    if (j < r.w) s_tile[warp][lane] = __ldg(&a.pos[j]);
                    __syncwarp();
                    const uint32_t cnt = min(32u, r.w - t);
                    if (open) {
                        for (uint32_t q = 0; q < cnt; ++q) {
                            const float4 p = s_tile[warp][q];
                            if (t + q != ip) {
                                float tx, ty, tz;
                                particle_term<kExact>(__fsub_rn(p.x, me.x), __fsub_rn(p.y, me.y),
                                                      __fsub_rn(p.z, me.z), p.w, g, eps2, tx, ty, tz);
                                acc.add(tx, ty, tz);
                            }
                        }
                        inter += cnt - ((ip - t) < cnt ? 1u : 0u);
                    }
                    __syncwarp();
                }
            }
            if (exhausted) {
                if (sp == 0) {
                    more = false;
                } else {
                    __syncwarp();
                    cur = s_stack[warp][--sp];
                }
            }
        }

        if (valid) {
            const float cl = a.clampv, dt = a.dt;
            const float ax = fminf(fmaxf(acc.ax, -cl), cl);
            const float ay = fminf(fmaxf(acc.ay, -cl), cl);
            const float az = fminf(fmaxf(acc.az, -cl), cl);
            a.acc[ip] = make_float4(ax, ay, az, 0.f);
            // Kick-drift: updateSpheres' v += a dt, x += v dt (no damping).
            float4 v = a.vel_in[ip];
            v.x = __fadd_rn(v.x, __fmul_rn(ax, dt));
            v.y = __fadd_rn(v.y, __fmul_rn(ay, dt));
            v.z = __fadd_rn(v.z, __fmul_rn(az, dt));
            a.vel_out[ip] = v;
            a.id_out[ip] = a.id_in[ip];
            if (kPrec) {
                const size_t n = a.n;
                const double ddt = (double)dt;
                a.x64_out[ip] = __dadd_rn(a.x64_in[ip], __dmul_rn((double)v.x, ddt));
                a.x64_out[n + ip] = __dadd_rn(a.x64_in[n + ip], __dmul_rn((double)v.y, ddt));
                a.x64_out[2 * n + ip] = __dadd_rn(a.x64_in[2 * n + ip], __dmul_rn((double)v.z, ddt));
                a.pos_out[ip] = me;
            } else {
                a.pos_out[ip] = make_float4(__fadd_rn(me.x, __fmul_rn(v.x, dt)),
                                            __fadd_rn(me.y, __fmul_rn(v.y, dt)),
                                            __fadd_rn(me.z, __fmul_rn(v.z, dt)), me.w);
            }
        }
        if (!kPersistent) break;
    }
    // Statistics: one atomic per warp.
    unsigned long long i64 = inter, v64 = visits, c64 = cell_inter;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        i64 += __shfl_xor_sync(kFullMask, i64, o);
        v64 += __shfl_xor_sync(kFullMask, v64, o);
        c64 += __shfl_xor_sync(kFullMask, c64, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stats[0], i64);
        atomicAdd(&a.stats[1], v64);
        atomicAdd(&a.stats[2], c64);
    }
    (void)lt;
}


namespace {

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <bool kExact, bool kPrec, bool kBatched, bool kPersistent, int kWarps>
cudaError_t launch_phys_t(const TraverseArgs& a, cudaStream_t st) {
    auto kernel = traverse_phys_kernel<kExact, kPrec, kBatched, kPersistent, kWarps>;
    const uint32_t chunks = (a.n + 31u) / 32u;
    uint32_t blocks;
    if (kPersistent) {
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarps * 32, 0);
        if (e != cudaSuccess) return e;
        blocks = (uint32_t)std::max(1, per_sm) * (uint32_t)sm_count();
        blocks = std::min<uint32_t>(blocks, (chunks + kWarps - 1) / kWarps);
        cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), st);
    } else {
        blocks = (chunks + kWarps - 1) / kWarps;
    }
    if (blocks == 0) return cudaSuccess;
    kernel<<<blocks, kWarps * 32, 0, st>>>(a);
    return cudaGetLastError();
}

template <bool kExact, bool kPrec, bool kBatched, bool kPersistent>
cudaError_t launch_phys_w(const TraverseArgs& a, int warps, cudaStream_t st) {
    switch (warps) {
        case 2: return launch_phys_t<kExact, kPrec, kBatched, kPersistent, 2>(a, st);
        case 8: return launch_phys_t<kExact, kPrec, kBatched, kPersistent, 8>(a, st);
        default: return launch_phys_t<kExact, kPrec, kBatched, kPersistent, 4>(a, st);
    }
}

template <bool kExact, bool kPrec, bool kBatched>
cudaError_t launch_phys_p(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st) {
    return c.persistent ? launch_phys_w<kExact, kPrec, kBatched, true>(a, c.warps, st)
                        : launch_phys_w<kExact, kPrec, kBatched, false>(a, c.warps, st);
}

template <bool kExact, bool kPrec>
cudaError_t launch_phys_b(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st) {
    return c.batched ? launch_phys_p<kExact, kPrec, true>(a, c, st)
                     : launch_phys_p<kExact, kPrec, false>(a, c, st);
}

}  // namespace

cudaError_t launch_traverse_ref(const TraverseArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    traverse_ref_kernel<<<(a.n + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_traverse_phys(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    if (c.exact)
        return c.precision ? launch_phys_b<true, true>(a, c, st) : launch_phys_b<true, false>(a, c, st);
    return c.precision ? launch_phys_b<false, true>(a, c, st) : launch_phys_b<false, false>(a, c, st);
}

}  // namespace astro
