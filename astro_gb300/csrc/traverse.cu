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

// Interaction terms of the PHYSICAL preset (G = g):
//   particle / monopole:  t = G m d / (r^2 + eps^2)^(3/2)
//   quadrupole addition:  t += G [ 5/2 (d.Qd) d / r^7 - Qd / r^5 ]
// with d the displacement towards the source and Q traceless
// (Qzz = -Qxx - Qyy). kExact rounds every operation separately, in the
// order of the CPU restatement; otherwise rsqrt and FMAs are used.
template <bool kExact>
__device__ __forceinline__ void cell_term(float dx, float dy, float dz, float r2t, float m,
                                          bool quad, float4 q, float qyz, float g, float eps2,
                                          float& tx, float& ty, float& tz) {
    if (kExact) {
        const float r2 = __fadd_rn(r2t, eps2);
        const float inv = __fdiv_rn(1.0f, __fsqrt_rn(r2));
        const float inv2 = __fmul_rn(inv, inv);
        const float inv3 = __fmul_rn(inv2, inv);
        const float sc = __fmul_rn(__fmul_rn(g, m), inv3);
        tx = __fmul_rn(dx, sc);
        ty = __fmul_rn(dy, sc);
        tz = __fmul_rn(dz, sc);
        if (quad) {
            const float inv5 = __fmul_rn(inv3, inv2), inv7 = __fmul_rn(inv5, inv2);
            const float qzz = -__fadd_rn(q.x, q.y);
            const float qx = __fadd_rn(__fadd_rn(__fmul_rn(q.x, dx), __fmul_rn(q.z, dy)), __fmul_rn(q.w, dz));
            const float qy = __fadd_rn(__fadd_rn(__fmul_rn(q.z, dx), __fmul_rn(q.y, dy)), __fmul_rn(qyz, dz));
            const float qz = __fadd_rn(__fadd_rn(__fmul_rn(q.w, dx), __fmul_rn(qyz, dy)), __fmul_rn(qzz, dz));
            const float dqd = __fadd_rn(__fadd_rn(__fmul_rn(dx, qx), __fmul_rn(dy, qy)), __fmul_rn(dz, qz));
            const float w = __fmul_rn(__fmul_rn(2.5f, dqd), inv7);
            tx = __fadd_rn(tx, __fmul_rn(g, __fsub_rn(__fmul_rn(w, dx), __fmul_rn(qx, inv5))));
            ty = __fadd_rn(ty, __fmul_rn(g, __fsub_rn(__fmul_rn(w, dy), __fmul_rn(qy, inv5))));
            tz = __fadd_rn(tz, __fmul_rn(g, __fsub_rn(__fmul_rn(w, dz), __fmul_rn(qz, inv5))));
        }
    } else {
        const float inv = rsqrtf(r2t + eps2);
        const float inv2 = inv * inv;
        const float inv3 = inv2 * inv;
        const float sc = g * m * inv3;
        tx = dx * sc;
        ty = dy * sc;
        tz = dz * sc;
        if (quad) {
            const float inv5 = inv3 * inv2, inv7 = inv5 * inv2;
            const float qzz = -(q.x + q.y);
            const float qx = fmaf(q.x, dx, fmaf(q.z, dy, q.w * dz));
            const float qy = fmaf(q.z, dx, fmaf(q.y, dy, qyz * dz));
            const float qz = fmaf(q.w, dx, fmaf(qyz, dy, qzz * dz));
            const float dqd = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
            const float w = 2.5f * dqd * inv7;
            const float gi5 = g * inv5, gw = g * w;
            tx = fmaf(gw, dx, fmaf(-gi5, qx, tx));
            ty = fmaf(gw, dy, fmaf(-gi5, qy, ty));
            tz = fmaf(gw, dz, fmaf(-gi5, qz, tz));
        }
    }
}

template <bool kExact>
__device__ __forceinline__ void particle_term(float dx, float dy, float dz, float m, float g,
                                              float eps2, float& tx, float& ty, float& tz) {
    if (kExact) {
        const float r2t =
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        cell_term<true>(dx, dy, dz, r2t, m, false, make_float4(0.f, 0.f, 0.f, 0.f), 0.f, g, eps2,
                        tx, ty, tz);
    } else {
        const float inv = rsqrtf(fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2))));
        const float sc = g * m * (inv * inv * inv);
        tx = dx * sc;
        ty = dy * sc;
        tz = dz * sc;
    }
}

// ---------------------------------------------------------- far nodes ----
// The field of an accepted node at d = D - rho, D = com - group centre, to
// second order in the offset rho (the same terms as cell_term, without G):
//   a_i(D - rho) = a_i - J_ij rho_j + 1/2 H_ijk rho_j rho_k
// With R = (|D|^2 + eps^2)^(-1/2), q = QD, s = D.QD:
//   a_i   = al D_i - R^5 q_i
//   J_ij  = ga (q_i D_j + q_j D_i) - be D_i D_j - R^5 Q_ij + al [i=j]
//   H_ijk = nu D_i D_j D_k + ka S(qDD) + ga (S(QD) + S(q delta)) - be S(delta D)
// al = m R^3 + 5/2 s R^7, be = 3 m R^5 + 35/2 s R^9, ga = 5 R^7,
// ka = -35 R^9, nu = 15 m R^7 + 315/2 s R^11; S(.) sums the three distinct
// placements of the indices. Coefficients: a {x, y, z}, J {xx, yy, zz, xy,
// xz, yz}, H {xxx, yyy, zzz, xxy, xxz, xyy, yyz, xzz, yzz, xyz}. kExact
// rounds every product and sum separately in the CPU restatement's order
// (fma(a, b, c) there is a * b + c); otherwise FMAs and rsqrt are used.
constexpr int kFarCoefs = 19;

template <bool kExact>
__device__ __forceinline__ float xmul(float a, float b) { return kExact ? __fmul_rn(a, b) : a * b; }
template <bool kExact>
__device__ __forceinline__ float xadd(float a, float b) { return kExact ? __fadd_rn(a, b) : a + b; }
template <bool kExact>
__device__ __forceinline__ float xfma(float a, float b, float c) {
    return kExact ? __fadd_rn(__fmul_rn(a, b), c) : fmaf(a, b, c);
}

struct FarTerms {
    float D[3], qv[3], Q[3][3], R5, al, be, ga, ka, nu;
};

template <bool kExact, int i, int j>
__device__ __forceinline__ float far_j(const FarTerms& f) {
    float v = xfma<kExact>(f.ga, xfma<kExact>(f.qv[i], f.D[j], xmul<kExact>(f.qv[j], f.D[i])),
                           -xfma<kExact>(f.be, xmul<kExact>(f.D[i], f.D[j]),
                                         xmul<kExact>(f.R5, f.Q[i][j])));
    if (i == j) v = xadd<kExact>(v, f.al);
    return v;
}

template <bool kExact, int i, int j, int k>
__device__ __forceinline__ float far_h(const FarTerms& f) {
    const float dij = xmul<kExact>(f.D[i], f.D[j]);
    const float sqdd = xfma<kExact>(
        f.qv[i], xmul<kExact>(f.D[j], f.D[k]),
        xfma<kExact>(f.qv[j], xmul<kExact>(f.D[i], f.D[k]), xmul<kExact>(f.qv[k], dij)));
    const float sqd = xfma<kExact>(f.Q[i][j], f.D[k],
                                   xfma<kExact>(f.Q[i][k], f.D[j], xmul<kExact>(f.Q[j][k], f.D[i])));
    const float ddd = xmul<kExact>(dij, f.D[k]);
    if constexpr (kExact) {
        // The restatement multiplies by the 0/1 Kronecker factors.
        constexpr float cij = i == j ? 1.f : 0.f, cik = i == k ? 1.f : 0.f, cjk = j == k ? 1.f : 0.f;
        const float sqdel = xfma<true>(cjk, f.qv[i], xfma<true>(cik, f.qv[j], __fmul_rn(cij, f.qv[k])));
        const float sdel = xfma<true>(cij, f.D[k], xfma<true>(cik, f.D[j], __fmul_rn(cjk, f.D[i])));
        return xfma<true>(f.nu, ddd,
                          xfma<true>(f.ka, sqdd,
                                     xfma<true>(f.ga, __fadd_rn(sqd, sqdel), -__fmul_rn(f.be, sdel))));
    } else if constexpr (i != j && j != k) {
        // Sorted, all different: no Kronecker terms.
        return fmaf(f.nu, ddd, fmaf(f.ka, sqdd, f.ga * sqd));
    } else {
        // Sorted (i <= j <= k): i = j = k, i = j < k or i < j = k.
        float sqdel, sdel;
        if constexpr (i == j && j == k) {
            sqdel = 3.0f * f.qv[i];
            sdel = 3.0f * f.D[i];
        } else if constexpr (i == j) {
            sqdel = f.qv[k];
            sdel = f.D[k];
        } else {
            sqdel = f.qv[i];
            sdel = f.D[i];
        }
        return fmaf(f.nu, ddd, fmaf(f.ka, sqdd, fmaf(f.ga, sqd + sqdel, -(f.be * sdel))));
    }
}

// Adds the far-node coefficients of a node (centre of mass and mass cm,
// quadrupole {Qxx, Qyy, Qxy, Qxz}, Qyz, Qzz) about the group centre gc into fc.
template <bool kExact, bool kQuad>
__device__ __forceinline__ void far_coefs(float4 cm, float4 q, float qyz, float qzz, float gcx,
                                          float gcy, float gcz, float eps2, float (&fc)[kFarCoefs]) {
    FarTerms f;
    f.D[0] = xadd<kExact>(cm.x, -gcx);
    f.D[1] = xadd<kExact>(cm.y, -gcy);
    f.D[2] = xadd<kExact>(cm.z, -gcz);
    const float m = cm.w;
    const float r2 = xadd<kExact>(
        xfma<kExact>(f.D[0], f.D[0], xfma<kExact>(f.D[1], f.D[1], xmul<kExact>(f.D[2], f.D[2]))),
        eps2);
    const float R = kExact ? __fdiv_rn(1.0f, __fsqrt_rn(r2)) : rsqrtf(r2);
    const float R2 = xmul<kExact>(R, R), R3 = xmul<kExact>(R2, R), R5 = xmul<kExact>(R3, R2),
                R7 = xmul<kExact>(R5, R2);
    f.R5 = R5;
    if (kQuad || kExact) {
        const float qxx = kQuad ? q.x : 0.f, qyy = kQuad ? q.y : 0.f, qxy = kQuad ? q.z : 0.f,
                    qxz = kQuad ? q.w : 0.f, qyz_ = kQuad ? qyz : 0.f, qzz_ = kQuad ? qzz : -0.f;
        f.Q[0][0] = qxx; f.Q[0][1] = qxy; f.Q[0][2] = qxz;
        f.Q[1][0] = qxy; f.Q[1][1] = qyy; f.Q[1][2] = qyz_;
        f.Q[2][0] = qxz; f.Q[2][1] = qyz_; f.Q[2][2] = qzz_;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            f.qv[i] = xfma<kExact>(f.Q[i][0], f.D[0],
                                   xfma<kExact>(f.Q[i][1], f.D[1], xmul<kExact>(f.Q[i][2], f.D[2])));
        const float sq = xfma<kExact>(f.D[0], f.qv[0],
                                      xfma<kExact>(f.D[1], f.qv[1], xmul<kExact>(f.D[2], f.qv[2])));
        const float R9 = xmul<kExact>(R7, R2), R11 = xmul<kExact>(R9, R2);
        f.al = xfma<kExact>(m, R3, xmul<kExact>(xmul<kExact>(2.5f, sq), R7));
        f.be = xfma<kExact>(xmul<kExact>(3.0f, m), R5, xmul<kExact>(xmul<kExact>(17.5f, sq), R9));
        f.ga = xmul<kExact>(5.0f, R7);
        f.ka = -xmul<kExact>(35.0f, R9);
        f.nu = xfma<kExact>(xmul<kExact>(15.0f, m), R7, xmul<kExact>(xmul<kExact>(157.5f, sq), R11));
    } else {
        // Monopole only (fast form): Q = 0, q = 0, s = 0.
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            f.qv[i] = 0.f;
#pragma unroll
            for (int j = 0; j < 3; ++j) f.Q[i][j] = 0.f;
        }
        f.al = m * R3;
        f.be = 3.0f * m * R5;
        f.ga = 0.f;
        f.ka = 0.f;
        f.nu = 15.0f * m * R7;
    }
    if constexpr (!kExact) {
        // Fast form: the same coefficients from shared products, each FMA
        // chain ending in its sum. With P = D D^T, u = ga q, M = ga Q and
        // t = nu/3 D + ka q:
        //   J_ij  = u_i D_j + u_j D_i - be P_ij - R^5 Q_ij (+ al if i = j)
        //   H_ijk = t_i P_jk + t_j P_ik + t_k P_ij + M_ij D_k + M_ik D_j + M_jk D_i
        //           + (u_k - be D_k) [i=j] + (u_j - be D_j) [i=k] + (u_i - be D_i) [j=k]
        const float* D = f.D;
        const float P[3][3] = {{D[0] * D[0], D[0] * D[1], D[0] * D[2]},
                               {D[0] * D[1], D[1] * D[1], D[1] * D[2]},
                               {D[0] * D[2], D[1] * D[2], D[2] * D[2]}};
        const float nbe = -f.be, nR5 = -R5, nu3 = f.nu * (1.0f / 3.0f);
        float u[3], t[3], v[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            u[i] = f.ga * f.qv[i];
            t[i] = fmaf(nu3, D[i], f.ka * f.qv[i]);
            v[i] = fmaf(nbe, D[i], u[i]);  // u_i - be D_i
            fc[i] = fmaf(f.al, D[i], fmaf(nR5, f.qv[i], fc[i]));
        }
        float M[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) M[i][j] = f.ga * f.Q[i][j];
        auto jc = [&](int i, int j, float acc) {
            acc = fmaf(nR5, f.Q[i][j], fmaf(nbe, P[i][j], acc));
            return fmaf(u[i], D[j], fmaf(u[j], D[i], acc));
        };
        fc[3] = jc(0, 0, fc[3] + f.al);
        fc[4] = jc(1, 1, fc[4] + f.al);
        fc[5] = jc(2, 2, fc[5] + f.al);
        fc[6] = jc(0, 1, fc[6]);
        fc[7] = jc(0, 2, fc[7]);
        fc[8] = jc(1, 2, fc[8]);
        auto hc = [&](int i, int j, int k, float acc) {
            acc = fmaf(t[i], P[j][k], fmaf(t[j], P[i][k], fmaf(t[k], P[i][j], acc)));
            return fmaf(M[i][j], D[k], fmaf(M[i][k], D[j], fmaf(M[j][k], D[i], acc)));
        };
        fc[9] = hc(0, 0, 0, fmaf(3.0f, v[0], fc[9]));
        fc[10] = hc(1, 1, 1, fmaf(3.0f, v[1], fc[10]));
        fc[11] = hc(2, 2, 2, fmaf(3.0f, v[2], fc[11]));
        fc[12] = hc(0, 0, 1, fc[12] + v[1]);
        fc[13] = hc(0, 0, 2, fc[13] + v[2]);
        fc[14] = hc(0, 1, 1, fc[14] + v[0]);
        fc[15] = hc(1, 1, 2, fc[15] + v[2]);
        fc[16] = hc(0, 2, 2, fc[16] + v[0]);
        fc[17] = hc(1, 2, 2, fc[17] + v[1]);
        fc[18] = hc(0, 1, 2, fc[18]);
        return;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
        fc[i] = xadd<kExact>(fc[i], xfma<kExact>(f.al, f.D[i], -xmul<kExact>(R5, f.qv[i])));
    fc[3] = xadd<kExact>(fc[3], far_j<kExact, 0, 0>(f));
    fc[4] = xadd<kExact>(fc[4], far_j<kExact, 1, 1>(f));
    fc[5] = xadd<kExact>(fc[5], far_j<kExact, 2, 2>(f));
    fc[6] = xadd<kExact>(fc[6], far_j<kExact, 0, 1>(f));
    fc[7] = xadd<kExact>(fc[7], far_j<kExact, 0, 2>(f));
    fc[8] = xadd<kExact>(fc[8], far_j<kExact, 1, 2>(f));
    fc[9] = xadd<kExact>(fc[9], far_h<kExact, 0, 0, 0>(f));
    fc[10] = xadd<kExact>(fc[10], far_h<kExact, 1, 1, 1>(f));
    fc[11] = xadd<kExact>(fc[11], far_h<kExact, 2, 2, 2>(f));
    fc[12] = xadd<kExact>(fc[12], far_h<kExact, 0, 0, 1>(f));
    fc[13] = xadd<kExact>(fc[13], far_h<kExact, 0, 0, 2>(f));
    fc[14] = xadd<kExact>(fc[14], far_h<kExact, 0, 1, 1>(f));
    fc[15] = xadd<kExact>(fc[15], far_h<kExact, 1, 1, 2>(f));
    fc[16] = xadd<kExact>(fc[16], far_h<kExact, 0, 2, 2>(f));
    fc[17] = xadd<kExact>(fc[17], far_h<kExact, 1, 2, 2>(f));
    fc[18] = xadd<kExact>(fc[18], far_h<kExact, 0, 1, 2>(f));
}

// The expansion fc at offset rho from the group centre (without G).
template <bool kExact>
__device__ __forceinline__ void far_eval(const float (&fc)[kFarCoefs], float rx, float ry, float rz,
                                         float& ox, float& oy, float& oz) {
    const float pxx = xmul<kExact>(rx, rx), pyy = xmul<kExact>(ry, ry), pzz = xmul<kExact>(rz, rz);
    const float pxy = xmul<kExact>(rx, ry), pxz = xmul<kExact>(rx, rz), pyz = xmul<kExact>(ry, rz);
    const float* J = fc + 3;
    const float* H = fc + 9;
    auto comp = [&](float a, float j0, float j1, float j2, float h0, float h1, float h2, float h3,
                    float h4, float h5) {
        const float jr = xfma<kExact>(j0, rx, xfma<kExact>(j1, ry, xmul<kExact>(j2, rz)));
        const float cross = xfma<kExact>(h3, pxy, xfma<kExact>(h4, pxz, xmul<kExact>(h5, pyz)));
        const float hh = xfma<kExact>(
            h0, pxx, xfma<kExact>(h1, pyy, xfma<kExact>(h2, pzz, xmul<kExact>(2.0f, cross))));
        return xfma<kExact>(0.5f, hh, xadd<kExact>(a, -jr));
    };
    // Rows: J {x: xx xy xz, y: xy yy yz, z: xz yz zz}; H {x: xxx xyy xzz xxy xxz xyz,
    // y: xxy yyy yzz xyy xyz yyz, z: xxz yyz zzz xyz xzz yzz}.
    ox = comp(fc[0], J[0], J[3], J[4], H[0], H[5], H[7], H[3], H[4], H[9]);
    oy = comp(fc[1], J[3], J[1], J[5], H[3], H[1], H[8], H[5], H[9], H[6]);
    oz = comp(fc[2], J[4], J[5], J[2], H[4], H[6], H[2], H[9], H[7], H[8]);
}

// Per-lane acceleration sum: plain or compensated (Kahan) per component.
template <bool kExact, bool kKahan>
struct Accum {
    float ax = 0.f, ay = 0.f, az = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;

    __device__ __forceinline__ void add1(float& s, float& c, float t) {
        if (kKahan) {
            if (kExact) {
                const float y = __fsub_rn(t, c);
                const float u = __fadd_rn(s, y);
                c = __fsub_rn(__fsub_rn(u, s), y);
                s = u;
            } else {
                const float y = t - c;
                const float u = s + y;
                c = (u - s) - y;
                s = u;
            }
        } else {
            s = kExact ? __fadd_rn(s, t) : s + t;
        }
    }
    __device__ __forceinline__ void add(float tx, float ty, float tz) {
        add1(ax, cx, tx);
        add1(ay, cy, ty);
        add1(az, cz, tz);
    }

    // Blocked form (group walk, exact): with Kahan, terms are added plainly
    // within blocks of 32 consecutive list positions and each block's
    // partial is Kahan-added by step(); every position steps, including a
    // particle's own skipped one. Without Kahan, push() is add().
    float bx = 0.f, by = 0.f, bz = 0.f;
    uint32_t k = 0;
    __device__ __forceinline__ void push(float tx, float ty, float tz) {
        if (kKahan) {
            bx = kExact ? __fadd_rn(bx, tx) : bx + tx;
            by = kExact ? __fadd_rn(by, ty) : by + ty;
            bz = kExact ? __fadd_rn(bz, tz) : bz + tz;
        } else {
            add(tx, ty, tz);
        }
    }
    __device__ __forceinline__ void close() {
        add(bx, by, bz);
        bx = by = bz = 0.f;
    }
    __device__ __forceinline__ void step() {
        if (kKahan && (++k & 31u) == 0u) close();
    }
    __device__ __forceinline__ void finish() {
        if (kKahan && (k & 31u) != 0u) close();
    }
};

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


// Group walk. One warp per group of <= 32 consecutive sorted particles (a
// tree cell or a pack of sibling cells, built with the tree). The warp walks
// the tree breadth first from the system's root, testing 32 frontier nodes
// at a time against the group's bounding box: accepted nodes go to the cell
// list (records staged in shared memory), opened leaves and buckets to the
// leaf list, other opened nodes put their children (one run of consecutive
// node indices each) in the next frontier (per-warp buffers in global
// memory); accepted nodes far from the group go to the far list, expanded
// after the walk. The cell and leaf lists are evaluated by all lanes,
// one particle per lane, whenever they fill and at the end: cells into one
// sum, leaf particles (32 at a time through shared memory) into another.
// Cell list capacity per warp: the largest that keeps a block's static
// shared memory under 48 KB.
constexpr int cell_cap(int warps) { return warps >= 8 ? 96 : 128; }
constexpr int kLeafCap = 32;

// A staged accepted cell: centre of mass and mass, and with quadrupoles
// {Qxx, Qyy, Qxy, Qxz} and {Qyz, Qzz}; one record, so the evaluation loop
// walks a single shared-memory array.
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
// Stages a node's quadrupole {Qxx, Qyy, Qxy, Qxz}, Qyz (Qzz = -(Qxx + Qyy)).
// kNegated stores every component negated, for the packed-pair evaluation:
// it then needs no negation and rounds each term exactly as with the plain
// components (IEEE round-to-nearest is symmetric in sign).
template <bool kNegated>
__device__ __forceinline__ void stage_quad(CellSlot<true>& cs, const float4 q, const float qyz) {
    if constexpr (!kNegated) {
        cs.q = q;
        cs.q2 = make_float4(qyz, -(q.x + q.y), 0.f, 0.f);
    } else {
        cs.q = make_float4(-q.x, -q.y, -q.z, -q.w);
        cs.q2 = make_float4(-qyz, q.x + q.y, 0.f, 0.f);
    }
}
// Resident warps per SM the group walk's register allocation is sized for
// (0: the compiler's choice). 24 (80 registers, a few spilled words in the
// far-node loop) measured 1-5% faster than the compiler's 96 registers at
// 20 warps.
#ifndef ASTRO_GROUP_WARPS_PER_SM
#define ASTRO_GROUP_WARPS_PER_SM 24
#endif


#if ASTRO_GROUP_WARPS_PER_SM > 0
#define ASTRO_GROUP_BOUNDS(w) __launch_bounds__((w) * 32, ASTRO_GROUP_WARPS_PER_SM / (w))
#else
#define ASTRO_GROUP_BOUNDS(w) __launch_bounds__((w) * 32)
#endif

template <bool kExact, bool kPrec, bool kQuad, int kWarps>
__global__ ASTRO_GROUP_BOUNDS(kWarps) void traverse_group_kernel(TraverseArgs a) {
    constexpr int kCellCap = cell_cap(kWarps);
    // The precision form's fast path evaluates cells and leaf particles two
    // at a time in packed FP32 pairs: 12% faster there, 2-4% slower in the
    // plain form (more spilled registers), which keeps one at a time.
    constexpr bool kPair = kPrec && !kExact;
    __shared__ CellSlot<kQuad> s_cell[kWarps][kCellCap];
    __shared__ uint2 s_leaf[kWarps][kLeafCap];
    __shared__ float4 s_tile[kWarps][32];
    __shared__ uint32_t s_jdx[kWarps][32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t gw = blockIdx.x * kWarps + warp;
    uint32_t* buf0 = a.frontier + (size_t)gw * (a.far2 > 0.f ? 3 : 2) * a.frontier_cap;
    uint32_t* buf1 = buf0 + a.frontier_cap;
    uint32_t* far_list = buf1 + a.frontier_cap;
    const uint32_t ngroups = *a.group_count;
    const float g = a.g, eps2 = a.eps2;
    uint32_t inter = 0, visits = 0, cell_inter = 0, far_inter = 0, far_nodes = 0;

    while (true) {
        uint32_t gi = 0;
        if (lane == 0) gi = atomicAdd(a.queue, 1u);
        gi = __shfl_sync(kFullMask, gi, 0);
        if (gi >= ngroups) break;
        if (a.group_chunk > 0) {
            // Queue tickets visit whole chunks of consecutive groups in a
            // scrambled chunk order (a bijection: 1000003 is prime and
            // larger than the chunk count); the partial last chunk stays.
            const uint32_t chunk = a.group_chunk, nfull = ngroups / chunk;
            if (gi < nfull * chunk)
                gi = (uint32_t)(((uint64_t)(gi / chunk) * 1000003ull) % nfull) * chunk + gi % chunk;
        }
        const uint2 gr = a.groups[gi];
        const uint32_t gcount = gr.y - gr.x;
        // A group of at most 16 particles runs as reps = 32 / gcount copies
        // (lane = rep * gcount + particle), each copy summing every reps-th
        // listed source; the copies' partial sums are added at the end. The
        // exact form keeps one copy, for the CPU restatement's order.
        const uint32_t reps = kExact ? 1u : max(1u, 32u / gcount);
        const uint32_t rep = lane / gcount;
        const bool valid = rep < reps;   // the lane holds a copy of a particle
        const bool owner = rep == 0;     // the copy that writes the particle
        const uint32_t ip = gr.x + (lane - rep * gcount);
        const float4 me = valid ? a.pos[ip] : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint32_t sys = a.nsys > 1 ? (uint32_t)(a.sorted_keys[gr.x] >> (3u * a.lbits)) : 0u;
        const float* crit_layer = a.sys[sys].crit2;
        // Group bounding box.
        float lo_x = valid ? me.x : INFINITY, lo_y = valid ? me.y : INFINITY,
              lo_z = valid ? me.z : INFINITY;
        float hi_x = valid ? me.x : -INFINITY, hi_y = valid ? me.y : -INFINITY,
              hi_z = valid ? me.z : -INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo_x = fminf(lo_x, __shfl_xor_sync(kFullMask, lo_x, o));
            lo_y = fminf(lo_y, __shfl_xor_sync(kFullMask, lo_y, o));
            lo_z = fminf(lo_z, __shfl_xor_sync(kFullMask, lo_z, o));
            hi_x = fmaxf(hi_x, __shfl_xor_sync(kFullMask, hi_x, o));
            hi_y = fmaxf(hi_y, __shfl_xor_sync(kFullMask, hi_y, o));
            hi_z = fmaxf(hi_z, __shfl_xor_sync(kFullMask, hi_z, o));
        }
        Accum<kExact, kPrec> cells, leaves;
        uint32_t n_cell = 0, n_leaf = 0;

        // Far nodes: centre and half diagonal of the group's box. The walk
        // lists far nodes in the warp's third frontier-sized buffer; after
        // the walk lane l expands far nodes l, l + 32, ... into its partial.
        const bool far_on = a.far2 > 0.f;
        const float gcx = __fmul_rn(__fadd_rn(lo_x, hi_x), 0.5f);
        const float gcy = __fmul_rn(__fadd_rn(lo_y, hi_y), 0.5f);
        const float gcz = __fmul_rn(__fadd_rn(lo_z, hi_z), 0.5f);
        const float hrx = __fmul_rn(__fsub_rn(hi_x, lo_x), 0.5f);
        const float hry = __fmul_rn(__fsub_rn(hi_y, lo_y), 0.5f);
        const float hrz = __fmul_rn(__fsub_rn(hi_z, lo_z), 0.5f);
        const float rg2 = __fadd_rn(__fmul_rn(hrx, hrx), __fadd_rn(__fmul_rn(hry, hry), __fmul_rn(hrz, hrz)));
        uint32_t far_total = 0;

        // Cell list: every lane sums its particle against each staged cell.
        // The fast path leaves G out of the terms and applies it once at the end.
        auto flush_cells = [&]() {
            __syncwarp();
            if (valid) {
                if (kExact) {
                    for (uint32_t e = 0; e < n_cell; ++e) {
                        const CellSlot<kQuad>& cs = s_cell[warp][e];
                        const float4 c = cs.cm;
                        const float dx = __fsub_rn(c.x, me.x), dy = __fsub_rn(c.y, me.y),
                                    dz = __fsub_rn(c.z, me.z);
                        const float r2t = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                    __fmul_rn(dz, dz));
                        float tx, ty, tz;
                        if constexpr (kQuad)
                            cell_term<true>(dx, dy, dz, r2t, c.w, true, cs.q, cs.q2.x, g, eps2, tx, ty,
                                            tz);
                        else
                            cell_term<true>(dx, dy, dz, r2t, c.w, false,
                                            make_float4(0.f, 0.f, 0.f, 0.f), 0.f, g, eps2, tx, ty, tz);
                        cells.push(tx, ty, tz);
                        cells.step();
                    }
                } else {
                    // Precision form: this flush's terms go into a partial
                    // that is Kahan-added once.
                    float px = 0.f, py = 0.f, pz = 0.f;
                    float& rx = kPrec ? px : cells.ax;
                    float& ry = kPrec ? py : cells.ay;
                    float& rz = kPrec ? pz : cells.az;
                    auto cell = [&](const CellSlot<kQuad>& cs) {
                        const float4 c = cs.cm;
                        const float dx = c.x - me.x, dy = c.y - me.y, dz = c.z - me.z;
                        const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
                        const float u = inv * inv, inv3 = u * inv;
                        if constexpr (kQuad) {
                            // inv^3 (M + 5/2 u^2 d.Qd) d - inv^5 Qd, u = 1/r^2:
                            // two FMAs per component into the sums. With the
                            // staged components negated (kPair), qx.. = -(Qd)
                            // and dqd = -d.Qd.
                            const float4 q = cs.q;
                            const float4 q2 = cs.q2;
                            const float qx = fmaf(q.x, dx, fmaf(q.z, dy, q.w * dz));
                            const float qy = fmaf(q.z, dx, fmaf(q.y, dy, q2.x * dz));
                            const float qz = fmaf(q.w, dx, fmaf(q2.x, dy, q2.y * dz));
                            const float dqd = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
                            const float sa = inv3 * fmaf((kPair ? -2.5f : 2.5f) * u * u, dqd, c.w);
                            const float sb = kPair ? inv3 * u : -(inv3 * u);
                            rx = fmaf(sb, qx, fmaf(sa, dx, rx));
                            ry = fmaf(sb, qy, fmaf(sa, dy, ry));
                            rz = fmaf(sb, qz, fmaf(sa, dz, rz));
                        } else {
                            const float sa = inv3 * c.w;
                            rx = fmaf(sa, dx, rx);
                            ry = fmaf(sa, dy, ry);
                            rz = fmaf(sa, dz, rz);
                        }
                    };
                    if (!kPair && reps == 1) {
#pragma unroll 4
                        for (uint32_t e = 0; e < n_cell; ++e) cell(s_cell[warp][e]);
                    } else if (kPair && reps == 1) {
                        // Two cells per step in packed FP32 pairs (one
                        // instruction for both): every term is rounded as in
                        // `cell`; even and odd cells are summed apart and
                        // joined at the end of the flush.
                        const float2 mx = make_float2(-me.x, -me.x), my = make_float2(-me.y, -me.y),
                                     mz = make_float2(-me.z, -me.z);
                        float2 sx = make_float2(0.f, 0.f), sy = sx, sz = sx;
                        uint32_t e = 0;
#pragma unroll 1
                        for (; e + 1 < n_cell; e += 2) {
                            const CellSlot<kQuad>& A = s_cell[warp][e];
                            const CellSlot<kQuad>& B = s_cell[warp][e + 1];
                            const float4 ca = A.cm, cb = B.cm;
                            const float2 dx = __fadd2_rn(make_float2(ca.x, cb.x), mx);
                            const float2 dy = __fadd2_rn(make_float2(ca.y, cb.y), my);
                            const float2 dz = __fadd2_rn(make_float2(ca.z, cb.z), mz);
                            const float2 r2 = __ffma2_rn(
                                dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, make_float2(eps2, eps2))));
                            const float2 inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                            const float2 u = __fmul2_rn(inv, inv), inv3 = __fmul2_rn(u, inv);
                            if constexpr (kQuad) {
                                const float4 qa = A.q, qb = B.q, pa = A.q2, pb = B.q2;
                                const float2 qxx = make_float2(qa.x, qb.x), qyy = make_float2(qa.y, qb.y),
                                             qxy = make_float2(qa.z, qb.z), qxz = make_float2(qa.w, qb.w),
                                             qyz = make_float2(pa.x, pb.x), qzz = make_float2(pa.y, pb.y);
                                const float2 qx = __ffma2_rn(qxx, dx, __ffma2_rn(qxy, dy, __fmul2_rn(qxz, dz)));
                                const float2 qy = __ffma2_rn(qxy, dx, __ffma2_rn(qyy, dy, __fmul2_rn(qyz, dz)));
                                const float2 qz = __ffma2_rn(qxz, dx, __ffma2_rn(qyz, dy, __fmul2_rn(qzz, dz)));
                                const float2 dqd = __ffma2_rn(dx, qx, __ffma2_rn(dy, qy, __fmul2_rn(dz, qz)));
                                const float2 uu = __fmul2_rn(__fmul2_rn(make_float2(-2.5f, -2.5f), u), u);
                                const float2 sa =
                                    __fmul2_rn(inv3, __ffma2_rn(uu, dqd, make_float2(ca.w, cb.w)));
                                const float2 sb = __fmul2_rn(inv3, u);
                                sx = __ffma2_rn(sb, qx, __ffma2_rn(sa, dx, sx));
                                sy = __ffma2_rn(sb, qy, __ffma2_rn(sa, dy, sy));
                                sz = __ffma2_rn(sb, qz, __ffma2_rn(sa, dz, sz));
                            } else {
                                const float2 sa = __fmul2_rn(inv3, make_float2(ca.w, cb.w));
                                sx = __ffma2_rn(sa, dx, sx);
                                sy = __ffma2_rn(sa, dy, sy);
                                sz = __ffma2_rn(sa, dz, sz);
                            }
                        }
                        rx += sx.x + sx.y;
                        ry += sy.x + sy.y;
                        rz += sz.x + sz.y;
                        if (e < n_cell) cell(s_cell[warp][e]);
                    } else {
#pragma unroll 2
                        for (uint32_t e = rep; e < n_cell; e += reps) cell(s_cell[warp][e]);
                    }
                    if (kPrec) cells.add(px, py, pz);
                }
                if (owner) {
                    inter += n_cell;
                    cell_inter += n_cell;
                }
            }
            __syncwarp();
            n_cell = 0;
        };
        // Leaf list: the listed particle ranges are concatenated and staged
        // 32 particles at a time (a shuffle binary search over the ranges'
        // prefix sums finds each lane's particle), keeping the walk order.
        auto flush_leaves = [&]() {
            uint32_t rb = 0, rlen = 0;
            if (lane < n_leaf) {
                const uint2 rg = s_leaf[warp][lane];
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
            const bool skip_self_free = !kExact && eps2 > 0.f;
            for (uint32_t t0 = 0; t0 < total; t0 += 32u) {
                const uint32_t pos = t0 + lane;
                uint32_t e = 0;
#pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1) {
                    const uint32_t cand = e + step;
                    const uint32_t pc = __shfl_sync(kFullMask, pre, cand & 31u);
                    if (cand < n_leaf && pc <= pos) e = cand;
                }
                const uint32_t eb = __shfl_sync(kFullMask, rb, e);
                const uint32_t ep = __shfl_sync(kFullMask, pre, e);
                __syncwarp();
                if (pos < total) {
                    const uint32_t j = eb + (pos - ep);
                    s_tile[warp][lane] = __ldg(&a.pos[j]);
                    s_jdx[warp][lane] = j;
                }
                __syncwarp();
                const uint32_t cnt = min(32u, total - t0);
                if (valid) {
                    // Precision form, fast path: the tile's terms go into a
                    // partial that is Kahan-added once.
                    float px = 0.f, py = 0.f, pz = 0.f;
                    float& rx = kPrec ? px : leaves.ax;
                    float& ry = kPrec ? py : leaves.ay;
                    float& rz = kPrec ? pz : leaves.az;
                    if (skip_self_free) {
                        // eps > 0: the self term is exactly zero, so no test is needed.
                        auto pp = [&](const float4 p) {
                            const float dx = p.x - me.x, dy = p.y - me.y, dz = p.z - me.z;
                            const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
                            const float sc = p.w * (inv * inv * inv);
                            rx = fmaf(dx, sc, rx);
                            ry = fmaf(dy, sc, ry);
                            rz = fmaf(dz, sc, rz);
                        };
                        if (!kPair && reps == 1) {
#pragma unroll 4
                            for (uint32_t q = 0; q < cnt; ++q) pp(s_tile[warp][q]);
                        } else if (kPair && reps == 1) {
                            // Two sources per step in packed FP32 pairs, each
                            // term rounded as in `pp`; even and odd sources
                            // summed apart and joined after the tile.
                            const float2 mx = make_float2(-me.x, -me.x), my = make_float2(-me.y, -me.y),
                                         mz = make_float2(-me.z, -me.z);
                            float2 sx = make_float2(0.f, 0.f), sy = sx, sz = sx;
                            uint32_t q = 0;
#pragma unroll 1
                            for (; q + 1 < cnt; q += 2) {
                                const float4 pa = s_tile[warp][q], pb = s_tile[warp][q + 1];
                                const float2 dx = __fadd2_rn(make_float2(pa.x, pb.x), mx);
                                const float2 dy = __fadd2_rn(make_float2(pa.y, pb.y), my);
                                const float2 dz = __fadd2_rn(make_float2(pa.z, pb.z), mz);
                                const float2 r2 = __ffma2_rn(
                                    dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, make_float2(eps2, eps2))));
                                const float2 inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                                const float2 sc = __fmul2_rn(make_float2(pa.w, pb.w),
                                                             __fmul2_rn(__fmul2_rn(inv, inv), inv));
                                sx = __ffma2_rn(dx, sc, sx);
                                sy = __ffma2_rn(dy, sc, sy);
                                sz = __ffma2_rn(dz, sc, sz);
                            }
                            rx += sx.x + sx.y;
                            ry += sy.x + sy.y;
                            rz += sz.x + sz.y;
                            if (q < cnt) pp(s_tile[warp][q]);
                        } else {
#pragma unroll 4
                            for (uint32_t q = rep; q < cnt; q += reps) pp(s_tile[warp][q]);
                        }
                        if (owner) inter += cnt;
                    } else if (kExact) {
                        for (uint32_t q = 0; q < cnt; ++q) {
                            if (s_jdx[warp][q] != ip) {
                                const float4 p = s_tile[warp][q];
                                float tx, ty, tz;
                                particle_term<true>(__fsub_rn(p.x, me.x), __fsub_rn(p.y, me.y),
                                                    __fsub_rn(p.z, me.z), p.w, g, eps2, tx, ty, tz);
                                leaves.push(tx, ty, tz);
                                ++inter;
                            }
                            leaves.step();
                        }
                    } else {
                        for (uint32_t q = rep; q < cnt; q += reps) {
                            if (s_jdx[warp][q] == ip) continue;
                            const float4 p = s_tile[warp][q];
                            float tx, ty, tz;
                            particle_term<false>(p.x - me.x, p.y - me.y, p.z - me.z, p.w, 1.0f, eps2,
                                                 tx, ty, tz);
                            rx += tx;
                            ry += ty;
                            rz += tz;
                            ++inter;
                        }
                    }
                    if (kPrec && !kExact) leaves.add(px, py, pz);
                }
            }
            __syncwarp();
            n_leaf = 0;
        };

        // Two forms of the same breadth-first walk (same nodes, same order):
        // a frontier of runs of consecutive child nodes, or of node indices;
        // which is faster depends on the workload (astro_params.walk_frontier).
        // The per-node test and staging are written out in both forms: shared
        // through one lambda they compiled to a register allocation with more
        // spills and a traversal up to 2.4% slower.
        if (a.walk_runs) {
        // The frontier holds runs of consecutive node indices (first, count)
        // in walk order: the children of an opened node are consecutive, so
        // each opened node adds one run, and a chunk of 32 nodes is found by
        // a shuffle search over 32 runs loaded at once, without a load of
        // its own.
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
                    const bool has = pos < rtotal;
                    // The run holding position pos: the last one starting at or before it.
                    uint32_t e = 0;
#pragma unroll
                    for (uint32_t step = 16; step > 0; step >>= 1) {
                        const uint32_t cand = e + step;
                        const uint32_t pc = __shfl_sync(kFullMask, rpre, cand & 31u);
                        if (cand < nrun && pc <= pos) e = cand;
                    }
                    const uint32_t first = __shfl_sync(kFullMask, run.x, e);
                    const uint32_t estart = __shfl_sync(kFullMask, rpre, e);
                    const uint32_t nd = has ? first + (pos - estart) : 0u;
                    float4 c = make_float4(0.f, 0.f, 0.f, 0.f), q4 = c;
                    uint4 r = make_uint4(0u, 0u, 0u, 0u);
                    float crit = 0.f, qyz = 0.f;
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
                        const float Dx = __fsub_rn(c.x, gcx), Dy = __fsub_rn(c.y, gcy),
                                    Dz = __fsub_rn(c.z, gcz);
                        const float D2 = __fadd_rn(__fmul_rn(Dx, Dx),
                                                   __fadd_rn(__fmul_rn(Dy, Dy), __fmul_rn(Dz, Dz)));
                        far = __fmul_rn(a.far2, D2) > rg2;
                    }
                    const bool acc = accepted && !far;
                    const uint32_t tested = __popc(__ballot_sync(kFullMask, has));
                    if (owner) visits += tested;
                    // Far nodes, in frontier order.
                    const uint32_t bfar = __ballot_sync(kFullMask, far);
                    if (bfar) {
                        if (far_total + __popc(bfar) <= a.frontier_cap) {
                            if (far) far_list[far_total + __popc(bfar & lt)] = nd;
                            far_total += __popc(bfar);
                        } else if (lane == 0) {
                            atomicOr(a.err, kErrFrontier);
                        }
                    }
                    // Accepted cells, in frontier order.
                    const uint32_t bacc = __ballot_sync(kFullMask, acc);
                    if (bacc) {
                        if (n_cell + __popc(bacc) > (uint32_t)kCellCap) flush_cells();
                        if (acc) {
                            const uint32_t slot = n_cell + __popc(bacc & lt);
                            s_cell[warp][slot].cm = c;
                            if constexpr (kQuad) {
                                q4 = __ldg(&a.node_q[nd]);
                                qyz = __ldg(&a.node_qyz[nd]);
                                stage_quad<kPair>(s_cell[warp][slot], q4, qyz);
                            }
                        }
                        n_cell += __popc(bacc);
                    }
                    // Opened leaves and buckets, in frontier order.
                    const uint32_t bleaf = __ballot_sync(kFullMask, leaf);
                    if (bleaf) {
                        if (n_leaf + __popc(bleaf) > (uint32_t)kLeafCap) flush_leaves();
                        if (leaf) s_leaf[warp][n_leaf + __popc(bleaf & lt)] = make_uint2(r.z, r.w);
                        n_leaf += __popc(bleaf);
                    }
                    // Children of opened nodes: one run each, in frontier order.
                    const uint32_t bopen = __ballot_sync(kFullMask, opn);
                    if (bopen) {
                        if (nnext + __popc(bopen) <= run_cap) {
                            if (opn) nxt[nnext + __popc(bopen & lt)] = make_uint2(r.x, r.y - r.x);
                            nnext += __popc(bopen);
                        } else if (lane == 0) {
                            atomicOr(a.err, kErrFrontier);
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
                const uint32_t nd = has ? cur[k] : 0u;
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
                    const float Dx = __fsub_rn(c.x, gcx), Dy = __fsub_rn(c.y, gcy),
                                Dz = __fsub_rn(c.z, gcz);
                    const float D2 = __fadd_rn(__fmul_rn(Dx, Dx),
                                               __fadd_rn(__fmul_rn(Dy, Dy), __fmul_rn(Dz, Dz)));
                    far = __fmul_rn(a.far2, D2) > rg2;
                }
                const bool acc = accepted && !far;
                const uint32_t tested = __popc(__ballot_sync(kFullMask, has));
                if (owner) visits += tested;
                // Far nodes, in frontier order.
                const uint32_t bfar = __ballot_sync(kFullMask, far);
                if (bfar) {
                    if (far_total + __popc(bfar) <= a.frontier_cap) {
                        if (far) far_list[far_total + __popc(bfar & lt)] = nd;
                        far_total += __popc(bfar);
                    } else if (lane == 0) {
                        atomicOr(a.err, kErrFrontier);
                    }
                }
                // Accepted cells, in frontier order.
                const uint32_t bacc = __ballot_sync(kFullMask, acc);
                if (bacc) {
                    if (n_cell + __popc(bacc) > (uint32_t)kCellCap) flush_cells();
                    if (acc) {
                        const uint32_t slot = n_cell + __popc(bacc & lt);
                        s_cell[warp][slot].cm = c;
                        if constexpr (kQuad)
                            stage_quad<kPair>(s_cell[warp][slot], __ldg(&a.node_q[nd]), __ldg(&a.node_qyz[nd]));
                    }
                    n_cell += __popc(bacc);
                }
                // Opened leaves and buckets, in frontier order.
                const uint32_t bleaf = __ballot_sync(kFullMask, leaf);
                if (bleaf) {
                    if (n_leaf + __popc(bleaf) > (uint32_t)kLeafCap) flush_leaves();
                    if (leaf) s_leaf[warp][n_leaf + __popc(bleaf & lt)] = make_uint2(r.z, r.w);
                    n_leaf += __popc(bleaf);
                }
                // Children of opened nodes form the next frontier, in order.
                const uint32_t cnt = opn ? r.y - r.x : 0u;
                uint32_t incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
                    if (lane >= (uint32_t)o) incl += y;
                }
                const uint32_t total = __shfl_sync(kFullMask, incl, 31);
                if (nnext + total <= a.frontier_cap) {
                    const uint32_t o0 = nnext + incl - cnt;
                    for (uint32_t j = 0; j < cnt; ++j) nxt[o0 + j] = r.x + j;
                    nnext += total;
                } else if (lane == 0) {
                    atomicOr(a.err, kErrFrontier);
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
        flush_cells();
        flush_leaves();
        // The self-free fast loop counted the particle's own entry once.
        if (!kExact && eps2 > 0.f && owner) --inter;

        // Far nodes: lane l sums the coefficients of far nodes l, l + 32, ...
        // in walk order; the partials are combined pairwise (lane l + lane
        // l^o, o = 16 .. 1), leaving the sum in every lane; each particle
        // adds the expansion at its offset.
        float fx = 0.f, fy = 0.f, fz = 0.f;
        if (far_total > 0) {
            __syncwarp();
            float fc[kFarCoefs];
#pragma unroll
            for (int k = 0; k < kFarCoefs; ++k) fc[k] = 0.f;
            for (uint32_t f = lane; f < far_total; f += 32u) {
                const uint32_t nd = far_list[f];
                const float4 c = __ldg(&a.node_cm[nd]);
                if constexpr (kQuad) {
                    const float4 q = __ldg(&a.node_q[nd]);
                    far_coefs<kExact, true>(c, q, __ldg(&a.node_qyz[nd]), -(q.x + q.y), gcx, gcy, gcz,
                                            eps2, fc);
                } else {
                    far_coefs<kExact, false>(c, make_float4(0.f, 0.f, 0.f, 0.f), 0.f, 0.f, gcx, gcy,
                                             gcz, eps2, fc);
                }
            }
#pragma unroll
            for (int k = 0; k < kFarCoefs; ++k) {
                float v = fc[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v = xadd<kExact>(v, __shfl_xor_sync(kFullMask, v, o));
                fc[k] = v;
            }
            far_eval<kExact>(fc, xadd<kExact>(me.x, -gcx), xadd<kExact>(me.y, -gcy),
                             xadd<kExact>(me.z, -gcz), fx, fy, fz);
            if (owner) {
                inter += far_total;
                cell_inter += far_total;
                far_inter += far_total;
            }
            if (lane == 0) far_nodes += far_total;
        }

        float sx, sy, sz;
        if (kExact) {
            cells.finish();
            leaves.finish();
            sx = __fadd_rn(cells.ax, leaves.ax);
            sy = __fadd_rn(cells.ay, leaves.ay);
            sz = __fadd_rn(cells.az, leaves.az);
            if (far_total > 0) {
                sx = __fadd_rn(sx, __fmul_rn(g, fx));
                sy = __fadd_rn(sy, __fmul_rn(g, fy));
                sz = __fadd_rn(sz, __fmul_rn(g, fz));
            }
        } else {
            // Compensated sums: the running sum minus its pending correction.
            sx = (cells.ax - cells.cx) + (leaves.ax - leaves.cx);
            sy = (cells.ay - cells.cy) + (leaves.ay - leaves.cy);
            sz = (cells.az - cells.cz) + (leaves.az - leaves.cz);
            if (reps > 1) {
                __syncwarp();
                if (valid) s_tile[warp][lane] = make_float4(sx, sy, sz, 0.f);
                __syncwarp();
                if (owner)
                    for (uint32_t r = 1; r < reps; ++r) {
                        const float4 t = s_tile[warp][lane + r * gcount];
                        sx += t.x;
                        sy += t.y;
                        sz += t.z;
                    }
                __syncwarp();
            }
            sx = (sx + fx) * g;
            sy = (sy + fy) * g;
            sz = (sz + fz) * g;
        }
        if (owner) {
            const float cl = a.clampv, dt = a.dt;
            const float ax = fminf(fmaxf(sx, -cl), cl);
            const float ay = fminf(fmaxf(sy, -cl), cl);
            const float az = fminf(fmaxf(sz, -cl), cl);
            a.acc[ip] = make_float4(ax, ay, az, 0.f);
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
    }
    unsigned long long i64 = inter, v64 = visits, c64 = cell_inter, f64 = far_inter;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        i64 += __shfl_xor_sync(kFullMask, i64, o);
        v64 += __shfl_xor_sync(kFullMask, v64, o);
        c64 += __shfl_xor_sync(kFullMask, c64, o);
        f64 += __shfl_xor_sync(kFullMask, f64, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stats[0], i64);
        atomicAdd(&a.stats[1], v64);
        atomicAdd(&a.stats[2], c64);
        if (far_nodes) atomicAdd(&a.stats[3], (unsigned long long)far_nodes);
        if (f64) atomicAdd(&a.stats[4], f64);
    }
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

template <bool kExact, bool kPrec, bool kQuad, int kWarps>
uint32_t group_blocks() {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, traverse_group_kernel<kExact, kPrec, kQuad, kWarps>, kWarps * 32, 0);
    return (uint32_t)std::max(1, per_sm) * (uint32_t)sm_count();
}

template <bool kExact, bool kPrec, bool kQuad, int kWarps>
cudaError_t launch_group_t(const TraverseArgs& a, cudaStream_t st) {
    const uint32_t blocks = group_blocks<kExact, kPrec, kQuad, kWarps>();
    cudaError_t e = cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    traverse_group_kernel<kExact, kPrec, kQuad, kWarps><<<blocks, kWarps * 32, 0, st>>>(a);
    return cudaGetLastError();
}

template <bool kExact, bool kPrec, bool kQuad>
cudaError_t launch_group_w(const TraverseArgs& a, int warps, cudaStream_t st) {
    return warps == 8 ? launch_group_t<kExact, kPrec, kQuad, 8>(a, st)
                      : launch_group_t<kExact, kPrec, kQuad, 4>(a, st);
}

template <bool kExact, bool kPrec>
cudaError_t launch_group_q(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st) {
    return c.quad ? launch_group_w<kExact, kPrec, true>(a, c.warps, st)
                  : launch_group_w<kExact, kPrec, false>(a, c.warps, st);
}

}  // namespace

uint32_t group_walk_warps(const TraverseConfig& c) {
    // Warps of the persistent launch of the instantiation this config selects.
    uint32_t blocks;
    const bool w8 = c.warps == 8;
#define ASTRO_GB(E, P, Q) (w8 ? group_blocks<E, P, Q, 8>() : group_blocks<E, P, Q, 4>())
    if (c.exact) {
        if (c.precision) blocks = c.quad ? ASTRO_GB(true, true, true) : ASTRO_GB(true, true, false);
        else blocks = c.quad ? ASTRO_GB(true, false, true) : ASTRO_GB(true, false, false);
    } else {
        if (c.precision) blocks = c.quad ? ASTRO_GB(false, true, true) : ASTRO_GB(false, true, false);
        else blocks = c.quad ? ASTRO_GB(false, false, true) : ASTRO_GB(false, false, false);
    }
#undef ASTRO_GB
    return blocks * (w8 ? 8u : 4u);
}

cudaError_t launch_traverse_groups(const TraverseArgs& a, const TraverseConfig& c, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    if (c.exact)
        return c.precision ? launch_group_q<true, true>(a, c, st) : launch_group_q<true, false>(a, c, st);
    return c.precision ? launch_group_q<false, true>(a, c, st) : launch_group_q<false, false>(a, c, st);
}

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
