// Interaction terms shared by the traversal kernels (traverse.cu,
// traverse_group.cu): the fast 1/sqrt, the cell and particle terms, the
// far-node expansion, compensated accumulators and the packed-pair terms.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace astro {

// The fast traversal's 1/sqrt: a single rsqrt.approx.ftz operation. It is
// used only where the argument is a normal float (r^2 >= eps^2 >= FLT_MIN);
// there it returns what rsqrtf() returns, without the fix-up rsqrtf() wraps
// around the same operation for subnormal arguments.
constexpr float kFltMin = 1.17549435e-38f;
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template <bool kFtz>
__device__ __forceinline__ float rsq(float x) {
    if constexpr (kFtz) return rsqrt_ftz(x);
    else return rsqrtf(x);
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


// Packed-pair terms of the fast path: two sources at once (one instruction
// for both), each term rounded as the one-at-a-time form rounds it. (x, y, z,
// m) are the sources, (nmx, nmy, nmz) the negated target position, e2 eps^2;
// the terms (without G) are added to (sx, sy, sz).
__device__ __forceinline__ void mono_pair(float2 x, float2 y, float2 z, float2 m, float2 nmx,
                                          float2 nmy, float2 nmz, float2 e2, float2& sx, float2& sy,
                                          float2& sz) {
    const float2 dx = __fadd2_rn(x, nmx), dy = __fadd2_rn(y, nmy), dz = __fadd2_rn(z, nmz);
    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
    const float2 inv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
    const float2 sc = __fmul2_rn(m, __fmul2_rn(__fmul2_rn(inv, inv), inv));
    sx = __ffma2_rn(dx, sc, sx);
    sy = __ffma2_rn(dy, sc, sy);
    sz = __ffma2_rn(dz, sc, sz);
}
// A cell with its quadrupole, given negated (nxx = -Qxx, ..., nzz = -Qzz):
// inv^3 (M + 5/2 u^2 d.Qd) d - inv^5 Qd with u = 1/r^2, where qx.. = -(Qd)
// and dqd = -d.Qd, so no negation is needed (IEEE round-to-nearest is
// symmetric in sign).
__device__ __forceinline__ void cell_pair_quad(float2 x, float2 y, float2 z, float2 m, float2 nxx,
                                               float2 nyy, float2 nxy, float2 nxz, float2 nyz,
                                               float2 nzz, float2 nmx, float2 nmy, float2 nmz,
                                               float2 e2, float2& sx, float2& sy, float2& sz) {
    const float2 dx = __fadd2_rn(x, nmx), dy = __fadd2_rn(y, nmy), dz = __fadd2_rn(z, nmz);
    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
    const float2 inv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
    const float2 u = __fmul2_rn(inv, inv), inv3 = __fmul2_rn(u, inv);
    const float2 qx = __ffma2_rn(nxx, dx, __ffma2_rn(nxy, dy, __fmul2_rn(nxz, dz)));
    const float2 qy = __ffma2_rn(nxy, dx, __ffma2_rn(nyy, dy, __fmul2_rn(nyz, dz)));
    const float2 qz = __ffma2_rn(nxz, dx, __ffma2_rn(nyz, dy, __fmul2_rn(nzz, dz)));
    const float2 dqd = __ffma2_rn(dx, qx, __ffma2_rn(dy, qy, __fmul2_rn(dz, qz)));
    const float2 uu = __fmul2_rn(__fmul2_rn(make_float2(-2.5f, -2.5f), u), u);
    const float2 sa = __fmul2_rn(inv3, __ffma2_rn(uu, dqd, m));
    const float2 sb = __fmul2_rn(inv3, u);
    sx = __ffma2_rn(sb, qx, __ffma2_rn(sa, dx, sx));
    sy = __ffma2_rn(sb, qy, __ffma2_rn(sa, dy, sy));
    sz = __ffma2_rn(sb, qz, __ffma2_rn(sa, dz, sz));
}

}  // namespace astro
