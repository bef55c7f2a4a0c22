// ORACLE — test infrastructure only (see astro_oracle.h). Not part of the product.
//
// PHYSICAL preset: the reference's pipeline (Renderer.draw, Renderer.swift:
// 495-755) with physical units. Stage by stage:
//   bounding box    per system, FP32 (FP64 in the precision form)
//   encode          generateMortonCodes (MortonCode.metal:26-52) with a
//                   bounding-box quantiser into [0, 2^21) and the system id
//                   above the 3*lbits key bits
//   sort            MetalKernelsRadixSort.sort (RadixSort.swift:98-185),
//                   one-bit split passes
//   run detection   markUniques/scatterUniques per layer (Octree.metal:282-334)
//   aggregation     aggregateLeafNodes / aggregateNodes (Octree.metal:53-202)
//                   as raw sums (S = sum m x, M = sum m) in sorted order, the
//                   last leaf ending at the particle count
//   traversal       barnesHut (BarnesHut.metal:22-101) with the geometric cell
//                   size, Plummer softening and particle-particle sums in
//                   opened leaves and buckets
//   integration     updateSpheres' kick-drift (BarnesHut.metal:189-194)
//                   without damping or type multipliers: v += a dt, x += v dt,
//                   i.e. leapfrog with velocities at half steps
// State order: the particle arrays are kept in the Morton order of the last
// step (upload order at first). Each step stable-sorts the keys of the
// current order and permutes the state by the result, so ties are broken by
// the previous order. Particle ids map the state back to upload order.
// Arithmetic: FP32 round-to-nearest without contraction, 1/sqrt as a
// correctly rounded sqrt followed by a division, sums in ascending order.
#include "astro_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr uint64_t kInvalidCode = ASTRO_INVALID_MORTON_CODE;
constexpr uint32_t kInvalidChild = ASTRO_INVALID_CHILD;
constexpr float kQuantCells = 2097152.0f;  // 2^21 cells per axis
constexpr uint32_t kQuantMax = 2097151u;

inline uint32_t float_to_uint_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

inline uint32_t quantise(float x, float lo, float scale) {
    float t = (x - lo) * scale;
    return std::min(float_to_uint_sat(t), kQuantMax);
}

uint32_t system_bits(uint32_t nsys) {
    uint32_t b = 0;
    while ((1ull << b) < nsys) ++b;
    return b;
}

struct SysQuant {
    float lo[3];
    float scale;
    float ext;
    float crit2[ASTRO_MAX_LAYERS];
    double origin[3];
};

struct PhysState {
    astro_params p{};
    uint32_t n = 0, nsys = 1, lbits = 6, layers = 7, sysbits = 0;
    bool prec = false;
    std::vector<uint32_t> sys_off, sys_of;
    std::vector<float> pos, vel, acc, rel;  // float4 per particle, current order
    std::vector<uint32_t> id;               // upload index of each particle
    std::vector<double> x64;                // 3 per particle (precision form)
    std::vector<SysQuant> quant;
    std::vector<uint64_t> keys, sorted;
    std::vector<uint32_t> perm;
    std::vector<uint32_t> sizes, offsets, counts;
    uint64_t capacity = 0;
    std::vector<float> cm;       // com.xyz, mass per node
    std::vector<float> sum32;    // Sx, Sy, Sz, M per node (plain)
    std::vector<double> sum64;   // Sx, Sy, Sz, M per node (precision)
    std::vector<uint32_t> pbeg, pend, cbeg, cend;
    std::vector<float> quad;     // Qxx, Qyy, Qxy, Qxz, Qyz per node (quadrupole flag)
    std::vector<float> ncrit2;   // per-node opening radius^2 (delta flag)
    uint64_t interactions = 0, visits = 0, far_nodes = 0, far_interactions = 0;

    void layout(const uint32_t* sys_sizes) {
        sys_off.assign(nsys + 1, 0);
        for (uint32_t s = 0; s < nsys; ++s) sys_off[s + 1] = sys_off[s] + sys_sizes[s];
        sys_of.resize(n);
        for (uint32_t s = 0; s < nsys; ++s)
            for (uint32_t i = sys_off[s]; i < sys_off[s + 1]; ++i) sys_of[i] = s;
        // Closed-form capacity of Renderer.swift:373-386, summed per system.
        sizes.assign(layers, 0);
        offsets.assign(layers, 0);
        uint64_t off = 0;
        for (uint32_t l = 0; l < layers; ++l) {
            uint32_t bits = 3u * (lbits - l);
            uint64_t possible = bits >= 40 ? (1ull << 40) : (1ull << bits);
            uint64_t size = 0;
            for (uint32_t s = 0; s < nsys; ++s) size += std::min<uint64_t>(sys_sizes[s], possible);
            sizes[l] = (uint32_t)size;
            offsets[l] = (uint32_t)off;
            off += size;
        }
        capacity = off;
        counts.assign(layers, 0);
        cm.assign(4 * capacity, 0.0f);
        sum32.assign(prec ? 0 : 4 * capacity, 0.0f);
        sum64.assign(prec ? 4 * capacity : 0, 0.0);
        pbeg.assign(capacity, 0);
        pend.assign(capacity, 0);
        cbeg.assign(capacity, 0);
        cend.assign(capacity, 0);
        quad.assign(5 * capacity, 0.0f);
        ncrit2.assign(capacity, 0.0f);
    }

    // Bounding box, quantiser and opening thresholds per system.
    void setup_quant() {
        quant.assign(nsys, SysQuant{});
        for (uint32_t s = 0; s < nsys; ++s) {
            SysQuant& q = quant[s];
            float lo[3], hi[3];
            if (prec) {
                double lo64[3], hi64[3];
                for (int a = 0; a < 3; ++a) {
                    lo64[a] = INFINITY;
                    hi64[a] = -INFINITY;
                }
                for (uint32_t i = sys_off[s]; i < sys_off[s + 1]; ++i)
                    for (int a = 0; a < 3; ++a) {
                        lo64[a] = std::min(lo64[a], x64[3ull * i + a]);
                        hi64[a] = std::max(hi64[a], x64[3ull * i + a]);
                    }
                for (int a = 0; a < 3; ++a) {
                    q.origin[a] = (lo64[a] + hi64[a]) * 0.5;
                    lo[a] = (float)(lo64[a] - q.origin[a]);
                    hi[a] = (float)(hi64[a] - q.origin[a]);
                }
                for (uint32_t i = sys_off[s]; i < sys_off[s + 1]; ++i) {
                    for (int a = 0; a < 3; ++a)
                        rel[4ull * i + a] = (float)(x64[3ull * i + a] - q.origin[a]);
                    rel[4ull * i + 3] = pos[4ull * i + 3];
                }
            } else {
                for (int a = 0; a < 3; ++a) {
                    lo[a] = INFINITY;
                    hi[a] = -INFINITY;
                    q.origin[a] = 0.0;
                }
                for (uint32_t i = sys_off[s]; i < sys_off[s + 1]; ++i)
                    for (int a = 0; a < 3; ++a) {
                        lo[a] = std::min(lo[a], pos[4ull * i + a]);
                        hi[a] = std::max(hi[a], pos[4ull * i + a]);
                    }
                for (uint32_t i = sys_off[s]; i < sys_off[s + 1]; ++i)
                    for (int a = 0; a < 4; ++a) rel[4ull * i + a] = pos[4ull * i + a];
            }
            float ext = 0.0f;
            for (int a = 0; a < 3; ++a) {
                q.lo[a] = lo[a];
                ext = std::max(ext, hi[a] - lo[a]);
            }
            if (!(ext > 0.0f) || !std::isfinite(ext)) ext = 1.0f;
            q.ext = ext;
            q.scale = kQuantCells / ext;
            for (uint32_t l = 0; l < layers; ++l) {
                float size = std::ldexp(ext, (int)l - (int)lbits);
                float c = size / p.theta;
                q.crit2[l] = c * c;
            }
        }
    }

    void encode() {
        const uint32_t unused_bits = 63u - 3u * lbits;
        keys.resize(n);
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            uint32_t i = (uint32_t)ii, s = sys_of[i];
            const SysQuant& q = quant[s];
            uint32_t qx = quantise(rel[4ull * i + 0], q.lo[0], q.scale);
            uint32_t qy = quantise(rel[4ull * i + 1], q.lo[1], q.scale);
            uint32_t qz = quantise(rel[4ull * i + 2], q.lo[2], q.scale);
            uint64_t code = oracle_interleave_bits(qx, qy, qz) >> unused_bits;
            keys[i] = ((uint64_t)s << (3u * lbits)) | code;
        }
    }

    void sort(uint32_t split_passes) {
        std::vector<uint32_t> iota(n);
        for (uint32_t i = 0; i < n; ++i) iota[i] = i;
        sorted.resize(n);
        perm.resize(n);
        uint32_t passes = split_passes ? split_passes : 3u * lbits + sysbits;
        oracle_split_sort(keys.data(), iota.data(), sorted.data(), perm.data(), n, passes);
        // Permute the state into the new order.
        std::vector<float> p2(4ull * n), v2(4ull * n), r2(4ull * n);
        std::vector<uint32_t> id2(n);
        std::vector<double> x2(prec ? 3ull * n : 0);
        for (uint32_t j = 0; j < n; ++j) {
            uint32_t s = perm[j];
            for (int a = 0; a < 4; ++a) {
                p2[4ull * j + a] = pos[4ull * s + a];
                v2[4ull * j + a] = vel[4ull * s + a];
                r2[4ull * j + a] = rel[4ull * s + a];
            }
            if (prec)
                for (int a = 0; a < 3; ++a) x2[3ull * j + a] = x64[3ull * s + a];
            id2[j] = id[s];
        }
        pos.swap(p2);
        vel.swap(v2);
        rel.swap(r2);
        id.swap(id2);
        if (prec) x64.swap(x2);
    }

    // Run detection per layer (markUniques / scatterUniques, Octree.metal:282-334):
    // layer 0 runs of equal keys, layer l runs of equal code >> 3 among the
    // layer l-1 nodes. Children and particle ranges are contiguous.
    void topology() {
        std::vector<uint32_t> flags, scan;
        flags.assign(n, 0);
        scan.assign(n, 0);
        for (uint32_t i = 0; i < n; ++i) flags[i] = (i == 0 || sorted[i] != sorted[i - 1]) ? 1u : 0u;
        oracle_exclusive_scan(flags.data(), scan.data(), n);
        uint32_t u0 = scan[n - 1] + flags[n - 1];
        counts[0] = u0;
        for (uint32_t i = 0; i < n; ++i)
            if (flags[i]) pbeg[scan[i]] = i;
        for (uint32_t j = 0; j < u0; ++j) pend[j] = (j + 1 < u0) ? pbeg[j + 1] : n;
        for (uint32_t l = 1; l < layers; ++l) {
            uint32_t prev = counts[l - 1], in_off = offsets[l - 1], out_off = offsets[l];
            flags.assign(prev, 0);
            scan.assign(prev, 0);
            for (uint32_t j = 0; j < prev; ++j) {
                uint64_t c = sorted[pbeg[in_off + j]] >> (3u * l);
                uint64_t cp = j ? sorted[pbeg[in_off + j - 1]] >> (3u * l) : 0;
                flags[j] = (j == 0 || c != cp) ? 1u : 0u;
            }
            oracle_exclusive_scan(flags.data(), scan.data(), prev);
            uint32_t u = scan[prev - 1] + flags[prev - 1];
            counts[l] = u;
            for (uint32_t j = 0; j < prev; ++j)
                if (flags[j]) cbeg[out_off + scan[j]] = in_off + j;
            for (uint32_t k = 0; k < u; ++k) {
                uint32_t node = out_off + k;
                cend[node] = (k + 1 < u) ? cbeg[node + 1] : in_off + prev;
                pbeg[node] = pbeg[cbeg[node]];
                pend[node] = pend[cend[node] - 1];
            }
        }
    }

    void aggregate() {
        for (uint32_t l = 0; l < layers; ++l) {
            uint32_t off = offsets[l], u = counts[l];
#pragma omp parallel for schedule(dynamic, 64)
            for (int64_t kk = 0; kk < (int64_t)u; ++kk) {
                uint32_t node = off + (uint32_t)kk;
                if (prec) {
                    double sx = 0, sy = 0, sz = 0, m = 0;
                    if (l == 0) {
                        // FP64 sums over the FP32 frame relative to the system
                        // origin; float x float products are exact in FP64.
                        for (uint32_t i = pbeg[node]; i < pend[node]; ++i) {
                            double mi = (double)rel[4ull * i + 3];
                            m += mi;
                            sx += mi * (double)rel[4ull * i + 0];
                            sy += mi * (double)rel[4ull * i + 1];
                            sz += mi * (double)rel[4ull * i + 2];
                        }
                    } else {
                        for (uint32_t c = cbeg[node]; c < cend[node]; ++c) {
                            sx += sum64[4ull * c + 0];
                            sy += sum64[4ull * c + 1];
                            sz += sum64[4ull * c + 2];
                            m += sum64[4ull * c + 3];
                        }
                    }
                    double* o = &sum64[4ull * node];
                    o[0] = sx;
                    o[1] = sy;
                    o[2] = sz;
                    o[3] = m;
                    // Centre of mass through one reciprocal of the mass: the
                    // FP32 reciprocal refined by one FP64 Newton step.
                    float* c = &cm[4ull * node];
                    double inv = 0.0;
                    if (m > 0) {
                        const double r0 = (double)(1.0f / (float)m);
                        inv = std::fma(r0, std::fma(-m, r0, 1.0), r0);
                    }
                    c[0] = m > 0 ? (float)(sx * inv) : 0.0f;
                    c[1] = m > 0 ? (float)(sy * inv) : 0.0f;
                    c[2] = m > 0 ? (float)(sz * inv) : 0.0f;
                    c[3] = (float)m;
                } else {
                    float sx = 0, sy = 0, sz = 0, m = 0;
                    if (l == 0) {
                        for (uint32_t i = pbeg[node]; i < pend[node]; ++i) {
                            const float* q = &pos[4ull * i];
                            m += q[3];
                            sx += q[3] * q[0];
                            sy += q[3] * q[1];
                            sz += q[3] * q[2];
                        }
                    } else {
                        for (uint32_t c = cbeg[node]; c < cend[node]; ++c) {
                            sx += sum32[4ull * c + 0];
                            sy += sum32[4ull * c + 1];
                            sz += sum32[4ull * c + 2];
                            m += sum32[4ull * c + 3];
                        }
                    }
                    float* o = &sum32[4ull * node];
                    o[0] = sx;
                    o[1] = sy;
                    o[2] = sz;
                    o[3] = m;
                    float* c = &cm[4ull * node];
                    const float inv = m > 0 ? 1.0f / m : 0.0f;
                    c[0] = m > 0 ? sx * inv : 0.0f;
                    c[1] = m > 0 ? sy * inv : 0.0f;
                    c[2] = m > 0 ? sz * inv : 0.0f;
                    c[3] = m;
                }
            }
        }
    }

    static constexpr uint32_t kFlagDelta = 0x8u;      // ASTRO_FLAG_OPEN_DELTA
    static constexpr uint32_t kFlagQuad = 0x10u;      // ASTRO_FLAG_QUADRUPOLE
    static constexpr uint32_t kFlagPerParticle = 0x20u;  // ASTRO_FLAG_PER_PARTICLE
    static constexpr uint32_t kLanes = 32;            // far-node partials (one per lane of a warp)
    static constexpr uint32_t kDefaultGroup = 32;     // group size of params.group_size = 0

    // One accumulator (plain or Kahan) per component.
    struct Acc {
        float s[3] = {0, 0, 0}, c[3] = {0, 0, 0};
        void add(bool kahan, const float t[3]) {
            for (int a = 0; a < 3; ++a) {
                if (kahan) {
                    float y = t[a] - c[a];
                    float u = s[a] + y;
                    c[a] = (u - s[a]) - y;
                    s[a] = u;
                } else {
                    s[a] += t[a];
                }
            }
        }
    };

    // Blocked compensated sum of the group walk: terms are added plainly
    // within blocks of kBlock consecutive list positions, and each block's
    // partial is Kahan-added to the running sum. Every list position
    // counts, including a particle's own (skipped) position in the leaf
    // list, so block boundaries depend on positions only. Without Kahan
    // every term goes straight into the sum.
    struct BlockAcc {
        static constexpr uint32_t kBlock = 32;
        float s[3] = {0, 0, 0}, c[3] = {0, 0, 0}, b[3] = {0, 0, 0};
        uint32_t k = 0;
        void close() {
            for (int a = 0; a < 3; ++a) {
                float y = b[a] - c[a];
                float u = s[a] + y;
                c[a] = (u - s[a]) - y;
                s[a] = u;
                b[a] = 0.0f;
            }
        }
        void add(bool kahan, const float t[3]) {
            for (int a = 0; a < 3; ++a) {
                if (kahan) b[a] += t[a];
                else s[a] += t[a];
            }
        }
        void step(bool kahan) {
            if (kahan && ++k % kBlock == 0) close();
        }
        void finish(bool kahan) {
            if (kahan && k % kBlock != 0) close();
        }
    };

    // Softened monopole of mass m at displacement d (r2t = |d|^2), plus the
    // quadrupole term of q = {Qxx, Qyy, Qxy, Qxz, Qyz} (Qzz = -Qxx - Qyy)
    // when q is not NULL:
    //   a = G m d / r^3 + G [ 5/2 (d.Qd) d / r^7 - Qd / r^5 ],  r^2 = |d|^2 + eps^2.
    void term(float dx, float dy, float dz, float r2t, float m, const float* q, float out[3]) const {
        const float g = p.g, eps2 = p.softening * p.softening;
        float r2 = r2t + eps2;
        float inv = 1.0f / std::sqrt(r2);
        float inv2 = inv * inv;
        float inv3 = inv2 * inv;
        float sc = (g * m) * inv3;
        out[0] = dx * sc;
        out[1] = dy * sc;
        out[2] = dz * sc;
        if (q) {
            float inv5 = inv3 * inv2, inv7 = inv5 * inv2;
            float qzz = -(q[0] + q[1]);
            float qx = (q[0] * dx + q[2] * dy) + q[3] * dz;
            float qy = (q[2] * dx + q[1] * dy) + q[4] * dz;
            float qz = (q[3] * dx + q[4] * dy) + qzz * dz;
            float dqd = (dx * qx + dy * qy) + dz * qz;
            float w = (2.5f * dqd) * inv7;
            out[0] = out[0] + g * ((w * dx) - (qx * inv5));
            out[1] = out[1] + g * ((w * dy) - (qy * inv5));
            out[2] = out[2] + g * ((w * dz) - (qz * inv5));
        }
    }

    // Far nodes of the group walk. The field of a node (mass m, traceless
    // quadrupole Q, as in term()) at displacement d = D - rho from a point
    // rho off the expansion centre, D = com - centre, is taken to second
    // order in rho:
    //   a_i(D - rho) = a_i - J_ij rho_j + 1/2 H_ijk rho_j rho_k,
    // a the field at D, J and H its first and second derivatives. With
    // R = (|D|^2 + eps^2)^(-1/2), q = QD and s = D.Qd:
    //   a_i  = al D_i - R^5 q_i
    //   J_ij = ga (q_i D_j + q_j D_i) - be D_i D_j - R^5 Q_ij + al [i=j]
    //   H_ijk = nu D_i D_j D_k + ka S(qDD) + ga (S(QD) + S(q delta)) - be S(delta D)
    // al = m R^3 + 5/2 s R^7, be = 3 m R^5 + 35/2 s R^9, ga = 5 R^7,
    // ka = -35 R^9, nu = 15 m R^7 + 315/2 s R^11, and S(.) the sum over the
    // three distinct placements of the indices (S(delta D) = delta_ij D_k +
    // delta_ik D_j + delta_jk D_i). The 19 coefficients are stored as
    // a {x, y, z}, J {xx, yy, zz, xy, xz, yz}, H {xxx, yyy, zzz, xxy, xxz,
    // xyy, yyz, xzz, yzz, xyz}. fma(a, b, c) below is a * b + c with both
    // operations rounded, the order the CUDA kernels follow.
    static constexpr int kFarCoefs = 19;
    static float fma2(float a, float b, float c) { return a * b + c; }
    void far_coefs(const float* c, const float* q, const float gc[3], float out[kFarCoefs]) const {
        const float eps2 = p.softening * p.softening;
        const float D[3] = {c[0] - gc[0], c[1] - gc[1], c[2] - gc[2]};
        const float m = c[3];
        const float r2 = fma2(D[0], D[0], fma2(D[1], D[1], D[2] * D[2])) + eps2;
        const float R = 1.0f / std::sqrt(r2);
        const float R2 = R * R, R3 = R2 * R, R5 = R3 * R2, R7 = R5 * R2, R9 = R7 * R2,
                    R11 = R9 * R2;
        const float Q[3][3] = {{q[0], q[2], q[3]}, {q[2], q[1], q[4]}, {q[3], q[4], -(q[0] + q[1])}};
        float qv[3];
        for (int i = 0; i < 3; ++i) qv[i] = fma2(Q[i][0], D[0], fma2(Q[i][1], D[1], Q[i][2] * D[2]));
        const float sq = fma2(D[0], qv[0], fma2(D[1], qv[1], D[2] * qv[2]));
        const float al = fma2(m, R3, (2.5f * sq) * R7);
        const float be = fma2(3.0f * m, R5, (17.5f * sq) * R9);
        const float ga = 5.0f * R7;
        const float ka = -(35.0f * R9);
        const float nu = fma2(15.0f * m, R7, (157.5f * sq) * R11);
        for (int i = 0; i < 3; ++i) out[i] = fma2(al, D[i], -(R5 * qv[i]));
        static const int jx[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
        for (int t = 0; t < 6; ++t) {
            const int i = jx[t][0], j = jx[t][1];
            float v = fma2(ga, fma2(qv[i], D[j], qv[j] * D[i]), -fma2(be, D[i] * D[j], R5 * Q[i][j]));
            if (i == j) v = v + al;
            out[3 + t] = v;
        }
        static const int hx[10][3] = {{0, 0, 0}, {1, 1, 1}, {2, 2, 2}, {0, 0, 1}, {0, 0, 2},
                                      {0, 1, 1}, {1, 1, 2}, {0, 2, 2}, {1, 2, 2}, {0, 1, 2}};
        for (int t = 0; t < 10; ++t) {
            const int i = hx[t][0], j = hx[t][1], k = hx[t][2];
            const float cij = i == j ? 1.0f : 0.0f, cik = i == k ? 1.0f : 0.0f,
                        cjk = j == k ? 1.0f : 0.0f;
            const float dij = D[i] * D[j];
            const float sqdd = fma2(qv[i], D[j] * D[k], fma2(qv[j], D[i] * D[k], qv[k] * dij));
            const float sqd = fma2(Q[i][j], D[k], fma2(Q[i][k], D[j], Q[j][k] * D[i]));
            const float sqdel = fma2(cjk, qv[i], fma2(cik, qv[j], cij * qv[k]));
            const float sdel = fma2(cij, D[k], fma2(cik, D[j], cjk * D[i]));
            out[9 + t] = fma2(nu, dij * D[k], fma2(ka, sqdd, fma2(ga, sqd + sqdel, -(be * sdel))));
        }
    }

    // The expansion of coefficients f about the group centre at offset rho,
    // times G.
    void far_eval(const float f[kFarCoefs], const float rho[3], float out[3]) const {
        const float pxx = rho[0] * rho[0], pyy = rho[1] * rho[1], pzz = rho[2] * rho[2];
        const float pxy = rho[0] * rho[1], pxz = rho[0] * rho[2], pyz = rho[1] * rho[2];
        // Per component: J row {j_x, j_y, j_z} and H row {xx, yy, zz, xy, xz, yz}.
        static const int jr[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
        static const int hr[3][6] = {{0, 5, 7, 3, 4, 9}, {3, 1, 8, 5, 9, 6}, {4, 6, 2, 9, 7, 8}};
        for (int i = 0; i < 3; ++i) {
            const float* J = f + 3;
            const float* H = f + 9;
            const float jr_ = fma2(J[jr[i][0]], rho[0], fma2(J[jr[i][1]], rho[1], J[jr[i][2]] * rho[2]));
            const float cross = fma2(H[hr[i][3]], pxy, fma2(H[hr[i][4]], pxz, H[hr[i][5]] * pyz));
            const float hh = fma2(H[hr[i][0]], pxx, fma2(H[hr[i][1]], pyy, fma2(H[hr[i][2]], pzz, 2.0f * cross)));
            out[i] = p.g * fma2(0.5f, hh, f[i] - jr_);
        }
    }

    float node_crit2(uint32_t nd, uint32_t l, uint32_t s) const {
        return (p.flags & kFlagDelta) ? ncrit2[nd] : quant[s].crit2[l];
    }

    void finish(uint32_t ip, const float a[3]) {
        const float cl = p.force_clamp;
        float* o = &acc[4ull * ip];
        for (int k = 0; k < 3; ++k) o[k] = std::fmin(std::fmax(a[k], -cl), cl);
        o[3] = 0.0f;
    }

    // barnesHut (BarnesHut.metal:22-101) per particle in sorted order:
    // children pushed in order and popped last first, as the reference's
    // stack does; one accumulator in visiting order.
    void traverse_per_particle() {
        const bool kahan = prec, quad_on = (p.flags & kFlagQuad) != 0;
        uint64_t tot_inter = 0, tot_visits = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : tot_inter, tot_visits)
        for (int64_t ipp = 0; ipp < (int64_t)n; ++ipp) {
            uint32_t ip = (uint32_t)ipp, s = sys_of[ip];
            const float px = rel[4ull * ip], py = rel[4ull * ip + 1], pz = rel[4ull * ip + 2];
            Acc A;
            float t[3];
            uint64_t inter = 0, vis = 0;
            std::vector<uint32_t> st_node, st_layer;
            st_node.push_back(offsets[lbits] + s);
            st_layer.push_back(lbits);
            while (!st_node.empty()) {
                uint32_t nd = st_node.back(), l = st_layer.back();
                st_node.pop_back();
                st_layer.pop_back();
                ++vis;
                const float* c = &cm[4ull * nd];
                float dx = c[0] - px, dy = c[1] - py, dz = c[2] - pz;
                float r2t = dx * dx + dy * dy + dz * dz;
                if (r2t > node_crit2(nd, l, s)) {
                    term(dx, dy, dz, r2t, c[3], quad_on ? &quad[5ull * nd] : nullptr, t);
                    A.add(kahan, t);
                    ++inter;
                } else if (l == 0 || pend[nd] - pbeg[nd] <= p.bucket) {
                    for (uint32_t j = pbeg[nd]; j < pend[nd]; ++j) {
                        if (j == ip) continue;
                        const float* q = &rel[4ull * j];
                        float ex = q[0] - px, ey = q[1] - py, ez = q[2] - pz;
                        term(ex, ey, ez, ex * ex + ey * ey + ez * ez, q[3], nullptr, t);
                        A.add(kahan, t);
                        ++inter;
                    }
                } else {
                    for (uint32_t ch = cbeg[nd]; ch < cend[nd]; ++ch) {
                        st_node.push_back(ch);
                        st_layer.push_back(l - 1);
                    }
                }
            }
            finish(ip, A.s);
            tot_inter += inter;
            tot_visits += vis;
        }
        interactions = tot_inter;
        visits = tot_visits;
    }

    // Groups for the group walk: every particle in exactly one group of at
    // most kGroup consecutive (sorted) particles of one system, kGroup =
    // params.group_size (0 = 32; at most 64, two particles per lane).
    //  - a node with more than kGroup particles packs its consecutive small
    //    children (at most kGroup particles each) greedily, in child order;
    //  - a top-layer node with at most kGroup particles is a group;
    //  - a leaf with more than kGroup particles is cut into kGroup chunks,
    //    which are walked against the box of the whole leaf.
    // Each group: its particles [first, second) and the particles [wb, we)
    // whose bounding box its walk tests.
    struct Group {
        uint32_t first, second, wb, we;
    };
    std::vector<Group> make_groups() const {
        const uint32_t kGroup = p.group_size ? p.group_size : kDefaultGroup;
        std::vector<Group> groups;
        for (uint32_t l = 0; l < layers; ++l)
            for (uint32_t k = 0; k < counts[l]; ++k) {
                uint32_t node = offsets[l] + k, pc = pend[node] - pbeg[node];
                if (pc <= kGroup) {
                    if (l == lbits) groups.push_back({pbeg[node], pend[node], pbeg[node], pend[node]});
                    continue;
                }
                if (l == 0) {
                    for (uint32_t b = pbeg[node]; b < pend[node]; b += kGroup)
                        groups.push_back({b, std::min(b + kGroup, pend[node]), pbeg[node], pend[node]});
                    continue;
                }
                uint32_t gb = 0, ge = 0;
                for (uint32_t ch = cbeg[node]; ch < cend[node]; ++ch) {
                    uint32_t cc = pend[ch] - pbeg[ch];
                    if (cc <= kGroup) {
                        if (ge == gb) {
                            gb = pbeg[ch];
                            ge = pend[ch];
                        } else if ((ge - gb) + cc <= kGroup) {
                            ge = pend[ch];
                        } else {
                            groups.push_back({gb, ge, gb, ge});
                            gb = pbeg[ch];
                            ge = pend[ch];
                        }
                    } else if (ge != gb) {
                        groups.push_back({gb, ge, gb, ge});
                        gb = ge = 0;
                    }
                }
                if (ge != gb) groups.push_back({gb, ge, gb, ge});
            }
        return groups;
    }

    // Group walk: the tree is walked once per group, breadth first from the
    // system's root, against the group's bounding box. A node is accepted
    // when the box lies outside its opening radius; an opened leaf or bucket
    // goes to the particle list; other opened nodes contribute their
    // children to the next level. Each particle then sums the accepted cells
    // (in walk order) and, separately, the particles of the listed leaves and
    // buckets (in walk order, itself excluded); a = cells + particles.
    // With params.far_ratio > 0 an accepted node whose centre of mass lies
    // further than r_g / far_ratio from the centre of the group's box (r_g
    // its half diagonal) is a far node: its expansion coefficients
    // (far_coefs) go into one of 32 partial sums, far node f into partial
    // f mod 32 in walk order; the partials are combined by the pairwise
    // exchange 16, 8, 4, 2, 1 (partial l + partial l^o), and each particle
    // adds the expansion at its offset: a = (cells + particles) + far.
    void traverse_groups() {
        const bool kahan = prec, quad_on = (p.flags & kFlagQuad) != 0;
        const auto groups = make_groups();
        const float fr2 = p.far_ratio * p.far_ratio;
        uint64_t tot_inter = 0, tot_visits = 0, tot_far_nodes = 0, tot_far_inter = 0;
#pragma omp parallel for schedule(dynamic, 16) \
    reduction(+ : tot_inter, tot_visits, tot_far_nodes, tot_far_inter)
        for (int64_t gi = 0; gi < (int64_t)groups.size(); ++gi) {
            const uint32_t gb = groups[gi].first, ge = groups[gi].second;
            const uint32_t s = sys_of[gb];
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (uint32_t i = groups[gi].wb; i < groups[gi].we; ++i)
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], rel[4ull * i + a]);
                    hi[a] = std::max(hi[a], rel[4ull * i + a]);
                }
            float gc[3], hr[3];
            for (int a = 0; a < 3; ++a) {
                gc[a] = (lo[a] + hi[a]) * 0.5f;
                hr[a] = (hi[a] - lo[a]) * 0.5f;
            }
            const float rg2 = fma2(hr[0], hr[0], fma2(hr[1], hr[1], hr[2] * hr[2]));
            std::vector<uint32_t> frontier{offsets[lbits] + s}, next, cells, leaves, far;
            uint64_t tested = 0;
            for (int l = (int)lbits; !frontier.empty(); --l) {
                next.clear();
                for (uint32_t nd : frontier) {
                    ++tested;
                    const float* c = &cm[4ull * nd];
                    float d[3];
                    for (int a = 0; a < 3; ++a) d[a] = std::max(std::max(lo[a] - c[a], c[a] - hi[a]), 0.0f);
                    float dist2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    if (dist2 > node_crit2(nd, (uint32_t)l, s)) {
                        bool is_far = false;
                        if (fr2 > 0.0f) {
                            const float D[3] = {c[0] - gc[0], c[1] - gc[1], c[2] - gc[2]};
                            is_far = fr2 * fma2(D[0], D[0], fma2(D[1], D[1], D[2] * D[2])) > rg2;
                        }
                        (is_far ? far : cells).push_back(nd);
                    } else if (l == 0 || pend[nd] - pbeg[nd] <= p.bucket) {
                        leaves.push_back(nd);
                    } else {
                        for (uint32_t ch = cbeg[nd]; ch < cend[nd]; ++ch) next.push_back(ch);
                    }
                }
                frontier.swap(next);
            }
            float fsum[kFarCoefs] = {};
            if (!far.empty()) {
                float part[kLanes][kFarCoefs] = {};
                static const float kZeroQ[5] = {0, 0, 0, 0, 0};
                for (size_t f = 0; f < far.size(); ++f) {
                    float co[kFarCoefs];
                    far_coefs(&cm[4ull * far[f]], quad_on ? &quad[5ull * far[f]] : kZeroQ, gc, co);
                    for (int k = 0; k < kFarCoefs; ++k) part[f % kLanes][k] += co[k];
                }
                for (uint32_t o = kLanes / 2; o > 0; o >>= 1) {
                    float nxt[kLanes][kFarCoefs];
                    for (uint32_t l = 0; l < kLanes; ++l)
                        for (int k = 0; k < kFarCoefs; ++k) nxt[l][k] = part[l][k] + part[l ^ o][k];
                    std::memcpy(part, nxt, sizeof(part));
                }
                std::memcpy(fsum, part[0], sizeof(fsum));
                // One expansion per walk: the chunks of a leaf share one.
                if (groups[gi].first == groups[gi].wb) tot_far_nodes += far.size();
            }
            for (uint32_t ip = gb; ip < ge; ++ip) {
                const float px = rel[4ull * ip], py = rel[4ull * ip + 1], pz = rel[4ull * ip + 2];
                BlockAcc A, B;
                float t[3];
                uint64_t inter = far.size();
                tot_far_inter += far.size();
                for (uint32_t nd : cells) {
                    const float* c = &cm[4ull * nd];
                    float dx = c[0] - px, dy = c[1] - py, dz = c[2] - pz;
                    term(dx, dy, dz, dx * dx + dy * dy + dz * dz, c[3],
                         quad_on ? &quad[5ull * nd] : nullptr, t);
                    A.add(kahan, t);
                    A.step(kahan);
                    ++inter;
                }
                A.finish(kahan);
                for (uint32_t nd : leaves)
                    for (uint32_t j = pbeg[nd]; j < pend[nd]; ++j) {
                        if (j != ip) {
                            const float* q = &rel[4ull * j];
                            float ex = q[0] - px, ey = q[1] - py, ez = q[2] - pz;
                            term(ex, ey, ez, ex * ex + ey * ey + ez * ez, q[3], nullptr, t);
                            B.add(kahan, t);
                            ++inter;
                        }
                        B.step(kahan);
                    }
                B.finish(kahan);
                float a3[3] = {A.s[0] + B.s[0], A.s[1] + B.s[1], A.s[2] + B.s[2]};
                if (!far.empty()) {
                    const float rho[3] = {px - gc[0], py - gc[1], pz - gc[2]};
                    float fa[3];
                    far_eval(fsum, rho, fa);
                    for (int a = 0; a < 3; ++a) a3[a] = a3[a] + fa[a];
                }
                finish(ip, a3);
                tot_inter += inter;
                tot_visits += tested;
            }
        }
        interactions = tot_inter;
        visits = tot_visits;
        far_nodes = tot_far_nodes;
        far_interactions = tot_far_inter;
    }

    // Kick-drift (BarnesHut.metal:189-194 without damping and type scale).
    void integrate(float dt) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; ++i)
            for (int a = 0; a < 3; ++a) {
                float v = vel[4ull * i + a] + acc[4ull * i + a] * dt;
                vel[4ull * i + a] = v;
                if (prec)
                    x64[3ull * i + a] = x64[3ull * i + a] + (double)v * (double)dt;
                else
                    pos[4ull * i + a] = pos[4ull * i + a] + v * dt;
            }
    }

    // Quadrupole moments about each node's centre of mass (parallel-axis
    // sums over children, traceless: Qzz = -Qxx - Qyy) and the
    // delta-corrected opening radius (size / theta + w |com - cell centre|)^2,
    // w = params.open_delta_weight.
    void moments() {
        const bool want_q = (p.flags & kFlagQuad) != 0, want_d = (p.flags & kFlagDelta) != 0;
        if (!want_q && !want_d) return;
        for (uint32_t l = 0; l < layers; ++l) {
            uint32_t off = offsets[l], u = counts[l];
#pragma omp parallel for schedule(dynamic, 64)
            for (int64_t kk = 0; kk < (int64_t)u; ++kk) {
                uint32_t node = off + (uint32_t)kk;
                const float* c = &cm[4ull * node];
                const uint32_t s = sys_of[pbeg[node]];
                // The node's cell: geometric centre and edge.
                float center[3], size;
                {
                    uint64_t code = (sorted[pbeg[node]] & ((1ull << (3 * lbits)) - 1)) >> (3 * l);
                    uint32_t cc[3] = {0, 0, 0};
                    for (uint32_t b = 0; b < lbits - l; ++b)
                        for (int a = 0; a < 3; ++a) cc[a] |= (uint32_t)((code >> (3 * b + a)) & 1) << b;
                    size = std::ldexp(quant[s].ext, (int)l - (int)lbits);
                    float half = 0.5f * size;
                    for (int a = 0; a < 3; ++a) center[a] = quant[s].lo[a] + (float)(2 * cc[a] + 1) * half;
                }
                if (want_q) {
                    float q[5] = {0, 0, 0, 0, 0};
                    auto add = [&](float m, float dx, float dy, float dz) {
                        float r2 = dx * dx + dy * dy + dz * dz;
                        q[0] += m * (3 * dx * dx - r2);
                        q[1] += m * (3 * dy * dy - r2);
                        q[2] += m * (3 * dx * dy);
                        q[3] += m * (3 * dx * dz);
                        q[4] += m * (3 * dy * dz);
                    };
                    if (l == 0) {
                        // A leaf: first and second mass moments about the
                        // cell centre in one pass, shifted to the centre of
                        // mass: P = S - e D^T - D e^T + M e e^T, e = com -
                        // centre; Q = 3 P - tr(P) I.
                        float d[3] = {0, 0, 0}, sm[6] = {0, 0, 0, 0, 0, 0};  // xx yy zz xy xz yz
                        for (uint32_t i = pbeg[node]; i < pend[node]; ++i) {
                            const float* x = &rel[4ull * i];
                            const float u[3] = {x[0] - center[0], x[1] - center[1], x[2] - center[2]};
                            const float t[3] = {x[3] * u[0], x[3] * u[1], x[3] * u[2]};
                            for (int a = 0; a < 3; ++a) d[a] += t[a];
                            sm[0] += t[0] * u[0];
                            sm[1] += t[1] * u[1];
                            sm[2] += t[2] * u[2];
                            sm[3] += t[0] * u[1];
                            sm[4] += t[0] * u[2];
                            sm[5] += t[1] * u[2];
                        }
                        const float e[3] = {c[0] - center[0], c[1] - center[1], c[2] - center[2]};
                        const float mm = c[3];
                        auto shifted = [&](float sab, int a, int b) {
                            return ((sab - e[a] * d[b]) - e[b] * d[a]) + e[a] * (mm * e[b]);
                        };
                        const float pxx = shifted(sm[0], 0, 0), pyy = shifted(sm[1], 1, 1),
                                    pzz = shifted(sm[2], 2, 2), pxy = shifted(sm[3], 0, 1),
                                    pxz = shifted(sm[4], 0, 2), pyz = shifted(sm[5], 1, 2);
                        const float tr = (pxx + pyy) + pzz;
                        q[0] = 3.0f * pxx - tr;
                        q[1] = 3.0f * pyy - tr;
                        q[2] = 3.0f * pxy;
                        q[3] = 3.0f * pxz;
                        q[4] = 3.0f * pyz;
                    } else {
                        for (uint32_t ch = cbeg[node]; ch < cend[node]; ++ch) {
                            const float* cc = &cm[4ull * ch];
                            add(cc[3], cc[0] - c[0], cc[1] - c[1], cc[2] - c[2]);
                            for (int a = 0; a < 5; ++a) q[a] += quad[5ull * ch + a];
                        }
                    }
                    for (int a = 0; a < 5; ++a) quad[5ull * node + a] = q[a];
                }
                if (want_d) {
                    float d[3];
                    for (int a = 0; a < 3; ++a) d[a] = c[a] - center[a];
                    float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    float crit = size / p.theta + p.open_delta_weight * std::sqrt(dd);
                    ncrit2[node] = crit * crit;
                }
            }
        }
    }

    void step(uint32_t split_passes, float dt) {
        setup_quant();
        encode();
        sort(split_passes);
        topology();
        aggregate();
        moments();
        if (p.flags & kFlagPerParticle) traverse_per_particle();
        else traverse_groups();
        integrate(dt);
    }

    void write_outputs(oracle_outputs* out) {
        if (!out) return;
        if (out->codes)
            for (uint32_t j = 0; j < n; ++j) out->codes[id[j]] = sorted[j];
        if (out->sorted_codes) std::memcpy(out->sorted_codes, sorted.data(), 8ull * n);
        if (out->sorted_indices) std::memcpy(out->sorted_indices, id.data(), 4ull * n);
        if (out->layer_counts) std::memcpy(out->layer_counts, counts.data(), 4ull * layers);
        if (out->layer_sizes) std::memcpy(out->layer_sizes, sizes.data(), 4ull * layers);
        if (out->layer_offsets) std::memcpy(out->layer_offsets, offsets.data(), 4ull * layers);
        if (out->acc4)
            for (uint32_t j = 0; j < n; ++j)
                std::memcpy(&out->acc4[4ull * id[j]], &acc[4ull * j], 16);
        out->interactions = interactions;
        out->far_nodes = far_nodes;
        out->far_interactions = far_interactions;
        out->node_visits = visits;
        if (out->nodes) {
            // Every slot, or the listed ones (nodes_index) in their order.
            const uint64_t count = out->nodes_index ? out->nodes_count : capacity;
            for (uint64_t i = 0; i < count; ++i) {
                const uint64_t slot = out->nodes_index ? out->nodes_index[i] : i;
                OctreeNode& o = out->nodes[i];
                std::memset(&o, 0, sizeof(o));
                o.mortonCode = kInvalidCode;
                for (int c = 0; c < 8; ++c) o.children[c] = kInvalidChild;
                uint32_t l = 0;
                while (l + 1 < layers && slot >= offsets[l + 1]) ++l;
                if (slot >= capacity || slot < offsets[l] || slot - offsets[l] >= counts[l]) continue;
                const uint32_t node = (uint32_t)slot;
                o.mortonCode = sorted[pbeg[node]] >> (3u * l);
                for (int a = 0; a < 3; ++a) o.centerOfMass[a] = cm[4ull * node + a];
                o.totalMass = cm[4ull * node + 3];
                o.layer = l;
                if (l > 0)
                    for (uint32_t c = cbeg[node], q = 0; c < cend[node] && q < 8; ++c, ++q)
                        o.children[q] = c;
            }
        }
    }
};

}  // namespace

extern "C" void oracle_far_expand(const astro_params* p, const float* cm4, const float* q5,
                                  const float* gc3, const float* rho3, float* coefs19, float* acc3) {
    PhysState st;
    st.p = *p;
    float co[PhysState::kFarCoefs];
    st.far_coefs(cm4, q5, gc3, co);
    if (coefs19) std::memcpy(coefs19, co, sizeof(co));
    if (acc3) st.far_eval(co, rho3, acc3);
}

extern "C" int oracle_phys_run(const astro_params* p, PositionMass* pm, VelocityRadius* vr,
                               uint32_t n, const uint32_t* sys_sizes, uint32_t nsys, float dt,
                               uint32_t nsteps, uint32_t split_passes, double* pos64,
                               oracle_outputs* out) {
    if (!p || !pm || !vr || n == 0 || p->lbits < 1 || p->lbits > 21) return -1;
    uint32_t one = n;
    if (!sys_sizes) {
        sys_sizes = &one;
        nsys = 1;
    }
    uint64_t total = 0;
    for (uint32_t s = 0; s < nsys; ++s) {
        if (sys_sizes[s] == 0) return -1;
        total += sys_sizes[s];
    }
    if (total != n) return -1;
    PhysState st;
    st.p = *p;
    st.n = n;
    st.nsys = nsys;
    st.lbits = p->lbits;
    st.layers = p->lbits + 1;
    st.sysbits = nsys > 1 ? system_bits(nsys) : 0;
    if (3u * st.lbits + st.sysbits > 64) return -1;
    st.prec = p->form == ASTRO_FORM_PRECISION;
    st.pos.resize(4ull * n);
    st.vel.resize(4ull * n);
    st.acc.assign(4ull * n, 0.0f);
    st.rel.resize(4ull * n);
    st.id.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            st.pos[4ull * i + a] = pm[i].position[a];
            st.vel[4ull * i + a] = vr[i].velocity[a];
        }
        st.pos[4ull * i + 3] = pm[i].mass;
        st.vel[4ull * i + 3] = vr[i].radius;
        st.id[i] = i;
    }
    if (st.prec) {
        st.x64.resize(3ull * n);
        for (uint32_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) st.x64[3ull * i + a] = (double)pm[i].position[a];
    }
    st.layout(sys_sizes);
    for (uint32_t s = 0; s < nsteps; ++s) st.step(split_passes, dt);
    st.write_outputs(out);
    for (uint32_t j = 0; j < n; ++j) {
        uint32_t i = st.id[j];
        for (int a = 0; a < 3; ++a) {
            pm[i].position[a] = st.prec ? (float)st.x64[3ull * j + a] : st.pos[4ull * j + a];
            vr[i].velocity[a] = st.vel[4ull * j + a];
        }
        if (pos64 && st.prec)
            for (int a = 0; a < 3; ++a) pos64[3ull * i + a] = st.x64[3ull * j + a];
    }
    return 0;
}

extern "C" void oracle_direct_accel_f64(const PositionMass* pm, const double* pos64, uint32_t n,
                                        const uint32_t* sys_sizes, uint32_t nsys,
                                        const uint32_t* sample_idx, uint32_t n_sample, double g,
                                        double eps, double* acc3) {
    std::vector<uint32_t> off(1, 0);
    if (!sys_sizes) {
        off.push_back(n);
    } else {
        for (uint32_t s = 0; s < nsys; ++s) off.push_back(off.back() + sys_sizes[s]);
    }
    auto X = [&](uint32_t i, int a) {
        return pos64 ? pos64[3ull * i + a] : (double)pm[i].position[a];
    };
    const double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t k = 0; k < (int64_t)n_sample; ++k) {
        uint32_t i = sample_idx[k];
        uint32_t s = (uint32_t)(std::upper_bound(off.begin(), off.end(), i) - off.begin()) - 1;
        double xi = X(i, 0), yi = X(i, 1), zi = X(i, 2);
        double ax = 0, ay = 0, az = 0;
        for (uint32_t j = off[s]; j < off[s + 1]; ++j) {
            if (j == i) continue;
            double dx = X(j, 0) - xi, dy = X(j, 1) - yi, dz = X(j, 2) - zi;
            double r2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv = 1.0 / std::sqrt(r2);
            double w = g * (double)pm[j].mass * inv * inv * inv;
            ax += w * dx;
            ay += w * dy;
            az += w * dz;
        }
        acc3[3 * k] = ax;
        acc3[3 * k + 1] = ay;
        acc3[3 * k + 2] = az;
    }
}
