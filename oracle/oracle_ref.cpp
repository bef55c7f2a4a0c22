// ORACLE — test infrastructure only (see astro_oracle.h). Not part of the product.
//
// REFERENCE preset: the Metal kernels of the osbo/astro step restated as
// loops over gid, dispatched in the order Renderer.draw encodes them
// (Astro/Renderer.swift:495-755). Each function names the reference lines it
// follows. Arithmetic is FP32 round-to-nearest without contraction.
#include "astro_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint64_t kInvalidCode = ASTRO_INVALID_MORTON_CODE;  // bridge.h:91-94
constexpr uint32_t kInvalidChild = ASTRO_INVALID_CHILD;       // Octree.metal:10
constexpr uint32_t kScanBlock = 512;                          // RadixSort.metal:5

// MSL leaves an out-of-range float->uint conversion implementation-defined
// (MortonCode.metal:35-37). Here it is defined as a saturating
// round-toward-zero conversion: NaN and values <= 0 give 0, values >= 2^32
// give 0xFFFFFFFF. The CUDA kernels use the same conversion.
inline uint32_t float_to_uint_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

OctreeNode empty_node() {  // clearOctreeNodeBuffer, Octree.metal:253-269
    OctreeNode n;
    std::memset(&n, 0, sizeof(n));
    n.mortonCode = kInvalidCode;
    for (int i = 0; i < 8; ++i) n.children[i] = kInvalidChild;
    n.layer = 0;
    return n;
}

// prefixSum, RadixSort.metal:44-85: one 512-thread threadgroup scanning 1024
// values in threadgroup memory (up-sweep, then down-sweep), written shifted by
// zeroff so the block result is exclusive; aux[b] receives the block total.
void prefix_sum_block(const uint32_t* input, uint32_t* output, uint32_t* aux, uint32_t len,
                      uint32_t zeroff, uint32_t b) {
    uint32_t s[2 * kScanBlock];
    for (uint32_t t = 0; t < kScanBlock; ++t) {
        uint64_t t1 = (uint64_t)t + 2ull * b * kScanBlock, t2 = t1 + kScanBlock;
        s[t] = t1 < len ? input[t1] : 0u;
        s[t + kScanBlock] = t2 < len ? input[t2] : 0u;
    }
    for (uint32_t stride = 1; stride <= kScanBlock; stride <<= 1)
        for (uint32_t t = 0; t < kScanBlock; ++t) {
            uint64_t index = (uint64_t)(t + 1) * stride * 2 - 1;
            if (index < 2 * kScanBlock) s[index] += s[index - stride];
        }
    for (uint32_t stride = kScanBlock >> 1; stride > 0; stride >>= 1)
        for (uint32_t t = 0; t < kScanBlock; ++t) {
            uint64_t index = (uint64_t)(t + 1) * stride * 2 - 1;
            if (index + stride < 2 * kScanBlock) s[index + stride] += s[index];
        }
    for (uint32_t t = 0; t < kScanBlock; ++t) {
        uint64_t t1 = (uint64_t)t + 2ull * b * kScanBlock, t2 = t1 + kScanBlock;
        if (t1 + zeroff < len) output[t1 + zeroff] = s[t];
        if (t2 + zeroff < len)
            output[t2 + zeroff] = (t == kScanBlock - 1 && zeroff) ? 0u : s[t + kScanBlock];
    }
    if (zeroff && b == 0 && len > 0) output[0] = 0;
    if (aux) aux[b] = s[2 * kScanBlock - 1];
}

// prefixFixup, RadixSort.metal:30-42.
void prefix_fixup_block(uint32_t* input, const uint32_t* aux, uint32_t len, uint32_t b) {
    uint32_t block_sum = aux[b];
    for (uint32_t t = 0; t < kScanBlock; ++t) {
        uint64_t start = (uint64_t)t + 2ull * b * kScanBlock;
        if (start < len) input[start] += block_sum;
        if (start + kScanBlock < len) input[start + kScanBlock] += block_sum;
    }
}

// ScanKernel.encodeScanTo, RadixSort.swift:225-279 (zeroff = 1). The
// reference scans the block sums with one threadgroup, which caps len at
// 1,048,576; here the block sums are scanned by the same routine
// recursively, which lifts the cap and changes nothing below it.
void encode_scan(const uint32_t* input, uint32_t* output, uint32_t len) {
    if (len == 0) return;
    uint32_t nblocks = (len + 2 * kScanBlock - 1) / (2 * kScanBlock);
    std::vector<uint32_t> aux(nblocks), aux2(nblocks);
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblocks; ++b)
        prefix_sum_block(input, output, aux.data(), len, 1, (uint32_t)b);
    if (nblocks <= 1) return;
    encode_scan(aux.data(), aux2.data(), nblocks);
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblocks; ++b)
        prefix_fixup_block(output, aux2.data(), len, (uint32_t)b);
}

// SplitKernel.encodeSplitTo, RadixSort.swift:312-349: split_prep
// (RadixSort.metal:89-100), the scan, split_scatter (RadixSort.metal:102-131).
void split_pass(const uint64_t* in, const uint32_t* in_idx, uint64_t* out, uint32_t* out_idx,
                uint32_t bit, uint32_t count, uint32_t* e, uint32_t* f) {
#pragma omp parallel for schedule(static)
    for (int64_t tid = 0; tid < (int64_t)count; ++tid) e[tid] = (in[tid] & (1ull << bit)) == 0;
    encode_scan(e, f, count);
    uint32_t total_falses = f[count - 1] + e[count - 1];
#pragma omp parallel for schedule(static)
    for (int64_t tid = 0; tid < (int64_t)count; ++tid) {
        bool is_bit_set = (in[tid] & (1ull << bit)) != 0;
        uint32_t dst = is_bit_set ? total_falses + ((uint32_t)tid - f[tid]) : f[tid];
        out[dst] = in[tid];
        out_idx[dst] = in_idx[tid];
    }
}

}  // namespace

extern "C" {

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n <= 0) n = omp_get_num_procs();
    omp_set_num_threads(n);
    return n;
#else
    (void)n;
    return 1;
#endif
}

// interleaveBitsOptimized, MortonCode.metal:7-23: bit i of x, y, z goes to
// key bit 3i, 3i+1, 3i+2 for i < 21.
uint64_t oracle_interleave_bits(uint32_t x, uint32_t y, uint32_t z) {
    x &= 0x1FFFFFu;
    y &= 0x1FFFFFu;
    z &= 0x1FFFFFu;
    uint64_t result = 0;
    for (int i = 0; i < 21; ++i) {
        result |= (uint64_t)(x & (1u << i)) << (2 * i);
        result |= (uint64_t)(y & (1u << i)) << (2 * i + 1);
        result |= (uint64_t)(z & (1u << i)) << (2 * i + 2);
    }
    return result;
}

// generateMortonCodes, MortonCode.metal:26-52, with the bound check the
// reference omits and the key width 3*lbits (lbits = 6 there).
void oracle_generate_morton_codes(const PositionMass* pos, uint64_t* codes, uint64_t* unsorted,
                                  uint32_t count, uint32_t lbits, float offset) {
    const uint32_t unused_bits = 63u - 3u * lbits;
#pragma omp parallel for schedule(static)
    for (int64_t gid = 0; gid < (int64_t)count; ++gid) {
        const PositionMass& d = pos[gid];
        uint32_t x = float_to_uint_sat(d.position[0] + offset);
        uint32_t y = float_to_uint_sat(d.position[1] + offset);
        uint32_t z = float_to_uint_sat(d.position[2] + offset);
        uint64_t code = oracle_interleave_bits(x, y, z) >> unused_bits;
        codes[gid] = code;
        unsorted[gid] = code;
    }
}

void oracle_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t len) {
    encode_scan(in, out, len);
}

// MetalKernelsRadixSort.sort, RadixSort.swift:98-185: copy count pairs into
// the ping-pong temporaries, run npasses one-bit splits from bit 0 (64 in the
// reference), copy the result out.
void oracle_split_sort(const uint64_t* in_keys, const uint32_t* in_idx, uint64_t* out_keys,
                       uint32_t* out_idx, uint32_t count, uint32_t npasses) {
    if (count == 0) return;
    std::vector<uint64_t> ka(in_keys, in_keys + count), kb(count);
    std::vector<uint32_t> ia(in_idx, in_idx + count), ib(count), e(count), f(count);
    for (uint32_t bit = 0; bit < npasses; ++bit) {
        split_pass(ka.data(), ia.data(), kb.data(), ib.data(), bit, count, e.data(), f.data());
        ka.swap(kb);
        ia.swap(ib);
    }
    std::memcpy(out_keys, ka.data(), sizeof(uint64_t) * count);
    std::memcpy(out_idx, ia.data(), sizeof(uint32_t) * count);
}

// Renderer.makeBuffers, Renderer.swift:373-386: layer l holds at most
// min(count, 2^(3*(lbits-l))) nodes; with several systems the bound is summed
// per system (the batched form). Offsets are the running sum; the root of
// system s is node offsets[lbits] + s.
uint64_t oracle_layer_layout(uint32_t count, uint32_t nsys, uint32_t lbits, uint32_t* sizes,
                             uint32_t* offsets) {
    (void)nsys;
    uint64_t off = 0;
    for (uint32_t l = 0; l <= lbits; ++l) {
        uint32_t bits_remaining = 3u * (lbits - l);
        uint64_t possible = bits_remaining >= 40 ? (1ull << 40) : (1ull << bits_remaining);
        uint64_t size = std::min<uint64_t>(count, possible);
        if (sizes) sizes[l] = (uint32_t)size;
        if (offsets) offsets[l] = (uint32_t)off;
        off += size;
    }
    return off;
}

// lightingPass (BarnesHut.metal:103-167): for s < min(numStars, 5) (the
// unrolled "if (numStars >= s+1)" blocks), in order:
//   dist = length(x_s - x); d = max(dist / LIGHT_ATTENUATION_DISTANCE, 1e-9)
//   (bridge.h:98: 4e5); light += rgb_s * (1 / (d * d));
// rgb = light; alpha = type 2 ? min(max(r, max(g, b)), 0.25) : 1 (:161-166).
// The lights are read first: no colour written here feeds another particle.
void oracle_lighting(const PositionMass* pm, ColorType* ct, uint32_t n, uint32_t num_stars) {
    const uint32_t nl = std::min(std::min(num_stars, 5u), n);
    float lp[5][3], lc[5][3];
    for (uint32_t s = 0; s < nl; ++s)
        for (int a = 0; a < 3; ++a) {
            lp[s][a] = pm[s].position[a];
            lc[s][a] = ct[s].color[a];
        }
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t type = ct[i].type;
        if (type != 1u && type != 2u) continue;
        float light[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t s = 0; s < nl; ++s) {
            const float dx = lp[s][0] - pm[i].position[0];
            const float dy = lp[s][1] - pm[i].position[1];
            const float dz = lp[s][2] - pm[i].position[2];
            const float dist = std::sqrt(dx * dx + dy * dy + dz * dz);
            const float d = std::max(dist / 4e5f, 1e-9f);
            const float att = 1.0f / (d * d);
            for (int a = 0; a < 3; ++a) light[a] = light[a] + lc[s][a] * att;
        }
        for (int a = 0; a < 3; ++a) ct[i].color[a] = light[a];
        ct[i].color[3] = type == 2u ? std::min(std::max(light[0], std::max(light[1], light[2])), 0.25f)
                                    : 1.0f;
    }
}

}  // extern "C"

namespace {

// The Renderer's compute state (Renderer.swift:56-70,336-391) for one frame.
struct RefFrame {
    astro_params p{};
    uint32_t n = 0, n_tree = 0, layers = 0;
    std::vector<uint32_t> sizes, offsets;
    uint64_t capacity = 0;
    std::vector<uint64_t> morton, unsorted_codes, sorted_codes;
    std::vector<uint32_t> unsorted_idx, sorted_idx, unique_idx, flags, scan;
    uint32_t parent_count = 0, child_count = 0;
    std::vector<OctreeNode> nodes;
    std::vector<float> force;  // float3 with 16-byte stride
    std::vector<uint32_t> types;
    std::vector<float> colors;  // ColorType colours (4 per particle; zero when none given)

    void init(const astro_params& prm, uint32_t n_, uint32_t n_tree_, const ColorType* ct) {
        p = prm;
        n = n_;
        n_tree = n_tree_;
        layers = p.lbits + 1;
        sizes.assign(layers, 0);
        offsets.assign(layers, 0);
        capacity = oracle_layer_layout(n_tree, 1, p.lbits, sizes.data(), offsets.data());
        morton.assign(n_tree, 0);
        unsorted_codes.assign(n_tree, 0);
        sorted_codes.assign(n_tree, 0);
        unsorted_idx.assign(n_tree, 0);
        sorted_idx.assign(n_tree, 0);
        unique_idx.assign(n_tree, 0);
        flags.assign(n_tree, 0);
        scan.assign(n_tree, 0);
        nodes.assign(capacity, empty_node());
        force.assign(4ull * n, 0.0f);
        types.resize(n);
        for (uint32_t i = 0; i < n; ++i) types[i] = ct ? ct[i].type : (i < n_tree ? 1u : 2u);
        colors.assign(4ull * n, 0.0f);
        if (ct)
            for (uint32_t i = 0; i < n; ++i)
                for (int a = 0; a < 4; ++a) colors[4ull * i + a] = ct[i].color[a];
    }

    // countUniqueMortonCodes, Renderer.swift:570-625: clears, markUniques
    // (Octree.metal:282-303), the scan, scatterUniques (Octree.metal:306-318),
    // copyLastScanToParentCount (Octree.metal:321-334).
    void count_unique(bool aggregate, uint32_t count) {
        std::fill(flags.begin(), flags.begin() + count, 0u);
        std::fill(scan.begin(), scan.begin() + count, 0u);
        std::fill(unique_idx.begin(), unique_idx.begin() + count, 0u);
        const uint64_t* k = sorted_codes.data();
        for (uint32_t gid = 0; gid < count; ++gid) {
            if (k[gid] == kInvalidCode) {
                flags[gid] = 0;
                continue;
            }
            bool is_unique;
            if (gid == 0) is_unique = true;
            else if (aggregate) is_unique = (k[gid] >> 3) != (k[gid - 1] >> 3);
            else is_unique = k[gid] != k[gid - 1];
            flags[gid] = is_unique ? 1u : 0u;
        }
        encode_scan(flags.data(), scan.data(), count);
        for (uint32_t gid = 0; gid < count; ++gid)
            if (flags[gid]) unique_idx[scan[gid]] = gid;
        uint32_t last = count - 1;
        child_count = parent_count;
        parent_count = scan[last] + flags[last];
    }

    // radixSorter.sort as called per layer (Renderer.swift:522-528,730-736):
    // the count is parent_count; the sorted buffers keep their cleared tail.
    void sort_layer(uint32_t split_passes) {
        uint32_t count = parent_count;
        oracle_split_sort(unsorted_codes.data(), unsorted_idx.data(), sorted_codes.data(),
                          sorted_idx.data(), count, split_passes);
    }

    // aggregateLeafNodes, Octree.metal:53-117. The last run ends at
    // numUnique, not at the particle count (Octree.metal:71): with duplicate
    // keys the last leaf sums the wrong range. Reproduced as written.
    void aggregate_leaf_nodes(const PositionMass* pm) {
        uint32_t num_unique = parent_count;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t g = 0; g < (int64_t)num_unique; ++g) {
            uint32_t gid = (uint32_t)g;
            uint32_t start = unique_idx[gid];
            uint32_t end = (gid + 1 < num_unique) ? unique_idx[gid + 1] : num_unique;
            float cx = 0.0f, cy = 0.0f, cz = 0.0f, mass = 0.0f;
            float ec[4] = {0.0f, 0.0f, 0.0f, 0.0f}, en[3] = {0.0f, 0.0f, 0.0f};
            uint32_t suns = 0;
            for (uint32_t i = start; i < end; ++i) {
                const uint32_t si = sorted_idx[i];
                const PositionMass& s = pm[si];
                mass += s.mass;
                cx += s.position[0] * s.mass;
                cy += s.position[1] * s.mass;
                cz += s.position[2] * s.mass;
                if (types[si] == 0) {  // Octree.metal:85-89
                    for (int a = 0; a < 4; ++a) ec[a] += colors[4ull * si + a];
                    for (int a = 0; a < 3; ++a) en[a] += s.position[a];
                    ++suns;
                }
            }
            OctreeNode node = empty_node();
            node.mortonCode = sorted_codes[start];
            if (mass > 0.0f) {
                node.centerOfMass[0] = cx / mass;
                node.centerOfMass[1] = cy / mass;
                node.centerOfMass[2] = cz / mass;
            }
            node.totalMass = mass;
            // Octree.metal:93-98: the centre divides by max(suns, 1e-9).
            const float suns_safe = std::max((float)suns, 1e-9f);
            for (int a = 0; a < 4; ++a) node.emittedColor[a] = ec[a];
            for (int a = 0; a < 3; ++a) node.emittedColorCenter[a] = en[a] / suns_safe;
            node.layer = 0;
            nodes[gid] = node;
            unsorted_codes[gid] = node.mortonCode;
            unsorted_idx[gid] = gid;
        }
    }

    // aggregateNodes, Octree.metal:120-202: children are the run's nodes of
    // the layer below (first 8), mass and centre of mass weighted by child
    // mass, code = first child code >> 3.
    void aggregate_nodes(uint32_t input_offset, uint32_t output_offset, uint32_t layer) {
        uint32_t num_unique = parent_count;
#pragma omp parallel for schedule(static)
        for (int64_t g = 0; g < (int64_t)num_unique; ++g) {
            uint32_t gid = (uint32_t)g;
            uint32_t start = unique_idx[gid];
            uint32_t end = (gid + 1 < num_unique) ? unique_idx[gid + 1] : child_count;
            float cx = 0.0f, cy = 0.0f, cz = 0.0f, mass = 0.0f;
            float ec[4] = {0.0f, 0.0f, 0.0f, 0.0f}, en[3] = {0.0f, 0.0f, 0.0f};
            uint32_t suns = 0;
            uint32_t children[8];
            for (int i = 0; i < 8; ++i) children[i] = kInvalidChild;
            int child_n = 0;
            for (uint32_t i = start; i < end; ++i) {
                uint32_t node_index = sorted_idx[i] + input_offset;
                const OctreeNode& c = nodes[node_index];
                mass += c.totalMass;
                cx += c.centerOfMass[0] * c.totalMass;
                cy += c.centerOfMass[1] * c.totalMass;
                cz += c.centerOfMass[2] * c.totalMass;
                if (c.emittedColor[3] > 0.0f) {  // Octree.metal:155-159
                    for (int a = 0; a < 4; ++a) ec[a] += c.emittedColor[a];
                    for (int a = 0; a < 3; ++a) en[a] += c.emittedColorCenter[a];
                    ++suns;
                }
                if (child_n < 8) children[child_n++] = node_index;
            }
            OctreeNode node = empty_node();
            node.mortonCode = sorted_codes[start] >> 3;
            if (mass > 0.0f) {
                node.centerOfMass[0] = cx / mass;
                node.centerOfMass[1] = cy / mass;
                node.centerOfMass[2] = cz / mass;
            }
            node.totalMass = mass;
            // Octree.metal:171-177: the centre is averaged over the children
            // that emit.
            for (int a = 0; a < 4; ++a) node.emittedColor[a] = ec[a];
            for (int a = 0; a < 3; ++a)
                node.emittedColorCenter[a] = suns > 0 ? en[a] / (float)suns : en[a];
            node.layer = layer;
            for (int i = 0; i < 8; ++i) node.children[i] = children[i];
            nodes[output_offset + gid] = node;
        }
        for (uint32_t gid = 0; gid < num_unique; ++gid) {
            unsorted_codes[gid] = nodes[output_offset + gid].mortonCode;
            unsorted_idx[gid] = gid;
        }
    }

    // barnesHut, BarnesHut.metal:22-101. The node size 1 << (21 + layer) is
    // an int shift that overflows from layer 10 on; it is taken here as the
    // power of two 2^(21+layer), identical for layers 0..9.
    void barnes_hut(const PositionMass* pm) {
        const uint32_t root = offsets[layers - 1];
        const float g = p.g, softening = p.softening, theta = p.theta;
        const float leaf_min = p.leaf_min_dist2, clampv = p.force_clamp;
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t gg = 0; gg < (int64_t)n; ++gg) {
            uint32_t gid = (uint32_t)gg;
            uint32_t stack[1024];
            uint32_t sp = 0;
            stack[sp++] = root;
            float fx = 0.0f, fy = 0.0f, fz = 0.0f;
            const float px = pm[gid].position[0], py = pm[gid].position[1],
                        pz = pm[gid].position[2];
            float my_type = (float)types[gid];
            uint64_t my_code = kInvalidCode;
            if (my_type != 2.0f && gid < n_tree) my_code = morton[gid];
            while (sp > 0) {
                uint32_t node_idx = stack[--sp];
                const OctreeNode& node = nodes[node_idx];
                if (node.mortonCode == kInvalidCode) continue;
                float dx = node.centerOfMass[0] - px;
                float dy = node.centerOfMass[1] - py;
                float dz = node.centerOfMass[2] - pz;
                float dist_sqr = dx * dx + dy * dy + dz * dz + softening;
                dist_sqr = std::fmax(dist_sqr, 1e-6f);
                float dist = std::sqrt(dist_sqr);
                dist = std::fmax(dist, 1e-6f);
                float side_length = std::ldexp(1.0f, 21 + (int)node.layer);
                bool is_leaf = node.layer == 0;
                uint32_t shift = 3 * node.layer;
                bool is_self = false;
                if (my_type != 2.0f) is_self = ((my_code >> shift) == node.mortonCode) && is_leaf;
                if (is_leaf) {
                    if (!is_self && dist_sqr > leaf_min) {
                        float gm = g * node.totalMass, den = dist_sqr * dist;
                        fx += gm * dx / den;
                        fy += gm * dy / den;
                        fz += gm * dz / den;
                    }
                } else if (side_length / dist < theta) {
                    float gm = g * node.totalMass, den = dist_sqr * dist;
                    fx += gm * dx / den;
                    fy += gm * dy / den;
                    fz += gm * dz / den;
                } else {
                    for (int c = 0; c < 8; ++c) {
                        uint32_t child = node.children[c];
                        if (child != kInvalidChild && sp < 1024) stack[sp++] = child;
                    }
                }
            }
            float* out = &force[4ull * gid];
            out[0] = std::fmin(std::fmax(fx, -clampv), clampv);
            out[1] = std::fmin(std::fmax(fy, -clampv), clampv);
            out[2] = std::fmin(std::fmax(fz, -clampv), clampv);
            out[3] = 0.0f;
        }
    }

    // updateSpheres, BarnesHut.metal:169-196.
    void update_spheres(PositionMass* pm, VelocityRadius* vr, float dt) {
#pragma omp parallel for schedule(static)
        for (int64_t gg = 0; gg < (int64_t)n; ++gg) {
            uint32_t gid = (uint32_t)gg;
            float ax = force[4ull * gid], ay = force[4ull * gid + 1], az = force[4ull * gid + 2];
            uint32_t t = types[gid];
            if (t <= 2) {
                float s = p.type_accel_scale[t];
                ax *= s;
                ay *= s;
                az *= s;
            }
            float* v = vr[gid].velocity;
            float vx = v[0] * p.damping, vy = v[1] * p.damping, vz = v[2] * p.damping;
            vx += ax * dt;
            vy += ay * dt;
            vz += az * dt;
            v[0] = vx;
            v[1] = vy;
            v[2] = vz;
            float* x = pm[gid].position;
            x[0] += vx * dt;
            x[1] += vy * dt;
            x[2] += vz * dt;
        }
    }

    // Renderer.draw, compute section (Renderer.swift:505-533): the tree
    // build of one frame. live_counts[l] records parentCount after layer l.
    void build(const PositionMass* pm, uint32_t split_passes) {
        live_counts.assign(layers, 0);
        if (n_tree == 0) return;
        std::fill(sorted_codes.begin(), sorted_codes.end(), kInvalidCode);
        std::fill(sorted_idx.begin(), sorted_idx.end(), 0u);
        std::fill(nodes.begin(), nodes.end(), empty_node());
        oracle_generate_morton_codes(pm, morton.data(), unsorted_codes.data(), n_tree, p.lbits,
                                     p.quant_offset);
        for (uint32_t i = 0; i < n_tree; ++i) unsorted_idx[i] = i;  // fillIndices
        parent_count = n_tree;
        sort_layer(split_passes);
        count_unique(false, n_tree);
        live_counts[0] = parent_count;
        leaf_sorted_codes = sorted_codes;
        leaf_sorted_idx = sorted_idx;
        aggregate_leaf_nodes(pm);
        // buildInternalNodes, Renderer.swift:714-755.
        for (uint32_t layer = 1; layer < layers; ++layer) {
            std::fill(sorted_codes.begin(), sorted_codes.end(), kInvalidCode);
            std::fill(sorted_idx.begin(), sorted_idx.end(), 0u);
            sort_layer(split_passes);
            count_unique(true, n_tree);
            live_counts[layer] = parent_count;
            aggregate_nodes(offsets[layer - 1], offsets[layer], layer);
        }
    }

    std::vector<uint32_t> live_counts;
    std::vector<uint64_t> leaf_sorted_codes;
    std::vector<uint32_t> leaf_sorted_idx;
};

}  // namespace

extern "C" int oracle_ref_run(const astro_params* p, PositionMass* pm, VelocityRadius* vr,
                              const ColorType* ct, uint32_t n, uint32_t n_tree, float dt,
                              uint32_t nsteps, uint32_t split_passes, oracle_outputs* out) {
    if (!p || !pm || !vr || n_tree > n || p->lbits < 1 || p->lbits > 21 || split_passes > 64)
        return -1;
    RefFrame f;
    f.init(*p, n, n_tree, ct);
    for (uint32_t s = 0; s < nsteps; ++s) {
        f.build(pm, split_passes);             // Renderer.swift:511-533
        if (n > 0) f.barnes_hut(pm);           // Renderer.swift:536-539
        if (s + 1 == nsteps && out) {          // state of the last frame before integration
            if (out->codes) std::memcpy(out->codes, f.morton.data(), 8ull * n_tree);
            if (out->sorted_codes && n_tree)
                std::memcpy(out->sorted_codes, f.leaf_sorted_codes.data(), 8ull * n_tree);
            if (out->sorted_indices && n_tree)
                std::memcpy(out->sorted_indices, f.leaf_sorted_idx.data(), 4ull * n_tree);
            if (out->layer_counts)
                std::memcpy(out->layer_counts, f.live_counts.data(), 4ull * f.layers);
            if (out->layer_sizes) std::memcpy(out->layer_sizes, f.sizes.data(), 4ull * f.layers);
            if (out->layer_offsets)
                std::memcpy(out->layer_offsets, f.offsets.data(), 4ull * f.layers);
            if (out->nodes)
                std::memcpy(out->nodes, f.nodes.data(), sizeof(OctreeNode) * f.capacity);
            if (out->acc4) std::memcpy(out->acc4, f.force.data(), 16ull * n);
        }
        if (n > 0) f.update_spheres(pm, vr, dt);  // Renderer.swift:540
    }
    return 0;
}
