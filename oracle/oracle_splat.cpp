// CPU restatement of the headless splat (test infrastructure only: it is the
// checker of astro_splat, never part of the product path).
//
// The scene pass of the reference's renderer, drawn sequentially in particle
// order — sphere_vertex / dust_point_vertex (Spheres.metal:23-64):
//   clip = projectionMatrix * (viewMatrix * float4(position - cameraPosition, 1))
// stars and planets (types 0, 1: sphere meshes of extent 1 scaled by the
// radius, Renderer.swift:120-127) as opaque discs of radius radius/2 projected
// at the centre's depth; dust (type 2) as point sprites of `radius` pixels
// (Spheres.metal:56) blended with source alpha (Renderer.swift:288-295); depth
// test "less" with depth writes (Renderer.swift:143-144), depth cleared to 1
// (:768), colours stored as half floats after every write (the rgba16Float
// attachment, :276,285). Every operation below is one rounded FP32 operation,
// in the order the CUDA kernels use.
#include "astro_oracle.h"

#include <cmath>
#include <cstring>

namespace {

float mat_row(const float* m, int r, float x, float y, float z, float w) {
    float s = m[r] * x;
    s = s + m[4 + r] * y;
    s = s + m[8 + r] * z;
    return s + m[12 + r] * w;
}

// IEEE binary16 round to nearest even, returned as a float.
float round_to_half(float x) {
    if (std::isnan(x) || std::isinf(x)) return x;
    const float ax = std::fabs(x);
    float r;
    if (ax >= 65520.0f) {
        r = INFINITY;
    } else if (ax < 6.103515625e-05f) {  // below the smallest normal half: step 2^-24
        r = std::nearbyint(ax * 16777216.0f) / 16777216.0f;
    } else {
        int e = 0;
        std::frexp(ax, &e);  // ax = f * 2^e, f in [0.5, 1): 11 significant bits kept
        const float q = std::ldexp(1.0f, e - 11);
        r = std::nearbyint(ax / q) * q;
    }
    return std::signbit(x) ? -r : r;
}

struct Prim {
    float x, y, z, size;
    unsigned kind;  // 0 culled, 1 disc, 2 point
};

Prim project(const PositionMass& pm, const VelocityRadius& vr, uint32_t type, const float* view,
             const float* proj, const float* cam, uint32_t width, uint32_t height) {
    const float rx = pm.position[0] - cam[0], ry = pm.position[1] - cam[1], rz = pm.position[2] - cam[2];
    float v[4], c[4];
    for (int r = 0; r < 4; ++r) v[r] = mat_row(view, r, rx, ry, rz, 1.0f);
    for (int r = 0; r < 4; ++r) c[r] = mat_row(proj, r, v[0], v[1], v[2], v[3]);
    const bool point = type == 2u;
    Prim p{0.0f, 0.0f, 0.0f, 0.0f, point ? 2u : 1u};
    const float w = c[3];
    if (!(w > 0.0f) || !(c[2] >= 0.0f) || !(c[2] <= w)) p.kind = 0u;
    if (point && !(c[0] >= -w && c[0] <= w && c[1] >= -w && c[1] <= w)) p.kind = 0u;
    if (p.kind) {
        const float nx = c[0] / w, ny = c[1] / w, nz = c[2] / w;
        p.x = ((nx + 1.0f) * 0.5f) * (float)width;
        p.y = ((1.0f - ny) * 0.5f) * (float)height;
        p.z = nz;
        if (point) {
            p.size = vr.radius;
        } else {
            const float world_r = 0.5f * vr.radius;
            p.size = ((world_r * proj[5]) / w) * (0.5f * (float)height);
        }
        if (!(p.size > 0.0f) || !std::isfinite(p.x) || !std::isfinite(p.y)) p.kind = 0u;
    }
    return p;
}

bool covers(const Prim& q, int px, int py) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    if (q.kind == 2u) {
        const float h = q.size * 0.5f;
        return cx >= q.x - h && cx < q.x + h && cy >= q.y - h && cy < q.y + h;
    }
    const float dx = cx - q.x, dy = cy - q.y;
    return dx * dx + dy * dy < q.size * q.size;
}

void span(float c, float h, uint32_t size, int& lo, int& hi) {
    const float a = std::floor((c - h) - 0.5f);
    const float b = std::ceil((c + h) - 0.5f);
    lo = a < 0.0f ? 0 : (a > (float)size ? (int)size : (int)a);
    hi = b < 0.0f ? -1 : (b >= (float)size ? (int)size - 1 : (int)b);
}

}  // namespace

extern "C" void oracle_splat(const PositionMass* pm, const VelocityRadius* vr, const ColorType* ct,
                             uint32_t n, const float* view, const float* proj, const float* cam,
                             uint32_t width, uint32_t height, const float* clear, float* rgba,
                             float* depth) {
    const size_t pixels = (size_t)width * height;
    for (size_t p = 0; p < pixels; ++p) {
        for (int k = 0; k < 4; ++k) rgba[4 * p + k] = round_to_half(clear[k]);
        depth[p] = 1.0f;
    }
    for (uint32_t i = 0; i < n; ++i) {
        const Prim q = project(pm[i], vr[i], ct[i].type, view, proj, cam, width, height);
        if (!q.kind) continue;
        const float h = q.kind == 2u ? q.size * 0.5f : q.size;
        int x0, x1, y0, y1;
        span(q.x, h, width, x0, x1);
        span(q.y, h, height, y0, y1);
        for (int py = y0; py <= y1; ++py)
            for (int px = x0; px <= x1; ++px) {
                if (!covers(q, px, py)) continue;
                const size_t p = (size_t)py * width + (size_t)px;
                if (!(q.z < depth[p])) continue;
                const float* s = ct[i].color;
                float* d = &rgba[4 * p];
                if (q.kind == 2u) {
                    const float inv = 1.0f - s[3];
                    for (int k = 0; k < 3; ++k) d[k] = round_to_half(s[k] * s[3] + d[k] * inv);
                    d[3] = round_to_half(s[3] * s[3] + d[3] * inv);
                } else {
                    for (int k = 0; k < 4; ++k) d[k] = round_to_half(s[k]);
                }
                depth[p] = q.z;
            }
    }
}
