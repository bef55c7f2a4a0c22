// Headless particle splat: the scene pass of the reference's renderer
// (Astro/Spheres.metal:23-64 vertex math, Renderer.swift:780-830 draw order,
// :143-144 depth state, :276-295 pipelines) drawn into a device image.
//
// Every particle is projected as sphere_vertex / dust_point_vertex do:
//   clip = P * (V * float4(x - camera, 1))
// Stars and planets (types 0, 1) are the reference's sphere meshes (extent 1,
// scaled by the radius: world radius radius/2); here each is a disc of that
// projected radius at its centre's depth, drawn opaque. Dust (type 2) is a
// point sprite of `radius` pixels, blended with source alpha. Fragments are
// keyed (pixel, particle), sorted with the library's radix sort, and every
// pixel folds its fragments in particle order — the reference's draw order
// (stars, planets, dust by instance) — with the depth test "less", depth
// writes on, and the colour rounded to half precision after every write (the
// rgba16Float attachment). Correctly rounded operations throughout, in the
// order of the CPU restatement (oracle/oracle_splat.cpp).
#include <algorithm>

#include <cuda_fp16.h>

#include "build_kernels.cuh"
#include "common.cuh"

namespace astro {

namespace {

__device__ __forceinline__ float mat_row(const float* m, int r, float x, float y, float z, float w) {
    // (m * v)[r] for a column-major 4x4 m, summed over columns 0..3 in order.
    float s = __fmul_rn(m[r], x);
    s = __fadd_rn(s, __fmul_rn(m[4 + r], y));
    s = __fadd_rn(s, __fmul_rn(m[8 + r], z));
    return __fadd_rn(s, __fmul_rn(m[12 + r], w));
}

__device__ __forceinline__ float to_half(float x) { return __half2float(__float2half_rn(x)); }

// One projected primitive: window x, y, depth, and the point size (pixels) or
// the disc radius (pixels); kind 0 = culled, 1 = disc, 2 = point.
__global__ void splat_project_kernel(SplatArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 p = a.pos[i];
    const float rel_x = __fsub_rn(p.x, a.cam[0]), rel_y = __fsub_rn(p.y, a.cam[1]),
                rel_z = __fsub_rn(p.z, a.cam[2]);
    float v[4], c[4];
    for (int r = 0; r < 4; ++r) v[r] = mat_row(a.view, r, rel_x, rel_y, rel_z, 1.0f);
    for (int r = 0; r < 4; ++r) c[r] = mat_row(a.proj, r, v[0], v[1], v[2], v[3]);
    const uint32_t type = a.types[i];
    const float radius = a.vel[i].w;
    const bool point = type == 2u;
    uint32_t kind = point ? 2u : 1u;
    const float w = c[3];
    if (!(w > 0.0f) || !(c[2] >= 0.0f) || !(c[2] <= w)) kind = 0u;
    if (point && !(c[0] >= -w && c[0] <= w && c[1] >= -w && c[1] <= w)) kind = 0u;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (kind) {
        const float nx = __fdiv_rn(c[0], w), ny = __fdiv_rn(c[1], w), nz = __fdiv_rn(c[2], w);
        out.x = __fmul_rn(__fmul_rn(__fadd_rn(nx, 1.0f), 0.5f), (float)a.width);
        out.y = __fmul_rn(__fmul_rn(__fsub_rn(1.0f, ny), 0.5f), (float)a.height);
        out.z = nz;
        if (point) {
            out.w = radius;
        } else {
            const float world_r = __fmul_rn(0.5f, radius);
            out.w = __fmul_rn(__fdiv_rn(__fmul_rn(world_r, a.proj[5]), w),
                              __fmul_rn(0.5f, (float)a.height));
        }
        if (!(out.w > 0.0f) || !isfinite(out.x) || !isfinite(out.y)) kind = 0u;
    }
    a.prim[i] = out;
    a.kind[i] = kind;
}

// Pixel range [lo, hi] whose centres can lie in [c - h, c + h], clamped.
__device__ __forceinline__ void span(float c, float h, uint32_t size, int& lo, int& hi) {
    const float a = floorf(__fsub_rn(__fsub_rn(c, h), 0.5f));
    const float b = ceilf(__fsub_rn(__fadd_rn(c, h), 0.5f));
    lo = a < 0.0f ? 0 : (a > (float)size ? (int)size : (int)a);
    hi = b < 0.0f ? -1 : (b >= (float)size ? (int)size - 1 : (int)b);
}

__device__ __forceinline__ bool covers(uint32_t kind, float4 q, int px, int py) {
    const float cx = __fadd_rn((float)px, 0.5f), cy = __fadd_rn((float)py, 0.5f);
    if (kind == 2u) {
        const float h = __fmul_rn(q.w, 0.5f);
        return cx >= __fsub_rn(q.x, h) && cx < __fadd_rn(q.x, h) && cy >= __fsub_rn(q.y, h) &&
               cy < __fadd_rn(q.y, h);
    }
    const float dx = __fsub_rn(cx, q.x), dy = __fsub_rn(cy, q.y);
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < __fmul_rn(q.w, q.w);
}

// One warp per primitive: its lanes stride over the covered box and append
// (pixel << 32 | particle) keys; writes past cap are counted, not stored.
__global__ void splat_emit_kernel(SplatArgs a) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < a.n; i += warps) {
        const uint32_t kind = a.kind[i];
        if (kind == 0u) continue;
        const float4 q = a.prim[i];
        const float h = kind == 2u ? __fmul_rn(q.w, 0.5f) : q.w;
        int x0, x1, y0, y1;
        span(q.x, h, a.width, x0, x1);
        span(q.y, h, a.height, y0, y1);
        if (x1 < x0 || y1 < y0) continue;
        const uint32_t bw = (uint32_t)(x1 - x0 + 1);
        const uint64_t cells = (uint64_t)bw * (uint32_t)(y1 - y0 + 1);
        for (uint64_t k = lane; k < cells; k += 32u) {
            const int px = x0 + (int)(k % bw), py = y0 + (int)(k / bw);
            if (!covers(kind, q, px, py)) continue;
            const uint32_t slot = atomicAdd(a.cursor, 1u);
            if (slot < a.cap)
                a.keys[slot] = ((uint64_t)((uint32_t)py * a.width + (uint32_t)px) << 32) | i;
        }
    }
}

__global__ void splat_clear_kernel(SplatArgs a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.width * a.height) return;
    a.image[p] = make_float4(to_half(a.clear[0]), to_half(a.clear[1]), to_half(a.clear[2]),
                             to_half(a.clear[3]));
    a.depth[p] = a.clear_depth;
}

// One thread per pixel run of the sorted keys: depth test and blend in
// particle order.
__global__ void splat_fold_kernel(SplatArgs a, const uint64_t* __restrict__ keys, uint32_t count) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= count) return;
    const uint32_t pix = (uint32_t)(keys[f] >> 32);
    if (f > 0 && (uint32_t)(keys[f - 1] >> 32) == pix) return;
    float4 dst = a.image[pix];
    float z = a.depth[pix];
    for (uint32_t g = f; g < count && (uint32_t)(keys[g] >> 32) == pix; ++g) {
        const uint32_t i = (uint32_t)(keys[g] & 0xFFFFFFFFull);
        const float zf = a.prim[i].z;
        if (!(zf < z)) continue;
        const float4 src = a.colors[i];
        if (a.kind[i] == 2u) {
            const float inv = __fsub_rn(1.0f, src.w);
            dst.x = to_half(__fadd_rn(__fmul_rn(src.x, src.w), __fmul_rn(dst.x, inv)));
            dst.y = to_half(__fadd_rn(__fmul_rn(src.y, src.w), __fmul_rn(dst.y, inv)));
            dst.z = to_half(__fadd_rn(__fmul_rn(src.z, src.w), __fmul_rn(dst.z, inv)));
            dst.w = to_half(__fadd_rn(__fmul_rn(src.w, src.w), __fmul_rn(dst.w, inv)));
        } else {
            dst = make_float4(to_half(src.x), to_half(src.y), to_half(src.z), to_half(src.w));
        }
        z = zf;
    }
    a.image[pix] = dst;
    a.depth[pix] = z;
}

}  // namespace

cudaError_t launch_splat_project(const SplatArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    splat_project_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_splat_emit(const SplatArgs& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(((uint64_t)a.n * 32 + 255) / 256, 152u * 64u);
    splat_emit_kernel<<<blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_splat_clear(const SplatArgs& a, cudaStream_t st) {
    const uint32_t pixels = a.width * a.height;
    splat_clear_kernel<<<(pixels + 255) / 256, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_splat_fold(const SplatArgs& a, const uint64_t* keys, uint32_t count,
                              cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    splat_fold_kernel<<<(count + 255) / 256, 256, 0, st>>>(a, keys, count);
    return cudaGetLastError();
}

}  // namespace astro
