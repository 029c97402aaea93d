// dfpt_device.cuh - device code of the renderer core (sm_103a).
//
// This header is compiled twice: by dfpt_kernels_fast.cu (namespace dfpt_fast, FMA contraction
// allowed) and by dfpt_kernels_strict.cu (namespace dfpt_strict, -fmad=false) whose arithmetic
// is one IEEE rounding per operation, the Java float semantics of the reference kernel, so
// ray-cast hit ids, distances and normals come out bit-identical to a strict FP32 restatement.
//
// Reference: src/main/java/org/dayflower/pathtracer/kernel/GPURendererKernel.java (cited below
// as GRK:line), AbstractKernel.java (AK:line), AbstractImageKernel.java (AIK:line).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfpt_device_types.h"
#include "dfpt_internal.h"
#include "dfpt_noise_tables.h"

#ifndef DFPT_NS
#error "define DFPT_NS before including dfpt_device.cuh"
#endif

namespace DFPT_NS {

// ---------------------------------------------------------------------------------------------
// Constants (AK:56, GRK:76-78, MathF PI family: float products/quotients of (float)Math.PI).
constexpr float INF = 100000.0f;
constexpr float PI_F = 3.14159274101257324219f;
constexpr float TWO_PI = PI_F * 2.0f;
constexpr float INV_PI = 1.0f / PI_F;
constexpr float INV_TWO_PI = 1.0f / TWO_PI;
constexpr float PI_OVER_180 = PI_F / 180.0f;
constexpr float COLOR_RECIPROCAL = 1.0f / 255.0f;
constexpr float EPSILON_AK = 0.02f;

// Noise tables in global memory (divergent gathers go through L1, not the serialising constant
// cache); filled from DFPT_PERMUTATION / DFPT_GRADIENT3 when a handle is created.
__device__ int g_perm[512];
__device__ float g_grad3[36];
__device__ __forceinline__ int perm(int i) { return __ldg(g_perm + i); }
__device__ __forceinline__ float grad(int i) { return __ldg(g_grad3 + i); }

// Java Math.min/max: NaN propagates (PTX min.NaN / max.NaN, sm_80+).
__device__ __forceinline__ float jmin(float a, float b) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float jmax(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
// Three-operand forms (sm_100 and later): the minimum / maximum of a set, NaN when any operand is
// NaN, -0 below +0, so jmin3(a, b, c) == jmin(a, jmin(b, c)) for every input, in one instruction.
__device__ __forceinline__ float jmin3(float a, float b, float c) {
    float r;
    asm("min.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float jmax3(float a, float b, float c) {
    float r;
    asm("max.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// Aparapi's rsqrt is 1 / sqrt: both correctly rounded here (no fast-math).
__device__ __forceinline__ float rsqrt_j(float x) { return 1.0f / sqrtf(x); }
// sin, cos, asin, atan2 and pow of float arguments. The reference's Java path evaluates them as
// java.lang.Math in double and casts the result to float; the strict set does the same (CUDA's
// double functions, one rounding to float), so its results equal the strict-FP32 oracle's. The fast
// sets call the float functions.
#if defined(DFPT_STRICT_MATH)
__device__ __forceinline__ float sin_j(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float cos_j(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float asin_j(float x) { return (float)asin((double)x); }
__device__ __forceinline__ float atan2_j(float y, float x) { return (float)atan2((double)y, (double)x); }
__device__ __forceinline__ float pow_j(float a, float b) { return (float)pow((double)a, (double)b); }
#else
__device__ __forceinline__ float sin_j(float x) { return sinf(x); }
__device__ __forceinline__ float cos_j(float x) { return cosf(x); }
__device__ __forceinline__ float asin_j(float x) { return asinf(x); }
__device__ __forceinline__ float atan2_j(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ float pow_j(float a, float b) { return powf(a, b); }
#endif
__device__ __forceinline__ float saturate_j(float v, float a, float b) {
    const float lo = jmin(a, b), hi = jmax(a, b);
    return v < lo ? lo : v > hi ? hi : v;
}
__device__ __forceinline__ float modulo_j(float v) { return v - floorf(v); }                    // AK:420
__device__ __forceinline__ float remainder_j(float x, float y) { return x - (float)(int)(x / y) * y; }  // AK:529
__device__ __forceinline__ int f2i(float f) { return (int)f; }  // cvt.rzi saturates, NaN -> 0 (Java)
__device__ __forceinline__ float lerp_j(float a, float b, float t) { return (1.0f - t) * a + t * b; }
__device__ __forceinline__ float blerp_j(float v00, float v01, float v10, float v11, float tx, float ty) {
    return lerp_j(lerp_j(v00, v01, tx), lerp_j(v10, v11, tx), ty);
}

// ---------------------------------------------------------------------------------------------
// Random numbers. Counter mode: Philox4x32-10 (Salmon et al., SC'11) keyed by (pixel, seed),
// counted by (pass, draw/4); a path draws its numbers in the reference's order, one per call.
// LCG mode: the reference's per-pixel 48-bit LCG (AK:438-440, 1101-1110).

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

struct Rng {
    uint64_t state;  // LCG: 48-bit state; counter: draws made this pass
    uint32_t pixel, pass, seed_lo, seed_hi;
    int kind;
    uint4 block;
    uint32_t block_id;

    __device__ __forceinline__ float next() {
        if (kind == DFPT_RNG_LCG) {
            state = (state * 0x5DEECE66Dull + 0xBull) & ((1ull << 48) - 1ull);
            return (float)(uint32_t)(state >> 24) * (1.0f / 16777216.0f);
        }
        const uint32_t i = (uint32_t)state;
        state = (uint64_t)(i + 1u);
        const uint32_t bid = i >> 2;
        if (bid != block_id) {
            block = philox4x32_10(make_uint4(pass, bid, seed_hi, 0x44465054u), make_uint2(pixel, seed_lo));
            block_id = bid;
        }
        const uint32_t lane = i & 3u;
        const uint32_t x = lane == 0 ? block.x : lane == 1 ? block.y : lane == 2 ? block.z : block.w;
        return (float)(x >> 8) * (1.0f / 16777216.0f);
    }
};

__device__ __forceinline__ Rng make_rng(const DevParams& P, uint32_t pixel, uint32_t pass, uint64_t state) {
    Rng r;
    r.state = state;
    r.pixel = pixel;
    r.pass = pass;
    r.seed_lo = P.seed_lo;
    r.seed_hi = P.seed_hi;
    r.kind = P.rng_kind;
    r.block_id = 0xFFFFFFFFu;
    r.block = make_uint4(0, 0, 0, 0);
    return r;
}

// ---------------------------------------------------------------------------------------------
// Simplex noise (Gustavson) and fBm as the reference writes them (AK:600-716, 762-900).

__device__ __forceinline__ int fast_floor(float v) {
    const int i = (int)v;
    return v < (float)i ? i - 1 : i;
}

__device__ float simplex2(float x, float y) {
    const float F2 = 0.3660254037844386f, G2 = 0.21132486540518713f;
    const float s = (x + y) * F2;
    const int i = fast_floor(x + s), j = fast_floor(y + s);
    const float t = (float)(i + j) * G2;
    const float x0 = x - ((float)i - t), y0 = y - ((float)j - t);
    const int i1 = x0 > y0 ? 1 : 0, j1 = x0 > y0 ? 0 : 1;
    const float x1 = x0 - (float)i1 + G2, y1 = y0 - (float)j1 + G2;
    const float x2 = x0 - 1.0f + 2.0f * G2, y2 = y0 - 1.0f + 2.0f * G2;
    const int ii = i & 0xFF, jj = j & 0xFF;
    const int gi0 = perm(ii + perm(jj)) % 12;
    const int gi1 = perm(ii + i1 + perm(jj + j1)) % 12;
    const int gi2 = perm(ii + 1 + perm(jj + 1)) % 12;
    const float t0 = 0.5f - x0 * x0 - y0 * y0;
    const float n0 = t0 < 0.0f ? 0.0f : (t0 * t0) * (t0 * t0) * (grad(gi0 * 3) * x0 + grad(gi0 * 3 + 1) * y0);
    const float t1 = 0.5f - x1 * x1 - y1 * y1;
    const float n1 = t1 < 0.0f ? 0.0f : (t1 * t1) * (t1 * t1) * (grad(gi1 * 3) * x1 + grad(gi1 * 3 + 1) * y1);
    const float t2 = 0.5f - x2 * x2 - y2 * y2;
    const float n2 = t2 < 0.0f ? 0.0f : (t2 * t2) * (t2 * t2) * (grad(gi2 * 3) * x2 + grad(gi2 * 3 + 1) * y2);
    return 70.0f * (n0 + n1 + n2);
}

__device__ float simplex3(float x, float y, float z) {
    const float F3 = 1.0f / 3.0f, G3 = 1.0f / 6.0f;
    const float s = (x + y + z) * F3;
    const int i = fast_floor(x + s), j = fast_floor(y + s), k = fast_floor(z + s);
    const float t = (float)(i + j + k) * G3;
    const float x0 = x - ((float)i - t), y0 = y - ((float)j - t), z0 = z - ((float)k - t);
    int i1, j1, k1, i2, j2, k2;
    if (x0 >= y0) {
        if (y0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
        else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
        else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
    } else {
        if (y0 < z0) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
        else if (x0 < z0) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
        else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
    }
    const float x1 = x0 - (float)i1 + G3, y1 = y0 - (float)j1 + G3, z1 = z0 - (float)k1 + G3;
    const float x2 = x0 - (float)i2 + 2.0f * G3, y2 = y0 - (float)j2 + 2.0f * G3, z2 = z0 - (float)k2 + 2.0f * G3;
    const float x3 = x0 - 1.0f + 3.0f * G3, y3 = y0 - 1.0f + 3.0f * G3, z3 = z0 - 1.0f + 3.0f * G3;
    const int ii = i & 0xFF, jj = j & 0xFF, kk = k & 0xFF;
    const int gi0 = perm(ii + perm(jj + perm(kk))) % 12;
    const int gi1 = perm(ii + i1 + perm(jj + j1 + perm(kk + k1))) % 12;
    const int gi2 = perm(ii + i2 + perm(jj + j2 + perm(kk + k2))) % 12;
    const int gi3 = perm(ii + 1 + perm(jj + 1 + perm(kk + 1))) % 12;
    float n = 0.0f, tt;
    tt = 0.6f - x0 * x0 - y0 * y0 - z0 * z0;
    const float n0 = tt < 0.0f ? 0.0f : (tt * tt) * (tt * tt) * (grad(gi0 * 3) * x0 + grad(gi0 * 3 + 1) * y0 + grad(gi0 * 3 + 2) * z0);
    tt = 0.6f - x1 * x1 - y1 * y1 - z1 * z1;
    const float n1 = tt < 0.0f ? 0.0f : (tt * tt) * (tt * tt) * (grad(gi1 * 3) * x1 + grad(gi1 * 3 + 1) * y1 + grad(gi1 * 3 + 2) * z1);
    tt = 0.6f - x2 * x2 - y2 * y2 - z2 * z2;
    const float n2 = tt < 0.0f ? 0.0f : (tt * tt) * (tt * tt) * (grad(gi2 * 3) * x2 + grad(gi2 * 3 + 1) * y2 + grad(gi2 * 3 + 2) * z2);
    tt = 0.6f - x3 * x3 - y3 * y3 - z3 * z3;
    const float n3 = tt < 0.0f ? 0.0f : (tt * tt) * (tt * tt) * (grad(gi3 * 3) * x3 + grad(gi3 * 3 + 1) * y3 + grad(gi3 * 3 + 2) * z3);
    n = 32.0f * (n0 + n1 + n2 + n3);
    return n;
}

// simplexFractionalBrownianMotionXYZ (AK:695-716)
__device__ float fbm3(float frequency, float gain, float minimum, float maximum, int octaves, float x, float y, float z) {
    float amp = 1.0f, max_amp = 0.0f, freq = frequency, noise = 0.0f;
    for (int i = 0; i < octaves; ++i) {
        noise += simplex3(x * freq, y * freq, z * freq) * amp;
        max_amp += amp;
        amp *= gain;
        freq *= 2.0f;
    }
    noise /= max_amp;
    return noise * (maximum - minimum) / 2.0f + (maximum + minimum) / 2.0f;
}

// simplexFractalXY (AK:560-575), used by the ray marcher's height function (GRK:726-728)
__device__ float fractal2(float amplitude, float frequency, float gain, float lacunarity, int octaves, float x, float y) {
    float result = 0.0f, amp = amplitude, freq = frequency;
    for (int i = 0; i < octaves; ++i) {
        result += amp * simplex2(x * freq, y * freq);
        amp *= gain;
        freq *= lacunarity;
    }
    return result;
}

// ---------------------------------------------------------------------------------------------
// Shape intersections (GRK:1414-1594). tmin/tmax exclusive, INF on a miss.

__device__ __forceinline__ float isect_plane(float ox, float oy, float oz, float dx, float dy, float dz, float4 a, float4 n, float tmax) {
    const float dp = n.x * dx + n.y * dy + n.z * dz;
    if (dp < 0.0f || dp > 0.0f) {
        const float t = ((a.x - ox) * n.x + (a.y - oy) * n.y + (a.z - oz) * n.z) / dp;
        if (t > 0.001f && t < tmax) return t;
    }
    return INF;
}

__device__ __forceinline__ float isect_sphere(float ox, float oy, float oz, float dx, float dy, float dz, float4 s, float tmax) {
    const float px = ox - s.x, py = oy - s.y, pz = oz - s.z;
    const float r2 = s.w * s.w;
    const float a = dx * dx + dy * dy + dz * dz;
    const float b = 2.0f * (px * dx + py * dy + pz * dz);
    const float c = (px * px + py * py + pz * pz) - r2;
    const float disc2 = b * b - 4.0f * a * c;
    if (disc2 >= 0.0f) {
        const float disc = sqrtf(disc2);
        const float q = -0.5f * (b < 0.0f ? b - disc : b + disc);
        const float r0 = q / a;
        const float r1 = q == 0.0f ? r0 : c / q;
        const float t0 = jmin(r0, r1), t1 = jmax(r0, r1);
        if (t0 > 0.001f && t0 < tmax) return t0;
        if (t1 > 0.001f && t1 < tmax) return t1;
    }
    return INF;
}

// Moller-Trumbore with the reference's tolerances; e0 = b - a and e1 = c - a precomputed.
__device__ __forceinline__ float isect_triangle(float ox, float oy, float oz, float dx, float dy, float dz, float4 a, float4 e0, float4 e1, float tmax) {
    const float v0x = dy * e1.z - dz * e1.y;
    const float v0y = dz * e1.x - dx * e1.z;
    const float v0z = dx * e1.y - dy * e1.x;
    const float det = e0.x * v0x + e0.y * v0y + e0.z * v0z;
    float t = INF;
    if (det < -0.0001f || det > 0.0001f) {
        const float inv = 1.0f / det;
        const float v1x = ox - a.x, v1y = oy - a.y, v1z = oz - a.z;
        const float u = (v1x * v0x + v1y * v0y + v1z * v0z) * inv;
        if (u >= 0.0f && u <= 1.0f) {
            const float v2x = v1y * e0.z - v1z * e0.y;
            const float v2y = v1z * e0.x - v1x * e0.z;
            const float v2z = v1x * e0.y - v1y * e0.x;
            const float v = (dx * v2x + dy * v2y + dz * v2z) * inv;
            t = v >= 0.0f && u + v <= 1.0f ? (e1.x * v2x + e1.y * v2y + e1.z * v2z) * inv : 0.001f;
            t = t > 0.001f && t < tmax ? t : INF;
        }
    }
    return t;
}

// Ray march of the (parameter-free) sin(x)sin(z) terrain (GRK:1470-1505).
__device__ float isect_terrain(float ox, float oy, float oz, float dx, float dy, float dz) {
    const float scale_r = 1.0f / 10.0f;
    float t = 0.0f, t_delta = 0.01f, lh = 0.0f, ly = 0.0f;
    for (float tc = 0.001f; tc < 10.0f; tc += t_delta) {
        const float px = ox * scale_r + dx * tc;
        const float py = oy * scale_r + dy * tc;
        const float pz = oz * scale_r + dz * tc;
        const float h = sin_j(px) * sin_j(pz);
        if (py < h) {
            t = tc - t_delta + t_delta * (lh - ly) / (py - ly - h + lh);
            tc = 10.0f;
        }
        t_delta = 0.01f * tc;
        lh = h;
        ly = py;
    }
    return t > EPSILON_AK ? t : INF;
}

struct Hit {
    float t;
    int prim;        // primitive index (primitive offset / 3), -1 on a miss
    int shape_type;  // Triangle (4) for mesh hits
    int shape_offset;
};

struct TraceStats {
    uint32_t nodes, tris;
};

// Slab distances of the node test, (b - o) * (1 / d) per axis (GRK:1093-1095, 1122-1129). The strict kernel
// set keeps that form. The fast set computes b * inv + (-o * inv), one FMA per slab with -o * inv
// taken once per mesh, and clamps inv to +-1e30 so that a zero direction component gives huge
// distances of the right sign rather than inf - inf; distances differ from the strict form by
// rounding only (the fast set is held to statistical parity).
struct SlabRay {
    float ix, iy, iz;  // 1 / d per axis
    float px, py, pz;  // fast: -o * inv; strict: o
};
__device__ __forceinline__ SlabRay slab_ray(float ox, float oy, float oz, float dx, float dy, float dz) {
    SlabRay r;
    r.ix = 1.0f / dx;
    r.iy = 1.0f / dy;
    r.iz = 1.0f / dz;
#ifdef DFPT_FMA_SLABS
    r.ix = copysignf(fminf(fabsf(r.ix), 1.0e30f), r.ix);
    r.iy = copysignf(fminf(fabsf(r.iy), 1.0e30f), r.iy);
    r.iz = copysignf(fminf(fabsf(r.iz), 1.0e30f), r.iz);
    r.px = -ox * r.ix;
    r.py = -oy * r.iy;
    r.pz = -oz * r.iz;
#else
    r.px = ox;
    r.py = oy;
    r.pz = oz;
#endif
    return r;
}
__device__ __forceinline__ float slab(float b, float inv, float p) {
#ifdef DFPT_FMA_SLABS
    return fmaf(b, inv, p);
#else
    return (b - p) * inv;
#endif
}

// Threaded-BVH walk of one mesh (GRK:1097-1194) in the reference's preorder: a node's box is
// tested when it is visited, with the closest distance found so far; descend to the next node
// (its left child) or skip to `next`. Returns true when an any-hit query found its hit.
// V selects the implementation: 0 loads each node when it is reached; 1 issues the loads of both
// possible successors (node + 1 and next) before the current node's slab test, so the dependent
// load of the walk overlaps the test. Both visit the same nodes in the same order.
template <bool ANY, int K>
__device__ __forceinline__ bool mesh_walk_pair(const DevScene& S, int root, int prim, float oxo, float oyo, float ozo,
                                               float dxo, float dyo, float dzo, Hit& h, TraceStats& st);

template <bool ANY, int K>
__device__ __forceinline__ bool mesh_walk_pair_compact(const DevScene& S, int root, int prim, float oxo, float oyo, float ozo,
                                                       float dxo, float dyo, float dzo, Hit& h, TraceStats& st);

template <bool ANY, int V>
__device__ __forceinline__ bool mesh_walk(const DevScene& S, int root, int prim, float oxo, float oyo, float ozo, float dxo,
                                          float dyo, float dzo, Hit& h, TraceStats& st) {
    // Variant 4: pair records with an 8-entry stack for closest-hit queries (when the scene's trees
    // allow it). Any-hit queries keep the threaded walk: with no closest distance yet they enter
    // every box on the ray, the pending right children outgrow the stack, and they gain nothing
    // from the cached intervals.
    if constexpr (V == 4 && !ANY) {
        if (S.use_pairs) return mesh_walk_pair<ANY, 8>(S, root, prim, oxo, oyo, ozo, dxo, dyo, dzo, h, st);
    }
    // Variant 5: the pair walk with an 8-entry stack of 8-byte entries (mesh_walk_pair_compact),
    // closest-hit queries only. Any-hit queries over pair records
    // measured 2.4x slower than the threaded walk: every box on a shadow ray is entered and the
    // pending right children overflow the stack.
    if constexpr (V == 5 && !ANY) {
        if (S.use_pairs == 2) return mesh_walk_pair_compact<ANY, 8>(S, root, prim, oxo, oyo, ozo, dxo, dyo, dzo, h, st);
    }
    const SlabRay sr = slab_ray(oxo, oyo, ozo, dxo, dyo, dzo);
    int node = root;
    float4 n0 = __ldg(S.nodes + 2 * node), n1 = __ldg(S.nodes + 2 * node + 1);
    while (node != -1) {
        st.nodes++;
        const int next = __float_as_int(n0.w);
        const int leaf = __float_as_int(n1.w);
        float4 d0, d1, s0, s1;
        if (V == 1) {
            // node + 1 exists for every inner node (its left child); next is -1 or a later node.
            const int dn = leaf == -1 ? node + 1 : node;
            const int sn = next != -1 ? next : node;
            d0 = __ldg(S.nodes + 2 * dn);
            d1 = __ldg(S.nodes + 2 * dn + 1);
            s0 = __ldg(S.nodes + 2 * sn);
            s1 = __ldg(S.nodes + 2 * sn + 1);
        }
        const float t0x = slab(n0.x, sr.ix, sr.px), t0y = slab(n0.y, sr.iy, sr.py), t0z = slab(n0.z, sr.iz, sr.pz);
        const float t1x = slab(n1.x, sr.ix, sr.px), t1y = slab(n1.y, sr.iy, sr.py), t1z = slab(n1.z, sr.iz, sr.pz);
        const float tmax = jmin3(jmax(t0x, t1x), jmax(t0y, t1y), jmax(t0z, t1z));
        const float tmin = jmax3(jmin(t0x, t1x), jmin(t0y, t1y), jmin(t0z, t1z));
        const float tb = tmin > tmax ? -1.0f : tmin > 0.001f && tmin < h.t ? tmin : tmax > 0.001f && tmax < h.t ? tmax : -1.0f;
        if (tb >= 0.0f && leaf != -1) {
            // Leaf: its triangles in order (-2 marks an empty leaf).
            for (int k = leaf; k >= 0;) {
                const float4 a = __ldg(S.tris + 3 * k);
                const float4 e0 = __ldg(S.tris + 3 * k + 1);
                const float4 e1 = __ldg(S.tris + 3 * k + 2);
                st.tris++;
                const float t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, a, e0, e1, h.t);
                if (t < h.t) {
                    h.t = t;
                    h.prim = prim;
                    h.shape_type = DFPT_SHAPE_TRIANGLE;
                    h.shape_offset = __float_as_int(a.w);
                }
                if (ANY && h.prim != -1) return true;
                k = __float_as_int(e0.w) != 0 ? -1 : k + 1;
            }
        }
        const bool descend = tb >= 0.0f && leaf == -1;
        node = descend ? node + 1 : next;
        if (node == -1) break;
        if (V == 1) {
            n0 = descend ? d0 : s0;
            n1 = descend ? d1 : s1;
        } else {
            n0 = __ldg(S.nodes + 2 * node);
            n1 = __ldg(S.nodes + 2 * node + 1);
        }
    }
    return false;
}

// The reference's box test (GRK:1132-1134) on a slab interval: the node is entered when the
// interval is not empty and its entry, or else its exit, lies in (0.001, closest). For fixed
// (tmin, tmax) it can only turn from true to false as the closest distance shrinks.
__device__ __forceinline__ bool box_accepts(float tmin, float tmax, float closest) {
    return !(tmin > tmax) && ((tmin > 0.001f && tmin < closest) || (tmax > 0.001f && tmax < closest));
}
__device__ __forceinline__ void slab_interval(float ax, float ay, float az, float bx, float by, float bz, const SlabRay& sr,
                                              float& tmin, float& tmax) {
    const float t0x = slab(ax, sr.ix, sr.px), t0y = slab(ay, sr.iy, sr.py), t0z = slab(az, sr.iz, sr.pz);
    const float t1x = slab(bx, sr.ix, sr.px), t1y = slab(by, sr.iy, sr.py), t1z = slab(bz, sr.iz, sr.pz);
    tmax = jmin3(jmax(t0x, t1x), jmax(t0y, t1y), jmax(t0z, t1z));
    tmin = jmax3(jmin(t0x, t1x), jmin(t0y, t1y), jmin(t0z, t1z));
}

// The threaded walk over pair records (DevScene::pairs), with a short stack in shared memory. An
// entered inner node's record gives both children's boxes in one load. The left child is tested
// at once (it follows its parent in preorder, with the same closest distance); the right child's
// slab interval is computed now and its test is decided when the walk reaches it in preorder -
// after the left subtree - with the closest distance of that moment, so every test has exactly
// the operands of mesh_walk's. A right child that fails already is never pushed (it would fail
// then too). When the K-entry stack overflows its oldest entries are dropped; once it runs empty
// the walk continues from next() of the last finished node in the threaded records. Each lane
// may call it alone.
template <bool ANY, int K>
__device__ __forceinline__ bool mesh_walk_pair(const DevScene& S, int root, int prim, float oxo, float oyo, float ozo,
                                               float dxo, float dyo, float dzo, Hit& h, TraceStats& st) {
    __shared__ int4 stk[K * 256];  // [entry][thread]: {first triangle, node, tmin bits, tmax bits}
    const int tid = threadIdx.x;
    const SlabRay sr = slab_ray(oxo, oyo, ozo, dxo, dyo, dzo);
    int cur, leaf, last = root;
    int top = 0, bottom = 0;  // live entries [bottom, top), slot e % K; bottom > 0 once any was dropped
    {
        const float4 n0 = __ldg(S.nodes + 2 * root), n1 = __ldg(S.nodes + 2 * root + 1);
        st.nodes++;
        float tmin, tmax;
        slab_interval(n0.x, n0.y, n0.z, n1.x, n1.y, n1.z, sr, tmin, tmax);
        if (!box_accepts(tmin, tmax, h.t)) return false;  // a mesh root's next is -1
        cur = root;
        leaf = __float_as_int(n1.w);
    }
    for (;;) {
        // `cur` was entered; `leaf` is its first triangle (-1 inner, -2 empty leaf).
        bool descend = false;
        if (leaf != -1) {
            for (int k = leaf; k >= 0;) {
                const float4 a = __ldg(S.tris + 3 * k);
                const float4 e0 = __ldg(S.tris + 3 * k + 1);
                const float4 e1 = __ldg(S.tris + 3 * k + 2);
                st.tris++;
                const float t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, a, e0, e1, h.t);
                if (t < h.t) {
                    h.t = t;
                    h.prim = prim;
                    h.shape_type = DFPT_SHAPE_TRIANGLE;
                    h.shape_offset = __float_as_int(a.w);
                }
                if (ANY && h.prim != -1) return true;
                k = __float_as_int(e0.w) != 0 ? -1 : k + 1;
            }
            last = cur;
        } else {
            const float4* P = S.pairs + 4 * (size_t)cur;
            const float4 p0 = __ldg(P), p1 = __ldg(P + 1), p2 = __ldg(P + 2);
            const int4 p3 = __ldg(reinterpret_cast<const int4*>(P + 3));
            float lmin, lmax, rmin, rmax;
            slab_interval(p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, sr, lmin, lmax);
            slab_interval(p1.z, p1.w, p2.x, p2.y, p2.z, p2.w, sr, rmin, rmax);
            st.nodes++;
            const bool accept_r = box_accepts(rmin, rmax, h.t);
            if (box_accepts(lmin, lmax, h.t)) {
                if (accept_r) {
                    if (top - bottom == K) ++bottom;
                    stk[(top % K) * 256 + tid] = make_int4(p3.y, p3.z, __float_as_int(rmin), __float_as_int(rmax));
                    ++top;
                } else {
                    st.nodes++;  // the right child's test, decided (rejected) already
                }
                cur = cur + 1;
                leaf = p3.x;
                descend = true;
            } else {
                st.nodes++;
                if (accept_r) {
                    cur = p3.z;
                    leaf = p3.y;
                    descend = true;
                } else {
                    last = p3.z;
                }
            }
        }
        if (descend) continue;
        // The next node in preorder: the nearest pending right child, else next() of `last`.
        for (;;) {
            if (top > bottom) {
                --top;
                const int4 e = stk[(top % K) * 256 + tid];
                st.nodes++;
                if (box_accepts(__int_as_float(e.z), __int_as_float(e.w), h.t)) {
                    cur = e.y;
                    leaf = e.x;
                    break;
                }
                last = e.y;
            } else if (bottom > 0) {
                const int nxt = __float_as_int(__ldg(S.nodes + 2 * last).w);
                if (nxt == -1) return false;
                const float4 n0 = __ldg(S.nodes + 2 * nxt), n1 = __ldg(S.nodes + 2 * nxt + 1);
                st.nodes++;
                float tmin, tmax;
                slab_interval(n0.x, n0.y, n0.z, n1.x, n1.y, n1.z, sr, tmin, tmax);
                if (box_accepts(tmin, tmax, h.t)) {
                    cur = nxt;
                    leaf = __float_as_int(n1.w);
                    break;
                }
                last = nxt;
            } else {
                return false;
            }
        }
    }
}

// mesh_walk_pair with 8-byte stack entries {code, key}. code >= 0 is an inner node; code < 0 is a
// leaf whose first triangle is ~code (the leaf's node index is in that triangle record's c - a
// slot). key is the one slab distance the deferred test still depends on: for an interval the
// box test accepted at push time (so tmin <= tmax or one side is NaN, and tmax > 0.001 whenever
// tmin <= 0.001), box_accepts(tmin, tmax, c) for any later closest distance c equals
// (tmin > 0.001 ? tmin : tmax) < c. Up to S.pair_stack entries (1..K) are live; a full stack drops
// its oldest entry, and once the live entries run out the walk continues from next() of the last
// finished node in the threaded records, so every node is still tested at its preorder position
// with the closest distance of that moment: the hits equal mesh_walk's at any stack depth. The
// visit counter can count a node twice after a drop: the threaded continuation re-tests a right
// child rejected at its parent's step (it is rejected again). Needs DevScene::use_pairs == 2 (no
// empty leaves) and blocks of at most 256 threads.
template <bool ANY, int K>
__device__ __forceinline__ bool mesh_walk_pair_compact(const DevScene& S, int root, int prim, float oxo, float oyo, float ozo,
                                                       float dxo, float dyo, float dzo, Hit& h, TraceStats& st) {
    static_assert((K & (K - 1)) == 0, "K must be a power of two");
    __shared__ int2 cstk[K * 256];  // [entry][thread]
    const int tid = threadIdx.x;
    const SlabRay sr = slab_ray(oxo, oyo, ozo, dxo, dyo, dzo);
    int cur, leaf, last = root;  // last < 0: a leaf whose node is in triangle ~last's record
    int top = 0, bottom = 0;     // live entries [bottom, top), slot e & (K - 1)
    const int cap = S.pair_stack < K ? S.pair_stack : K;
    {
        const float4 n0 = __ldg(S.nodes + 2 * root), n1 = __ldg(S.nodes + 2 * root + 1);
        st.nodes++;
        float tmin, tmax;
        slab_interval(n0.x, n0.y, n0.z, n1.x, n1.y, n1.z, sr, tmin, tmax);
        if (!box_accepts(tmin, tmax, h.t)) return false;  // a mesh root's next is -1
        cur = root;
        leaf = __float_as_int(n1.w);
    }
    for (;;) {
        // `cur` was entered (unknown for a leaf taken from the stack); `leaf` is its first
        // triangle, -1 for an inner node.
        bool descend = false;
        if (leaf >= 0) {
            for (int k = leaf;; ++k) {
                const float4 a = __ldg(S.tris + 3 * k);
                const float4 e0 = __ldg(S.tris + 3 * k + 1);
                const float4 e1 = __ldg(S.tris + 3 * k + 2);
                st.tris++;
                const float t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, a, e0, e1, h.t);
                if (t < h.t) {
                    h.t = t;
                    h.prim = prim;
                    h.shape_type = DFPT_SHAPE_TRIANGLE;
                    h.shape_offset = __float_as_int(a.w);
                }
                if (ANY && h.prim != -1) return true;
                if (__float_as_int(e0.w) != 0) {
                    last = __float_as_int(e1.w);
                    break;
                }
            }
        } else {
            const float4* P = S.pairs + 4 * (size_t)cur;
            const float4 p0 = __ldg(P), p1 = __ldg(P + 1), p2 = __ldg(P + 2);
            const int4 p3 = __ldg(reinterpret_cast<const int4*>(P + 3));
            float lmin, lmax, rmin, rmax;
            slab_interval(p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, sr, lmin, lmax);
            slab_interval(p1.z, p1.w, p2.x, p2.y, p2.z, p2.w, sr, rmin, rmax);
            st.nodes++;
            const bool accept_r = box_accepts(rmin, rmax, h.t);
            if (box_accepts(lmin, lmax, h.t)) {
                if (accept_r) {
                    if (top - bottom == cap) ++bottom;
                    const float key = rmin > 0.001f ? rmin : rmax;
                    cstk[(top & (K - 1)) * 256 + tid] = make_int2(p3.y >= 0 ? ~p3.y : p3.z, __float_as_int(key));
                    ++top;
                } else {
                    st.nodes++;  // the right child's test, decided (rejected) already
                }
                cur = cur + 1;
                leaf = p3.x;
                descend = true;
            } else {
                st.nodes++;
                if (accept_r) {
                    cur = p3.z;
                    leaf = p3.y;
                    descend = true;
                } else {
                    last = p3.z;
                }
            }
        }
        if (descend) continue;
        // The next node in preorder: the nearest pending right child, else next() of `last`.
        for (;;) {
            if (top > bottom) {
                --top;
                const int2 e = cstk[(top & (K - 1)) * 256 + tid];
                st.nodes++;
                if (__int_as_float(e.y) < h.t) {
                    cur = e.x;
                    leaf = e.x >= 0 ? -1 : ~e.x;
                    break;
                }
                last = e.x;
            } else if (bottom > 0) {
                if (last < 0) last = __float_as_int(__ldg(S.tris + 3 * (~last) + 2).w);
                const int nxt = __float_as_int(__ldg(S.nodes + 2 * last).w);
                if (nxt == -1) return false;
                const float4 n0 = __ldg(S.nodes + 2 * nxt), n1 = __ldg(S.nodes + 2 * nxt + 1);
                st.nodes++;
                float tmin, tmax;
                slab_interval(n0.x, n0.y, n0.z, n1.x, n1.y, n1.z, sr, tmin, tmax);
                if (box_accepts(tmin, tmax, h.t)) {
                    cur = nxt;
                    leaf = __float_as_int(n1.w);
                    break;
                }
                last = nxt;
            } else {
                return false;
            }
        }
    }
}

// Warp-synchronous form of the same walk: every lane keeps its own position in the preorder
// sequence, and the warp always serves the smallest position among its active lanes; the lanes
// standing on that node test it (one broadcast load), the others wait. Each lane therefore
// visits exactly the nodes, in exactly the order, of mesh_walk, with the closest distance it
// has at that moment; only the interleaving across lanes changes. All 32 lanes must call it
// together; `active` marks lanes with a ray that still needs this mesh.
template <bool ANY>
__device__ __forceinline__ bool mesh_walk_warp(const DevScene& S, int root, int prim, bool active, float oxo, float oyo, float ozo,
                                               float dxo, float dyo, float dzo, Hit& h, TraceStats& st) {
    const SlabRay sr = slab_ray(oxo, oyo, ozo, dxo, dyo, dzo);
    int cur = active ? root : -1;
    bool found = false;
    for (;;) {
        const unsigned key = cur < 0 ? 0xFFFFFFFFu : (unsigned)cur;
        const unsigned m = __reduce_min_sync(0xFFFFFFFFu, key);
        if (m == 0xFFFFFFFFu) break;
        if (key == m) {
            const int node = (int)m;
            const float4 n0 = __ldg(S.nodes + 2 * node), n1 = __ldg(S.nodes + 2 * node + 1);
            st.nodes++;
            const int next = __float_as_int(n0.w);
            const int leaf = __float_as_int(n1.w);
            const float t0x = slab(n0.x, sr.ix, sr.px), t0y = slab(n0.y, sr.iy, sr.py), t0z = slab(n0.z, sr.iz, sr.pz);
            const float t1x = slab(n1.x, sr.ix, sr.px), t1y = slab(n1.y, sr.iy, sr.py), t1z = slab(n1.z, sr.iz, sr.pz);
            const float tmax = jmin3(jmax(t0x, t1x), jmax(t0y, t1y), jmax(t0z, t1z));
            const float tmin = jmax3(jmin(t0x, t1x), jmin(t0y, t1y), jmin(t0z, t1z));
            const float tb = tmin > tmax ? -1.0f : tmin > 0.001f && tmin < h.t ? tmin : tmax > 0.001f && tmax < h.t ? tmax : -1.0f;
            bool stop = false;
            if (tb >= 0.0f && leaf != -1) {
                for (int k = leaf; k >= 0;) {
                    const float4 a = __ldg(S.tris + 3 * k);
                    const float4 e0 = __ldg(S.tris + 3 * k + 1);
                    const float4 e1 = __ldg(S.tris + 3 * k + 2);
                    st.tris++;
                    const float t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, a, e0, e1, h.t);
                    if (t < h.t) {
                        h.t = t;
                        h.prim = prim;
                        h.shape_type = DFPT_SHAPE_TRIANGLE;
                        h.shape_offset = __float_as_int(a.w);
                    }
                    if (ANY && h.prim != -1) { stop = true; break; }
                    k = __float_as_int(e0.w) != 0 ? -1 : k + 1;
                }
            }
            if (stop) {
                found = true;
                cur = -1;
            } else {
                cur = (tb >= 0.0f && leaf == -1) ? node + 1 : next;
            }
        }
    }
    return found;
}

// trace() for all 32 lanes of a warp together (the warp-synchronous walk); `valid` marks lanes
// with a ray. Same results as trace<ANY, 0> for every valid lane.
template <bool ANY>
__device__ Hit trace_warp(const DevScene& S, bool valid, float ox, float oy, float oz, float dx, float dy, float dz, TraceStats& st) {
    Hit h;
    h.t = INF;
    h.prim = -1;
    h.shape_type = -1;
    h.shape_offset = -1;
    bool done = !valid;
    const int np = S.primitive_count;
    for (int i = 0; i < np; ++i) {
        const int4 info = __ldg(S.prim_info + i);
        const float4* W = reinterpret_cast<const float4*>(S.w2o) + i * 4;
        const float4 r0 = __ldg(W), r1 = __ldg(W + 1), r2 = __ldg(W + 2);
        const float oxo = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
        const float oyo = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
        const float ozo = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
        const float dxo = r0.x * dx + r0.y * dy + r0.z * dz;
        const float dyo = r1.x * dx + r1.y * dy + r1.z * dz;
        const float dzo = r2.x * dx + r2.y * dy + r2.z * dz;
        float t = INF;
        const int type = info.x;
        if (type == DFPT_SHAPE_TRIANGLE_MESH) {
            if (mesh_walk_warp<ANY>(S, info.w, i, !done, oxo, oyo, ozo, dxo, dyo, dzo, h, st)) done = true;
        } else if (!done) {
            if (type == DFPT_SHAPE_PLANE) {
                t = isect_plane(oxo, oyo, ozo, dxo, dyo, dzo, __ldg(S.plane_a + info.w), __ldg(S.plane_n + info.w), h.t);
            } else if (type == DFPT_SHAPE_SPHERE) {
                t = isect_sphere(oxo, oyo, ozo, dxo, dyo, dzo, __ldg(S.sphere4 + info.w), h.t);
            } else if (type == DFPT_SHAPE_TERRAIN) {
                t = isect_terrain(oxo, oyo, ozo, dxo, dyo, dzo);
            } else if (type == DFPT_SHAPE_TRIANGLE) {
                st.tris++;
                t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, __ldg(S.tris + 3 * info.w), __ldg(S.tris + 3 * info.w + 1),
                                   __ldg(S.tris + 3 * info.w + 2), h.t);
            }
            if (t < h.t) {
                h.t = t;
                h.prim = i;
                h.shape_type = type;
                h.shape_offset = info.y;
            }
            if (ANY && h.prim != -1) done = true;
        }
    }
    return h;
}

// One primitive of doIntersectPrimitives (GRK:1048-1256): the ray in object space, then the
// shape's test against the closest distance so far. Returns true when an any-hit query is done.
template <bool ANY, int V>
__device__ __forceinline__ bool prim_test(const DevScene& S, int i, float ox, float oy, float oz, float dx, float dy, float dz, Hit& h,
                                          TraceStats& st) {
    const int4 info = __ldg(S.prim_info + i);
    const float4* W = reinterpret_cast<const float4*>(S.w2o) + i * 4;
    const float4 r0 = __ldg(W), r1 = __ldg(W + 1), r2 = __ldg(W + 2);
    const float oxo = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
    const float oyo = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
    const float ozo = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
    const float dxo = r0.x * dx + r0.y * dy + r0.z * dz;
    const float dyo = r1.x * dx + r1.y * dy + r1.z * dz;
    const float dzo = r2.x * dx + r2.y * dy + r2.z * dz;
    float t = INF;
    const int type = info.x;
    if (type == DFPT_SHAPE_TRIANGLE_MESH) {
        // The mesh updates the closest hit in place; t stays INF for the check below.
        if (mesh_walk<ANY, V>(S, info.w, i, oxo, oyo, ozo, dxo, dyo, dzo, h, st)) return true;
    } else if (type == DFPT_SHAPE_PLANE) {
        t = isect_plane(oxo, oyo, ozo, dxo, dyo, dzo, __ldg(S.plane_a + info.w), __ldg(S.plane_n + info.w), h.t);
    } else if (type == DFPT_SHAPE_SPHERE) {
        t = isect_sphere(oxo, oyo, ozo, dxo, dyo, dzo, __ldg(S.sphere4 + info.w), h.t);
    } else if (type == DFPT_SHAPE_TERRAIN) {
        t = isect_terrain(oxo, oyo, ozo, dxo, dyo, dzo);
    } else if (type == DFPT_SHAPE_TRIANGLE) {
        st.tris++;
        t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, __ldg(S.tris + 3 * info.w), __ldg(S.tris + 3 * info.w + 1),
                           __ldg(S.tris + 3 * info.w + 2), h.t);
    }
    if (t < h.t) {
        h.t = t;
        h.prim = i;
        h.shape_type = type;
        h.shape_offset = info.y;
    }
    return ANY && h.prim != -1;
}

// Slab test of a padded world box against the ray's half line t >= 0: the entry distance, or
// +inf when the line misses. An axis whose direction component is (nearly) zero is a slab the
// ray stays in or out of for every t, tested on the origin directly (no 0 * inf).
__device__ __forceinline__ void cull_slab(float lo, float hi, float o, float d, float inv, float& tmin, float& tmax) {
    if (fabsf(d) < 1.0e-20f) {
        if (!(o >= lo && o <= hi)) {
            tmin = INFINITY;
            tmax = -INFINITY;
        }
        return;
    }
    const float t0 = (lo - o) * inv, t1 = (hi - o) * inv;
    tmin = fmaxf(tmin, fminf(t0, t1));
    tmax = fminf(tmax, fmaxf(t0, t1));
}
__device__ __forceinline__ float box_entry(float4 lo, float4 hi, float ox, float oy, float oz, float dx, float dy, float dz, float ix,
                                           float iy, float iz) {
    float tmin = 0.0f, tmax = INFINITY;
    cull_slab(lo.x, hi.x, ox, dx, ix, tmin, tmax);
    cull_slab(lo.y, hi.y, oy, dy, iy, tmin, tmax);
    cull_slab(lo.z, hi.z, oz, dz, iz, tmin, tmax);
    return tmin <= tmax ? tmin : INFINITY;
}

// doIntersectPrimitives (GRK:1048-1256): a linear loop over primitives, each ray transformed
// to object space; meshes walk the threaded (preorder, skip-pointer) BVH exactly as flattened.
// ANY = isTesting: return at the first primitive with a hit. With culling mode 1 each primitive's
// padded world box is tested first and the primitive skipped when the ray's half line misses it
// or enters it beyond the closest distance found so far (see trace_culled for why that leaves
// the result unchanged); the loop order is the reference's.
template <bool ANY, int V = 0>
__device__ Hit trace(const DevScene& S, float ox, float oy, float oz, float dx, float dy, float dz, TraceStats& st) {
    Hit h;
    h.t = INF;
    h.prim = -1;
    h.shape_type = -1;
    h.shape_offset = -1;
    const int np = S.primitive_count;
    if (S.use_culling == 1) {
        const float ix = 1.0f / dx, iy = 1.0f / dy, iz = 1.0f / dz;
        for (int i = 0; i < np; ++i) {
            const float4 lo = __ldg(S.prim_box + 2 * i), hi = __ldg(S.prim_box + 2 * i + 1);
            if (box_entry(lo, hi, ox, oy, oz, dx, dy, dz, ix, iy, iz) > h.t) continue;
            if (prim_test<ANY, V>(S, i, ox, oy, oz, dx, dy, dz, h, st)) return h;
        }
        return h;
    }
    for (int i = 0; i < np; ++i)
        if (prim_test<ANY, V>(S, i, ox, oy, oz, dx, dy, dz, h, st)) return h;
    return h;
}

// The same loop over only the primitives the ray can reach, still in primitive order. A
// primitive whose padded world box the ray's half line misses, or enters beyond the closest
// distance found so far, cannot change the closest hit - its object-space root box or shape
// test would reject it (the world box holds the primitive's geometry under the inverse of its
// world-to-object matrix, padded for rounding) - so skipping it leaves every later test with
// the closest distance the full loop would have. The reachable primitives are collected from
// the culling BVH, sorted, merged with the unbounded ones, and tested with prim_test. More than
// DFPT_CULL_CANDIDATES of them (or a deeper tree than the stack) falls back to the full loop.
template <bool ANY, int V>
__device__ Hit trace_culled(const DevScene& S, float ox, float oy, float oz, float dx, float dy, float dz, TraceStats& st) {
    const float ix = 1.0f / dx, iy = 1.0f / dy, iz = 1.0f / dz;
    int cand[DFPT_CULL_CANDIDATES];
    int nc = 0;
    bool overflow = false;
    int stack[DFPT_CULL_STACK];
    int sp = 0;
    int node = 0;
    for (;;) {
        const float4 a = __ldg(S.cull_nodes + 2 * node), b = __ldg(S.cull_nodes + 2 * node + 1);
        if (box_entry(a, b, ox, oy, oz, dx, dy, dz, ix, iy, iz) < INFINITY) {
            const int l = __float_as_int(a.w), r = __float_as_int(b.w);
            if (l < 0) {
                for (int k = -l - 1, e = -l - 1 + r; k < e; ++k) {
                    if (nc == DFPT_CULL_CANDIDATES) { overflow = true; break; }
                    const int p = __ldg(S.cull_prims + k);
                    int j = nc++;
                    while (j > 0 && cand[j - 1] > p) { cand[j] = cand[j - 1]; --j; }
                    cand[j] = p;
                }
                if (overflow) break;
            } else {
                if (sp == DFPT_CULL_STACK) { overflow = true; break; }
                stack[sp++] = r;
                node = l;
                continue;
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    if (overflow) {
        // The full loop, with the per-primitive box test (mode 1).
        DevScene flat = S;
        flat.use_culling = 1;
        return trace<ANY, V>(flat, ox, oy, oz, dx, dy, dz, st);
    }
    Hit h;
    h.t = INF;
    h.prim = -1;
    h.shape_type = -1;
    h.shape_offset = -1;
    int ia = 0, ic = 0;
    const int na = S.always_count;
    while (ia < na || ic < nc) {
        const int pa = ia < na ? __ldg(S.always + ia) : 0x7FFFFFFF;
        const int pc = ic < nc ? cand[ic] : 0x7FFFFFFF;
        int i;
        if (pa < pc) {
            i = pa;
            ++ia;
        } else {
            i = pc;
            ++ic;
            const float4 lo = __ldg(S.prim_box + 2 * i), hi = __ldg(S.prim_box + 2 * i + 1);
            if (box_entry(lo, hi, ox, oy, oz, dx, dy, dz, ix, iy, iz) > h.t) continue;
        }
        if (prim_test<ANY, V>(S, i, ox, oy, oz, dx, dy, dz, h, st)) return h;
    }
    return h;
}

// Lane-refill traversal: every lane of a warp carries its own ray through a small state machine
// (the primitive loop of trace() and the threaded walk of mesh_walk, one node visit per step) and
// a lane whose ray is finished takes the next ray of the queue while the others go on, so the
// warp's lanes stay busy until the queue is empty instead of waiting for the slowest of 32 rays.
// Each ray goes through exactly the operations of trace<ANY, 0> (with the per-primitive box test
// when the scene selects culling), in the same order, so the results are the same. All 32 lanes call it
// together. `load(i, o, d)` reads queue entry i, `finish(i, o, d, hit)` consumes its result; the
// scene comes from `scene(i)` (the kernel's own, or the entry's scene in a batch).
template <bool ANY, class SceneOf, class Load, class Finish>
__device__ __forceinline__ void trace_refill(int n, int* fetch, SceneOf scene, Load load, Finish finish, TraceStats& st) {
    const unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    int idx = -1, prim = 0, node = -1;
    float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 1, 0);
    float oxo = 0, oyo = 0, ozo = 0, dxo = 0, dyo = 0, dzo = 1;
    SlabRay sr{0, 0, 1, 0, 0, 0};
    float4 n0 = make_float4(0, 0, 0, 0), n1 = make_float4(0, 0, 0, 0);
    Hit h;
    h.t = INF; h.prim = -1; h.shape_type = -1; h.shape_offset = -1;
    bool exhausted = false;
    for (;;) {
        // Refill when at least half the lanes are idle (or all of them).
        const unsigned idle = __ballot_sync(FULL, idx < 0);
        if (!exhausted && __popc(idle) >= 16) {
            int base = 0;
            if (lane == 0) base = atomicAdd(fetch, __popc(idle));
            base = __shfl_sync(FULL, base, 0);
            if (base + __popc(idle) >= n) exhausted = true;
            if (idx < 0) {
                const int j = base + __popc(idle & ((1u << lane) - 1u));
                if (j < n) {
                    idx = j;
                    load(j, o, d);
                    prim = 0;
                    node = -1;
                    h.t = INF; h.prim = -1; h.shape_type = -1; h.shape_offset = -1;
                }
            }
        }
        const unsigned busy = __ballot_sync(FULL, idx >= 0);
        if (busy == 0) {
            if (exhausted) break;
            continue;
        }
        if (idx < 0) continue;
        const DevScene& S = scene(idx, d);
        if (node < 0) {
            // Between primitives: finish the ray or set up the next primitive.
            if (prim >= S.primitive_count) {
                finish(idx, o, d, h);
                idx = -1;
                continue;
            }
            const int i = prim;
            if (S.use_culling != 0) {
                // Box test per primitive (the BVH-candidate mode gives the same hits this way).
                const float4 lo = __ldg(S.prim_box + 2 * i), hi = __ldg(S.prim_box + 2 * i + 1);
                if (box_entry(lo, hi, o.x, o.y, o.z, d.x, d.y, d.z, 1.0f / d.x, 1.0f / d.y, 1.0f / d.z) > h.t) {
                    ++prim;
                    continue;
                }
            }
            const int4 info = __ldg(S.prim_info + i);
            if (info.x != DFPT_SHAPE_TRIANGLE_MESH) {
                if (prim_test<ANY, 0>(S, i, o.x, o.y, o.z, d.x, d.y, d.z, h, st)) {
                    finish(idx, o, d, h);
                    idx = -1;
                    continue;
                }
                ++prim;
                continue;
            }
            const float4* W = reinterpret_cast<const float4*>(S.w2o) + i * 4;
            const float4 r0 = __ldg(W), r1 = __ldg(W + 1), r2 = __ldg(W + 2);
            oxo = r0.x * o.x + r0.y * o.y + r0.z * o.z + r0.w;
            oyo = r1.x * o.x + r1.y * o.y + r1.z * o.z + r1.w;
            ozo = r2.x * o.x + r2.y * o.y + r2.z * o.z + r2.w;
            dxo = r0.x * d.x + r0.y * d.y + r0.z * d.z;
            dyo = r1.x * d.x + r1.y * d.y + r1.z * d.z;
            dzo = r2.x * d.x + r2.y * d.y + r2.z * d.z;
            sr = slab_ray(oxo, oyo, ozo, dxo, dyo, dzo);
            node = info.w;
            n0 = __ldg(S.nodes + 2 * node);
            n1 = __ldg(S.nodes + 2 * node + 1);
            continue;
        }
        // One node of mesh_walk.
        st.nodes++;
        const int next = __float_as_int(n0.w);
        const int leaf = __float_as_int(n1.w);
        const float t0x = slab(n0.x, sr.ix, sr.px), t0y = slab(n0.y, sr.iy, sr.py), t0z = slab(n0.z, sr.iz, sr.pz);
        const float t1x = slab(n1.x, sr.ix, sr.px), t1y = slab(n1.y, sr.iy, sr.py), t1z = slab(n1.z, sr.iz, sr.pz);
        const float tmax = jmin3(jmax(t0x, t1x), jmax(t0y, t1y), jmax(t0z, t1z));
        const float tmin = jmax3(jmin(t0x, t1x), jmin(t0y, t1y), jmin(t0z, t1z));
        const float tb = tmin > tmax ? -1.0f : tmin > 0.001f && tmin < h.t ? tmin : tmax > 0.001f && tmax < h.t ? tmax : -1.0f;
        bool stop = false;
        if (tb >= 0.0f && leaf != -1) {
            for (int k = leaf; k >= 0;) {
                const float4 a = __ldg(S.tris + 3 * k);
                const float4 e0 = __ldg(S.tris + 3 * k + 1);
                const float4 e1 = __ldg(S.tris + 3 * k + 2);
                st.tris++;
                const float t = isect_triangle(oxo, oyo, ozo, dxo, dyo, dzo, a, e0, e1, h.t);
                if (t < h.t) {
                    h.t = t;
                    h.prim = prim;
                    h.shape_type = DFPT_SHAPE_TRIANGLE;
                    h.shape_offset = __float_as_int(a.w);
                }
                if (ANY && h.prim != -1) { stop = true; break; }
                k = __float_as_int(e0.w) != 0 ? -1 : k + 1;
            }
        }
        if (stop) {
            finish(idx, o, d, h);
            idx = -1;
            continue;
        }
        node = (tb >= 0.0f && leaf == -1) ? node + 1 : next;
        if (node < 0) {
            ++prim;
        } else {
            n0 = __ldg(S.nodes + 2 * node);
            n1 = __ldg(S.nodes + 2 * node + 1);
        }
    }
}

// Closest hit of one ray with the per-lane walk, through the culling structure when the scene has one.
__device__ __forceinline__ Hit trace_s(const DevScene& S, float ox, float oy, float oz, float dx, float dy, float dz, TraceStats& st) {
    return S.use_culling == 2 ? trace_culled<false, 0>(S, ox, oy, oz, dx, dy, dz, st) : trace<false, 0>(S, ox, oy, oz, dx, dy, dz, st);
}

// Selects the walk: V 0/1 per-lane (every lane may call it alone), V 2 warp-synchronous (all 32
// lanes call it; invalid lanes pass valid = false).
template <bool ANY, int V>
__device__ __forceinline__ Hit trace_v(const DevScene& S, bool valid, float ox, float oy, float oz, float dx, float dy, float dz, TraceStats& st) {
    if constexpr (V == 2) {
        return trace_warp<ANY>(S, valid, ox, oy, oz, dx, dy, dz, st);
    } else {
        if (valid) return S.use_culling == 2 ? trace_culled<ANY, V>(S, ox, oy, oz, dx, dy, dz, st) : trace<ANY, V>(S, ox, oy, oz, dx, dy, dz, st);
    }
    Hit h;
    h.t = INF;
    h.prim = -1;
    h.shape_type = -1;
    h.shape_offset = -1;
    return h;
}

}  // namespace DFPT_NS
