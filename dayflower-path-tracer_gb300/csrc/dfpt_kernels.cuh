// dfpt_kernels.cuh - surface evaluation, shading and the wavefront kernels.
//
// Included by dfpt_kernels_fast.cu and dfpt_kernels_strict.cu after dfpt_device.cuh, inside the
// namespace chosen by DFPT_NS. References: GRK = GPURendererKernel.java, AIK =
// AbstractImageKernel.java (src/main/java/org/dayflower/pathtracer/kernel/).
#pragma once

#include "dfpt_device.cuh"
#include "dfpt_launch.h"

namespace DFPT_NS {

// ---------------------------------------------------------------------------------------------
// The intersection record the shading reads (GRK:79-94): point, shading normal, UV, tangent.
struct Surf {
    float px, py, pz;
    float nx, ny, nz;
    float u, v;
    float tx, ty, tz;
};

__device__ __forceinline__ float3 p3(const DevScene& S, int off) {
    return make_float3(__ldg(S.point3fs + off), __ldg(S.point3fs + off + 1), __ldg(S.point3fs + off + 2));
}
__device__ __forceinline__ float3 v3(const DevScene& S, int off) {
    return make_float3(__ldg(S.vector3fs + off), __ldg(S.vector3fs + off + 1), __ldg(S.vector3fs + off + 2));
}
__device__ __forceinline__ float texf(const DevScene& S, int off) { return __ldg(S.textures + off); }

// Image texture lookup without filtering (GRK:1894-1929).
__device__ int image_texture_simple(const DevScene& S, int to, float u, float v) {
    const float width = texf(S, to + 4), height = texf(S, to + 5);
    const float su = texf(S, to + 6), sv = texf(S, to + 7);
    const float ca = texf(S, to + 2), sa = texf(S, to + 3);
    const float u0 = (u * ca - v * sa), v0 = (v * ca + u * sa);
    const float u1 = remainder_j(u0 * su * width, width), v1 = remainder_j(v0 * sv * height, height);
    const float u2 = u1 >= 0.0f ? u1 : width - fabsf(u1);
    const float v2 = v1 >= 0.0f ? v1 : height - fabsf(v1);
    const int x = f2i(u2), y = f2i(v2);
    const int w = f2i(width), res = f2i(width * height);
    const int index = y * w + x;
    return index >= 0 && index < res ? f2i(texf(S, to + 8 + index)) : 0;
}

// Object-space surface properties of the hit, the transform to world space and normal mapping
// (GRK:1258-1400, 2349-2650, 2658-2846, 3998-4073).
__device__ Surf surface(const DevScene& S, const DevParams& P, float ox, float oy, float oz, float dx, float dy, float dz, const Hit& h) {
    const float4* W = reinterpret_cast<const float4*>(S.w2o) + h.prim * 4;
    const float4 w0 = __ldg(W), w1 = __ldg(W + 1), w2 = __ldg(W + 2);
    const float4* O = reinterpret_cast<const float4*>(S.o2w) + h.prim * 4;
    const float4 m0 = __ldg(O), m1 = __ldg(O + 1), m2 = __ldg(O + 2);
    const float oxo = w0.x * ox + w0.y * oy + w0.z * oz + w0.w;
    const float oyo = w1.x * ox + w1.y * oy + w1.z * oz + w1.w;
    const float ozo = w2.x * ox + w2.y * oy + w2.z * oz + w2.w;
    const float dxo = w0.x * dx + w0.y * dy + w0.z * dz;
    const float dyo = w1.x * dx + w1.y * dy + w1.z * dz;
    const float dzo = w2.x * dx + w2.y * dy + w2.z * dz;
    const float t = h.t;
    Surf s;
    s.tx = s.ty = s.tz = 0.0f;
    s.u = s.v = 0.0f;
    const int off = h.shape_offset;
    if (h.shape_type == DFPT_SHAPE_PLANE) {
        const float3 a = p3(S, __ldg(S.planes + off)), b = p3(S, __ldg(S.planes + off + 1)), c = p3(S, __ldg(S.planes + off + 2));
        const float3 n = v3(S, __ldg(S.planes + off + 3));
        s.px = oxo + dxo * t; s.py = oyo + dyo * t; s.pz = ozo + dzo * t;
        const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
        const bool isX = ax > ay && ax > az;
        const bool isY = ay > az;
        const float a1x = isX ? a.y : isY ? a.z : a.x;
        const float a1y = isX ? a.z : isY ? a.x : a.y;
        const float b1x = isX ? c.y - a.x : isY ? c.z - a.x : c.x - a.x;
        const float b1y = isX ? c.z - a.y : isY ? c.x - a.y : c.y - a.y;
        const float c1x = isX ? b.y - a.x : isY ? b.z - a.x : b.x - a.x;
        const float c1y = isX ? b.z - a.y : isY ? b.x - a.y : b.y - a.y;
        const float det = b1x * c1y - b1y * c1x;
        const float dr = 1.0f / det;
        const float bnu = -b1y * dr, bnv = b1x * dr, bnd = (b1y * a1x - b1x * a1y) * dr;
        const float cnu = c1y * dr, cnv = -c1x * dr, cnd = (c1x * a1y - c1y * a1x) * dr;
        const float hu = isX ? s.py : isY ? s.pz : s.px;
        const float hv = isX ? s.pz : isY ? s.px : s.py;
        s.u = hu * bnu + hv * bnv + bnd;
        s.v = hu * cnu + hv * cnv + cnd;
        s.nx = n.x; s.ny = n.y; s.nz = n.z;
    } else if (h.shape_type == DFPT_SHAPE_SPHERE) {
        const float3 c = p3(S, f2i(__ldg(S.spheres + off)));
        s.px = oxo + dxo * t; s.py = oyo + dyo * t; s.pz = ozo + dzo * t;
        const float n0x = s.px - c.x, n0y = s.py - c.y, n0z = s.pz - c.z;
        const float r = rsqrt_j(n0x * n0x + n0y * n0y + n0z * n0z);
        s.nx = n0x * r; s.ny = n0y * r; s.nz = n0z * r;
        s.u = 0.5f + atan2_j(-s.nz, -s.nx) * INV_TWO_PI;
        s.v = 0.5f - asin_j(-s.ny) * INV_PI;
    } else if (h.shape_type == DFPT_SHAPE_TERRAIN) {
        const float sr = 1.0f / 10.0f;
        s.px = oxo * sr + dxo * t; s.py = oyo * sr + dyo * t; s.pz = ozo * sr + dzo * t;
        const float e = 0.02f;
        const float nx = (sin_j(s.px - e) * sin_j(s.pz)) - (sin_j(s.px + e) * sin_j(s.pz));
        const float ny = 2.0f * e;
        const float nz = (sin_j(s.px) * sin_j(s.pz - e)) - (sin_j(s.px) * sin_j(s.pz + e));
        const float r = rsqrt_j(nx * nx + ny * ny + nz * nz);
        s.nx = nx * r; s.ny = ny * r; s.nz = nz * r;
        s.u = s.px; s.v = s.pz;
    } else {  // Triangle
        // The vertex values come from the triangle's shading record (one contiguous 144-byte
        // record, the same floats) when the scene has them, else through the reference's indices.
        const int* T = S.triangles + off;
        const float4* R = S.shade_tris ? S.shade_tris + 9 * (size_t)(off / 12) : nullptr;
        float3 a, b, c;
        float uax, uay, ubx, uby, ucx, ucy;
        if (R) {
            const float4 r0 = __ldg(R), r1 = __ldg(R + 1), r2 = __ldg(R + 2), r3 = __ldg(R + 3);
            a = make_float3(r0.x, r0.y, r0.z);
            b = make_float3(r0.w, r1.x, r1.y);
            c = make_float3(r1.z, r1.w, r2.x);
            uax = r2.y; uay = r2.z; ubx = r2.w; uby = r3.x; ucx = r3.y; ucy = r3.z;
        } else {
            a = p3(S, __ldg(T + 0)); b = p3(S, __ldg(T + 1)); c = p3(S, __ldg(T + 2));
            const int ta = __ldg(T + 6), tb = __ldg(T + 7), tc = __ldg(T + 8);
            uax = __ldg(S.point2fs + ta); uay = __ldg(S.point2fs + ta + 1);
            ubx = __ldg(S.point2fs + tb); uby = __ldg(S.point2fs + tb + 1);
            ucx = __ldg(S.point2fs + tc); ucy = __ldg(S.point2fs + tc + 1);
        }
        s.px = oxo + dxo * t; s.py = oyo + dyo * t; s.pz = ozo + dzo * t;
        const float abx = b.x - a.x, aby = b.y - a.y, abz = b.z - a.z;
        const float acx = c.x - a.x, acy = c.y - a.y, acz = c.z - a.z;
        const float v0x = dyo * acz - dzo * acy, v0y = dzo * acx - dxo * acz, v0z = dxo * acy - dyo * acx;
        const float v1x = oxo - a.x, v1y = oyo - a.y, v1z = ozo - a.z;
        const float v2x = v1y * abz - v1z * aby, v2y = v1z * abx - v1x * abz, v2z = v1x * aby - v1y * abx;
        const float det = abx * v0x + aby * v0y + abz * v0z;
        const float dr = 1.0f / det;
        const float bu = (v1x * v0x + v1y * v0y + v1z * v0z) * dr;
        const float bv = (dxo * v2x + dyo * v2y + dzo * v2z) * dr;
        const float bw = 1.0f - bu - bv;
        s.u = bw * uax + bu * ubx + bv * ucx;
        s.v = bw * uay + bu * uby + bv * ucy;
        float n0x = 0.0f, n0y = 0.0f, n0z = 0.0f, t0x = 0.0f, t0y = 0.0f, t0z = 0.0f;
        if (P.shader_type == DFPT_SHADER_FLAT) {
            n0x = aby * acz - abz * acy;
            n0y = abz * acx - abx * acz;
            n0z = abx * acy - aby * acx;
        } else if (P.shader_type == DFPT_SHADER_GOURAUD) {
            float3 na, nb, nc, tga, tgb, tgc;
            if (R) {
                const float4 r3 = __ldg(R + 3), r4 = __ldg(R + 4), r5 = __ldg(R + 5), r6 = __ldg(R + 6), r7 = __ldg(R + 7),
                             r8 = __ldg(R + 8);
                na = make_float3(r3.w, r4.x, r4.y);
                nb = make_float3(r4.z, r4.w, r5.x);
                nc = make_float3(r5.y, r5.z, r5.w);
                tga = make_float3(r6.x, r6.y, r6.z);
                tgb = make_float3(r6.w, r7.x, r7.y);
                tgc = make_float3(r7.z, r7.w, r8.x);
            } else {
                na = v3(S, __ldg(T + 3)); nb = v3(S, __ldg(T + 4)); nc = v3(S, __ldg(T + 5));
                tga = v3(S, __ldg(T + 9)); tgb = v3(S, __ldg(T + 10)); tgc = v3(S, __ldg(T + 11));
            }
            n0x = na.x * bw + nb.x * bu + nc.x * bv;
            n0y = na.y * bw + nb.y * bu + nc.y * bv;
            n0z = na.z * bw + nb.z * bu + nc.z * bv;
            t0x = tga.x * bw + tgb.x * bu + tgc.x * bv;
            t0y = tga.y * bw + tgb.y * bu + tgc.y * bv;
            t0z = tga.z * bw + tgb.z * bu + tgc.z * bv;
        }
        const float nr = rsqrt_j(n0x * n0x + n0y * n0y + n0z * n0z);
        s.nx = n0x * nr; s.ny = n0y * nr; s.nz = n0z * nr;
        const float tr = rsqrt_j(t0x * t0x + t0y * t0y + t0z * t0z);
        s.tx = t0x * tr; s.ty = t0y * tr; s.tz = t0z * tr;
    }
    // To world space: the point by object-to-world, directions by the transposed
    // world-to-object (not renormalised).
    const float wpx = m0.x * s.px + m0.y * s.py + m0.z * s.pz + m0.w;
    const float wpy = m1.x * s.px + m1.y * s.py + m1.z * s.pz + m1.w;
    const float wpz = m2.x * s.px + m2.y * s.py + m2.z * s.pz + m2.w;
    const float wnx = w0.x * s.nx + w1.x * s.ny + w2.x * s.nz;
    const float wny = w0.y * s.nx + w1.y * s.ny + w2.y * s.nz;
    const float wnz = w0.z * s.nx + w1.z * s.ny + w2.z * s.nz;
    const float wtx = w0.x * s.tx + w1.x * s.ty + w2.x * s.tz;
    const float wty = w0.y * s.tx + w1.y * s.ty + w2.y * s.tz;
    const float wtz = w0.z * s.tx + w1.z * s.ty + w2.z * s.tz;
    s.px = wpx; s.py = wpy; s.pz = wpz;
    s.nx = wnx; s.ny = wny; s.nz = wnz;
    s.tx = wtx; s.ty = wty; s.tz = wtz;

    const int4 info = __ldg(S.prim_info + h.prim);
    const int so = info.z;
    if (P.normal_mapping == 1) {
        // Normal mapping via image texture (GRK:2714-2846).
        const int nto = f2i(__ldg(S.surfaces + so + 3));
        if (f2i(texf(S, nto)) == DFPT_TEXTURE_IMAGE) {
            const int rgb = image_texture_simple(S, nto, s.u, s.v);
            const float r = ((((rgb >> 16) & 0xFF) * COLOR_RECIPROCAL) - 0.5f) * 2.0f;
            const float g = ((((rgb >> 8) & 0xFF) * COLOR_RECIPROCAL) - 0.5f) * 2.0f;
            const float bb = ((((rgb >> 0) & 0xFF) * COLOR_RECIPROCAL) - 0.0f) * 2.0f;
            const float wx = s.nx, wy = s.ny, wz = s.nz;
            float sx, sy, sz;
            if (info.x == DFPT_SHAPE_SPHERE) {
                const float v0x = -2.0f * PI_F * wy, v0y = 2.0f * PI_F * wx, v0z = 0.0f;
                const float u0x = v0y * wz - v0z * wy, u0y = v0z * wx - v0x * wz, u0z = v0x * wy - v0y * wx;
                const float ur = rsqrt_j(u0x * u0x + u0y * u0y + u0z * u0z);
                const float u1x = u0x * ur, u1y = u0y * ur, u1z = u0z * ur;
                const float v1x = wy * u1z - wz * u1y, v1y = wz * u1x - wx * u1z, v1z = wx * u1y - wy * u1x;
                const float vr = rsqrt_j(v1x * v1x + v1y * v1y + v1z * v1z);
                const float v2x = v1x * vr, v2y = v1y * vr, v2z = v1z * vr;
                sx = r * u1x + g * v2x + bb * wx; sy = r * u1y + g * v2y + bb * wy; sz = r * u1z + g * v2z + bb * wz;
            } else if (info.x == DFPT_SHAPE_TRIANGLE) {
                const float ux = s.tx, uy = s.ty, uz = s.tz;
                const float v0x = wy * uz - wz * uy, v0y = wz * ux - wx * uz, v0z = wx * uy - wy * ux;
                const float vr = rsqrt_j(v0x * v0x + v0y * v0y + v0z * v0z);
                const float v1x = v0x * vr, v1y = v0y * vr, v1z = v0z * vr;
                sx = r * ux + g * v1x + bb * wx; sy = r * uy + g * v1y + bb * wy; sz = r * uz + g * v1z + bb * wz;
            } else {
                const float awx = fabsf(wx), awy = fabsf(wy), awz = fabsf(wz);
                const bool isWX = awx < awy && awx < awz;
                const bool isWY = awy < awz;
                const float v0x = isWX ? 0.0f : isWY ? wz : wy;
                const float v0y = isWX ? wz : isWY ? 0.0f : -wx;
                const float v0z = isWX ? -wy : isWY ? -wx : 0.0f;
                const float vr = rsqrt_j(v0x * v0x + v0y * v0y + v0z * v0z);
                const float v1x = v0x * vr, v1y = v0y * vr, v1z = v0z * vr;
                const float u0x = v1y * wz - v1z * wy, u0y = v1z * wx - v1x * wz, u0z = v1x * wy - v1y * wx;
                const float ur = rsqrt_j(u0x * u0x + u0y * u0y + u0z * u0z);
                const float u1x = u0x * ur, u1y = u0y * ur, u1z = u0z * ur;
                sx = r * u1x + g * v1x + bb * wx; sy = r * u1y + g * v1y + bb * wy; sz = r * u1z + g * v1z + bb * wz;
            }
            const float sr = rsqrt_j(sx * sx + sy * sy + sz * sz);
            s.nx = sx * sr; s.ny = sy * sr; s.nz = sz * sr;
        }
        // Normal mapping via noise (GRK:2658-2712).
        const float amount = __ldg(S.surfaces + so + 4), scale = __ldg(S.surfaces + so + 5);
        if (amount > 0.0f && scale > 0.0f) {
            const float sr = 1.0f / scale;
            const float x1 = s.px * sr, y1 = s.py * sr, z1 = s.pz * sr;
            const float nx = fbm3(scale, 0.5f, -0.26f, 0.26f, 16, x1, y1, z1);
            const float ny = fbm3(scale, 0.5f, -0.26f, 0.26f, 16, y1, z1, x1);
            const float nz = fbm3(scale, 0.5f, -0.26f, 0.26f, 16, z1, x1, y1);
            const float qx = s.nx + nx * amount, qy = s.ny + ny * amount, qz = s.nz + nz * amount;
            const float qr = rsqrt_j(qx * qx + qy * qy + qz * qz);
            s.nx = qx * qr; s.ny = qy * qr; s.nz = qz * qr;
        }
    }
    return s;
}

// ---------------------------------------------------------------------------------------------
// Textures: packed 0xRRGGBB (GRK:1596-1960).

__device__ __forceinline__ int pack8(float r, float g, float b) {
    const int ri = f2i(saturate_j(r, 0.0f, 1.0f) * 255.0f + 0.5f);
    const int gi = f2i(saturate_j(g, 0.0f, 1.0f) * 255.0f + 0.5f);
    const int bi = f2i(saturate_j(b, 0.0f, 1.0f) * 255.0f + 0.5f);
    return ((ri & 0xFF) << 16) | ((gi & 0xFF) << 8) | (bi & 0xFF);
}
__device__ __forceinline__ float cr(int rgb) { return ((rgb >> 16) & 0xFF) * COLOR_RECIPROCAL; }
__device__ __forceinline__ float cg(int rgb) { return ((rgb >> 8) & 0xFF) * COLOR_RECIPROCAL; }
__device__ __forceinline__ float cb(int rgb) { return (rgb & 0xFF) * COLOR_RECIPROCAL; }

__device__ int texture_leaf(const DevScene& S, int to, const Surf& s) {
    const int type = f2i(texf(S, to));
    if (type == DFPT_TEXTURE_BULLSEYE) {
        const int ca = f2i(texf(S, to + 2)), cbb = f2i(texf(S, to + 3));
        const float len = sqrtf(s.px * s.px + s.py * s.py + s.pz * s.pz);
        const float value = remainder_j(len * 0.25f, 1.0f);
        float r = value > 0.5f ? cr(ca) : cr(cbb);
        float g = value > 0.5f ? cg(ca) : cg(cbb);
        float b = value > 0.5f ? cb(ca) : cb(cbb);
        const float m = value > 0.5f ? 0.8f : 1.2f;
        if (cr(ca) == cr(cbb) && cg(ca) == cg(cbb) && cb(ca) == cb(cbb)) { r *= m; g *= m; b *= m; }
        return pack8(r, g, b);
    } else if (type == DFPT_TEXTURE_CHECKERBOARD) {
        const int c0 = f2i(texf(S, to + 2)), c1 = f2i(texf(S, to + 3));
        const float ca = texf(S, to + 4), sa = texf(S, to + 5), su = texf(S, to + 6), sv = texf(S, to + 7);
        const float tu = modulo_j((s.u * ca - s.v * sa) * su);
        const float tv = modulo_j((s.v * ca + s.u * sa) * sv);
        const bool dark = (tu > 0.5f) ^ (tv > 0.5f);
        const float m = dark ? 0.8f : 1.2f;
        float r = dark ? cr(c0) : cr(c1), g = dark ? cg(c0) : cg(c1), b = dark ? cb(c0) : cb(c1);
        if (cr(c0) == cr(c1) && cg(c0) == cg(c1) && cb(c0) == cb(c1)) { r *= m; g *= m; b *= m; }
        return pack8(r, g, b);
    } else if (type == DFPT_TEXTURE_CONSTANT) {
        return f2i(texf(S, to + 2));
    } else if (type == DFPT_TEXTURE_FBM) {
        const int add = f2i(texf(S, to + 2)), mul = f2i(texf(S, to + 3));
        const float noise = fbm3(texf(S, to + 4), texf(S, to + 5), 0.0f, 1.0f, f2i(texf(S, to + 6)), s.px, s.py, s.pz);
        return pack8(noise * cr(mul) + cr(add), noise * cg(mul) + cg(add), noise * cb(mul) + cb(add));
    } else if (type == DFPT_TEXTURE_IMAGE) {
        const float width = texf(S, to + 4), height = texf(S, to + 5);
        const float su = texf(S, to + 6), sv = texf(S, to + 7);
        const float ca = texf(S, to + 2), sa = texf(S, to + 3);
        const float u0 = (s.u * ca - s.v * sa), v0 = (s.v * ca + s.u * sa);
        const float u1 = remainder_j(u0 * su * width, width), v1 = remainder_j(v0 * sv * height, height);
        const float u2 = u1 >= 0.0f ? u1 : width - fabsf(u1);
        const float v2 = v1 >= 0.0f ? v1 : height - fabsf(v1);
        const int x = f2i(u2), y = f2i(v2);
        const int w = f2i(width), res = f2i(width * height);
        const int i00 = y * w + x, i01 = y * w + (x + 1), i10 = (y + 1) * w + x, i11 = (y + 1) * w + (x + 1);
        const int c00 = i00 >= 0 && i00 < res ? f2i(texf(S, to + 8 + i00)) : 0;
        const int c01 = i01 >= 0 && i01 < res ? f2i(texf(S, to + 8 + i01)) : 0;
        const int c10 = i10 >= 0 && i10 < res ? f2i(texf(S, to + 8 + i10)) : 0;
        const int c11 = i11 >= 0 && i11 < res ? f2i(texf(S, to + 8 + i11)) : 0;
        const float fx = u2 - (float)x, fy = v2 - (float)y;
        return pack8(blerp_j(cr(c00), cr(c01), cr(c10), cr(c11), fx, fy), blerp_j(cg(c00), cg(c01), cg(c10), cg(c11), fx, fy),
                     blerp_j(cb(c00), cb(c01), cb(c10), cb(c11), fx, fy));
    } else if (type == DFPT_TEXTURE_SURFACE_NORMAL) {
        return pack8((s.nx + 1.0f) * 0.5f, (s.ny + 1.0f) * 0.5f, (s.nz + 1.0f) * 0.5f);
    } else if (type == DFPT_TEXTURE_UV) {
        return pack8(s.u, s.v, 0.0f);
    }
    return 0;
}

__device__ int texture_color(const DevScene& S, int to, const Surf& s) {
    if (f2i(texf(S, to)) == DFPT_TEXTURE_BLEND) {
        const int ta = f2i(texf(S, to + 2)), tb = f2i(texf(S, to + 3));
        const float f = texf(S, to + 4);
        const int a = texture_leaf(S, ta, s), b = texture_leaf(S, tb, s);
        return pack8((1.0f - f) * cr(a) + f * cr(b), (1.0f - f) * cg(a) + f * cg(b), (1.0f - f) * cb(a) + f * cb(b));
    }
    return texture_leaf(S, to, s);
}

// ---------------------------------------------------------------------------------------------
// Perez sky (GRK:2127-2236), evaluated in FP32 on the device; the reference evaluates the
// Perez functions in FP64. cos(acos(x)) is x on [-1, 1].
__device__ float3 sky_color(const DevParams& P, float dx, float dy, float dz) {
    float d0x = dx * P.sky_u[0] + dy * P.sky_u[1] + dz * P.sky_u[2];
    float d0y = dx * P.sky_v[0] + dy * P.sky_v[1] + dz * P.sky_v[2];
    float d0z = dx * P.sky_w[0] + dy * P.sky_w[1] + dz * P.sky_w[2];
    float3 c = make_float3(0.01f, 0.01f, 0.01f);
    if (d0z >= 0.0f && P.sky_active == 1) {
        d0z = jmax(d0z, 0.001f);
        const float lr = rsqrt_j(d0x * d0x + d0y * d0y + d0z * d0z);
        const float d1x = d0x * lr, d1y = d0y * lr, d1z = d0z * lr;
        const float dp = d1x * P.sun_dir[0] + d1y * P.sun_dir[1] + d1z * P.sun_dir[2];
        const float cos1 = fminf(fmaxf(d1z, -1.0f), 1.0f);
        const float theta1 = acosf(cos1);
        const float cos1r = 1.0f / (cos1 + 0.01f);
        const float cosg = fminf(fmaxf(dp, -1.0f), 1.0f);
        const float gamma = acosf(cosg);
        const float c0sq = P.cos_theta0 * P.cos_theta0;
        const float num_l = (1.0f + P.perez_l[0] * expf(P.perez_l[1] * cos1r)) * (1.0f + P.perez_l[2] * expf(P.perez_l[3] * gamma) + P.perez_l[4] * cosg * cosg);
        const float rel_l = P.zenith_l * num_l / P.den_l * 1.0e-4f;
        const float den_x = P.den_x_a * (1.0f + P.perez_x[2] * expf(P.perez_x[3] * theta1) + P.perez_x[4] * c0sq);
        const float num_x = (1.0f + P.perez_x[0] * expf(P.perez_x[1] * cos1r)) * (1.0f + P.perez_x[2] * expf(P.perez_x[3] * gamma) + P.perez_x[4] * cosg * cosg);
        const float x = P.zenith_x * num_x / den_x;
        const float den_y = P.den_y_a * (1.0f + P.perez_y[2] * expf(P.perez_y[3] * theta1) + P.perez_y[4] * c0sq);
        const float num_y = (1.0f + P.perez_y[0] * expf(P.perez_y[1] * cos1r)) * (1.0f + P.perez_y[2] * expf(P.perez_y[3] * gamma) + P.perez_y[4] * cosg * cosg);
        const float y = P.zenith_y * num_y / den_y;
        const float c0 = 1.0f / (0.0241f + 0.2562f * x - 0.7341f * y);
        const float c1 = (-1.3515f - 1.7703f * x + 5.9114f * y) * c0;
        const float c2 = (0.03f - 31.4424f * x + 30.0717f * y) * c0;
        const float X = 10246.121f + c1 * 187.75537f + c2 * 213.14803f;
        const float Y = 10676.695f + c1 * 192.59653f + c2 * 76.29494f;
        const float Z = 12372.504f + c1 * 3482.8765f + c2 * -235.71611f;
        const float Yr = 1.0f / Y;
        const float R = X * rel_l * Yr, G = rel_l, B = Z * rel_l * Yr;
        float r = 3.2410042f * R + -1.5373994f * G + -0.49861607f * B;
        float g = -0.9692241f * R + 1.8759298f * G + 0.041554242f * B;
        float b = 0.05563942f * R + -0.20401107f * G + 1.0571486f * B;
        const float w = jmax(0.0f, -jmin(0.0f, jmin(r, jmin(g, b))));
        c = make_float3(r + w, g + w, b + w);
    }
    return c;
}

// Sun sample of doCalculateColorForSun (GRK:2238-2347): a direction in the 500-radius cone
// around the sun direction; returns false when the sample faces away from the sun or surface.
__device__ bool sun_sample(const DevParams& P, float px, float py, float pz, float nx, float ny, float nz, float u, float v,
                           float& ldx, float& ldy, float& ldz, float& dot1) {
    const float sr2 = 500.0f * 500.0f;
    const float tx = P.sun_origin[0] - px, ty = P.sun_origin[1] - py, tz = P.sun_origin[2] - pz;
    const float tl2 = tx * tx + ty * ty + tz * tz;
    const float sin2 = sr2 / tl2;
    const float cos_max = sqrtf(jmax(0.0f, 1.0f - sin2));
    const float cos_t = u * (cos_max - 1.0f) + 1.0f;
    const float sin_t = sqrtf(jmax(0.0f, 1.0f - cos_t * cos_t));
    const float phi = TWO_PI * v;
    const float x = cos_j(phi) * sin_t, y = sin_j(phi) * sin_t, z = cos_t;
    const float wx = P.sun_dir_world[0], wy = P.sun_dir_world[1], wz = P.sun_dir_world[2];
    const float ax = fabsf(wx), ay = fabsf(wy), az = fabsf(wz);
    const float vx = ax < ay && ax < az ? 0.0f : ay < az ? wz : wy;
    const float vy = ax < ay && ax < az ? wz : ay < az ? 0.0f : -wx;
    const float vz = ax < ay && ax < az ? -wy : ay < az ? -wx : 0.0f;
    const float vr = rsqrt_j(vx * vx + vy * vy + vz * vz);
    const float vnx = vx * vr, vny = vy * vr, vnz = vz * vr;
    const float unx = vny * wz - vnz * wy, uny = vnz * wx - vnx * wz, unz = vnx * wy - vny * wx;
    const float rx = unx * x + vnx * y + wx * z;
    const float ry = uny * x + vny * y + wy * z;
    const float rz = unz * x + vnz * y + wz * z;
    const float rr = rsqrt_j(rx * rx + ry * ry + rz * rz);
    ldx = rx * rr; ldy = ry * rr; ldz = rz * rr;
    const float dot0 = ldx * wx + ldy * wy + ldz * wz;
    dot1 = ldx * nx + ldy * ny + ldz * nz;
    return dot0 > 0.0f && dot1 > 0.0f;
}

// Cosine-weighted hemisphere direction around w (GRK:3466-3500).
__device__ __forceinline__ void cosine_dir(float wx, float wy, float wz, float u, float v, float& ox, float& oy, float& oz) {
    const float phi = TWO_PI * u;
    const float ct = sqrtf(v), st = sqrtf(1.0f - v);
    const float x = cos_j(phi) * st, y = sin_j(phi) * st, z = ct;
    const bool isY = fabsf(wx) > 0.1f;
    const float ux = (isY ? 1.0f : 0.0f) * wz;
    const float uy = -((isY ? 0.0f : 1.0f) * wz);
    const float uz = (isY ? 0.0f : 1.0f) * wy - (isY ? 1.0f : 0.0f) * wx;
    const float ur = rsqrt_j(ux * ux + uy * uy + uz * uz);
    const float unx = ux * ur, uny = uy * ur, unz = uz * ur;
    const float vnx = wy * unz - wz * uny, vny = wz * unx - wx * unz, vnz = wx * uny - wy * unx;
    const float dx = unx * x + vnx * y + wx * z;
    const float dy = uny * x + vny * y + wy * z;
    const float dz = unz * x + vnz * y + wz * z;
    const float dr = rsqrt_j(dx * dx + dy * dy + dz * dz);
    ox = dx * dr; oy = dy * dr; oz = dz * dr;
}

// ---------------------------------------------------------------------------------------------
// Camera ray (GRK:573-724). Returns false for pixels outside a fisheye lens.
__device__ bool primary_ray(const DevScene& S, const DevParams& P, int pixel, bool jitter, Rng& rng, float4& o, float4& d) {
    const int y = pixel / P.width;
    const int x = pixel - y * P.width;
    const float* C = S.camera;
    const float ex = __ldg(C + 1), ey = __ldg(C + 2), ez = __ldg(C + 3);
    const float ux = __ldg(C + 7), uy = __ldg(C + 8), uz = __ldg(C + 9);
    const float vx = __ldg(C + 10), vy = __ldg(C + 11), vz = __ldg(C + 12);
    const float wx = __ldg(C + 13), wy = __ldg(C + 14), wz = __ldg(C + 15);
    const float fx = P.fov_tan_x;
    const float fy = P.fov_tan_y;
    const float hx = ux * fx, hy = uy * fx, hz = uz * fx;
    const float gx = vx * fy, gy = vy * fy, gz = vz * fy;
    float sx = 0.5f, sy = 0.5f;
    if (jitter) {
        sx = rng.next();
        sy = rng.next();
        sx = sx < 0.5f ? sqrtf(2.0f * sx) - 1.0f : 1.0f - sqrtf(2.0f - 2.0f * sx);
        sy = sy < 0.5f ? sqrtf(2.0f * sy) - 1.0f : 1.0f - sqrtf(2.0f - 2.0f * sy);
    }
    const float psx = (sx + (float)x) / (__ldg(C + 16) - 1.0f);
    const float psy = (sy + (float)y) / (__ldg(C + 17) - 1.0f);
    const float sx0 = 2.0f * psx - 1.0f, sy0 = 2.0f * psy - 1.0f;
    float w = 1.0f;
    if (__ldg(C + 18) == 2.0f) {
        const float dp = sx0 * sx0 + sy0 * sy0;
        if (dp > 1.0f) return false;
        w = sqrtf(1.0f - dp);
    }
    const float mx = ex + wx * w, my = ey + wy * w, mz = ez + wz * w;
    const float qx = mx + (hx * sx0) + (gx * sy0);
    const float qy = my + (hy * sx0) + (gy * sy0);
    const float qz = mz + (hz * sx0) + (gz * sy0);
    const float focal = __ldg(C + 6);
    const float ipx = ex + (qx - ex) * focal, ipy = ey + (qy - ey) * focal, ipz = ez + (qz - ez) * focal;
    const float aperture = __ldg(C + 0);
    float apx = ex, apy = ey, apz = ez;
    if (aperture > 0.00001f) {
        const float r1 = rng.next(), r2 = rng.next();
        const float angle = TWO_PI * r1;
        const float dist = aperture * sqrtf(r2);
        const float ax = cos_j(angle) * dist, ay = sin_j(angle) * dist;
        apx = ex + ux * ax + vx * ay;
        apy = ey + uy * ax + vy * ay;
        apz = ez + uz * ax + vz * ay;
    }
    const float tx = ipx - apx, ty = ipy - apy, tz = ipz - apz;
    const float tr = rsqrt_j(tx * tx + ty * ty + tz * tz);
    o = make_float4(apx, apy, apz, 0.0f);
    d = make_float4(tx * tr, ty * tr, tz * tr, 0.0f);
    return true;
}

// Warp-aggregated queue append: one atomic per warp; returns the slot or -1. Every lane of the
// warp must call it.
__device__ __forceinline__ int warp_push(int* counter, bool active) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, active);
    if (mask == 0u) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return active ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

__device__ __forceinline__ void warp_add_stats(const DevParams& P, unsigned long long* stats, int which, uint32_t a, uint32_t b, uint32_t c) {
    if (!P.counting) return;
    const unsigned long long sa = __reduce_add_sync(0xFFFFFFFFu, a);
    const unsigned long long sb = __reduce_add_sync(0xFFFFFFFFu, b);
    const unsigned long long sc = __reduce_add_sync(0xFFFFFFFFu, c);
    if ((threadIdx.x & 31) == 0) {
        if (sa) atomicAdd(stats + which, sa);
        if (sb) atomicAdd(stats + 2, sb);
        if (sc) atomicAdd(stats + 3, sc);
        if (which == 0 && sb) atomicAdd(stats + 4, sb);  // closest-hit share
        if (which == 0 && sc) atomicAdd(stats + 5, sc);
    }
}

// Warp-level dynamic work distribution: each warp takes the next 32 queue entries from a counter
// (reset at the start of the pass), so warps that drew short rays keep taking more. All 32 lanes
// iterate together (i >= n marks lanes without an entry).
#define WARP_DYNAMIC(i, n, counter)                                                            \
    for (int i##_base = 0;;)                                                                   \
        if ((i##_base = __shfl_sync(0xFFFFFFFFu, (threadIdx.x & 31) == 0 ? atomicAdd((counter), 32) : 0, 0)) >= (n)) break; \
        else for (int i = i##_base + (int)(threadIdx.x & 31), i##_once = 1; i##_once; i##_once = 0)

#define GRID_STRIDE_UNIFORM(i, n)                                                              \
    for (int i##_base = blockIdx.x * blockDim.x; i##_base < (n); i##_base += gridDim.x * blockDim.x) \
        for (int i = i##_base + (int)threadIdx.x, i##_once = 1; i##_once; i##_once = 0)

// Scene and parameters of a work item: the kernel's own (one scene) or the item's scene of a batch.
// A translation unit compiled with DFPT_ONE_SCENE runs the batch stages over one scene (waves of
// passes): its scene record is the kernel parameter, read from the constant bank, not a record in
// global memory per ray (which costs registers inside the traversal loop).
template <bool BATCH>
__device__ __forceinline__ const DevScene& scene_of(const DevScene& S0, const DevBatch& Q, int sid) {
#ifdef DFPT_ONE_SCENE
    (void)Q; (void)sid;
    return S0;
#else
    if constexpr (BATCH) return Q.scenes[sid];
    else { (void)Q; (void)sid; return S0; }
#endif
}
template <bool BATCH>
__device__ __forceinline__ const DevParams& params_of(const DevParams* P0, const DevBatch& Q, int sid) {
#ifdef DFPT_ONE_SCENE
    (void)Q; (void)sid;
    return *P0;
#else
    if constexpr (BATCH) return Q.params[sid];
    else { (void)Q; (void)sid; return *P0; }
#endif
}
// The scene holding global sample g: the last scene whose first sample is <= g.
__device__ __forceinline__ int batch_scene_of(const DevBatch& Q, long long g) {
    int lo = 0, hi = Q.n_scenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (Q.sample_begin[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------------------------
// Path tracer wavefront (doRenderWithPathTracer, GRK:3151-3705). Every stage is written once for
// both forms: one scene (BATCH = false; a path is a pixel, the pass index keys the RNG) and a batch
// of scenes (BATCH = true; a path is a wave slot, {scene, pixel, sample} come from the slot key).

// Waves with the counter RNG and no differentiation start their paths lean: the camera writes no
// throughput, radiance or RNG state, and shading at bounce 0 starts from throughput 1, radiance 0
// and the camera's draw count (two for the pixel jitter, two more with an aperture). The film
// ignores a rejected (fisheye) slot's radiance.
template <bool BATCH>
__device__ __forceinline__ bool lean_start(const DevParams& P) {
    return BATCH && P.rng_kind == DFPT_RNG_COUNTER && !P.diff;
}
#ifndef DFPT_ONE_SCENE
// Waves of several scenes: within each scene's segment [a, b) of the wave (scene-local sample
// indices, sample order: pass j, pixel x at j * np + x) the slots run pixel-major, a pixel's
// samples adjacent in pass order. Pixel x holds K + (x >= a % np) + (x < b % np) of the segment's
// samples (K = b / np - a / np - 1) and starts at pos(x), the sum of the counts of the pixels
// before it; seg_local_of_pos inverts pos over its three linear pieces.
__device__ __forceinline__ long long seg_pos(long long x, long long K, long long ra, long long rb) {
    return x * K + (x > ra ? x - ra : 0) + (x < rb ? x : rb);
}
__device__ __forceinline__ long long seg_pos_of_local(long long loc, long long a, long long b, long long np) {
    const long long ja = a / np, ra = a - ja * np, jb = b / np, rb = b - jb * np, K = jb - ja - 1;
    const long long j = loc / np, x = loc - j * np;
    return seg_pos(x, K, ra, rb) + (j - (ja + (x >= ra ? 0 : 1)));
}
__device__ __forceinline__ long long seg_local_of_pos(long long p, long long a, long long b, long long np) {
    const long long ja = a / np, ra = a - ja * np, jb = b / np, rb = b - jb * np, K = jb - ja - 1;
    const long long lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
    const long long s0 = K + 1, s1 = ra < rb ? K + 2 : K;
    const long long p_lo = lo * s0, p_hi = p_lo + (hi - lo) * s1;
    long long x;
    if (p < p_lo) x = p / s0;                     // p_lo > 0 implies s0 > 0
    else if (p < p_hi) x = lo + (p - p_lo) / s1;  // p_hi > p_lo implies s1 > 0
    else x = hi + (p - p_hi) / s0;                // reached only when s0 > 0
    const long long j = ja + (x >= ra ? 0 : 1) + (p - seg_pos(x, K, ra, rb));
    return j * np + x;
}
#endif

#ifdef DFPT_ONE_SCENE
// A handle's waves (one scene, sample order pass-major from a first sample at a pass boundary).
// When the capacity is a whole number of passes every wave holds whole passes, and its slots run
// pixel-major: the wave's samples of one pixel are adjacent, so a warp's primary rays leave one or
// two pixels. wave_passes returns the passes of the current wave, or 0 when the slots stay in
// sample order. `rel` is a sample's place in the wave in sample order.
__device__ __forceinline__ unsigned wave_passes(const DevBatch& Q, long long np) {
    if (Q.capacity % np != 0) return 0u;
    const long long base = Q.wave_base[0];
    const long long end = base + Q.capacity < Q.wave_base[1] ? base + Q.capacity : Q.wave_base[1];
    return (unsigned)((end - base) / np);
}
__device__ __forceinline__ unsigned slot_of_rel(unsigned rel, unsigned np, unsigned passes) {
    if (passes == 0u) return rel;
    const unsigned j = rel / np;
    return (rel - j * np) * passes + j;
}
__device__ __forceinline__ unsigned rel_of_slot(unsigned slot, unsigned np, unsigned passes) {
    if (passes == 0u) return slot;
    const unsigned x = slot / passes;
    return (slot - x * passes) * np + x;
}
#endif

// Slot order of a plain pass. With P.pixel_tiles the pass's queue slots run over 8 x 4 pixel tiles
// (tiles in row-major order, a tile's 32 pixels row by row), so a warp's primary rays leave a
// compact block of pixels instead of a 32-pixel strip; the bounces' queues keep that locality. A
// path keeps its slot; its pixel (RNG key, selection buffer, hit records, film) follows from it.
// Only for widths that are multiples of 8 and heights that are multiples of 4.
__device__ __forceinline__ int pixel_of_slot(const DevParams& P, int i) {
    if (!P.pixel_tiles) return i;
    const int t = i >> 5, l = i & 31, tw = P.width >> 3;
    const int ty = t / tw, tx = t - ty * tw;
    return ((ty << 2) + (l >> 3)) * P.width + (tx << 3) + (l & 7);
}
__device__ __forceinline__ int slot_of_pixel(const DevParams& P, int p) {
    if (!P.pixel_tiles) return p;
    const int y = p / P.width, x = p - y * P.width;
    return (((y >> 2) * (P.width >> 3) + (x >> 3)) << 5) | ((y & 3) << 3) | (x & 7);
}

__device__ __forceinline__ uint32_t camera_draws(const DevScene& S, const DevParams& P) {
    const bool pt = P.renderer_type == DFPT_RENDERER_PATH_TRACER ||
                    (P.renderer_type < DFPT_RENDERER_AMBIENT_OCCLUSION || P.renderer_type > DFPT_RENDERER_SURFACE_NORMALS);
    return (pt ? 2u : 0u) + (__ldg(S.camera) > 0.00001f ? 2u : 0u);
}

// A pixel the fisheye lens rejects has no primary ray: its hit record says "no hit".
__device__ __forceinline__ void record_rejected(const DevParams& P, DevPass& B, int pixel) {
    if (!P.record_hits) return;
    B.hit_prim_offset[pixel] = -1;
    B.hit_shape_type[pixel] = -1;
    B.hit_shape_offset[pixel] = -1;
    B.hit_distance[pixel] = 0.0f;
    B.hit_normal[3 * pixel] = 0.0f; B.hit_normal[3 * pixel + 1] = 0.0f; B.hit_normal[3 * pixel + 2] = 0.0f;
}

template <bool BATCH>
__global__ void __launch_bounds__(256) k_camera(DevScene S0, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q) {
    const int n = BATCH ? Q.capacity : B.n_pixels;
    const uint32_t pass = BATCH ? 0u : (uint32_t)*B.pass_index;
    long long base = 0, end = 0, pass0 = 0;
    if constexpr (BATCH) {
        base = Q.wave_base[0];
        end = Q.wave_base[1];
        pass0 = Q.wave_base[2];
    }
#ifdef DFPT_ONE_SCENE
    const unsigned wave_p = wave_passes(Q, (long long)Q.params[0].width * Q.params[0].height);
#endif
    // A thin lens keeps every pixel, so with one scene the queue is the slots in order (no atomics):
    // the valid slots are a prefix.
    const bool dense = (!BATCH || Q.n_scenes == 1) && __ldg(scene_of<BATCH>(S0, Q, 0).camera + 18) != 2.0f;
    if (dense && blockIdx.x == 0 && threadIdx.x == 0) {
        long long valid = n;
        if constexpr (BATCH) valid = end - base < (long long)n ? (end - base > 0 ? end - base : 0) : (long long)n;
        B.counts[0] = (int)valid;
    }
    GRID_STRIDE_UNIFORM(i, n) {
        bool valid = i < n;
        int sid = 0, pixel = i;
        uint32_t sample = pass;
        if constexpr (BATCH) {
            if (valid) {
#ifdef DFPT_ONE_SCENE
                // Slots past the wave's samples stay invalid (rel_of_slot maps only those below).
                const unsigned np0 = (unsigned)((long long)Q.params[0].width * Q.params[0].height);
                const long long g = wave_p == 0u ? base + i
                                    : (unsigned)i < wave_p * np0 ? base + rel_of_slot((unsigned)i, np0, wave_p) : end;
#else
                const long long g = base + i;
#endif
                if (g >= end) {
                    valid = false;
                } else {
                    sid = batch_scene_of(Q, g);
                    const long long np = (long long)Q.params[sid].width * Q.params[sid].height;
#ifdef DFPT_ONE_SCENE
                    const long long local = g - Q.sample_begin[sid];
#else
                    // The slot's place in its scene's segment of the wave, pixel-major.
                    const long long b0 = Q.sample_begin[sid], b1 = Q.sample_begin[sid + 1];
                    const long long wend = base + Q.capacity < end ? base + Q.capacity : end;
                    const long long sa = (base > b0 ? base : b0) - b0, sb = (wend < b1 ? wend : b1) - b0;
                    const long long local = seg_local_of_pos(g - (b0 + sa), sa, sb, np);
#endif
                    long long j;
                    if (local < 0x7FFFFFFFll) {  // 32-bit division where it fits (np < 2^28)
                        const unsigned q = (unsigned)local / (unsigned)np;
                        j = q;
                        pixel = (int)((unsigned)local - q * (unsigned)np);
                    } else {
                        j = local / np;
                        pixel = (int)(local - j * np);
                    }
                    sample = (uint32_t)(j + pass0);
#ifdef DFPT_ONE_SCENE
                    // One scene: shading derives the key from the slot; the adjoint replay reads it.
                    if (Q.params[0].diff) Q.slot_key[i] = make_int4(sid, pixel, (int)sample, 0);
#else
                    Q.slot_key[i] = make_int4(sid, pixel, (int)sample, 0);
#endif
                }
            }
        }
        const DevScene& S = scene_of<BATCH>(S0, Q, sid);
        const DevParams& P = params_of<BATCH>(Pp, Q, sid);
        if constexpr (!BATCH) pixel = pixel_of_slot(P, i);
        float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 0, 0);
        bool live = false;
        if (valid) {
            const bool pt = P.renderer_type == DFPT_RENDERER_PATH_TRACER ||
                            (P.renderer_type < DFPT_RENDERER_AMBIENT_OCCLUSION || P.renderer_type > DFPT_RENDERER_SURFACE_NORMALS);
            Rng rng = make_rng(P, (uint32_t)pixel, sample, (!BATCH && P.rng_kind == DFPT_RNG_LCG) ? B.rng[i] : 0ull);
            live = primary_ray(S, P, pixel, pt, rng, o, d);
            B.pixel_flags[i] = live ? 0 : 1;
            if (!BATCH && !live) record_rejected(P, B, pixel);
            if (!lean_start<BATCH>(P)) {
                B.rng[i] = rng.state;
                B.throughput[PSI(i)] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
                B.radiance[PSI(i)] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            if (P.diff) B.vis[i] = 0;
            if (!BATCH && P.wireframes == 1) {
                B.primary_o[i] = o;
                B.primary_d[i] = d;
            }
        }
        const int slot = dense ? (live ? i : -1) : warp_push(B.counts + 0, live);
        if (slot >= 0) {
            o.w = __int_as_float(i);
            d.w = BATCH ? __int_as_float(sid) : 0.0f;
            B.q_o[0][slot] = o;
            B.q_d[0][slot] = d;
        }
    }
}

// Traversal kernels are instantiated per tuning configuration (walk variant, block size, resident
// blocks per SM); see TRACE_CONFIGS.
template <bool BATCH, bool ANY, int V, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_trace(DevScene S0, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q, int bounce, int which_queue) {
    const DevParams& P = *Pp;  // run-wide flags (statistics counting)
    const int n = B.counts[bounce];
    const float4* __restrict__ qo = B.q_o[which_queue];
    const float4* __restrict__ qd = B.q_d[which_queue];
    if constexpr (V == 3) {
        TraceStats st{0, 0};
        uint32_t segs = 0;
        trace_refill<ANY>(
            n, B.counts + DFPT_COUNTS_FETCH + bounce,
            [&](int, const float4& d) -> const DevScene& { return scene_of<BATCH>(S0, Q, BATCH ? __float_as_int(d.w) : 0); },
            [&](int i, float4& o, float4& d) { o = qo[i]; d = qd[i]; },
            [&](int i, const float4&, const float4&, const Hit& h) {
                B.q_hit[i] = make_int4(__float_as_int(h.t), h.prim, h.shape_type, h.shape_offset);
                ++segs;
            },
            st);
        warp_add_stats(P, B.stats, ANY ? 1 : 0, segs, st.nodes, st.tris);
    } else {
        WARP_DYNAMIC(i, n, B.counts + DFPT_COUNTS_FETCH + bounce) {
            TraceStats st{0, 0};
            const bool valid = i < n;
            float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 1, 0);
            if (valid) {
                // Streaming accesses: each ray and hit is touched once here, and the BVH records
                // keep the L1.
                o = __ldcs(qo + i);
                d = __ldcs(qd + i);
            }
            const DevScene& S = scene_of<BATCH>(S0, Q, BATCH ? __float_as_int(d.w) : 0);
            const Hit h = trace_v<ANY, V>(S, valid, o.x, o.y, o.z, d.x, d.y, d.z, st);
            if (valid) __stcs(B.q_hit + i, make_int4(__float_as_int(h.t), h.prim, h.shape_type, h.shape_offset));
            warp_add_stats(P, B.stats, ANY ? 1 : 0, valid ? 1u : 0u, st.nodes, st.tris);
        }
    }
}

// A primitive's extension record (scenes that carry them): its Phong exponent, and a scale on its
// emission texture's 8-bit colour (HDR emitters).
__device__ __forceinline__ void primitive_extension(const DevScene& S, int prim, float& er, float& eg, float& eb, float& exponent) {
    const float4 x = __ldg(S.prim_ext + prim);
    exponent = x.x;
    er *= x.y; eg *= x.z; eb *= x.w;
}

// Differentiable mode: the primitive's parameters applied to its texture colors.
__device__ __forceinline__ void diff_surface(const DevParams& P, int prim, float& ar, float& ag, float& ab, float& er, float& eg,
                                             float& eb, float& exponent) {
    const float4 a = P.diff_albedo[prim], e = P.diff_emission[prim];
    ar *= a.x; ag *= a.y; ab *= a.z;
    er += e.x; eg += e.y; eb += e.z;
    exponent = P.diff_exponent[prim];
}

// Material sampling at one vertex (GRK:3323-3686): the next ray, and the throughput T multiplied
// by the vertex's factors. Reports whether the albedo was one of them and, for a Phong lobe, the
// sampled cosine (the path-replay adjoint differentiates through both).
struct Scatter {
    float4 o, d;       // next ray origin / direction (w unset)
    bool albedo;       // T was multiplied by the albedo
    float phong_ct;    // Phong: cosine to the lobe axis drawn from (n + 1) cos^n; else 0
};

__device__ __forceinline__ Scatter scatter(const Surf& s, int material, float wx, float wy, float wz, float4 o, float4 d, float dp2,
                                           float ar, float ag, float ab, float exponent, Rng& rng, float4& T) {
    Scatter out;
    out.albedo = false;
    out.phong_ct = 0.0f;
    float ox = o.x, oy = o.y, oz = o.z, dx = d.x, dy = d.y, dz = d.z;
    const float rx = dx - s.nx * dp2, ry = dy - s.ny * dp2, rz = dz - s.nz * dp2;
    if (material == DFPT_MATERIAL_CLEAR_COAT) {
        const float a = 1.5f - 1.0f, b = 1.5f + 1.0f, c = 1.0f / 1.5f;
        const float e = (a * a) / (b * b);
        const float d0 = wx * dx + wy * dy + wz * dz;
        const float tir = 1.0f - c * c * (1.0f - d0 * d0);
        if (tir < 0.0f) {
            ox = s.px + wx * 0.02f; oy = s.py + wy * 0.02f; oz = s.pz + wz * 0.02f;
            dx = rx; dy = ry; dz = rz;
        } else {
            const float a2 = 1.0f - (-d0);
            const float refl = e + (1.0f - e) * a2 * a2 * a2 * a2 * a2;
            const float trans = 1.0f - refl;
            const float pr = 0.25f + 0.5f * refl;
            const float rp = refl / pr, tp = trans / (1.0f - pr);
            const bool is_refl = rng.next() < pr;
            const float m = is_refl ? rp : tp;
            T.x *= m; T.y *= m; T.z *= m;
            if (is_refl) {
                ox = s.px + wx * 0.02f; oy = s.py + wy * 0.02f; oz = s.pz + wz * 0.02f;
                dx = rx; dy = ry; dz = rz;
            } else {
                const float u = rng.next(), v = rng.next();
                cosine_dir(wx, wy, wz, u, v, dx, dy, dz);
                ox = s.px + wx * 0.01f; oy = s.py + wy * 0.01f; oz = s.pz + wz * 0.01f;
                T.x *= ar; T.y *= ag; T.z *= ab;
                out.albedo = true;
            }
        }
    } else if (material == DFPT_MATERIAL_LAMBERTIAN) {
        const float u = rng.next(), v = rng.next();
        cosine_dir(wx, wy, wz, u, v, dx, dy, dz);
        ox = s.px + wx * 0.01f; oy = s.py + wy * 0.01f; oz = s.pz + wz * 0.01f;
        T.x *= ar; T.y *= ag; T.z *= ab;
        out.albedo = true;
    } else if (material == DFPT_MATERIAL_PHONG) {
        const float u = rng.next(), v = rng.next();
        const float phi = TWO_PI * u;
        const float ct = pow_j(1.0f - v, 1.0f / (exponent + 1.0f));
        out.phong_ct = ct;
        const float st = sqrtf(jmax(0.0f, 1.0f - ct * ct));
        const float x = cos_j(phi) * st, y = sin_j(phi) * st, z = ct;
        const float rwr = rsqrt_j(rx * rx + ry * ry + rz * rz);
        const float rnx = rx * rwr, rny = ry * rwr, rnz = rz * rwr;
        const bool isY = fabsf(rnx) > 0.1f;
        const float ux = (isY ? 1.0f : 0.0f) * rnz;
        const float uy = -((isY ? 0.0f : 1.0f) * rnz);
        const float uz = (isY ? 0.0f : 1.0f) * rny - (isY ? 1.0f : 0.0f) * rnx;
        const float ur = rsqrt_j(ux * ux + uy * uy + uz * uz);
        const float unx = ux * ur, uny = uy * ur, unz = uz * ur;
        const float vnx = rny * unz - rnz * uny, vny = rnz * unx - rnx * unz, vnz = rnx * uny - rny * unx;
        // The reference mixes the unnormalised reflection vector in here (GRK:3555-3557).
        const float px = unx * x + vnx * y + rx * z;
        const float py = uny * x + vny * y + ry * z;
        const float pz = unz * x + vnz * y + rz * z;
        const float pr = rsqrt_j(px * px + py * py + pz * pz);
        ox = s.px + rnx * 0.01f; oy = s.py + rny * 0.01f; oz = s.pz + rnz * 0.01f;
        dx = px * pr; dy = py * pr; dz = pz * pr;
        T.x *= ar; T.y *= ag; T.z *= ab;
        out.albedo = true;
    } else if (material == DFPT_MATERIAL_GLASS) {
        const float a = 1.5f - 1.0f, b = 1.5f + 1.0f, c = 1.0f / 1.5f, dd = 1.5f / 1.0f;
        const float e = (a * a) / (b * b);
        const bool going_in = s.nx * wx + s.ny * wy + s.nz * wz > 0.0f;
        const float nnt = going_in ? c : dd;
        const float dw = wx * dx + wy * dy + wz * dz;
        const float tir = 1.0f - nnt * nnt * (1.0f - dw * dw);
        if (tir < 0.0f) {
            ox = s.px + wx * 0.01f; oy = s.py + wy * 0.01f; oz = s.pz + wz * 0.01f;
            dx = rx; dy = ry; dz = rz;
        } else {
            const float st = sqrtf(tir);
            const float scl = going_in ? dw * nnt + st : -(dw * nnt + st);
            const float t0x = dx * nnt - s.nx * scl, t0y = dy * nnt - s.ny * scl, t0z = dz * nnt - s.nz * scl;
            const float tr = rsqrt_j(t0x * t0x + t0y * t0y + t0z * t0z);
            const float tdx = t0x * tr, tdy = t0y * tr, tdz = t0z * tr;
            const float a1 = going_in ? -dw : tdx * s.nx + tdy * s.ny + tdz * s.nz;
            const float a2 = 1.0f - a1;
            const float refl = e + (1.0f - e) * a2 * a2 * a2 * a2 * a2;
            const float trans = 1.0f - refl;
            const float pr = 0.25f + 0.5f * refl;
            const float rp = refl / pr, tp = trans / (1.0f - pr);
            const bool is_refl = rng.next() < pr;
            const float m = is_refl ? rp : tp;
            T.x *= m; T.y *= m; T.z *= m;
            const float eps = is_refl ? 0.01f : 0.000001f;
            ox = s.px + wx * eps; oy = s.py + wy * eps; oz = s.pz + wz * eps;
            dx = is_refl ? rx : tdx; dy = is_refl ? ry : tdy; dz = is_refl ? rz : tdz;
        }
    } else if (material == DFPT_MATERIAL_REFLECTION) {
        ox = s.px + s.nx * 0.000001f; oy = s.py + s.ny * 0.000001f; oz = s.pz + s.nz * 0.000001f;
        dx = rx; dy = ry; dz = rz;
        T.x *= ar; T.y *= ag; T.z *= ab;
        out.albedo = true;
    }
    out.o = make_float4(ox, oy, oz, 0.0f);
    out.d = make_float4(dx, dy, dz, 0.0f);
    return out;
}

// Ray binning between bounces: the bin of a ray is its direction bin (cube-map or octant) and its
// origin's cell in a grid over its scene's bounds (axis bits interleaved), under 3 bits of its scene's
// place in the wave when the wave holds several (consecutive) scenes; shadow rays, all headed for
// the sun, are binned by origin cell alone. Rays of a bin start near each other and head the same
// way, so a warp of them walks much the same nodes. Only the processing order changes: every ray
// keeps its path id and its own result. Keys stay below DFPT_SORT_BINS.
__device__ __forceinline__ int wave_first_scene(const DevBatch& Q) { return (int)Q.wave_tab[0]; }
__device__ __forceinline__ int cell_bits(const DevScene& S, float4 o, int bits);
// Cube-map direction bin: the major axis and its sign, the two minor components over the face in
// N steps each (6 N^2 values).
template <int N>
__device__ __forceinline__ int cube_dir_bin(float4 d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    const int major = ax >= ay && ax >= az ? 0 : ay >= az ? 1 : 2;
    const float m = major == 0 ? d.x : major == 1 ? d.y : d.z;
    const float u = major == 0 ? d.y : d.x, v = major == 2 ? d.y : d.z;
    const float r = (0.5f * N) / fmaxf(fabsf(m), 1e-30f);
    const int iu = min(N - 1, max(0, (int)(u * r + 0.5f * N))), iv = min(N - 1, max(0, (int)(v * r + 0.5f * N)));
    return ((major * 2 + (m < 0.0f ? 1 : 0)) * N + iu) * N + iv;
}
__device__ __forceinline__ int ray_bin_in_wave(const DevBatch& Q, int first, float4 o, float4 d) {
    const int sid = __float_as_int(d.w);
    if (Q.n_scenes == 1) {
#if DFPT_RAY_DIR_RES
        // One scene in the wave: a cube-map direction bin over the origin grid.
        return (cube_dir_bin<DFPT_RAY_DIR_RES>(d) << DFPT_RAY_CELL_BITS) | cell_bits(Q.scenes[sid], o, DFPT_RAY_CELL_BITS);
#else
        // One scene in the wave: no scene bits; the octant over the origin grid.
        const int oct = (d.x < 0.0f ? 1 : 0) | (d.y < 0.0f ? 2 : 0) | (d.z < 0.0f ? 4 : 0);
        return (oct << DFPT_RAY_CELL_BITS) | cell_bits(Q.scenes[sid], o, DFPT_RAY_CELL_BITS);
#endif
    }
#if DFPT_BATCH_DIR_BINS
    // Several scenes: 3 bits of the scene's place in the wave over a 6 x 4 x 4 direction bin
    // (7 bits) and a 16^3 grid.
    return (((sid - first) & 7) << 19) | (cube_dir_bin<4>(d) << 12) | cell_bits(Q.scenes[sid], o, 12);
#else
    // Several scenes: 3 bits of the scene's place in the wave over the octant and a 32^3 grid.
    const int oct = (d.x < 0.0f ? 1 : 0) | (d.y < 0.0f ? 2 : 0) | (d.z < 0.0f ? 4 : 0);
    return (((sid - first) & 7) << 18) | (oct << 15) | cell_bits(Q.scenes[sid], o, 15);
#endif
}

// A plain pass's bounce ray: a 6 x 4 x 4 cube-map direction bin over an origin grid of `bits`
// bits (a multiple of 3, at most 15).
__device__ __forceinline__ int plain_ray_bin(const DevScene& S, float4 o, float4 d, int bits) {
    return (cube_dir_bin<4>(d) << bits) | cell_bits(S, o, bits);
}

// Bin counts with one atomic per distinct bin of a warp.
__device__ __forceinline__ void bin_count(int* bins, int key) {
    const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
    if (key >= 0 && (int)(threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(bins + key, __popc(same));
}


// Origin cell over the scene bounds with `bits` bits in all (at most 24: bits / 3 per axis, the
// remainder to the axes of largest extent), axis bits interleaved from the least significant up.
__device__ __forceinline__ int cell_bits(const DevScene& S, float4 o, int bits) {
    const float lo[3] = {S.bounds_lo.x, S.bounds_lo.y, S.bounds_lo.z};
    const float hi[3] = {S.bounds_hi.x, S.bounds_hi.y, S.bounds_hi.z};
    const float p[3] = {o.x, o.y, o.z};
    const float ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    int nb[3] = {bits / 3, bits / 3, bits / 3};
    int extra = bits - 3 * (bits / 3);
    // The smallest axis gets no extra bit; with 2 extra, the other two get one each.
    const int small = ext[0] <= ext[1] && ext[0] <= ext[2] ? 0 : ext[1] <= ext[2] ? 1 : 2;
    for (int a = 0; a < 3 && extra > 0; ++a)
        if (a != small || extra == 3) { ++nb[a]; --extra; }
    int c[3];
    for (int a = 0; a < 3; ++a) {
        const float n = (float)(1 << nb[a]);
        const float u = (p[a] - lo[a]) * (n * __frcp_rn(ext[a]));  // any monotone mapping bins alike
        c[a] = u >= 0.0f ? (u < n - 1.0f ? (int)u : (1 << nb[a]) - 1) : 0;
    }
    int cell = 0, k = 0;
    for (int b = 0; b < 8; ++b)
        for (int a = 0; a < 3; ++a)
            if (b < nb[a]) cell |= ((c[a] >> b) & 1) << k++;
    return cell;
}

__device__ __forceinline__ int shadow_bin_in_wave(const DevBatch& Q, int first, float4 o, float4 d) {
    const int sid = __float_as_int(d.w);
    // One scene in the wave: the origin grid alone.
    if (Q.n_scenes == 1) return cell_bits(Q.scenes[sid], o, DFPT_SHADOW_CELL_BITS);
    // Several scenes: 3 bits of the scene's place in the wave over a 64^3 grid.
    return (((sid - first) & 7) << 18) | cell_bits(Q.scenes[sid], o, 18);
}

// One ray's shading at one bounce: miss -> sky; hit -> emission, sun sample (a shadow ray), Russian
// roulette, material sampling and the next ray (GRK:3185-3686). `o4`, `d4` are the ray (path id in
// o4.w), `hr` its closest hit; the path's state (throughput, radiance, RNG) is read and written in
// place. Returns the next ray in (emit_next, no, nd) and the sun shadow ray in (emit_shadow, so,
// sd, sc); the caller queues them.
template <bool BATCH>
__device__ __forceinline__ void shade_ray(const DevScene& S0, const DevParams* __restrict__ Pp, DevPass& B, const DevBatch& Q, int bounce,
                                          uint32_t pass, const float4 o4, const float4 d4, const int4 hr, int& path, bool& emit_next,
                                          float4& no, float4& nd, bool& emit_shadow, float4& so, float4& sd, float4& sc) {
    path = __float_as_int(o4.w);
    const int sid = BATCH ? __float_as_int(d4.w) : 0;
    const float sid_bits = BATCH ? d4.w : 0.0f;
    const DevScene& S = scene_of<BATCH>(S0, Q, sid);
    const DevParams& P = params_of<BATCH>(Pp, Q, sid);
    uint32_t rng_pixel = (uint32_t)(BATCH ? path : pixel_of_slot(P, path)), rng_pass = pass;
    if constexpr (BATCH) {
#ifdef DFPT_ONE_SCENE
        // One scene: the slot's pixel and pass follow from its index as k_camera derived
        // them (slot i of the wave is sample base + i), without the random slot-key load.
        const long long np = (long long)P.width * P.height;
        const long long local = Q.wave_base[0] + rel_of_slot((unsigned)path, (unsigned)np, wave_passes(Q, np)) - Q.sample_begin[0];
        if (local < 0x7FFFFFFFll) {
            const unsigned q = (unsigned)local / (unsigned)np;
            rng_pixel = (unsigned)local - q * (unsigned)np;
            rng_pass = (uint32_t)(q + Q.wave_base[2]);
        } else {
            const long long j = local / np;
            rng_pixel = (uint32_t)(local - j * np);
            rng_pass = (uint32_t)(j + Q.wave_base[2]);
        }
#else
        const int4 key = Q.slot_key[path];
        rng_pixel = (uint32_t)key.y;
        rng_pass = (uint32_t)key.z;
#endif
    }
    Hit h;
    h.t = __int_as_float(hr.x);
    h.prim = hr.y;
    h.shape_type = hr.z;
    h.shape_offset = hr.w;
    const bool fresh = bounce == 0 && lean_start<BATCH>(P);
    float4 T = fresh ? make_float4(1.0f, 1.0f, 1.0f, 0.0f) : B.throughput[PSI(path)];
    float4 L = fresh ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : B.radiance[PSI(path)];
    if (!BATCH && bounce == 0) B.primitive_offsets[rng_pixel] = h.prim >= 0 ? h.prim * 3 : -1;
    // A handle's waves of passes: the selection buffer holds the first hits of the call's
    // last pass (wave record entry 4; batches of scenes have no selection buffer).
    if (BATCH && bounce == 0 && B.primitive_offsets != nullptr && (long long)rng_pass == Q.wave_base[4])
        B.primitive_offsets[rng_pixel] = h.prim >= 0 ? h.prim * 3 : -1;
    if (h.t == INF || h.prim == -1) {
        const float3 sky = sky_color(P, d4.x, d4.y, d4.z);
        L.x += T.x * sky.x * INV_PI;
        L.y += T.y * sky.y * INV_PI;
        L.z += T.z * sky.z * INV_PI;
        B.radiance[PSI(path)] = L;
        if (!BATCH && bounce == 0 && P.record_hits) {
            B.hit_prim_offset[rng_pixel] = -1; B.hit_shape_type[rng_pixel] = -1; B.hit_shape_offset[rng_pixel] = -1;
            B.hit_distance[rng_pixel] = INF;
        }
    } else {
        Rng rng = make_rng(P, rng_pixel, rng_pass, fresh ? (uint64_t)camera_draws(S, P) : B.rng[path]);
        const Surf s = surface(S, P, o4.x, o4.y, o4.z, d4.x, d4.y, d4.z, h);
        if (!BATCH && bounce == 0 && P.record_hits) {
            const uint32_t px = rng_pixel;
            B.hit_prim_offset[px] = h.prim * 3; B.hit_shape_type[px] = h.shape_type; B.hit_shape_offset[px] = h.shape_offset;
            B.hit_distance[px] = h.t;
            B.hit_normal[3 * px] = s.nx; B.hit_normal[3 * px + 1] = s.ny; B.hit_normal[3 * px + 2] = s.nz;
        }
        const int so_off = __ldg(S.prim_info + h.prim).z;
        const float dp = s.nx * d4.x + s.ny * d4.y + s.nz * d4.z;
        const float dp2 = dp * 2.0f;
        const bool correct = dp < 0.0f;
        const float wx = correct ? s.nx : -s.nx, wy = correct ? s.ny : -s.ny, wz = correct ? s.nz : -s.nz;
        const int albedo = texture_color(S, f2i(__ldg(S.surfaces + so_off + 1)), s);
        const int emission = texture_color(S, f2i(__ldg(S.surfaces + so_off + 2)), s);
        float ar = cr(albedo), ag = cg(albedo), ab = cb(albedo);
        float er = cr(emission), eg = cg(emission), eb = cb(emission);
        const int material = f2i(__ldg(S.surfaces + so_off + 0));
        float exponent = 50.0f;  // the reference's fixed Phong exponent (GRK:3524)
        if (S.prim_ext) primitive_extension(S, h.prim, er, eg, eb, exponent);
        if (P.diff) diff_surface(P, h.prim, ar, ag, ab, er, eg, eb, exponent);
        if ((material == DFPT_MATERIAL_CLEAR_COAT || material == DFPT_MATERIAL_LAMBERTIAN || material == DFPT_MATERIAL_PHONG) &&
            P.sun_active == 1) {
            const float u = rng.next(), v = rng.next();
            float lx, ly, lz, dot1;
            if (sun_sample(P, s.px, s.py, s.pz, wx, wy, wz, u, v, lx, ly, lz, dot1)) {
                emit_shadow = true;
                so = make_float4(s.px, s.py, s.pz, __int_as_float(path));
                sd = make_float4(lx, ly, lz, sid_bits);
                sc = make_float4(T.x * (ar * 1.0f * dot1 * INV_PI), T.y * (ag * 1.0f * dot1 * INV_PI), T.z * (ab * 1.0f * dot1 * INV_PI),
                                 __int_as_float(bounce));
            }
        }
        L.x += T.x * er;
        L.y += T.y * eg;
        L.z += T.z * eb;
        const int depth = bounce + 1;
        bool alive = true;
        if (depth >= P.depth_rr) {
            const float q = jmax(ar, jmax(ag, ab));
            const float r = rng.next();
            // The reference then tests the same ray for any hit; it just hit, so the
            // test always hits and adds no sky (GRK:3293-3311).
            if (r >= q) alive = false;
            else {
                const float qr = 1.0f / q;
                ar *= qr; ag *= qr; ab *= qr;
            }
        }
        if (alive) {
            const Scatter sct = scatter(s, material, wx, wy, wz, o4, d4, dp2, ar, ag, ab, exponent, rng, T);
            emit_next = true;
            no = make_float4(sct.o.x, sct.o.y, sct.o.z, __int_as_float(path));
            nd = make_float4(sct.d.x, sct.d.y, sct.d.z, sid_bits);
        }
        B.throughput[PSI(path)] = T;
        B.radiance[PSI(path)] = L;
        B.rng[path] = rng.state;
    }
}

// One bounce of shading: miss -> sky; hit -> emission, sun sample (a shadow ray), Russian
// roulette, material sampling and the next ray (GRK:3185-3686).
template <bool BATCH>
#ifndef DFPT_SHADE_MINB
#define DFPT_SHADE_MINB 3  // resident blocks of 256 per SM the shading kernel is compiled for
#endif
__global__ void __launch_bounds__(256, DFPT_SHADE_MINB) k_shade(DevScene S0, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q, int bounce) {
    const int n = B.counts[bounce];
    const int qi = B.sorted_queues ? 0 : (bounce & 1);
    const uint32_t pass = BATCH ? 0u : (uint32_t)*B.pass_index;
    GRID_STRIDE_UNIFORM(i, n) {
        bool emit_next = false, emit_shadow = false;
        float4 no = make_float4(0, 0, 0, 0), nd = make_float4(0, 0, 0, 0);
        float4 so = make_float4(0, 0, 0, 0), sd = make_float4(0, 0, 0, 0), sc = make_float4(0, 0, 0, 0);
        int path = 0;
        if (i < n) shade_ray<BATCH>(S0, Pp, B, Q, bounce, pass, B.q_o[qi][i], B.q_d[qi][i], B.q_hit[i], path, emit_next, no, nd,
                                    emit_shadow, so, sd, sc);
        const int slot = warp_push(B.counts + bounce + 1, emit_next);
        if (slot >= 0) {
            B.q_o[qi ^ 1][slot] = no;
            B.q_d[qi ^ 1][slot] = nd;
        }
        if constexpr (BATCH) {
            // Ray binning: the histograms of the next bounce's rays and of the shadow rays.
            if (B.sorted_queues) {
                const int first = wave_first_scene(Q);
                bin_count(B.sort_count, emit_next ? ray_bin_in_wave(Q, first, no, nd) : -1);
                if (B.sort_count_shadow) bin_count(B.sort_count_shadow, emit_shadow ? shadow_bin_in_wave(Q, first, so, sd) : -1);
            }
        } else {
            // Plain passes may bin the next bounce's rays (the record of one bounce carries
            // sort_count) and the deferred shadow rays (origin cells).
            if (B.sort_count) bin_count(B.sort_count, emit_next ? plain_ray_bin(S0, no, nd, B.sort_ray_bits) : -1);
            if (B.sort_count_shadow) bin_count(B.sort_count_shadow, emit_shadow ? cell_bits(S0, so, DFPT_SHADOW_CELL_BITS) : -1);
        }
        const int sslot = warp_push(B.counts + DFPT_COUNTS_SHADOW, emit_shadow);
        if (sslot >= 0) {
            B.s_o[sslot] = so;
            B.s_d[sslot] = sd;
            B.s_c[sslot] = sc;
        }
    }
}

// Sun visibility: any hit (GRK:2324-2340); unoccluded samples add their contribution. The shadow
// rays of every bounce of the pass wait in one queue and are traced in a single launch after the
// last bounce (their contributions only add to the path radiance).
template <bool BATCH, int V, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_shadow(DevScene S0, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q, int bounce) {
    const DevParams& P = *Pp;
    const int n = B.counts[DFPT_COUNTS_SHADOW];
    (void)bounce;
    // Unoccluded: the pending contribution joins the path radiance. A path has up to one shadow
    // ray per bounce in this queue, so several threads may add to the same path: atomics (the
    // sum's order, and so its last bit, may vary).
    auto unoccluded = [&](int i, const float4& o, const float4& c) {
        const int path = __float_as_int(o.w);
        float* L = reinterpret_cast<float*>(B.radiance + PSI(path));
        atomicAdd(L, c.x);
        atomicAdd(L + 1, c.y);
        atomicAdd(L + 2, c.z);
        if (P.diff) atomicOr(B.vis + path, 1 << __float_as_int(c.w));
    };
    if constexpr (V == 3) {
        TraceStats st{0, 0};
        uint32_t segs = 0;
        trace_refill<true>(
            n, B.counts + DFPT_COUNTS_FETCH + DFPT_MAX_DEPTH + 1,
            [&](int, const float4& d) -> const DevScene& { return scene_of<BATCH>(S0, Q, BATCH ? __float_as_int(d.w) : 0); },
            [&](int i, float4& o, float4& d) { o = B.s_o[i]; d = B.s_d[i]; },
            [&](int i, const float4& o, const float4&, const Hit& h) {
                ++segs;
                if (h.t >= INF - 0.0001f) unoccluded(i, o, B.s_c[i]);
            },
            st);
        warp_add_stats(P, B.stats, 1, segs, st.nodes, st.tris);
    } else {
        WARP_DYNAMIC(i, n, B.counts + DFPT_COUNTS_FETCH + DFPT_MAX_DEPTH + 1) {
            TraceStats st{0, 0};
            const bool valid = i < n;
            float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 1, 0);
            if (valid) {
                o = __ldcs(B.s_o + i);  // read once: streaming
                d = __ldcs(B.s_d + i);
            }
            const DevScene& S = scene_of<BATCH>(S0, Q, BATCH ? __float_as_int(d.w) : 0);
            const Hit h = trace_v<true, V>(S, valid, o.x, o.y, o.z, d.x, d.y, d.z, st);
            if (valid && h.t >= INF - 0.0001f) unoccluded(i, o, __ldcs(B.s_c + i));
            warp_add_stats(P, B.stats, 1, valid ? 1u : 0u, st.nodes, st.tris);
        }
    }
}

// After the last bounce: any-hit test of the continuation ray, sky if it escapes (GRK:3689-3701).
template <bool BATCH, int V, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_final(DevScene S0, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q, int bounce) {
    const DevParams& P0 = *Pp;  // run-wide flags (statistics counting)
    const int n = B.counts[bounce];
    const int qi = B.sorted_queues ? 0 : (bounce & 1);
    // The continuation escaped: sky, as at a miss.
    auto escaped = [&](const float4& o, const float4& d) {
        const int sid = BATCH ? __float_as_int(d.w) : 0;
        const DevParams& P = params_of<BATCH>(Pp, Q, sid);
        const int path = __float_as_int(o.w);
        const float4 T = B.throughput[PSI(path)];
        const float3 sky = sky_color(P, d.x, d.y, d.z);
        float4 L = B.radiance[PSI(path)];
        L.x += T.x * sky.x * INV_PI;
        L.y += T.y * sky.y * INV_PI;
        L.z += T.z * sky.z * INV_PI;
        B.radiance[PSI(path)] = L;
    };
    if constexpr (V == 3) {
        TraceStats st{0, 0};
        uint32_t segs = 0;
        trace_refill<true>(
            n, B.counts + DFPT_COUNTS_FETCH + bounce,
            [&](int, const float4& d) -> const DevScene& { return scene_of<BATCH>(S0, Q, BATCH ? __float_as_int(d.w) : 0); },
            [&](int i, float4& o, float4& d) { o = B.q_o[qi][i]; d = B.q_d[qi][i]; },
            [&](int, const float4& o, const float4& d, const Hit& h) {
                ++segs;
                if (!(h.t < INF)) escaped(o, d);
            },
            st);
        warp_add_stats(P0, B.stats, 1, segs, st.nodes, st.tris);
    } else {
        WARP_DYNAMIC(i, n, B.counts + DFPT_COUNTS_FETCH + bounce) {
            TraceStats st{0, 0};
            const bool valid = i < n;
            float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 1, 0);
            if (valid) {
                o = B.q_o[qi][i];
                d = B.q_d[qi][i];
            }
            const DevScene& S = scene_of<BATCH>(S0, Q, BATCH ? __float_as_int(d.w) : 0);
            const Hit h = trace_v<true, V>(S, valid, o.x, o.y, o.z, d.x, d.y, d.z, st);
            if (valid && !(h.t < INF)) escaped(o, d);
            warp_add_stats(P0, B.stats, 1, valid ? 1u : 0u, st.nodes, st.tris);
        }
    }
}

// The last bounces of a plain pass in one launch. Each lane takes a path whose ray waits for bounce
// b0 and carries it to its end - closest hit, shading, the next ray - through bounces b0 .. nb - 1
// and the any-hit test of the continuation after the last (k_final). Late bounces hold few rays,
// and a launch per bounce costs the slowest ray of every bounce; here the paths' remaining walks
// overlap. A lane whose path ends takes the next waiting path from the queue (warp-aggregated
// fetch), so lanes stay busy while paths of different lengths finish; lanes of a warp may stand at
// different bounces. Each path takes exactly the steps of the per-bounce kernels (same hits, same
// draws, same order of its radiance sums); sun shadow rays join the deferred queue as there. Every
// lane calls the traversals, the fetch and the queue append together (warp-uniform loop).
template <int V, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_tail(DevScene S, const DevParams* __restrict__ Pp, DevPass B, int b0, int nb) {
    const DevParams& P = *Pp;
    const int n = B.counts[b0];
    const int qi = b0 & 1;
    const uint32_t pass = (uint32_t)*B.pass_index;
    const DevBatch Q{};
    int* const fetch = B.counts + DFPT_COUNTS_FETCH + b0;
    const int lane = threadIdx.x & 31;
    bool have = false;      // the lane holds a path: its ray waits at bounce b (b == nb: the final any-hit)
    bool drained = false;   // warp-uniform: the queue has no more paths
    int b = nb;
    float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 1, 0);
    for (;;) {
        if (!drained) {
            const unsigned need = __ballot_sync(0xFFFFFFFFu, !have);
            if (need) {
                const int leader = __ffs(need) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(fetch, __popc(need));
                base = __shfl_sync(0xFFFFFFFFu, base, leader);
                if (base + __popc(need) >= n) drained = true;
                const int idx = base + __popc(need & ((1u << lane) - 1u));
                if (!have && idx < n) {
                    o = __ldcs(B.q_o[qi] + idx);
                    d = __ldcs(B.q_d[qi] + idx);
                    b = b0;
                    have = true;
                }
            }
        }
        if (!__any_sync(0xFFFFFFFFu, have)) break;
        // One closest-hit bounce for the lanes whose ray waits at a bounce below nb.
        const bool step = have && b < nb;
        {
            TraceStats st{0, 0};
            const Hit h = trace_v<false, V>(S, step, o.x, o.y, o.z, d.x, d.y, d.z, st);
            warp_add_stats(P, B.stats, 0, step ? 1u : 0u, st.nodes, st.tris);
            bool emit_next = false, emit_shadow = false;
            float4 no = make_float4(0, 0, 0, 0), nd = make_float4(0, 0, 0, 0);
            float4 so = make_float4(0, 0, 0, 0), sd = make_float4(0, 0, 0, 0), sc = make_float4(0, 0, 0, 0);
            int path = 0;
            if (step)
                shade_ray<false>(S, Pp, B, Q, b, pass, o, d, make_int4(__float_as_int(h.t), h.prim, h.shape_type, h.shape_offset), path,
                                 emit_next, no, nd, emit_shadow, so, sd, sc);
            if (B.sort_count_shadow) bin_count(B.sort_count_shadow, emit_shadow ? cell_bits(S, so, DFPT_SHADOW_CELL_BITS) : -1);
            const int sslot = warp_push(B.counts + DFPT_COUNTS_SHADOW, emit_shadow);
            if (sslot >= 0) {
                B.s_o[sslot] = so;
                B.s_d[sslot] = sd;
                B.s_c[sslot] = sc;
            }
            if (step) {
                if (emit_next) {
                    o = no;
                    d = nd;
                    ++b;
                } else {
                    have = false;
                }
            }
        }
        // The continuation after the last bounce: any hit, else the sky (GRK:3689-3701).
        const bool fin = have && b == nb;
        if (__any_sync(0xFFFFFFFFu, fin)) {
            TraceStats st{0, 0};
            const Hit h = trace_v<true, V>(S, fin, o.x, o.y, o.z, d.x, d.y, d.z, st);
            warp_add_stats(P, B.stats, 1, fin ? 1u : 0u, st.nodes, st.tris);
            if (fin) {
                if (!(h.t < INF)) {
                    const int path = __float_as_int(o.w);
                    const float4 T = B.throughput[PSI(path)];
                    const float3 sky = sky_color(P, d.x, d.y, d.z);
                    float4 L = B.radiance[PSI(path)];
                    L.x += T.x * sky.x * INV_PI;
                    L.y += T.y * sky.y * INV_PI;
                    L.z += T.z * sky.z * INV_PI;
                    B.radiance[PSI(path)] = L;
                }
                have = false;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// The per-pixel modes: ray caster, ambient occlusion, surface normals, ray tracer, ray marcher.

// doShaderPhongReflectionModel0 (GRK:1962-2039), with the reference's closest-hit shadow test.
__device__ int phong0(const DevScene& S, const DevParams& P, bool test, float px, float py, float pz, float nx, float ny, float nz,
                      float vx, float vy, float vz, float ar, float ag, float ab, TraceStats& st) {
    float r = 0.0f, g = 0.0f, b = 0.0f;
    r += ar * 0.2f * 1.0f; g += ag * 0.2f * 1.0f; b += ab * 0.2f * 1.0f;
    const float lx = P.sun_origin[0] - px, ly = P.sun_origin[1] - py, lz = P.sun_origin[2] - pz;
    const float l2 = lx * lx + ly * ly + lz * lz;
    const float ll = sqrtf(l2);
    const float lr = 1.0f / ll;
    const float lnx = lx * lr, lny = ly * lr, lnz = lz * lr;
    float t = INF;
    if (test) t = trace_s(S, px, py, pz, lnx, lny, lnz, st).t;
    if (t >= INF || t > l2) {
        const float ldn = lnx * nx + lny * ny + lnz * nz;
        r += ar * 0.5f * jmax(ldn, 0.0f) * 1.0f;
        g += ag * 0.5f * jmax(ldn, 0.0f) * 1.0f;
        b += ab * 0.5f * jmax(ldn, 0.0f) * 1.0f;
        if (ldn > 0.0f) {
            const float rx = 2.0f * ldn * nx - lnx, ry = 2.0f * ldn * ny - lny, rz = 2.0f * ldn * nz - lnz;
            const float rr = rsqrt_j(rx * rx + ry * ry + rz * rz);
            const float rdv = rx * rr * vx + ry * rr * vy + rz * rr * vz;
            const float sh = pow_j(jmax(rdv, 0.0f), 250.0f);
            r += 0.5f * sh * 1.0f; g += 0.5f * sh * 1.0f; b += 0.5f * sh * 1.0f;
        }
    }
    r = saturate_j(r, 0.0f, 1.0f); g = saturate_j(g, 0.0f, 1.0f); b = saturate_j(b, 0.0f, 1.0f);
    return ((f2i(r * 255.0f + 0.5f) & 0xFF) << 16) | ((f2i(g * 255.0f + 0.5f) & 0xFF) << 8) | (f2i(b * 255.0f + 0.5f) & 0xFF);
}

__device__ __forceinline__ void record_primary(const DevParams& P, DevPass& B, int pixel, const Hit& h, const Surf* s) {
    if (!P.record_hits) return;
    B.hit_prim_offset[pixel] = h.prim >= 0 ? h.prim * 3 : -1;
    B.hit_shape_type[pixel] = h.prim >= 0 ? h.shape_type : -1;
    B.hit_shape_offset[pixel] = h.prim >= 0 ? h.shape_offset : -1;
    B.hit_distance[pixel] = h.t;
    if (s) {
        B.hit_normal[3 * pixel] = s->nx; B.hit_normal[3 * pixel + 1] = s->ny; B.hit_normal[3 * pixel + 2] = s->nz;
    }
}

__device__ float height_rm(const DevParams& P, float x, float z) {
    return fractal2(P.g_amplitude, P.g_frequency, P.g_gain, P.g_lacunarity, P.g_octaves, x, z);
}

__global__ void __launch_bounds__(128) k_simple(DevScene S, const DevParams* __restrict__ Pp, DevPass B) {
    const DevParams& P = *Pp;
    const int n = B.n_pixels;
    const uint32_t pass = (uint32_t)*B.pass_index;
    const int mode = P.renderer_type;
    GRID_STRIDE_UNIFORM(i, n) {
        TraceStats st{0, 0};
        uint32_t segs = 0;
        if (i < n) {
            Rng rng = make_rng(P, (uint32_t)i, pass, P.rng_kind == DFPT_RNG_LCG ? B.rng[i] : 0ull);
            float4 o4, d4;
            const bool live = primary_ray(S, P, i, false, rng, o4, d4);
            B.pixel_flags[i] = live ? 0 : 1;
            if (!live) record_rejected(P, B, i);
            if (P.wireframes == 1) { B.primary_o[i] = o4; B.primary_d[i] = d4; }
            float cr_ = 0.0f, cg_ = 0.0f, cb_ = 0.0f;
            if (live) {
                float ox = o4.x, oy = o4.y, oz = o4.z, dx = d4.x, dy = d4.y, dz = d4.z;
                if (mode == DFPT_RENDERER_RAY_MARCHER) {
                    // doRenderWithRayMarcher (GRK:3802-3864)
                    oy = height_rm(P, ox, oz) + 0.1f;
                    const float max_t = jmax(oy, 1.0f) * 20.0f;
                    const float3 sky = sky_color(P, dx, dy, dz);
                    cr_ = sky.x; cg_ = sky.y; cb_ = sky.z;
                    float del_t = 0.01f;
                    for (float t = 0.001f; t < max_t; t += del_t) {
                        const float px = ox + dx * t, py = oy + dy * t, pz = oz + dz * t;
                        const float hh = height_rm(P, px, pz);
                        if (py < hh) {
                            const float nx = height_rm(P, px - EPSILON_AK, pz) - height_rm(P, px + EPSILON_AK, pz);
                            const float ny = 2.0f * EPSILON_AK;
                            const float nz = height_rm(P, px, pz - EPSILON_AK) - height_rm(P, px, pz + EPSILON_AK);
                            const float nr = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
                            const float noise = fbm3(8.0f, 0.5f, 0.0f, 1.0f, 16, px, py, pz);
                            const float al = saturate_j(noise * 1.0f + 0.1f, 0.0f, 1.0f);
                            const int c = phong0(S, P, false, px, py, pz, nx * nr, ny * nr, nz * nr, -dx, -dy, -dz, al, al, al, st);
                            cr_ = cr(c); cg_ = cg(c); cb_ = cb(c);
                            t = max_t;
                        }
                        del_t = 0.01f * t;
                    }
                } else {
                    const int depth_max = mode == DFPT_RENDERER_RAY_TRACER ? 5 : 1;
                    for (int depth = 0; depth < depth_max; ++depth) {
                        const Hit h = trace_s(S, ox, oy, oz, dx, dy, dz, st);
                        segs++;
                        if (depth == 0) B.primitive_offsets[i] = h.prim >= 0 ? h.prim * 3 : -1;
                        if (h.t == INF || h.prim == -1) {
                            if (depth == 0) record_primary(P, B, i, h, nullptr);
                            if (mode != DFPT_RENDERER_AMBIENT_OCCLUSION) {
                                const float3 sky = sky_color(P, dx, dy, dz);
                                cr_ += sky.x; cg_ += sky.y; cb_ += sky.z;
                            }
                            break;
                        }
                        const Surf s = surface(S, P, ox, oy, oz, dx, dy, dz, h);
                        if (depth == 0) record_primary(P, B, i, h, &s);
                        if (mode == DFPT_RENDERER_SURFACE_NORMALS) {
                            cr_ = (s.nx + 1.0f) * 0.5f; cg_ = (s.ny + 1.0f) * 0.5f; cb_ = (s.nz + 1.0f) * 0.5f;
                            break;
                        }
                        const float dp = s.nx * dx + s.ny * dy + s.nz * dz;
                        const bool correct = dp < 0.0f;
                        const float wx = correct ? s.nx : -s.nx, wy = correct ? s.ny : -s.ny, wz = correct ? s.nz : -s.nz;
                        if (mode == DFPT_RENDERER_AMBIENT_OCCLUSION) {
                            // doRenderWithAmbientOcclusion (GRK:3029-3149)
                            const float w0r = rsqrt_j(wx * wx + wy * wy + wz * wz);
                            const float w1x = wx * w0r, w1y = wy * w0r, w1z = wz * w0r;
                            const bool isY = fabsf(w1x) > 0.1f;
                            const float u0x = isY ? 0.0f : 1.0f, u0y = isY ? 1.0f : 0.0f;
                            const float u1x = u0y * w1z, u1y = -(u0x * w1z), u1z = u0x * w1y - u0y * w1x;
                            const float ur = rsqrt_j(u1x * u1x + u1y * u1y + u1z * u1z);
                            const float u2x = u1x * ur, u2y = u1y * ur, u2z = u1z * ur;
                            const float v0x = w1y * u2z - w1z * u2y, v0y = w1z * u2x - w1x * u2z, v0z = w1x * u2y - w1y * u2x;
                            const float xi = rng.next(), xj = rng.next();
                            const float phi = TWO_PI * xi;
                            const float cp = cos_j(phi), sp = sin_j(phi), sth = sqrtf(xj), cth = sqrtf(1.0f - xj);
                            const float e0x = cp * sth, e0y = sp * sth, e0z = cth;
                            const float e1x = e0x * u2x + e0y * v0x + e0z * w1x;
                            const float e1y = e0x * u2y + e0y * v0y + e0z * w1y;
                            const float e1z = e0x * u2z + e0y * v0z + e0z * w1z;
                            const float er = rsqrt_j(e1x * e1x + e1y * e1y + e1z * e1z);
                            const float aox = s.px + w1x * 0.01f, aoy = s.py + w1y * 0.01f, aoz = s.pz + w1z * 0.01f;
                            const float t = trace_s(S, aox, aoy, aoz, e1x * er, e1y * er, e1z * er, st).t;
                            segs++;
                            const bool hit = t < P.ao_max_distance;
                            const float v = hit ? 1.0f : 0.0f;  // bright 1, dark 0
                            cr_ += (1.0f - v) * 1.0f + v * 0.0f;
                            cg_ += (1.0f - v) * 1.0f + v * 0.0f;
                            cb_ += (1.0f - v) * 1.0f + v * 0.0f;
                            break;
                        }
                        const int so_off = __ldg(S.prim_info + h.prim).z;
                        const int albedo = texture_color(S, f2i(__ldg(S.surfaces + so_off + 1)), s);
                        float ar, ag, ab;
                        if (mode == DFPT_RENDERER_RAY_TRACER) {
                            ar = ((albedo >> 16) & 0xFF) / 255.0f; ag = ((albedo >> 8) & 0xFF) / 255.0f; ab = (albedo & 0xFF) / 255.0f;
                        } else {
                            ar = cr(albedo); ag = cg(albedo); ab = cb(albedo);
                        }
                        const int c = phong0(S, P, true, s.px, s.py, s.pz, wx, wy, wz, -dx, -dy, -dz, ar, ag, ab, st);
                        segs++;
                        if (mode == DFPT_RENDERER_RAY_CASTER) {
                            cr_ = cr(c); cg_ = cg(c); cb_ = cb(c);
                            break;
                        }
                        // Ray tracer (GRK:3866-3996)
                        cr_ += cr(c); cg_ += cg(c); cb_ += cb(c);
                        const int material = f2i(__ldg(S.surfaces + so_off));
                        if (material != DFPT_MATERIAL_REFLECTION) break;
                        const float dp2 = dp * 2.0f;
                        ox = s.px + s.nx * 0.000001f; oy = s.py + s.ny * 0.000001f; oz = s.pz + s.nz * 0.000001f;
                        dx = dx - s.nx * dp2; dy = dy - s.ny * dp2; dz = dz - s.nz * dp2;
                    }
                }
            }
            B.radiance[PSI(i)] = make_float4(cr_, cg_, cb_, 0.0f);
            B.rng[i] = rng.state;
        }
        warp_add_stats(P, B.stats, 0, segs, st.nodes, st.tris);
    }
}

// Wireframe overlay (GRK:2910-3027): pixels on a triangle edge are set to black.
__global__ void __launch_bounds__(128) k_wireframe(DevScene S, const DevParams* __restrict__ Pp, DevPass B) {
    const DevParams& P = *Pp;
    const int n = B.n_pixels;
    GRID_STRIDE_UNIFORM(i, n) {
        if (i < n && B.pixel_flags[i] == 0) {
            TraceStats st{0, 0};
            const float4 o = B.primary_o[i], d = B.primary_d[i];
            const Hit h = trace_s(S, o.x, o.y, o.z, d.x, d.y, d.z, st);
            const float line_cos = P.wire_cos;
            if (h.t != INF && h.prim != -1 && h.shape_type == DFPT_SHAPE_TRIANGLE) {
                const Surf s = surface(S, P, o.x, o.y, o.z, d.x, d.y, d.z, h);
                const float* C = S.camera;
                const float ux = __ldg(C + 7), uy = __ldg(C + 8), uz = __ldg(C + 9);
                const float vx = __ldg(C + 10), vy = __ldg(C + 11), vz = __ldg(C + 12);
                const float wx = __ldg(C + 13), wy = __ldg(C + 14), wz = __ldg(C + 15);
                const float spx = s.px * ux + s.py * uy + s.pz * uz;
                const float spy = s.px * vx + s.py * vy + s.pz * vz;
                const float spz = s.px * wx + s.py * wy + s.pz * wz;
                const float spn = rsqrt_j(spx * spx + spy * spy + spz * spz);
                float cx[3], cy[3], cz[3];
                for (int k = 0; k < 3; ++k) {
                    const float3 q = p3(S, __ldg(S.triangles + h.shape_offset + k));
                    cx[k] = q.x * ux + q.y * uy + q.z * uz;
                    cy[k] = q.x * vx + q.y * vy + q.z * vz;
                    cz[k] = q.x * wx + q.y * wy + q.z * wz;
                }
                // Edges AC, BA, CB as (from, to) vertex pairs.
                const int ef[3] = {0, 1, 2}, et[3] = {2, 0, 1};
                bool edge = false;
                for (int k = 0; k < 3; ++k) {
                    const int f = ef[k], tt = et[k];
                    const float ds = ((cx[f] - cx[tt]) * (cx[f] - cx[tt])) + ((cy[f] - cy[tt]) * (cy[f] - cy[tt])) + ((cz[f] - cz[tt]) * (cz[f] - cz[tt]));
                    const float t0 = ((spx - cx[f]) * (cx[tt] - cx[f])) + ((spy - cy[f]) * (cy[tt] - cy[f])) + ((spz - cz[f]) * (cz[tt] - cz[f]));
                    const float t1 = t0 / ds;
                    const float qx = (1.0f - t1) * cx[f] + t1 * cx[tt];
                    const float qy = (1.0f - t1) * cy[f] + t1 * cy[tt];
                    const float qz = (1.0f - t1) * cz[f] + t1 * cz[tt];
                    const float qn = rsqrt_j(qx * qx + qy * qy + qz * qz);
                    const float dpq = qx * spx + qy * spy + qz * spz;
                    if (dpq * qn * spn >= line_cos) edge = true;
                }
                if (edge) B.pixel_flags[i] = 1;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Film accumulation (Kahan-compensated running sums) and the image pipeline: selection tint,
// tone map, sRGB redo-gamma, BGRA8 (GRK:279-307, AIK:333-472, 503-534, 702-774).

__device__ __forceinline__ float redo_gamma(const DevParams& P, float v) {
    return v <= 0.0f ? 0.0f : v >= 1.0f ? 1.0f : v <= P.cs_break ? v * P.cs_slope : P.cs_slope_match * powf(v, 1.0f / P.cs_gamma) - P.cs_segment;
}

__device__ __forceinline__ float filmic(float v, float exposure, float a, float b, float c, float d, float e, float subtract, float minimum) {
    const float m = jmax(v * exposure - subtract, minimum);
    return saturate_j((m * (a * m + b)) / (m * (c * m + d) + e), 0.0f, 1.0f);
}

// One sample into a pixel's Kahan-compensated sum (filmAddColor / filmSetColor, AIK:333-378):
// a rejected primary ray sets the pixel black; the first sample after a clear sets it.
__device__ __forceinline__ void film_add(float4 L, int flags, bool clear, float4& sum, float4& comp, int& cnt) {
    if (flags & 1) {
        sum = make_float4(0, 0, 0, 0); comp = make_float4(0, 0, 0, 0); cnt = 1;
    } else if (clear || cnt == 0) {
        sum = make_float4(L.x, L.y, L.z, 0); comp = make_float4(0, 0, 0, 0); cnt = 1;
    } else {
        float y, t;
        y = L.x - comp.x; t = sum.x + y; comp.x = (t - sum.x) - y; sum.x = t;
        y = L.y - comp.y; t = sum.y + y; comp.y = (t - sum.y) - y; sum.y = t;
        y = L.z - comp.z; t = sum.z + y; comp.z = (t - sum.z) - y; sum.z = t;
        cnt += 1;
    }
}

// Film average -> tone map -> sRGB -> BGRA8 (AIK:333-378, 410-534, 702-774), with the selection
// highlight on the green channel (GRK:282-290).
__device__ __forceinline__ uchar4 tone_map_bgra(const DevParams& P, float4 sum, int cnt, int po) {
    const float inv = 1.0f / (float)cnt;
    float r = sum.x * inv, g = sum.y * inv, b = sum.z * inv;
    g += (po > -1 && po == P.selected_primitive_offset) ? 1.0f : 0.0f;
    const float ex = P.exposure;
    switch (P.tone_mapper_type) {
        case DFPT_TONE_MAPPER_REINHARD:
            r = (r * ex) / (1.0f + r * ex); g = (g * ex) / (1.0f + g * ex); b = (b * ex) / (1.0f + b * ex);
            break;
        case DFPT_TONE_MAPPER_REINHARD_MODIFIED_1:
            r = 1.0f - expf(-r * ex); g = 1.0f - expf(-g * ex); b = 1.0f - expf(-b * ex);
            break;
        case DFPT_TONE_MAPPER_REINHARD_MODIFIED_2: {
            const float lw2r = 1.0f / (4.0f * 4.0f);
            const float rm = r * ex, gm = g * ex, bm = b * ex;
            r = rm * (1.0f + rm * lw2r) / (1.0f + rm); g = gm * (1.0f + gm * lw2r) / (1.0f + gm); b = bm * (1.0f + bm * lw2r) / (1.0f + bm);
            break;
        }
        case DFPT_TONE_MAPPER_FILMIC_CURVE_ACES_MODIFIED:
            r = filmic(r, ex, 2.51f, 0.03f, 2.43f, 0.59f, 0.14f, 0.0f, -FLT_MAX_F);
            g = filmic(g, ex, 2.51f, 0.03f, 2.43f, 0.59f, 0.14f, 0.0f, -FLT_MAX_F);
            b = filmic(b, ex, 2.51f, 0.03f, 2.43f, 0.59f, 0.14f, 0.0f, -FLT_MAX_F);
            break;
        default:
            break;
    }
    r = redo_gamma(P, r); g = redo_gamma(P, g); b = redo_gamma(P, b);
    const int ri = f2i(jmax(jmin(r * 255.0f + 0.5f, 255.0f), 0.0f));
    const int gi = f2i(jmax(jmin(g * 255.0f + 0.5f, 255.0f), 0.0f));
    const int bi = f2i(jmax(jmin(b * 255.0f + 0.5f, 255.0f), 0.0f));
    return make_uchar4((unsigned char)bi, (unsigned char)gi, (unsigned char)ri, 255);
}

__global__ void __launch_bounds__(256) k_film(const DevParams* __restrict__ Pp, DevPass B) {
    const DevParams& P = *Pp;
    const int n = B.n_pixels;
    const int pass = *B.pass_index;
    const bool clear = pass == P.clear_pass;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // Pixel i's path (its queue slot).
        const int path = slot_of_pixel(P, i);
        float4 sum = B.film_sum[i], comp = B.film_comp[i];
        int cnt = B.film_n[i];
        film_add(B.radiance[PSI(path)], B.pixel_flags[path], clear, sum, comp, cnt);
        if (P.diff) {
            const int k = pass - P.diff_pass0;
            if (k >= 0 && k < P.diff_spp) {
                B.diff_L[(size_t)k * n + i] = B.radiance[PSI(path)];
                B.diff_vis[(size_t)k * n + i] = (B.pixel_flags[path] & 1) ? 0 : B.vis[path];
            }
        }
        B.film_sum[i] = sum; B.film_comp[i] = comp; B.film_n[i] = cnt;
        reinterpret_cast<uchar4*>(B.bgra)[i] = tone_map_bgra(P, sum, cnt, B.primitive_offsets[i]);
    }
}

__global__ void k_end_pass(DevPass B) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *B.pass_index += 1;
}

// ---------------------------------------------------------------------------------------------
// Batch-only stages: the wave's film tasks, the film update, the final resolve, the wave advance.

// The scenes a wave touches, in order: {scene, local begin, local end, first film task}. A film task
// is one pixel of one scene that has at least one sample in the wave; a scene whose range in the
// wave covers fewer samples than pixels touches only that many pixels. Entry `E` holds the total.
__global__ void k_bwave(DevBatch Q) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const long long base = Q.wave_base[0];
    const long long end = base + Q.capacity < Q.wave_base[1] ? base + Q.capacity : Q.wave_base[1];
    int e = 0;
    long long tasks = 0;
    if (base < end) {
        for (int s = batch_scene_of(Q, base); s < Q.n_scenes && Q.sample_begin[s] < end; ++s) {
            const long long b0 = Q.sample_begin[s], b1 = Q.sample_begin[s + 1];
            const long long a = (base > b0 ? base : b0) - b0;
            const long long b = (end < b1 ? end : b1) - b0;
            const long long np = (long long)Q.params[s].width * Q.params[s].height;
            Q.wave_tab[4 * e + 0] = s;
            Q.wave_tab[4 * e + 1] = a;
            Q.wave_tab[4 * e + 2] = b;
            Q.wave_tab[4 * e + 3] = tasks;
            tasks += (b - a) < np ? (b - a) : np;
            ++e;
        }
    }
    Q.wave_tab[4 * e + 3] = tasks;
    *Q.wave_entries = e;
}

// One thread per film task: adds the pixel's samples of this wave in sample order, so each pixel
// sees the same Kahan sequence as one-scene rendering, pass after pass.
__global__ void __launch_bounds__(256) k_bfilm(DevBatch Q, DevPass B) {
    const int E = *Q.wave_entries;
    const long long tasks = Q.wave_tab[4 * E + 3];
    const long long base = Q.wave_base[0];
    const long long clear_sample = Q.wave_base[3];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tasks; t += (long long)gridDim.x * blockDim.x) {
        int e = 0;
        while (e + 1 < E && Q.wave_tab[4 * (e + 1) + 3] <= t) ++e;
        const int s = (int)Q.wave_tab[4 * e + 0];
        const long long a = Q.wave_tab[4 * e + 1], b = Q.wave_tab[4 * e + 2];
        const long long np = (long long)Q.params[s].width * Q.params[s].height;
        const long long first = a + (t - Q.wave_tab[4 * e + 3]);
        const long long pixel = first % np;
        const long long f = Q.film_begin[s] + pixel;
        const long long slot0 = Q.sample_begin[s] - base;
        float4 sum = B.film_sum[f], comp = B.film_comp[f];
        int cnt = B.film_n[f];
        const DevParams& P = Q.params[s];
        const long long pass0 = Q.wave_base[2];
#ifdef DFPT_ONE_SCENE
        const unsigned wave_p = wave_passes(Q, np);
#endif
        for (long long loc = first; loc < b; loc += np) {
#ifdef DFPT_ONE_SCENE
            const int slot = (int)slot_of_rel((unsigned)(slot0 + loc), (unsigned)np, wave_p);
#else
            const int slot = (int)(slot0 + a + seg_pos_of_local(loc, a, b, np));
#endif
            film_add(B.radiance[PSI(slot)], B.pixel_flags[slot], loc / np == clear_sample, sum, comp, cnt);
            if (P.diff) {
                // The differentiable forward's per-sample records (as k_film keeps them per pass).
                const long long k = pass0 + loc / np - P.diff_pass0;
                if (k >= 0 && k < P.diff_spp) {
                    B.diff_L[k * np + pixel] = B.radiance[PSI(slot)];
                    B.diff_vis[k * np + pixel] = (B.pixel_flags[slot] & 1) ? 0 : B.vis[slot];
                }
            }
        }
        B.film_sum[f] = sum; B.film_comp[f] = comp; B.film_n[f] = cnt;
    }
}

// Tone maps every scene's film into its BGRA8 image (once, after the last wave).
__global__ void __launch_bounds__(256) k_bresolve(DevBatch Q, DevPass B) {
    const long long n = Q.film_begin[Q.n_scenes];
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = Q.n_scenes - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (Q.film_begin[mid] <= f) lo = mid;
            else hi = mid - 1;
        }
        const int cnt = B.film_n[f];
        const int po = B.primitive_offsets != nullptr ? B.primitive_offsets[f] : -1;  // selection highlight (one scene)
        reinterpret_cast<uchar4*>(B.bgra)[f] = cnt > 0 ? tone_map_bgra(Q.params[lo], B.film_sum[f], cnt, po) : make_uchar4(0, 0, 0, 255);
    }
}

// Empties the shadow queue after its launch (waves trace each bounce's shadow rays at once).
__global__ void k_shadow_reset(DevPass B) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        B.counts[DFPT_COUNTS_SHADOW] = 0;
        B.counts[DFPT_COUNTS_FETCH + DFPT_MAX_DEPTH + 1] = 0;
    }
}

__global__ void k_bend_wave(DevBatch Q) {
    if (threadIdx.x == 0 && blockIdx.x == 0) Q.wave_base[0] += Q.capacity;
}

__global__ void __launch_bounds__(256) k_sort_hist(DevBatch Q, DevPass B, int bounce) {
    const int n = B.counts[bounce + 1];
    const int first = wave_first_scene(Q);
    GRID_STRIDE_UNIFORM(i, n) bin_count(B.sort_count, i < n ? ray_bin_in_wave(Q, first, B.q_o[1][i], B.q_d[1][i]) : -1);
}

// Moves the shadow queue (B.s_*) into the second set (out) in bin order.
__global__ void __launch_bounds__(256) k_sort_shadow_scatter(DevBatch Q, DevPass B, float4* out_o, float4* out_d, float4* out_c) {
    const int n = B.counts[DFPT_COUNTS_SHADOW];
    const int first = wave_first_scene(Q);
    GRID_STRIDE_UNIFORM(i, n) {
        int key = -1;
        float4 o, d, c;
        if (i < n) {
            o = B.s_o[i];
            d = B.s_d[i];
            c = B.s_c[i];
            key = shadow_bin_in_wave(Q, first, o, d);
        }
        const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (key >= 0 && (int)(threadIdx.x & 31) == leader) base = atomicAdd(B.sort_bins + key, __popc(same));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (key >= 0) {
            const int pos = base + __popc(same & ((1u << (threadIdx.x & 31)) - 1u));
            out_o[pos] = o;
            out_d[pos] = d;
            out_c[pos] = c;
        }
    }
}

// Exclusive scan of the bin counts into B.sort_bins, clearing the counts for the next count, in
// three launches over DFPT_SORT_CHUNKS chunks of 1024 bins: the chunk sums, their scan (one block),
// then each chunk's scan from its offset. Every access is coalesced (4 bins per thread).
__device__ __forceinline__ int block_exclusive_scan_256(int v, int& total) {
    __shared__ int warp_sum[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    int before = 0;
    total = 0;
    for (int k = 0; k < 8; ++k) {
        const int s = warp_sum[k];
        if (k < w) before += s;
        total += s;
    }
    __syncthreads();  // warp_sum is reused by the next call
    return before + x - v;
}
__global__ void __launch_bounds__(256) k_sort_chunk_sums(DevPass B, const int* __restrict__ counts) {
    const int4 c = reinterpret_cast<const int4*>(counts + (size_t)blockIdx.x * 1024)[threadIdx.x];
    int total;
    block_exclusive_scan_256(c.x + c.y + c.z + c.w, total);
    if (threadIdx.x == 0) B.sort_partials[blockIdx.x] = total;
}
// Scans the first `chunks` chunk sums (the rest of the bins are empty).
__global__ void __launch_bounds__(256) k_sort_chunk_offsets(DevPass B, int chunks) {
    constexpr int PER = DFPT_SORT_CHUNKS / 256;
    int v[PER], sum = 0;
    for (int j = 0; j < PER; ++j) {
        const int k = PER * threadIdx.x + j;
        v[j] = k < chunks ? B.sort_partials[k] : 0;
        sum += v[j];
    }
    int total;
    int run = block_exclusive_scan_256(sum, total);
    for (int j = 0; j < PER; ++j) {
        const int k = PER * threadIdx.x + j;
        if (k < chunks) B.sort_partials[k] = run;
        run += v[j];
    }
}
__global__ void __launch_bounds__(256) k_sort_chunk_scan(DevPass B, int* counts) {
    int4* cp = reinterpret_cast<int4*>(counts + (size_t)blockIdx.x * 1024) + threadIdx.x;
    const int4 c = *cp;
    *cp = make_int4(0, 0, 0, 0);
    int total;
    const int before = block_exclusive_scan_256(c.x + c.y + c.z + c.w, total) + B.sort_partials[blockIdx.x];
    reinterpret_cast<int4*>(B.sort_bins + (size_t)blockIdx.x * 1024)[threadIdx.x] =
        make_int4(before, before + c.x, before + c.x + c.y, before + c.x + c.y + c.z);
}
// A plain pass's deferred shadow rays into `out` in origin-cell order (the counts come from its
// shading, the offsets from the scan).
__global__ void __launch_bounds__(256) k_sort_shadow_scatter_plain(DevScene S, DevPass B, float4* out_o, float4* out_d, float4* out_c) {
    const int n = B.counts[DFPT_COUNTS_SHADOW];
    GRID_STRIDE_UNIFORM(i, n) {
        int key = -1;
        float4 o, d, c;
        if (i < n) {
            o = B.s_o[i];
            d = B.s_d[i];
            c = B.s_c[i];
            key = cell_bits(S, o, DFPT_SHADOW_CELL_BITS);
        }
        const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (key >= 0 && (int)(threadIdx.x & 31) == leader) base = atomicAdd(B.sort_bins + key, __popc(same));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (key >= 0) {
            const int pos = base + __popc(same & ((1u << (threadIdx.x & 31)) - 1u));
            out_o[pos] = o;
            out_d[pos] = d;
            out_c[pos] = c;
        }
    }
}
// The rays a plain pass's shading queued for `bounce` into `out` in bin order (direction bin over
// origin cell; the counts come from that shading, the offsets from the scan).
__global__ void __launch_bounds__(256) k_sort_rays_scatter_plain(DevScene S, DevPass B, int bounce, float4* out_o, float4* out_d) {
    const int n = B.counts[bounce];
    const int qi = bounce & 1;
    GRID_STRIDE_UNIFORM(i, n) {
        int key = -1;
        float4 o, d;
        if (i < n) {
            o = B.q_o[qi][i];
            d = B.q_d[qi][i];
            key = plain_ray_bin(S, o, d, B.sort_ray_bits);
        }
        const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (key >= 0 && (int)(threadIdx.x & 31) == leader) base = atomicAdd(B.sort_bins + key, __popc(same));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (key >= 0) {
            const int pos = base + __popc(same & ((1u << (threadIdx.x & 31)) - 1u));
            out_o[pos] = o;
            out_d[pos] = d;
        }
    }
}
// `chunks` chunks of 1024 bins hold every key (keys below chunks x 1024).
static void launch_sort_scan(const LaunchCtx& c, int* counts, int chunks = DFPT_SORT_CHUNKS) {
    k_sort_chunk_sums<<<chunks, 256, 0, c.stream>>>(*c.pass, counts);
    k_sort_chunk_offsets<<<1, 256, 0, c.stream>>>(*c.pass, chunks);
    k_sort_chunk_scan<<<chunks, 256, 0, c.stream>>>(*c.pass, counts);
}

__global__ void __launch_bounds__(256) k_sort_scatter(DevBatch Q, DevPass B, int bounce) {
    const int n = B.counts[bounce + 1];
    const int first = wave_first_scene(Q);
    GRID_STRIDE_UNIFORM(i, n) {
        int key = -1;
        float4 o, d;
        if (i < n) {
            o = B.q_o[1][i];
            d = B.q_d[1][i];
            key = ray_bin_in_wave(Q, first, o, d);
        }
        // Lanes with the same bin take consecutive places with one atomic.
        const unsigned same = __match_any_sync(0xFFFFFFFFu, key);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (key >= 0 && (int)(threadIdx.x & 31) == leader) base = atomicAdd(B.sort_bins + key, __popc(same));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (key >= 0) {
            const int pos = base + __popc(same & ((1u << (threadIdx.x & 31)) - 1u));
            B.q_o[0][pos] = o;
            B.q_d[0][pos] = d;
        }
    }
}

// FP64 mean of the film average (AIK film semantics: sum / samples per pixel).
__global__ void __launch_bounds__(256) k_film_mean(DevPass B, double* out3) {
    double r = 0.0, g = 0.0, b = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_pixels; i += gridDim.x * blockDim.x) {
        const float4 s = B.film_sum[i];
        const int c = B.film_n[i];
        if (c > 0) {
            const float inv = 1.0f / (float)c;
            r += (double)(s.x * inv); g += (double)(s.y * inv); b += (double)(s.z * inv);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        r += __shfl_down_sync(0xFFFFFFFFu, r, off);
        g += __shfl_down_sync(0xFFFFFFFFu, g, off);
        b += __shfl_down_sync(0xFFFFFFFFu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out3, r);
        atomicAdd(out3 + 1, g);
        atomicAdd(out3 + 2, b);
    }
}

__global__ void k_film_average(DevPass B, float* rgb, int* samples) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_pixels; i += gridDim.x * blockDim.x) {
        const float4 s = B.film_sum[i];
        const int c = B.film_n[i];
        const float inv = c > 0 ? 1.0f / (float)c : 0.0f;
        if (rgb) { rgb[3 * i] = s.x * inv; rgb[3 * i + 1] = s.y * inv; rgb[3 * i + 2] = s.z * inv; }
        if (samples) samples[i] = c;
    }
}

__global__ void k_init_tables(const int* perm256, const float* grad36) {
    const int i = threadIdx.x;
    if (i < 512) g_perm[i] = perm256[i & 255];
    if (i < 36) g_grad3[i] = grad36[i];
}

#ifdef DFPT_EXTENDED_KERNELS
#include "dfpt_adjoint.cuh"
#endif

// ---------------------------------------------------------------------------------------------
// Host-side launchers (the kernel set of this translation unit).

// Tuning configurations of the traversal kernels: {walk variant, block size, resident blocks}.
#define TRACE_CONFIGS(X) \
    X(0, 0, 256, 4) X(1, 1, 256, 4) X(2, 1, 256, 3) X(3, 0, 128, 8) X(4, 2, 256, 4) X(5, 2, 128, 8) X(6, 2, 256, 3) \
    X(7, 3, 256, 4) X(8, 3, 128, 8) X(9, 3, 256, 3) X(10, 3, 256, 2) \
    X(11, 0, 256, 6) X(12, 1, 256, 6) X(13, 0, 256, 8) X(14, 1, 256, 8) \
    X(15, 4, 256, 4) X(16, 5, 256, 4) X(17, 5, 256, 5)

// The scene argument of the batch stages: the context's scene in a one-scene set, else none (the
// kernels read each item's scene from the batch).
#ifdef DFPT_ONE_SCENE
#define BATCH_SCENE(c) (*(c).scene)
#else
#define BATCH_SCENE(c) DevScene{}
#endif

template <int V, int BLOCK, int MINB>
struct TraceCfg {
    static void carveout(int percent) {
#ifndef DFPT_ONE_SCENE
        cudaFuncSetAttribute(k_trace<false, false, V, BLOCK, MINB>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
#endif
#ifdef DFPT_EXTENDED_KERNELS
        cudaFuncSetAttribute(k_trace<true, false, (V == 2 ? 1 : V), BLOCK, MINB>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
#endif
    }
#ifndef DFPT_ONE_SCENE
    static void closest(const LaunchCtx& c, int bounce) {
        k_trace<false, false, V, BLOCK, MINB><<<c.grid_trace, BLOCK, 0, c.stream>>>(*c.scene, c.params, *c.pass, DevBatch{}, bounce, c.pass->sorted_queues ? 0 : (bounce & 1));
    }
    static void shadow(const LaunchCtx& c, int bounce) {
        k_shadow<false, V, BLOCK, MINB><<<c.grid_trace, BLOCK, 0, c.stream>>>(*c.scene, c.params, *c.pass, DevBatch{}, bounce);
    }
    static void final_(const LaunchCtx& c, int bounce) {
        k_final<false, V, BLOCK, MINB><<<c.grid_trace, BLOCK, 0, c.stream>>>(*c.scene, c.params, *c.pass, DevBatch{}, bounce);
    }
    static int grid(int sms) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<false, false, V, BLOCK, MINB>, BLOCK, 0);
        return sms * (b > 0 ? b : 1);
    }
    // The tail kernel: traversal and shading in one kernel, compiled for 2 resident blocks of 256,
    // and with the compact pair walk of the fast set also for 3 or 4 (c.tail_blocks: fewer
    // registers, more warps to hide the walk's load latency); its grid (SMs x resident blocks) is
    // found once per process. Its walk is the configuration's when that is the threaded walk (0)
    // or the compact pair walk (5), else the prefetching walk (1), so that three walks serve every
    // configuration (the other walks lost to these in whole launches).
    static constexpr int TVV = (V == 0 || V == 5) ? V : 1;
    template <int TB>
    static void tail_t(const LaunchCtx& c, int b0, int nb) {
        static int grid_tail = 0;
        if (grid_tail == 0) {
            int dev = 0, sms = 0, b = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_tail<TVV, 256, TB>, 256, 0);
            grid_tail = (sms > 0 ? sms : 1) * (b > 0 ? b : 1);
        }
        k_tail<TVV, 256, TB><<<grid_tail, 256, 0, c.stream>>>(*c.scene, c.params, *c.pass, b0, nb);
    }
    static void tail(const LaunchCtx& c, int b0, int nb) {
#ifdef DFPT_EXTENDED_KERNELS
        if constexpr (TVV == 5) {
            if (c.tail_blocks >= 4) { tail_t<4>(c, b0, nb); return; }
            if (c.tail_blocks == 3) { tail_t<3>(c, b0, nb); return; }
        }
#endif
        tail_t<2>(c, b0, nb);
    }
#endif
#ifdef DFPT_EXTENDED_KERNELS
    // Batch traversal: per-lane walks only (a warp may hold rays of several scenes).
    static constexpr int BV = V == 2 ? 1 : V;
    static void b_closest(const LaunchCtx& c, int bounce) {
        k_trace<true, false, BV, BLOCK, MINB><<<c.grid_trace, BLOCK, 0, c.stream>>>(BATCH_SCENE(c), c.params, *c.pass, *c.batch, bounce, c.pass->sorted_queues ? 0 : (bounce & 1));
    }
    static void b_shadow(const LaunchCtx& c, int bounce) {
        k_shadow<true, BV, BLOCK, MINB><<<c.grid_trace, BLOCK, 0, c.stream>>>(BATCH_SCENE(c), c.params, *c.pass, *c.batch, bounce);
    }
    static void b_final(const LaunchCtx& c, int bounce) {
        k_final<true, BV, BLOCK, MINB><<<c.grid_trace, BLOCK, 0, c.stream>>>(BATCH_SCENE(c), c.params, *c.pass, *c.batch, bounce);
    }
#ifdef DFPT_ONE_SCENE
    static int grid(int sms) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<true, false, BV, BLOCK, MINB>, BLOCK, 0);
        return sms * (b > 0 ? b : 1);
    }
#endif
#endif
};

#ifndef DFPT_ONE_SCENE
static void launch_trace_closest(const LaunchCtx& c, int bounce) {
    switch (c.trace_config) {
#define X(id, v, b, m) case id: TraceCfg<v, b, m>::closest(c, bounce); break;
        TRACE_CONFIGS(X)
#undef X
        default: TraceCfg<0, 256, 4>::closest(c, bounce);
    }
}
static void launch_shadow(const LaunchCtx& c, int bounce) {
    switch (c.trace_config) {
#define X(id, v, b, m) case id: TraceCfg<v, b, m>::shadow(c, bounce); break;
        TRACE_CONFIGS(X)
#undef X
        default: TraceCfg<0, 256, 4>::shadow(c, bounce);
    }
}
static void launch_tail(const LaunchCtx& c, int b0, int nb) {
    switch (c.trace_config) {
#define X(id, v, b, m) case id: TraceCfg<v, b, m>::tail(c, b0, nb); break;
        TRACE_CONFIGS(X)
#undef X
        default: TraceCfg<0, 256, 4>::tail(c, b0, nb);
    }
}
static void launch_final(const LaunchCtx& c, int bounce) {
    switch (c.trace_config) {
#define X(id, v, b, m) case id: TraceCfg<v, b, m>::final_(c, bounce); break;
        TRACE_CONFIGS(X)
#undef X
        default: TraceCfg<0, 256, 4>::final_(c, bounce);
    }
}
#endif
static void trace_carveout(int config, int percent) {
    switch (config) {
#define X(id, v, b, m) case id: TraceCfg<v, b, m>::carveout(percent); break;
        TRACE_CONFIGS(X)
#undef X
        default: break;
    }
}
static int trace_grid(int config, int sms) {
    switch (config) {
#define X(id, v, b, m) case id: return TraceCfg<v, b, m>::grid(sms);
        TRACE_CONFIGS(X)
#undef X
        default: return TraceCfg<0, 256, 4>::grid(sms);
    }
}

#ifndef DFPT_ONE_SCENE
static void launch_camera(const LaunchCtx& c) { k_camera<false><<<c.grid, 256, 0, c.stream>>>(*c.scene, c.params, *c.pass, DevBatch{}); }
static void launch_shade(const LaunchCtx& c, int bounce) { k_shade<false><<<c.grid, 256, 0, c.stream>>>(*c.scene, c.params, *c.pass, DevBatch{}, bounce); }
#endif

#ifdef DFPT_EXTENDED_KERNELS
#define BATCH_DISPATCH(fn)                                                                     \
    static void launch_b_##fn(const LaunchCtx& c, int bounce) {                                \
        switch (c.trace_config) {                                                              \
            TRACE_CONFIGS(BATCH_CASE_##fn)                                                     \
            default: TraceCfg<0, 256, 4>::b_##fn(c, bounce);                                   \
        }                                                                                      \
    }
#define BATCH_CASE_closest(id, v, b, m) case id: TraceCfg<v, b, m>::b_closest(c, bounce); break;
#define BATCH_CASE_shadow(id, v, b, m) case id: TraceCfg<v, b, m>::b_shadow(c, bounce); break;
#define BATCH_CASE_final(id, v, b, m) case id: TraceCfg<v, b, m>::b_final(c, bounce); break;
BATCH_DISPATCH(closest)
BATCH_DISPATCH(shadow)
BATCH_DISPATCH(final)
#undef BATCH_DISPATCH
#undef BATCH_CASE_closest
#undef BATCH_CASE_shadow
#undef BATCH_CASE_final
static void launch_b_camera(const LaunchCtx& c, int) { k_camera<true><<<c.grid, 256, 0, c.stream>>>(BATCH_SCENE(c), c.params, *c.pass, *c.batch); }
static void launch_b_shade(const LaunchCtx& c, int bounce) { k_shade<true><<<c.grid, 256, 0, c.stream>>>(BATCH_SCENE(c), c.params, *c.pass, *c.batch, bounce); }
static void launch_b_wave(const LaunchCtx& c, int) { k_bwave<<<1, 32, 0, c.stream>>>(*c.batch); }
static void launch_b_film(const LaunchCtx& c, int) { k_bfilm<<<c.grid, 256, 0, c.stream>>>(*c.batch, *c.pass); }
static void launch_b_resolve(const LaunchCtx& c, int) { k_bresolve<<<c.grid, 256, 0, c.stream>>>(*c.batch, *c.pass); }
static void launch_b_end(const LaunchCtx& c, int) { k_bend_wave<<<1, 32, 0, c.stream>>>(*c.batch); }
static void launch_b_shadow_reset(const LaunchCtx& c, int) { k_shadow_reset<<<1, 32, 0, c.stream>>>(*c.pass); }
// Bins the rays shading queued for bounce + 1 (queue 1 -> queue 0). k_shade counts the bins as it
// queues the rays (counted); the replay's shading does not, and a histogram pass counts them.
// Returns the kernels launched.
static int launch_b_sort(const LaunchCtx& c, int bounce, bool counted) {
    if (!counted) k_sort_hist<<<c.grid, 256, 0, c.stream>>>(*c.batch, *c.pass, bounce);
    launch_sort_scan(c, c.pass->sort_count);
    k_sort_scatter<<<c.grid, 256, 0, c.stream>>>(*c.batch, *c.pass, bounce);
    return counted ? 4 : 5;
}
// Bins the shadow queue into `to` (a pass record whose s_* point at the second set); k_shade
// counted the bins.
static int launch_b_sort_shadow(const LaunchCtx& c, const DevPass& to) {
    launch_sort_scan(c, c.pass->sort_count_shadow);
    k_sort_shadow_scatter<<<c.grid, 256, 0, c.stream>>>(*c.batch, *c.pass, to.s_o, to.s_d, to.s_c);
    return 4;
}

// Path-replay adjoint. Per-primitive partials live in shared memory when they fit in 44 KB.
template <bool BATCH>
static void launch_shade_adj_t(const LaunchCtx& c, int bounce) {
    const DevBatch Q = BATCH ? *c.batch : DevBatch{};
    const size_t bytes = (size_t)c.scene->primitive_count * DFPT_DIFF_PER_PRIM * sizeof(float);
    if (bytes <= 44 * 1024) k_shade_adj<BATCH, true><<<c.grid, 256, bytes, c.stream>>>(*c.scene, c.params, *c.pass, Q, bounce);
    else k_shade_adj<BATCH, false><<<c.grid, 256, 0, c.stream>>>(*c.scene, c.params, *c.pass, Q, bounce);
}
template <bool BATCH>
static void launch_final_adj_t(const LaunchCtx& c, int bounce) {
    // Per-lane walks (variant 1 prefetches); one block per gradient row.
    const DevBatch Q = BATCH ? *c.batch : DevBatch{};
    k_final_adj<BATCH, 1><<<c.grid, 256, 0, c.stream>>>(*c.scene, c.params, *c.pass, Q, bounce);
}
#ifndef DFPT_ONE_SCENE
static void launch_shade_adj(const LaunchCtx& c, int bounce) { launch_shade_adj_t<false>(c, bounce); }
static void launch_final_adj(const LaunchCtx& c, int bounce) { launch_final_adj_t<false>(c, bounce); }
#endif
static void launch_b_shade_adj(const LaunchCtx& c, int bounce) { launch_shade_adj_t<true>(c, bounce); }
static void launch_b_final_adj(const LaunchCtx& c, int bounce) { launch_final_adj_t<true>(c, bounce); }
static void launch_diff_reduce(const LaunchCtx& c, const double* rows, int n_rows, int row_len, double* out) {
    k_diff_reduce<<<(row_len + 255) / 256, 256, 0, c.stream>>>(rows, n_rows, row_len, out);
}
#endif
#ifndef DFPT_ONE_SCENE
static void launch_simple(const LaunchCtx& c) { k_simple<<<c.grid_simple, 128, 0, c.stream>>>(*c.scene, c.params, *c.pass); }
static void launch_wireframe(const LaunchCtx& c) { k_wireframe<<<c.grid_simple, 128, 0, c.stream>>>(*c.scene, c.params, *c.pass); }
static void launch_film(const LaunchCtx& c) { k_film<<<c.grid, 256, 0, c.stream>>>(c.params, *c.pass); }
static void launch_end_pass(const LaunchCtx& c) { k_end_pass<<<1, 32, 0, c.stream>>>(*c.pass); }
// Bins a plain pass's deferred shadow rays into `to` (a pass record whose s_* point at the second
// set); shading counted the bins. Returns the kernels launched.
static_assert(DFPT_SHADOW_CELL_BITS >= 10 && (1 << DFPT_SHADOW_CELL_BITS) <= DFPT_SORT_BINS,
              "the plain shadow scan covers whole chunks of 1024 bins within the bin array");
static int launch_sort_shadow(const LaunchCtx& c, const DevPass& to) {
    launch_sort_scan(c, c.pass->sort_count_shadow, (1 << DFPT_SHADOW_CELL_BITS) / 1024);
    k_sort_shadow_scatter_plain<<<c.grid, 256, 0, c.stream>>>(*c.scene, *c.pass, to.s_o, to.s_d, to.s_c);
    return 4;
}
// Bins the rays a plain pass queued for `bounce` into `to` (a pass record whose queue of that
// bounce's parity points at the second set); c.pass is the record the shading counted with.
static int launch_sort_rays(const LaunchCtx& c, int bounce, const DevPass& to) {
    const int qi = bounce & 1;
    launch_sort_scan(c, c.pass->sort_count, ((96 << c.pass->sort_ray_bits) + 1023) / 1024);
    k_sort_rays_scatter_plain<<<c.grid, 256, 0, c.stream>>>(*c.scene, *c.pass, bounce, to.q_o[qi], to.q_d[qi]);
    return 4;
}
static void launch_film_mean(const LaunchCtx& c, double* out3) { k_film_mean<<<c.grid, 256, 0, c.stream>>>(*c.pass, out3); }
static void launch_film_average(const LaunchCtx& c, float* rgb, int* samples) {
    k_film_average<<<c.grid, 256, 0, c.stream>>>(*c.pass, rgb, samples);
}
#endif
static void launch_init_tables(cudaStream_t s, const int* perm, const float* grad) { k_init_tables<<<1, 512, 0, s>>>(perm, grad); }

static void occupancy(int sms, int& grid, int& grid_trace, int& grid_simple) {
    int b1 = 0, b3 = 0;
#ifdef DFPT_ONE_SCENE
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_shade<true>, 256, 0);
    b3 = b1;
#else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_shade<false>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, k_simple, 128, 0);
#endif
    grid = sms * (b1 > 0 ? b1 : 1);
    grid_trace = trace_grid(0, sms);
    grid_simple = sms * (b3 > 0 ? b3 : 1);
}

KernelSet kernel_set() {
    KernelSet k;
#ifndef DFPT_ONE_SCENE
    k.camera = launch_camera;
    k.trace_closest = launch_trace_closest;
    k.shade = launch_shade;
    k.shadow = launch_shadow;
    k.final_ = launch_final;
    k.tail = launch_tail;
    k.simple = launch_simple;
    k.wireframe = launch_wireframe;
    k.film = launch_film;
    k.end_pass = launch_end_pass;
    k.sort_shadow = launch_sort_shadow;
    k.sort_rays = launch_sort_rays;
    k.film_mean = launch_film_mean;
    k.film_average = launch_film_average;
#endif
    k.init_tables = launch_init_tables;
    k.occupancy = occupancy;
    k.trace_grid = trace_grid;
    k.trace_carveout = trace_carveout;
#define X(id, v, b, m) +1
    k.trace_configs = 0 TRACE_CONFIGS(X);
#undef X
#ifdef DFPT_EXTENDED_KERNELS
    k.b_camera = launch_b_camera;
    k.b_trace_closest = launch_b_closest;
    k.b_shade = launch_b_shade;
    k.b_shadow = launch_b_shadow;
    k.b_final = launch_b_final;
    k.b_wave = launch_b_wave;
    k.b_film = launch_b_film;
    k.b_resolve = launch_b_resolve;
    k.b_end = launch_b_end;
    k.b_sort = launch_b_sort;
    k.b_sort_shadow = launch_b_sort_shadow;
    k.b_shadow_reset = launch_b_shadow_reset;
#ifndef DFPT_ONE_SCENE
    k.shade_adj = launch_shade_adj;
    k.final_adj = launch_final_adj;
#endif
    k.b_shade_adj = launch_b_shade_adj;
    k.b_final_adj = launch_b_final_adj;
    k.diff_reduce = launch_diff_reduce;
#endif
    return k;
}

}  // namespace DFPT_NS
