// oracle.cpp - CPU restatement of Dayflower's renderer kernel. TEST INFRASTRUCTURE ONLY.
//
// This is the checker the GPU core is compared against, never part of the product path: only
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it. It restates, function
// by function, src/main/java/org/dayflower/pathtracer/kernel/GPURendererKernel.java (GRK),
// AbstractKernel.java (AK) and AbstractImageKernel.java (AIK), templated on the real type:
//   R = float  : "strict FP32" - Java float semantics, one rounding per operation
//                (compiled with -ffp-contract=off), java.lang.Math in double then rounded;
//   R = double : the FP64 oracle (every float variable of the kernel promoted to double).
// Parity status: the reference cannot run here (Java + a closed Aparapi runtime, no JVM), and its
// repository holds no golden vectors, so this restatement is pinned by its source semantics and by
// known-answer tests derived from the reference's formulas (tests/golden) - "parity unpinned"
// against an executed reference.
#include <stdint.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/dfpt.h"

namespace {

// The reference's permutation table (AK:1130): Ken Perlin's with entry 156 = 23.
const int PERMUTATION[256] = {
    151, 160, 137, 91, 90, 15, 131, 13, 201, 95, 96, 53, 194, 233, 7, 225, 140, 36, 103, 30, 69, 142, 8, 99, 37, 240,
    21, 10, 23, 190, 6, 148, 247, 120, 234, 75, 0, 26, 197, 62, 94, 252, 219, 203, 117, 35, 11, 32, 57, 177, 33, 88,
    237, 149, 56, 87, 174, 20, 125, 136, 171, 168, 68, 175, 74, 165, 71, 134, 139, 48, 27, 166, 77, 146, 158, 231, 83,
    111, 229, 122, 60, 211, 133, 230, 220, 105, 92, 41, 55, 46, 245, 40, 244, 102, 143, 54, 65, 25, 63, 161, 1, 216, 80,
    73, 209, 76, 132, 187, 208, 89, 18, 169, 200, 196, 135, 130, 116, 188, 159, 86, 164, 100, 109, 198, 173, 186, 3, 64,
    52, 217, 226, 250, 124, 123, 5, 202, 38, 147, 118, 126, 255, 82, 85, 212, 207, 206, 59, 227, 47, 16, 58, 17, 182,
    189, 28, 42, 23, 183, 170, 213, 119, 248, 152, 2, 44, 154, 163, 70, 221, 153, 101, 155, 167, 43, 172, 9, 129, 22,
    39, 253, 19, 98, 108, 110, 79, 113, 224, 232, 178, 185, 112, 104, 218, 246, 97, 228, 251, 34, 242, 193, 238, 210,
    144, 12, 191, 179, 162, 241, 81, 51, 145, 235, 249, 14, 239, 107, 49, 192, 214, 31, 181, 199, 106, 157, 184, 84, 204,
    176, 115, 121, 50, 45, 127, 4, 150, 254, 138, 236, 205, 93, 222, 114, 67, 29, 24, 72, 243, 141, 128, 195, 78, 66,
    215, 61, 156, 180};
const float GRADIENT3[36] = {1, 1, 0, -1, 1, 0, 1, -1, 0, -1, -1, 0, 1, 0, 1, -1, 0, 1,
                             1, 0, -1, -1, 0, -1, 0, 1, 1, 0, -1, 1, 0, 1, -1, 0, -1, -1};

inline int perm(int i) { return PERMUTATION[i & 255]; }  // the 512-entry doubled table

// Java semantics helpers.
template <typename R> inline R jmin(R a, R b) { return (a != a) ? a : (b != b) ? b : (a <= b ? a : b); }
template <typename R> inline R jmax(R a, R b) { return (a != a) ? a : (b != b) ? b : (a >= b ? a : b); }
template <typename R> inline R jsqrt(R x) { return (R)std::sqrt((double)x); }
template <typename R> inline R jrsqrt(R x) { return (R)1 / jsqrt(x); }
template <typename R> inline R jsin(R x) { return (R)std::sin((double)x); }
template <typename R> inline R jcos(R x) { return (R)std::cos((double)x); }
template <typename R> inline R jtan(R x) { return (R)std::tan((double)x); }
template <typename R> inline R jpow(R a, R b) { return (R)std::pow((double)a, (double)b); }
template <typename R> inline R jexp(R x) { return (R)std::exp((double)x); }
template <typename R> inline R jatan2(R y, R x) { return (R)std::atan2((double)y, (double)x); }
template <typename R> inline R jfloor(R x) { return (R)std::floor((double)x); }
template <typename R> inline R jabs(R x) { return x < (R)0 ? -x : (x == (R)0 ? (R)0 : x); }
// Java (int) cast: truncation toward zero, saturating, NaN -> 0.
template <typename R> inline int jint(R x) {
    if (x != x) return 0;
    if (x >= (R)2147483647.0) return 2147483647;
    if (x <= (R)-2147483648.0) return (-2147483647 - 1);
    return (int)x;
}

// Constants of the float kernel (MathF PI family and GRK:76-78).
template <typename R> struct K {
    static constexpr float PIf = 3.14159274101257324219f;
    static R PI() { return (R)PIf; }
    static R TWO_PI() { return (R)(PIf * 2.0f); }
    static R INV_PI() { return (R)(1.0f / PIf); }
    static R INV_TWO_PI() { return (R)(1.0f / (PIf * 2.0f)); }
    static R PI_180() { return (R)(PIf / 180.0f); }
    static R CREC() { return (R)(1.0f / 255.0f); }
    static R INF() { return (R)100000.0f; }
};

// Philox4x32-10 counter-based stream (Salmon et al., SC'11); the draw order is the reference's.
void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

struct Random {
    int kind;  // DFPT_RNG_*
    uint64_t lcg;
    uint32_t pixel, pass, seed_lo, seed_hi, draws;
    // AbstractKernel.nextFloat (AK:438-440, 1101-1110) or the counter stream.
    float next() {
        if (kind == DFPT_RNG_LCG) {
            lcg = (lcg * 0x5DEECE66Dull + 0xBull) & ((1ull << 48) - 1ull);
            return (float)(int32_t)(lcg >> 24) * (1.0f / (float)(1 << 24));
        }
        uint32_t c[4] = {pass, draws >> 2, seed_hi, 0x44465054u};
        philox(c, pixel, seed_lo);
        const uint32_t x = c[draws & 3u];
        draws++;
        return (float)(x >> 8) * (1.0f / 16777216.0f);
    }
};

struct Scene {
    const dfpt_scene_desc* d;
    const dfpt_sky* sky;
    const dfpt_params* p;
    int width, height;
    float p3(int64_t i) const { return d->point3fs[i]; }
};

// The intersection record (GRK:79-94).
template <typename R> struct Isect {
    R distance;
    int primitive_offset, shape_type, shape_offset;
    R px, py, pz, nx, ny, nz, u, v, tx, ty, tz;  // point, shading normal, UV, tangent
};

struct Counters { uint64_t closest = 0, any = 0, nodes = 0, tris = 0, closest_nodes = 0, closest_tris = 0; };

// Differentiable-rendering inputs (per primitive: albedo multiplier, added emission, Phong
// exponent) and the record of one path, for the FP64 host adjoint.
struct DiffIn {
    const double* albedo;    // 3 per primitive
    const double* emission;  // 3 per primitive
    const double* exponent;  // 1 per primitive
};
struct TapeVertex {
    int prim, material;
    double T[3];              // throughput arriving at the vertex
    double tex[3], a0[3];     // albedo texture color, albedo used (before Russian roulette)
    bool sun, sun_vis;        // a sun sample was drawn / its shadow ray was unoccluded
    double sun_u, sun_v, sun_dot, p[3], w[3];
    bool albedo_mult;         // the vertex multiplied the throughput by the albedo
    double phong_ct, exponent;
    bool alive;
};
struct TapeEscape {
    int after;                // number of vertices before the escape
    double T[3], d[3];
};
struct Tape {
    std::vector<TapeVertex> v;
    std::vector<TapeEscape> esc;
    std::vector<std::pair<int, std::array<double, 3>>> contrib;  // (vertex index or depth, rgb)
    void clear() { v.clear(); esc.clear(); contrib.clear(); }
};

template <typename R> struct Kernel {
    const Scene& S;
    Random rng;
    Counters cnt;
    const DiffIn* diff = nullptr;  // per-primitive parameters (FP64 host adjoint)
    Tape* tape = nullptr;          // path record (FP64 host adjoint)
    R sun_u = 0, sun_v = 0, sun_dot = 0;
    bool sun_drawn = false, sun_seen = false;
    R ray[6];
    R color[3];  // colorTemporarySamples
    Isect<R> is;
    explicit Kernel(const Scene& s) : S(s) { is.tx = is.ty = is.tz = 0; }

    R nextf() { return (R)rng.next(); }

    // ---- AK helpers ----
    static R saturate(R v, R a, R b) { const R lo = jmin(a, b), hi = jmax(a, b); return v < lo ? lo : v > hi ? hi : v; }
    static R modulo(R v) { return v - jfloor(v); }
    static R remainder(R x, R y) { const int n = jint(x / y); return x - (R)n * y; }
    static R lerp(R a, R b, R t) { return ((R)1 - t) * a + t * b; }
    static R blerp(R a, R b, R c, R d, R tx, R ty) { return lerp(lerp(a, b, tx), lerp(c, d, tx), ty); }
    static int fast_floor(R v) { const int i = jint(v); return v < (R)i ? i - 1 : i; }

    static R simplex2(R x, R y) {
        const R F2 = (R)0.3660254037844386f, G2 = (R)0.21132486540518713f;
        const R s = (x + y) * F2;
        const int i = fast_floor(x + s), j = fast_floor(y + s);
        const R t = (R)(i + j) * G2;
        const R x0 = x - ((R)i - t), y0 = y - ((R)j - t);
        const int i1 = x0 > y0 ? 1 : 0, j1 = x0 > y0 ? 0 : 1;
        const R x1 = x0 - (R)i1 + G2, y1 = y0 - (R)j1 + G2;
        const R x2 = x0 - (R)1 + (R)2 * G2, y2 = y0 - (R)1 + (R)2 * G2;
        const int ii = i & 0xFF, jj = j & 0xFF;
        const int g0 = perm(ii + perm(jj)) % 12, g1 = perm(ii + i1 + perm(jj + j1)) % 12, g2 = perm(ii + 1 + perm(jj + 1)) % 12;
        R t0 = (R)0.5f - x0 * x0 - y0 * y0;
        const R n0 = t0 < (R)0 ? (R)0 : (t0 * t0) * (t0 * t0) * ((R)GRADIENT3[g0 * 3] * x0 + (R)GRADIENT3[g0 * 3 + 1] * y0);
        R t1 = (R)0.5f - x1 * x1 - y1 * y1;
        const R n1 = t1 < (R)0 ? (R)0 : (t1 * t1) * (t1 * t1) * ((R)GRADIENT3[g1 * 3] * x1 + (R)GRADIENT3[g1 * 3 + 1] * y1);
        R t2 = (R)0.5f - x2 * x2 - y2 * y2;
        const R n2 = t2 < (R)0 ? (R)0 : (t2 * t2) * (t2 * t2) * ((R)GRADIENT3[g2 * 3] * x2 + (R)GRADIENT3[g2 * 3 + 1] * y2);
        return (R)70 * (n0 + n1 + n2);
    }

    static R simplex3(R x, R y, R z) {
        const R F3 = (R)(1.0f / 3.0f), G3 = (R)(1.0f / 6.0f);
        const R s = (x + y + z) * F3;
        const int i = fast_floor(x + s), j = fast_floor(y + s), k = fast_floor(z + s);
        const R t = (R)(i + j + k) * G3;
        const R x0 = x - ((R)i - t), y0 = y - ((R)j - t), z0 = z - ((R)k - t);
        int i1 = 0, j1 = 0, k1 = 0, i2 = 0, j2 = 0, k2 = 0;
        if (x0 >= y0) {
            if (y0 >= z0) { i1 = 1; i2 = 1; j2 = 1; }
            else if (x0 >= z0) { i1 = 1; i2 = 1; k2 = 1; }
            else { k1 = 1; i2 = 1; k2 = 1; }
        } else {
            if (y0 < z0) { k1 = 1; j2 = 1; k2 = 1; }
            else if (x0 < z0) { j1 = 1; j2 = 1; k2 = 1; }
            else { j1 = 1; i2 = 1; j2 = 1; }
        }
        const R x1 = x0 - (R)i1 + G3, y1 = y0 - (R)j1 + G3, z1 = z0 - (R)k1 + G3;
        const R x2 = x0 - (R)i2 + (R)2 * G3, y2 = y0 - (R)j2 + (R)2 * G3, z2 = z0 - (R)k2 + (R)2 * G3;
        const R x3 = x0 - (R)1 + (R)3 * G3, y3 = y0 - (R)1 + (R)3 * G3, z3 = z0 - (R)1 + (R)3 * G3;
        const int ii = i & 0xFF, jj = j & 0xFF, kk = k & 0xFF;
        const int g[4] = {perm(ii + perm(jj + perm(kk))) % 12, perm(ii + i1 + perm(jj + j1 + perm(kk + k1))) % 12,
                          perm(ii + i2 + perm(jj + j2 + perm(kk + k2))) % 12, perm(ii + 1 + perm(jj + 1 + perm(kk + 1))) % 12};
        const R xs[4] = {x0, x1, x2, x3}, ys[4] = {y0, y1, y2, y3}, zs[4] = {z0, z1, z2, z3};
        R n[4];
        for (int c = 0; c < 4; ++c) {
            const R tt = (R)0.6f - xs[c] * xs[c] - ys[c] * ys[c] - zs[c] * zs[c];
            n[c] = tt < (R)0 ? (R)0 : (tt * tt) * (tt * tt) * ((R)GRADIENT3[g[c] * 3] * xs[c] + (R)GRADIENT3[g[c] * 3 + 1] * ys[c] + (R)GRADIENT3[g[c] * 3 + 2] * zs[c]);
        }
        return (R)32 * (n[0] + n[1] + n[2] + n[3]);
    }

    static R fbm3(R frequency, R gain, R minimum, R maximum, int octaves, R x, R y, R z) {
        R amp = 1, max_amp = 0, freq = frequency, noise = 0;
        for (int i = 0; i < octaves; ++i) {
            noise += simplex3(x * freq, y * freq, z * freq) * amp;
            max_amp += amp;
            amp *= gain;
            freq *= (R)2;
        }
        noise /= max_amp;
        return noise * (maximum - minimum) / (R)2 + (maximum + minimum) / (R)2;
    }

    R height(R x, R z) const {  // doGetY (GRK:726-728) -> simplexFractalXY
        R result = 0, amp = (R)S.p->global_amplitude, freq = (R)S.p->global_frequency;
        for (int i = 0; i < S.p->global_octaves; ++i) {
            result += amp * simplex2(x * freq, z * freq);
            amp *= (R)S.p->global_gain;
            freq *= (R)S.p->global_lacunarity;
        }
        return result;
    }

    // ---- doCreatePrimaryRay (GRK:573-724) ----
    bool create_primary_ray(int gid) {
        const float* cam = S.d->camera;
        const int y = gid / S.width, x = gid - y * S.width;
        const R eyeX = cam[1], eyeY = cam[2], eyeZ = cam[3];
        const R uX = cam[7], uY = cam[8], uZ = cam[9], vX = cam[10], vY = cam[11], vZ = cam[12], wX = cam[13], wY = cam[14], wZ = cam[15];
        const R fovX = jtan((R)cam[4] * (R)0.5f * K<R>::PI_180());
        const R fovY = jtan(-(R)cam[5] * (R)0.5f * K<R>::PI_180());
        const R hX = uX * fovX, hY = uY * fovX, hZ = uZ * fovX;
        const R vtX = vX * fovY, vtY = vY * fovY, vtZ = vZ * fovY;
        R sampleX = (R)0.5f, sampleY = (R)0.5f;
        if (S.p->renderer_type == DFPT_RENDERER_PATH_TRACER || !(S.p->renderer_type >= 1 && S.p->renderer_type <= 6)) {
            sampleX = nextf();
            sampleY = nextf();
            sampleX = sampleX < (R)0.5f ? jsqrt((R)2 * sampleX) - (R)1 : (R)1 - jsqrt((R)2 - (R)2 * sampleX);
            sampleY = sampleY < (R)0.5f ? jsqrt((R)2 * sampleY) - (R)1 : (R)1 - jsqrt((R)2 - (R)2 * sampleY);
        }
        const R sx = (sampleX + (R)x) / ((R)cam[16] - (R)1);
        const R sy = (sampleY + (R)y) / ((R)cam[17] - (R)1);
        const R sx0 = (R)2 * sx - (R)1, sy0 = (R)2 * sy - (R)1;
        R w = 1;
        if (cam[18] == 2.0f) {
            const R dp = sx0 * sx0 + sy0 * sy0;
            if (dp > (R)1) return false;
            w = jsqrt((R)1 - dp);
        }
        const R mX = eyeX + wX * w, mY = eyeY + wY * w, mZ = eyeZ + wZ * w;
        const R pX = mX + (hX * sx0) + (vtX * sy0), pY = mY + (hY * sx0) + (vtY * sy0), pZ = mZ + (hZ * sx0) + (vtZ * sy0);
        const R focal = cam[6];
        const R ipX = eyeX + (pX - eyeX) * focal, ipY = eyeY + (pY - eyeY) * focal, ipZ = eyeZ + (pZ - eyeZ) * focal;
        const R aperture = cam[0];
        R aX = eyeX, aY = eyeY, aZ = eyeZ;
        if (aperture > (R)0.00001f) {
            const R r1 = nextf(), r2 = nextf();
            const R angle = K<R>::TWO_PI() * r1;
            const R dist = aperture * jsqrt(r2);
            const R apX = jcos(angle) * dist, apY = jsin(angle) * dist;
            aX = eyeX + uX * apX + vX * apY;
            aY = eyeY + uY * apX + vY * apY;
            aZ = eyeZ + uZ * apX + vZ * apY;
        }
        const R dX = ipX - aX, dY = ipY - aY, dZ = ipZ - aZ;
        const R lr = jrsqrt(dX * dX + dY * dY + dZ * dZ);
        ray[0] = aX; ray[1] = aY; ray[2] = aZ;
        ray[3] = dX * lr; ray[4] = dY * lr; ray[5] = dZ * lr;
        return true;
    }

    // ---- shape intersections (GRK:1414-1594) ----
    static R isect_plane(R oX, R oY, R oZ, R dX, R dY, R dZ, R aX, R aY, R aZ, R nX, R nY, R nZ, R tMin, R tMax) {
        const R dp = nX * dX + nY * dY + nZ * dZ;
        if (dp < (R)0 || dp > (R)0) {
            const R t = ((aX - oX) * nX + (aY - oY) * nY + (aZ - oZ) * nZ) / dp;
            if (t > tMin && t < tMax) return t;
        }
        return K<R>::INF();
    }
    static R isect_sphere(R oX, R oY, R oZ, R dX, R dY, R dZ, R cX, R cY, R cZ, R radius, R tMin, R tMax) {
        const R pX = oX - cX, pY = oY - cY, pZ = oZ - cZ;
        const R r2 = radius * radius;
        const R a = dX * dX + dY * dY + dZ * dZ;
        const R b = (R)2 * (pX * dX + pY * dY + pZ * dZ);
        const R c = (pX * pX + pY * pY + pZ * pZ) - r2;
        const R disc2 = b * b - (R)4 * a * c;
        if (disc2 >= (R)0) {
            const R disc = jsqrt(disc2);
            const R q = (R)-0.5f * (b < (R)0 ? b - disc : b + disc);
            const R r0 = q / a;
            const R r1 = q == (R)0 ? r0 : c / q;
            const R t0 = jmin(r0, r1), t1 = jmax(r0, r1);
            if (t0 > tMin && t0 < tMax) return t0;
            if (t1 > tMin && t1 < tMax) return t1;
        }
        return K<R>::INF();
    }
    static R isect_triangle(R oX, R oY, R oZ, R dX, R dY, R dZ, R aX, R aY, R aZ, R bX, R bY, R bZ, R cX, R cY, R cZ, R tMin, R tMax) {
        const R e0X = bX - aX, e0Y = bY - aY, e0Z = bZ - aZ;
        const R e1X = cX - aX, e1Y = cY - aY, e1Z = cZ - aZ;
        const R v0X = dY * e1Z - dZ * e1Y, v0Y = dZ * e1X - dX * e1Z, v0Z = dX * e1Y - dY * e1X;
        const R det = e0X * v0X + e0Y * v0Y + e0Z * v0Z;
        R t = K<R>::INF();
        if (det < (R)-0.0001f || det > (R)0.0001f) {
            const R inv = (R)1 / det;
            const R v1X = oX - aX, v1Y = oY - aY, v1Z = oZ - aZ;
            const R u = (v1X * v0X + v1Y * v0Y + v1Z * v0Z) * inv;
            if (u >= (R)0 && u <= (R)1) {
                const R v2X = v1Y * e0Z - v1Z * e0Y, v2Y = v1Z * e0X - v1X * e0Z, v2Z = v1X * e0Y - v1Y * e0X;
                const R v = (dX * v2X + dY * v2Y + dZ * v2Z) * inv;
                t = v >= (R)0 && u + v <= (R)1 ? (e1X * v2X + e1Y * v2Y + e1Z * v2Z) * inv : tMin;
                t = t > tMin && t < tMax ? t : K<R>::INF();
            }
        }
        return t;
    }
    static R isect_terrain(R oX, R oY, R oZ, R dX, R dY, R dZ) {
        const R sr = (R)1 / (R)10;
        R t = 0, tDelta = (R)0.01f, lH = 0, lY = 0;
        for (R tc = (R)0.001f; tc < (R)10; tc += tDelta) {
            const R pX = oX * sr + dX * tc, pY = oY * sr + dY * tc, pZ = oZ * sr + dZ * tc;
            const R h = jsin(pX) * jsin(pZ);
            if (pY < h) {
                t = tc - tDelta + tDelta * (lH - lY) / (pY - lY - h + lH);
                tc = (R)10;
            }
            tDelta = (R)0.01f * tc;
            lH = h;
            lY = pY;
        }
        return t > (R)0.02f ? t : K<R>::INF();
    }

    void tri_positions(int off, R* a, R* b, R* c) const {
        const int* T = S.d->triangles + off;
        for (int k = 0; k < 3; ++k) { a[k] = S.p3(T[0] + k); b[k] = S.p3(T[1] + k); c[k] = S.p3(T[2] + k); }
    }

    // ---- doIntersectPrimitives (GRK:1048-1411) ----
    R intersect(R oX, R oY, R oZ, R dX, R dY, R dZ, bool testing) {
        if (testing) cnt.any++; else cnt.closest++;
        const dfpt_scene_desc* d = S.d;
        R closest = K<R>::INF();
        int cMatrix = -1, cPrim = -1, cType = -1, cOff = -1;
        const int count = (int)(d->primitives_count / 3);
        for (int i = 0; i < count; ++i) {
            R current = K<R>::INF();
            const int po = i * 3, mo = i * 16;
            const int type = d->primitives[po], off = d->primitives[po + 1];
            const float* W = d->primitives_world_to_object + mo;
            const R w11 = W[0], w12 = W[1], w13 = W[2], w14 = W[3], w21 = W[4], w22 = W[5], w23 = W[6], w24 = W[7], w31 = W[8], w32 = W[9], w33 = W[10], w34 = W[11];
            const R oXo = w11 * oX + w12 * oY + w13 * oZ + w14, oYo = w21 * oX + w22 * oY + w23 * oZ + w24, oZo = w31 * oX + w32 * oY + w33 * oZ + w34;
            const R dXo = w11 * dX + w12 * dY + w13 * dZ, dYo = w21 * dX + w22 * dY + w23 * dZ, dZo = w31 * dX + w32 * dY + w33 * dZ;
            const R iX = (R)1 / dXo, iY = (R)1 / dYo, iZ = (R)1 / dZo;
            if (type == DFPT_SHAPE_TRIANGLE_MESH) {
                const int abs_off = off;
                int rel = 0;
                while (rel != -1) {
                    const int at = abs_off + rel;
                    const int* B = d->bounding_volume_hierarchies;
                    cnt.nodes++;
                    if (!testing) cnt.closest_nodes++;
                    const R mnX = S.p3(B[at + 2]), mnY = S.p3(B[at + 2] + 1), mnZ = S.p3(B[at + 2] + 2);
                    const R mxX = S.p3(B[at + 3]), mxY = S.p3(B[at + 3] + 1), mxZ = S.p3(B[at + 3] + 2);
                    const R t0X = (mnX - oXo) * iX, t0Y = (mnY - oYo) * iY, t0Z = (mnZ - oZo) * iZ;
                    const R t1X = (mxX - oXo) * iX, t1Y = (mxY - oYo) * iY, t1Z = (mxZ - oZo) * iZ;
                    const R tMax = jmin(jmax(t0X, t1X), jmin(jmax(t0Y, t1Y), jmax(t0Z, t1Z)));
                    const R tMin = jmax(jmin(t0X, t1X), jmax(jmin(t0Y, t1Y), jmin(t0Z, t1Z)));
                    const R t = tMin > tMax ? (R)-1 : tMin > (R)0.001f && tMin < closest ? tMin : tMax > (R)0.001f && tMax < closest ? tMax : (R)-1;
                    if (t < (R)0) {
                        rel = B[at + 1];
                    } else if (B[at] == 1) {
                        rel = B[at + 4];
                    } else {
                        const int n = B[at + 4];
                        for (int j = 0; j < n; ++j) {
                            const int toff = B[at + 5 + j];
                            R a[3], b[3], c[3];
                            tri_positions(toff, a, b, c);
                            cnt.tris++;
                            if (!testing) cnt.closest_tris++;
                            current = isect_triangle(oXo, oYo, oZo, dXo, dYo, dZo, a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2], (R)0.001f, closest);
                            if (current < closest) { closest = current; cMatrix = mo; cPrim = po; cType = DFPT_SHAPE_TRIANGLE; cOff = toff; }
                            if (testing && cPrim != -1) return closest;
                        }
                        rel = B[at + 1];
                    }
                }
            } else if (type == DFPT_SHAPE_PLANE) {
                const int* Pl = d->planes + off;
                const float* N = d->vector3fs + Pl[3];
                current = isect_plane(oXo, oYo, oZo, dXo, dYo, dZo, S.p3(Pl[0]), S.p3(Pl[0] + 1), S.p3(Pl[0] + 2), N[0], N[1], N[2], (R)0.001f, closest);
            } else if (type == DFPT_SHAPE_SPHERE) {
                const int pos = jint(d->spheres[off]);
                current = isect_sphere(oXo, oYo, oZo, dXo, dYo, dZo, S.p3(pos), S.p3(pos + 1), S.p3(pos + 2), d->spheres[off + 1], (R)0.001f, closest);
            } else if (type == DFPT_SHAPE_TERRAIN) {
                current = isect_terrain(oXo, oYo, oZo, dXo, dYo, dZo);
            } else if (type == DFPT_SHAPE_TRIANGLE) {
                R a[3], b[3], c[3];
                tri_positions(off, a, b, c);
                cnt.tris++;
                if (!testing) cnt.closest_tris++;
                current = isect_triangle(oXo, oYo, oZo, dXo, dYo, dZo, a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2], (R)0.001f, closest);
            }
            if (current < closest) { closest = current; cMatrix = mo; cPrim = po; cType = type; cOff = off; }
            if (testing && cPrim != -1) return closest;
        }
        if (!testing) {
            if (cPrim != -1) {
                is.distance = closest;
                is.primitive_offset = cPrim;
                is.shape_type = cType;
                is.shape_offset = cOff;
                surface_properties(oX, oY, oZ, dX, dY, dZ, closest, cMatrix, cPrim, cType, cOff);
            } else {
                is.distance = K<R>::INF();
                is.primitive_offset = -1;
                is.shape_type = -1;
                is.shape_offset = -1;
            }
        }
        return closest;
    }

    // Surface properties in object space, then to world space, then normal mapping.
    void surface_properties(R oX, R oY, R oZ, R dX, R dY, R dZ, R t, int mo, int po, int type, int off) {
        const dfpt_scene_desc* d = S.d;
        const float* W = d->primitives_world_to_object + mo;
        const float* O = d->primitives_object_to_world + mo;
        const R w11 = W[0], w12 = W[1], w13 = W[2], w14 = W[3], w21 = W[4], w22 = W[5], w23 = W[6], w24 = W[7], w31 = W[8], w32 = W[9], w33 = W[10], w34 = W[11];
        const R oXo = w11 * oX + w12 * oY + w13 * oZ + w14, oYo = w21 * oX + w22 * oY + w23 * oZ + w24, oZo = w31 * oX + w32 * oY + w33 * oZ + w34;
        const R dXo = w11 * dX + w12 * dY + w13 * dZ, dYo = w21 * dX + w22 * dY + w23 * dZ, dZo = w31 * dX + w32 * dY + w33 * dZ;
        Isect<R>& I = is;
        if (type == DFPT_SHAPE_PLANE) {  // GRK:2349-2450
            const int* Pl = d->planes + off;
            const R aX = S.p3(Pl[0]), aY = S.p3(Pl[0] + 1), aZ = S.p3(Pl[0] + 2);
            const R bX = S.p3(Pl[1]), bY = S.p3(Pl[1] + 1), bZ = S.p3(Pl[1] + 2);
            const R cX = S.p3(Pl[2]), cY = S.p3(Pl[2] + 1), cZ = S.p3(Pl[2] + 2);
            const R nX = d->vector3fs[Pl[3]], nY = d->vector3fs[Pl[3] + 1], nZ = d->vector3fs[Pl[3] + 2];
            const R pX = oXo + dXo * t, pY = oYo + dYo * t, pZ = oZo + dZo * t;
            const R anX = jabs(nX), anY = jabs(nY), anZ = jabs(nZ);
            const bool isX = anX > anY && anX > anZ;
            const bool isY = anY > anZ;
            const R a1X = isX ? aY : isY ? aZ : aX, a1Y = isX ? aZ : isY ? aX : aY;
            const R b1X = isX ? cY - aX : isY ? cZ - aX : cX - aX, b1Y = isX ? cZ - aY : isY ? cX - aY : cY - aY;
            const R c1X = isX ? bY - aX : isY ? bZ - aX : bX - aX, c1Y = isX ? bZ - aY : isY ? bX - aY : bY - aY;
            const R det = b1X * c1Y - b1Y * c1X;
            const R dr = (R)1 / det;
            const R bNU = -b1Y * dr, bNV = b1X * dr, bND = (b1Y * a1X - b1X * a1Y) * dr;
            const R cNU = c1Y * dr, cNV = -c1X * dr, cND = (c1X * a1Y - c1Y * a1X) * dr;
            const R hU = isX ? pY : isY ? pZ : pX, hV = isX ? pZ : isY ? pX : pY;
            I.u = hU * bNU + hV * bNV + bND;
            I.v = hU * cNU + hV * cNV + cND;
            I.px = pX; I.py = pY; I.pz = pZ;
            I.nx = nX; I.ny = nY; I.nz = nZ;
        } else if (type == DFPT_SHAPE_SPHERE) {  // GRK:2452-2492
            const int pos = jint(d->spheres[off]);
            const R cX = S.p3(pos), cY = S.p3(pos + 1), cZ = S.p3(pos + 2);
            const R pX = oXo + dXo * t, pY = oYo + dYo * t, pZ = oZo + dZo * t;
            const R n0X = pX - cX, n0Y = pY - cY, n0Z = pZ - cZ;
            const R lr = jrsqrt(n0X * n0X + n0Y * n0Y + n0Z * n0Z);
            const R n1X = n0X * lr, n1Y = n0Y * lr, n1Z = n0Z * lr;
            I.u = (R)0.5f + jatan2(-n1Z, -n1X) * K<R>::INV_TWO_PI();
            I.v = (R)0.5f - (R)std::asin((double)(-n1Y)) * K<R>::INV_PI();  // asinpi; see the header note
            I.px = pX; I.py = pY; I.pz = pZ;
            I.nx = n1X; I.ny = n1Y; I.nz = n1Z;
        } else if (type == DFPT_SHAPE_TERRAIN) {  // GRK:2495-2539
            const R sr = (R)1 / (R)10;
            const R pX = oXo * sr + dXo * t, pY = oYo * sr + dYo * t, pZ = oZo * sr + dZo * t;
            const R e = (R)0.02f;
            const R nX = (jsin(pX - e) * jsin(pZ)) - (jsin(pX + e) * jsin(pZ));
            const R nY = (R)2 * e;
            const R nZ = (jsin(pX) * jsin(pZ - e)) - (jsin(pX) * jsin(pZ + e));
            const R lr = jrsqrt(nX * nX + nY * nY + nZ * nZ);
            I.px = pX; I.py = pY; I.pz = pZ;
            I.u = pX; I.v = pZ;
            I.nx = nX * lr; I.ny = nY * lr; I.nz = nZ * lr;
        } else {  // Triangle (GRK:2541-2650)
            const int* T = d->triangles + off;
            R a[3], b[3], c[3];
            tri_positions(off, a, b, c);
            const R pX = oXo + dXo * t, pY = oYo + dYo * t, pZ = oZo + dZo * t;
            const R abX = b[0] - a[0], abY = b[1] - a[1], abZ = b[2] - a[2];
            const R acX = c[0] - a[0], acY = c[1] - a[1], acZ = c[2] - a[2];
            const R v0X = dYo * acZ - dZo * acY, v0Y = dZo * acX - dXo * acZ, v0Z = dXo * acY - dYo * acX;
            const R v1X = oXo - a[0], v1Y = oYo - a[1], v1Z = oZo - a[2];
            const R v2X = v1Y * abZ - v1Z * abY, v2Y = v1Z * abX - v1X * abZ, v2Z = v1X * abY - v1Y * abX;
            const R det = abX * v0X + abY * v0Y + abZ * v0Z;
            const R dr = (R)1 / det;
            const R bu = (v1X * v0X + v1Y * v0Y + v1Z * v0Z) * dr;
            const R bv = (dXo * v2X + dYo * v2Y + dZo * v2Z) * dr;
            const R bw = (R)1 - bu - bv;
            const float* P2 = d->point2fs;
            I.u = bw * (R)P2[T[6]] + bu * (R)P2[T[7]] + bv * (R)P2[T[8]];
            I.v = bw * (R)P2[T[6] + 1] + bu * (R)P2[T[7] + 1] + bv * (R)P2[T[8] + 1];
            I.px = pX; I.py = pY; I.pz = pZ;
            R n0X = 0, n0Y = 0, n0Z = 0, t0X = 0, t0Y = 0, t0Z = 0;
            if (S.p->shader_type == DFPT_SHADER_FLAT) {
                n0X = abY * acZ - abZ * acY; n0Y = abZ * acX - abX * acZ; n0Z = abX * acY - abY * acX;
            } else if (S.p->shader_type == DFPT_SHADER_GOURAUD) {
                const float* V = d->vector3fs;
                n0X = (R)V[T[3]] * bw + (R)V[T[4]] * bu + (R)V[T[5]] * bv;
                n0Y = (R)V[T[3] + 1] * bw + (R)V[T[4] + 1] * bu + (R)V[T[5] + 1] * bv;
                n0Z = (R)V[T[3] + 2] * bw + (R)V[T[4] + 2] * bu + (R)V[T[5] + 2] * bv;
                t0X = (R)V[T[9]] * bw + (R)V[T[10]] * bu + (R)V[T[11]] * bv;
                t0Y = (R)V[T[9] + 1] * bw + (R)V[T[10] + 1] * bu + (R)V[T[11] + 1] * bv;
                t0Z = (R)V[T[9] + 2] * bw + (R)V[T[10] + 2] * bu + (R)V[T[11] + 2] * bv;
            }
            const R nr = jrsqrt(n0X * n0X + n0Y * n0Y + n0Z * n0Z);
            I.nx = n0X * nr; I.ny = n0Y * nr; I.nz = n0Z * nr;
            const R tr = jrsqrt(t0X * t0X + t0Y * t0Y + t0Z * t0Z);
            I.tx = t0X * tr; I.ty = t0Y * tr; I.tz = t0Z * tr;
        }
        // doTransformIntersectionToWorldSpace (GRK:3998-4073)
        const R o11 = O[0], o12 = O[1], o13 = O[2], o14 = O[3], o21 = O[4], o22 = O[5], o23 = O[6], o24 = O[7], o31 = O[8], o32 = O[9], o33 = O[10], o34 = O[11];
        const R pwX = o11 * I.px + o12 * I.py + o13 * I.pz + o14;
        const R pwY = o21 * I.px + o22 * I.py + o23 * I.pz + o24;
        const R pwZ = o31 * I.px + o32 * I.py + o33 * I.pz + o34;
        const R nwX = w11 * I.nx + w21 * I.ny + w31 * I.nz, nwY = w12 * I.nx + w22 * I.ny + w32 * I.nz, nwZ = w13 * I.nx + w23 * I.ny + w33 * I.nz;
        const R twX = w11 * I.tx + w21 * I.ty + w31 * I.tz, twY = w12 * I.tx + w22 * I.ty + w32 * I.tz, twZ = w13 * I.tx + w23 * I.ty + w33 * I.tz;
        I.px = pwX; I.py = pwY; I.pz = pwZ;
        I.nx = nwX; I.ny = nwY; I.nz = nwZ;
        I.tx = twX; I.ty = twY; I.tz = twZ;
        normal_map_image(po);
        normal_map_noise(po);
    }

    int image_simple(int to) const {  // GRK:1894-1929
        const float* Tx = S.d->textures;
        const R width = Tx[to + 4], height = Tx[to + 5], su = Tx[to + 6], sv = Tx[to + 7], ca = Tx[to + 2], sa = Tx[to + 3];
        const R u0 = (is.u * ca - is.v * sa), v0 = (is.v * ca + is.u * sa);
        const R u1 = remainder(u0 * su * width, width), v1 = remainder(v0 * sv * height, height);
        const R u2 = u1 >= (R)0 ? u1 : width - jabs(u1), v2 = v1 >= (R)0 ? v1 : height - jabs(v1);
        const int x = jint(u2), y = jint(v2), w = jint(width), res = jint(width * height);
        const int index = y * w + x;
        return index >= 0 && index < res ? jint(Tx[to + 8 + index]) : 0;
    }

    void normal_map_image(int po) {  // GRK:2714-2846
        const dfpt_scene_desc* d = S.d;
        const int so = d->primitives[po + 2];
        const int to = jint(d->surfaces[so + 3]);
        const int ttype = jint(d->textures[to]);
        if (S.p->normal_mapping == 1 && ttype == DFPT_TEXTURE_IMAGE) {
            const int rgb = image_simple(to);
            const R r = ((((rgb >> 16) & 0xFF) * K<R>::CREC()) - (R)0.5f) * (R)2;
            const R g = ((((rgb >> 8) & 0xFF) * K<R>::CREC()) - (R)0.5f) * (R)2;
            const R b = ((((rgb >> 0) & 0xFF) * K<R>::CREC()) - (R)0) * (R)2;
            const R wX = is.nx, wY = is.ny, wZ = is.nz;
            const int type = d->primitives[po];
            R sX, sY, sZ;
            if (type == DFPT_SHAPE_SPHERE) {
                const R v0X = (R)-2 * K<R>::PI() * wY, v0Y = (R)2 * K<R>::PI() * wX, v0Z = 0;
                const R u0X = v0Y * wZ - v0Z * wY, u0Y = v0Z * wX - v0X * wZ, u0Z = v0X * wY - v0Y * wX;
                const R ul = jrsqrt(u0X * u0X + u0Y * u0Y + u0Z * u0Z);
                const R u1X = u0X * ul, u1Y = u0Y * ul, u1Z = u0Z * ul;
                const R v1X = wY * u1Z - wZ * u1Y, v1Y = wZ * u1X - wX * u1Z, v1Z = wX * u1Y - wY * u1X;
                const R vl = jrsqrt(v1X * v1X + v1Y * v1Y + v1Z * v1Z);
                const R v2X = v1X * vl, v2Y = v1Y * vl, v2Z = v1Z * vl;
                sX = r * u1X + g * v2X + b * wX; sY = r * u1Y + g * v2Y + b * wY; sZ = r * u1Z + g * v2Z + b * wZ;
            } else if (type == DFPT_SHAPE_TRIANGLE) {
                const R uX = is.tx, uY = is.ty, uZ = is.tz;
                const R v0X = wY * uZ - wZ * uY, v0Y = wZ * uX - wX * uZ, v0Z = wX * uY - wY * uX;
                const R vl = jrsqrt(v0X * v0X + v0Y * v0Y + v0Z * v0Z);
                const R v1X = v0X * vl, v1Y = v0Y * vl, v1Z = v0Z * vl;
                sX = r * uX + g * v1X + b * wX; sY = r * uY + g * v1Y + b * wY; sZ = r * uZ + g * v1Z + b * wZ;
            } else {
                const R aX = jabs(wX), aY = jabs(wY), aZ = jabs(wZ);
                const bool isWX = aX < aY && aX < aZ, isWY = aY < aZ;
                const R v0X = isWX ? (R)0 : isWY ? wZ : wY, v0Y = isWX ? wZ : isWY ? (R)0 : -wX, v0Z = isWX ? -wY : isWY ? -wX : (R)0;
                const R vl = jrsqrt(v0X * v0X + v0Y * v0Y + v0Z * v0Z);
                const R v1X = v0X * vl, v1Y = v0Y * vl, v1Z = v0Z * vl;
                const R u0X = v1Y * wZ - v1Z * wY, u0Y = v1Z * wX - v1X * wZ, u0Z = v1X * wY - v1Y * wX;
                const R ul = jrsqrt(u0X * u0X + u0Y * u0Y + u0Z * u0Z);
                const R u1X = u0X * ul, u1Y = u0Y * ul, u1Z = u0Z * ul;
                sX = r * u1X + g * v1X + b * wX; sY = r * u1Y + g * v1Y + b * wY; sZ = r * u1Z + g * v1Z + b * wZ;
            }
            const R sl = jrsqrt(sX * sX + sY * sY + sZ * sZ);
            is.nx = sX * sl; is.ny = sY * sl; is.nz = sZ * sl;
        }
    }

    void normal_map_noise(int po) {  // GRK:2658-2712
        const dfpt_scene_desc* d = S.d;
        const int so = d->primitives[po + 2];
        const R amount = d->surfaces[so + 4], scale = d->surfaces[so + 5];
        if (S.p->normal_mapping == 1 && amount > (R)0 && scale > (R)0) {
            const R sr = (R)1 / scale;
            const R x1 = is.px * sr, y1 = is.py * sr, z1 = is.pz * sr;
            const R nX = fbm3(scale, (R)0.5f, (R)-0.26f, (R)0.26f, 16, x1, y1, z1);
            const R nY = fbm3(scale, (R)0.5f, (R)-0.26f, (R)0.26f, 16, y1, z1, x1);
            const R nZ = fbm3(scale, (R)0.5f, (R)-0.26f, (R)0.26f, 16, z1, x1, y1);
            const R qX = is.nx + nX * amount, qY = is.ny + nY * amount, qZ = is.nz + nZ * amount;
            const R ql = jrsqrt(qX * qX + qY * qY + qZ * qZ);
            is.nx = qX * ql; is.ny = qY * ql; is.nz = qZ * ql;
        }
    }

    // ---- textures (GRK:1596-1960) ----
    static int pack(R r, R g, R b) {
        const int ri = jint(saturate(r, (R)0, (R)1) * (R)255 + (R)0.5f);
        const int gi = jint(saturate(g, (R)0, (R)1) * (R)255 + (R)0.5f);
        const int bi = jint(saturate(b, (R)0, (R)1) * (R)255 + (R)0.5f);
        return ((ri & 0xFF) << 16) | ((gi & 0xFF) << 8) | (bi & 0xFF);
    }
    static R cr(int c) { return ((c >> 16) & 0xFF) * K<R>::CREC(); }
    static R cg(int c) { return ((c >> 8) & 0xFF) * K<R>::CREC(); }
    static R cb(int c) { return (c & 0xFF) * K<R>::CREC(); }

    int texture2(int to) const {
        const float* Tx = S.d->textures;
        const int type = jint(Tx[to]);
        if (type == DFPT_TEXTURE_BULLSEYE) {
            const int A = jint(Tx[to + 2]), B = jint(Tx[to + 3]);
            const R len = jsqrt(is.px * is.px + is.py * is.py + is.pz * is.pz);
            const R value = remainder(len * (R)0.25f, (R)1);
            R r = value > (R)0.5f ? cr(A) : cr(B), g = value > (R)0.5f ? cg(A) : cg(B), b = value > (R)0.5f ? cb(A) : cb(B);
            const R m = value > (R)0.5f ? (R)0.8f : (R)1.2f;
            if (cr(A) == cr(B) && cg(A) == cg(B) && cb(A) == cb(B)) { r *= m; g *= m; b *= m; }
            return pack(r, g, b);
        } else if (type == DFPT_TEXTURE_CHECKERBOARD) {
            const int C0 = jint(Tx[to + 2]), C1 = jint(Tx[to + 3]);
            const R ca = Tx[to + 4], sa = Tx[to + 5], su = Tx[to + 6], sv = Tx[to + 7];
            const R tu = modulo((is.u * ca - is.v * sa) * su), tv = modulo((is.v * ca + is.u * sa) * sv);
            const bool dark = (tu > (R)0.5f) ^ (tv > (R)0.5f);
            const R m = dark ? (R)0.8f : (R)1.2f;
            R r = dark ? cr(C0) : cr(C1), g = dark ? cg(C0) : cg(C1), b = dark ? cb(C0) : cb(C1);
            if (cr(C0) == cr(C1) && cg(C0) == cg(C1) && cb(C0) == cb(C1)) { r *= m; g *= m; b *= m; }
            return pack(r, g, b);
        } else if (type == DFPT_TEXTURE_CONSTANT) {
            return jint(Tx[to + 2]);
        } else if (type == DFPT_TEXTURE_FBM) {
            const int add = jint(Tx[to + 2]), mul = jint(Tx[to + 3]);
            const R noise = fbm3((R)Tx[to + 4], (R)Tx[to + 5], (R)0, (R)1, jint(Tx[to + 6]), is.px, is.py, is.pz);
            return pack(noise * cr(mul) + cr(add), noise * cg(mul) + cg(add), noise * cb(mul) + cb(add));
        } else if (type == DFPT_TEXTURE_IMAGE) {
            const R width = Tx[to + 4], height = Tx[to + 5], su = Tx[to + 6], sv = Tx[to + 7], ca = Tx[to + 2], sa = Tx[to + 3];
            const R u0 = (is.u * ca - is.v * sa), v0 = (is.v * ca + is.u * sa);
            const R u1 = remainder(u0 * su * width, width), v1 = remainder(v0 * sv * height, height);
            const R u2 = u1 >= (R)0 ? u1 : width - jabs(u1), v2 = v1 >= (R)0 ? v1 : height - jabs(v1);
            const int x = jint(u2), y = jint(v2), w = jint(width), res = jint(width * height);
            const int i00 = (y + 0) * w + (x + 0), i01 = (y + 0) * w + (x + 1), i10 = (y + 1) * w + (x + 0), i11 = (y + 1) * w + (x + 1);
            const int c00 = i00 >= 0 && i00 < res ? jint(Tx[to + 8 + i00]) : 0;
            const int c01 = i01 >= 0 && i01 < res ? jint(Tx[to + 8 + i01]) : 0;
            const int c10 = i10 >= 0 && i10 < res ? jint(Tx[to + 8 + i10]) : 0;
            const int c11 = i11 >= 0 && i11 < res ? jint(Tx[to + 8 + i11]) : 0;
            const R fx = u2 - (R)x, fy = v2 - (R)y;
            return pack(blerp(cr(c00), cr(c01), cr(c10), cr(c11), fx, fy), blerp(cg(c00), cg(c01), cg(c10), cg(c11), fx, fy),
                        blerp(cb(c00), cb(c01), cb(c10), cb(c11), fx, fy));
        } else if (type == DFPT_TEXTURE_SURFACE_NORMAL) {
            return pack((is.nx + (R)1) * (R)0.5f, (is.ny + (R)1) * (R)0.5f, (is.nz + (R)1) * (R)0.5f);
        } else if (type == DFPT_TEXTURE_UV) {
            return pack(is.u, is.v, (R)0);
        }
        return 0;
    }

    int texture(int to) const {
        const float* Tx = S.d->textures;
        if (jint(Tx[to]) == DFPT_TEXTURE_BLEND) {
            const int A = texture2(jint(Tx[to + 2])), B = texture2(jint(Tx[to + 3]));
            const R f = Tx[to + 4];
            return pack(((R)1 - f) * cr(A) + f * cr(B), ((R)1 - f) * cg(A) + f * cg(B), ((R)1 - f) * cb(A) + f * cb(B));
        }
        return texture2(to);
    }

    // ---- sky (GRK:2127-2236): Perez in FP64 as the reference ----
    void sky_color(R dX, R dY, R dZ) {
        const dfpt_sky* k = S.sky;
        R d0X = dX * (R)k->orthonormal_basis_u[0] + dY * (R)k->orthonormal_basis_u[1] + dZ * (R)k->orthonormal_basis_u[2];
        R d0Y = dX * (R)k->orthonormal_basis_v[0] + dY * (R)k->orthonormal_basis_v[1] + dZ * (R)k->orthonormal_basis_v[2];
        R d0Z = dX * (R)k->orthonormal_basis_w[0] + dY * (R)k->orthonormal_basis_w[1] + dZ * (R)k->orthonormal_basis_w[2];
        R r = (R)0.01f, g = (R)0.01f, b = (R)0.01f;
        if (d0Z >= (R)0 && k->is_sky_active == 1) {
            d0Z = jmax(d0Z, (R)0.001f);
            const R lr = jrsqrt(d0X * d0X + d0Y * d0Y + d0Z * d0Z);
            const R d1X = d0X * lr, d1Y = d0Y * lr, d1Z = d0Z * lr;
            const R dp = d1X * (R)k->sun_direction[0] + d1Y * (R)k->sun_direction[1] + d1Z * (R)k->sun_direction[2];
            const double theta0 = k->theta;
            const double theta1 = std::acos(std::max(std::min((double)d1Z, 1.0), -1.0));
            const double cos0 = std::cos(theta0), cos1 = std::cos(theta1);
            const double cos1r = 1.0 / (cos1 + 0.01);
            const double gamma = std::acos(std::max(std::min((double)dp, 1.0), -1.0));
            const double cosg = std::cos(gamma);
            const double* L = k->perez_relative_luminance;
            const double* X = k->perez_x;
            const double* Y = k->perez_y;
            const double den_l = ((1.0 + L[0] * std::exp(L[1])) * (1.0 + L[2] * std::exp(L[3] * theta0) + L[4] * cos0 * cos0));
            const double num_l = ((1.0 + L[0] * std::exp(L[1] * cos1r)) * (1.0 + L[2] * std::exp(L[3] * gamma) + L[4] * cosg * cosg));
            const double rel = k->zenith_relative_luminance * num_l / den_l * 1.0e-4;
            const double den_x = ((1.0 + X[0] * std::exp(X[1])) * (1.0 + X[2] * std::exp(X[3] * theta1) + X[4] * cos0 * cos0));
            const double num_x = ((1.0 + X[0] * std::exp(X[1] * cos1r)) * (1.0 + X[2] * std::exp(X[3] * gamma) + X[4] * cosg * cosg));
            const double x = k->zenith_x * num_x / den_x;
            const double den_y = ((1.0 + Y[0] * std::exp(Y[1])) * (1.0 + Y[2] * std::exp(Y[3] * theta1) + Y[4] * cos0 * cos0));
            const double num_y = ((1.0 + Y[0] * std::exp(Y[1] * cos1r)) * (1.0 + Y[2] * std::exp(Y[3] * gamma) + Y[4] * cosg * cosg));
            const double y = k->zenith_y * num_y / den_y;
            // The reference narrows x, y to float for the CIE step; the FP64 oracle keeps doubles.
            const R xf = (R)x, yf = (R)y;
            const R c0 = (R)1 / ((R)0.0241f + (R)0.2562f * xf - (R)0.7341f * yf);
            const R c1 = ((R)-1.3515f - (R)1.7703f * xf + (R)5.9114f * yf) * c0;
            const R c2 = ((R)0.03f - (R)31.4424f * xf + (R)30.0717f * yf) * c0;
            const R cX = (R)10246.121f + c1 * (R)187.75537f + c2 * (R)213.14803f;
            const R cY = (R)10676.695f + c1 * (R)192.59653f + c2 * (R)76.29494f;
            const R cZ = (R)12372.504f + c1 * (R)3482.8765f + c2 * (R)-235.71611f;
            const R cYr = (R)1 / cY;
            const R cR = (R)((double)cX * rel * (double)cYr), cG = (R)rel, cB = (R)((double)cZ * rel * (double)cYr);
            r = (R)3.2410042f * cR + (R)-1.5373994f * cG + (R)-0.49861607f * cB;
            g = (R)-0.9692241f * cR + (R)1.8759298f * cG + (R)0.041554242f * cB;
            b = (R)0.05563942f * cR + (R)-0.20401107f * cG + (R)1.0571486f * cB;
            const R w = jmax((R)0, -jmin((R)0, jmin(r, jmin(g, b))));
            r += w; g += w; b += w;
        }
        color[0] = r; color[1] = g; color[2] = b;
    }

    // ---- sun (GRK:2238-2347) ----
    void sun_color(bool active, R pX, R pY, R pZ, R nX, R nY, R nZ, R aR, R aG, R aB) {
        R r = 0, g = 0, b = 0;
        const dfpt_sky* k = S.sky;
        if (active) {
            const R sWX = k->sun_direction_world[0], sWY = k->sun_direction_world[1], sWZ = k->sun_direction_world[2];
            const R rad2 = (R)500 * (R)500;
            const R tX = (R)k->sun_origin[0] - pX, tY = (R)k->sun_origin[1] - pY, tZ = (R)k->sun_origin[2] - pZ;
            const R tl2 = tX * tX + tY * tY + tZ * tZ;
            const R u = nextf(), v = nextf();
            sun_drawn = true;
            sun_u = u; sun_v = v;
            const R sin2 = rad2 / tl2;
            const R cosMax = jsqrt(jmax((R)0, (R)1 - sin2));
            const R cosT = u * (cosMax - (R)1) + (R)1;
            const R sinT = jsqrt(jmax((R)0, (R)1 - cosT * cosT));
            const R phi = K<R>::TWO_PI() * v;
            const R x = jcos(phi) * sinT, y = jsin(phi) * sinT, z = cosT;
            const R aX = jabs(sWX), aY = jabs(sWY), aZ = jabs(sWZ);
            const R vX = aX < aY && aX < aZ ? (R)0 : aY < aZ ? sWZ : sWY;
            const R vY = aX < aY && aX < aZ ? sWZ : aY < aZ ? (R)0 : -sWX;
            const R vZ = aX < aY && aX < aZ ? -sWY : aY < aZ ? -sWX : (R)0;
            const R vl = jrsqrt(vX * vX + vY * vY + vZ * vZ);
            const R vnX = vX * vl, vnY = vY * vl, vnZ = vZ * vl;
            const R unX = vnY * sWZ - vnZ * sWY, unY = vnZ * sWX - vnX * sWZ, unZ = vnX * sWY - vnY * sWX;
            const R rX = unX * x + vnX * y + sWX * z, rY = unY * x + vnY * y + sWY * z, rZ = unZ * x + vnZ * y + sWZ * z;
            const R rl = jrsqrt(rX * rX + rY * rY + rZ * rZ);
            const R dX = rX * rl, dY = rY * rl, dZ = rZ * rl;
            const R dp0 = dX * sWX + dY * sWY + dZ * sWZ;
            const R dp1 = dX * nX + dY * nY + dZ * nZ;
            sun_dot = dp1;
            if (dp0 > (R)0 && dp1 > (R)0) {
                const R t = intersect(pX, pY, pZ, dX, dY, dZ, true);
                sun_seen = t >= K<R>::INF() - (R)0.0001f;
                if (t >= K<R>::INF() - (R)0.0001f) {
                    r = aR * (R)1 * dp1 * K<R>::INV_PI();
                    g = aG * (R)1 * dp1 * K<R>::INV_PI();
                    b = aB * (R)1 * dp1 * K<R>::INV_PI();
                }
            }
        }
        color[0] = r; color[1] = g; color[2] = b;
    }

    // ---- doRenderWithPathTracer (GRK:3151-3705) ----
    void path_trace(R* out, int gid, int* primitive_offsets) {
        const bool skyA = S.sky->is_sky_active == 1, sunA = S.sky->is_sun_active == 1;
        const int depthMax = S.p->pt_ray_depth_maximum, depthRR = S.p->pt_ray_depth_russian_roulette;
        int depth = 0;
        R oX = ray[0], oY = ray[1], oZ = ray[2], dX = ray[3], dY = ray[4], dZ = ray[5];
        R pR = 0, pG = 0, pB = 0, mR = 1, mG = 1, mB = 1;
        do {
            intersect(oX, oY, oZ, dX, dY, dZ, false);
            const R distance = is.distance;
            const int po = is.primitive_offset;
            if (depth == 0) primitive_offsets[gid] = po;
            if (distance == K<R>::INF() || po == -1) {
                sky_color(dX, dY, dZ);
                pR += mR * color[0] * K<R>::INV_PI(); pG += mG * color[1] * K<R>::INV_PI(); pB += mB * color[2] * K<R>::INV_PI();
                if (tape) {
                    tape->esc.push_back({depth, {(double)mR, (double)mG, (double)mB}, {(double)dX, (double)dY, (double)dZ}});
                    tape->contrib.push_back({depth, {(double)(mR * color[0] * K<R>::INV_PI()), (double)(mG * color[1] * K<R>::INV_PI()),
                                                     (double)(mB * color[2] * K<R>::INV_PI())}});
                }
                out[0] = pR; out[1] = pG; out[2] = pB;
                return;
            }
            const int so = S.d->primitives[po + 2];
            const R sX = is.px, sY = is.py, sZ = is.pz, nX = is.nx, nY = is.ny, nZ = is.nz;
            const R dp = nX * dX + nY * dY + nZ * dZ;
            const R dp2 = dp * (R)2;
            const bool correct = dp < (R)0;
            const R wX = correct ? nX : -nX, wY = correct ? nY : -nY, wZ = correct ? nZ : -nZ;
            const int aRGB = texture(jint(S.d->surfaces[so + 1]));
            R aR = cr(aRGB), aG = cg(aRGB), aB = cb(aRGB);
            const int eRGB = texture(jint(S.d->surfaces[so + 2]));
            R eR = cr(eRGB), eG = cg(eRGB), eB = cb(eRGB);
            const int material = jint(S.d->surfaces[so]);
            const R tR = aR, tG = aG, tB = aB;
            R exponent = (R)50;
            const int prim = po / 3;
            if (S.d->primitive_extensions) {
                // Per-primitive extension record {Phong exponent, emission scale r, g, b} (the
                // exponent PhongMaterial holds and SceneCompiler.java:760-768 drops; HDR emission).
                const float* x = S.d->primitive_extensions + 4 * (size_t)prim;
                exponent = (R)x[0];
                eR *= (R)x[1]; eG *= (R)x[2]; eB *= (R)x[3];
            }
            if (diff) {
                aR *= (R)diff->albedo[3 * prim]; aG *= (R)diff->albedo[3 * prim + 1]; aB *= (R)diff->albedo[3 * prim + 2];
                eR += (R)diff->emission[3 * prim]; eG += (R)diff->emission[3 * prim + 1]; eB += (R)diff->emission[3 * prim + 2];
                exponent = (R)diff->exponent[prim];
            }
            sun_drawn = sun_seen = false;
            if (material == DFPT_MATERIAL_CLEAR_COAT || material == DFPT_MATERIAL_LAMBERTIAN || material == DFPT_MATERIAL_PHONG) {
                sun_color(sunA, sX, sY, sZ, wX, wY, wZ, aR, aG, aB);
            } else {
                color[0] = color[1] = color[2] = 0;
            }
            pR += mR * (eR + color[0]); pG += mG * (eG + color[1]); pB += mB * (eB + color[2]);
            TapeVertex* tv = nullptr;
            if (tape) {
                TapeVertex x{};
                x.prim = prim;
                x.material = material;
                x.T[0] = (double)mR; x.T[1] = (double)mG; x.T[2] = (double)mB;
                x.tex[0] = (double)tR; x.tex[1] = (double)tG; x.tex[2] = (double)tB;
                x.a0[0] = (double)aR; x.a0[1] = (double)aG; x.a0[2] = (double)aB;
                x.sun = sun_drawn;
                x.sun_vis = sun_drawn && sun_seen && sun_dot > (R)0;
                x.sun_u = (double)sun_u; x.sun_v = (double)sun_v; x.sun_dot = (double)sun_dot;
                x.p[0] = (double)sX; x.p[1] = (double)sY; x.p[2] = (double)sZ;
                x.w[0] = (double)wX; x.w[1] = (double)wY; x.w[2] = (double)wZ;
                x.exponent = (double)exponent;
                x.alive = true;
                tape->v.push_back(x);
                tv = &tape->v.back();
                tape->contrib.push_back({depth, {(double)(mR * (eR + color[0])), (double)(mG * (eG + color[1])), (double)(mB * (eB + color[2]))}});
            }
            depth++;
            if (depth >= depthRR) {
                const R pdf = jmax(aR, jmax(aG, aB));
                const R rnd = nextf();
                if (rnd >= pdf) {
                    const bool hit = intersect(oX, oY, oZ, dX, dY, dZ, true) < K<R>::INF();
                    if (!hit) {
                        sky_color(dX, dY, dZ);
                        pR += mR * color[0] * K<R>::INV_PI(); pG += mG * color[1] * K<R>::INV_PI(); pB += mB * color[2] * K<R>::INV_PI();
                    }
                    if (tv) tv->alive = false;
                    out[0] = pR; out[1] = pG; out[2] = pB;
                    return;
                }
                const R pr = (R)1 / pdf;
                aR *= pr; aG *= pr; aB *= pr;
            }
            const R rX = dX - nX * dp2, rY = dY - nY * dp2, rZ = dZ - nZ * dp2;
            if (material == DFPT_MATERIAL_CLEAR_COAT) {
                const R a = (R)1.5f - (R)1, b = (R)1.5f + (R)1, c = (R)1 / (R)1.5f, e = (a * a) / (b * b);
                const R d0 = wX * dX + wY * dY + wZ * dZ;
                const R tir = (R)1 - c * c * ((R)1 - d0 * d0);
                if (tir < (R)0) {
                    oX = sX + wX * (R)0.02f; oY = sY + wY * (R)0.02f; oZ = sZ + wZ * (R)0.02f;
                    dX = rX; dY = rY; dZ = rZ;
                } else {
                    const R a1 = -d0, a2 = (R)1 - a1;
                    const R refl = e + ((R)1 - e) * a2 * a2 * a2 * a2 * a2;
                    const R trans = (R)1 - refl;
                    const R prob = (R)0.25f + (R)0.5f * refl;
                    const R rp = refl / prob, tp = trans / ((R)1 - prob);
                    const bool isR = nextf() < prob;
                    const R m = isR ? rp : tp;
                    mR *= m; mG *= m; mB *= m;
                    if (isR) {
                        oX = sX + wX * (R)0.02f; oY = sY + wY * (R)0.02f; oZ = sZ + wZ * (R)0.02f;
                        dX = rX; dY = rY; dZ = rZ;
                    } else {
                        cosine(wX, wY, wZ, dX, dY, dZ);
                        oX = sX + wX * (R)0.01f; oY = sY + wY * (R)0.01f; oZ = sZ + wZ * (R)0.01f;
                        mR *= aR; mG *= aG; mB *= aB;
                if (tv) tv->albedo_mult = true;
                    }
                }
            } else if (material == DFPT_MATERIAL_LAMBERTIAN) {
                cosine(wX, wY, wZ, dX, dY, dZ);
                oX = sX + wX * (R)0.01f; oY = sY + wY * (R)0.01f; oZ = sZ + wZ * (R)0.01f;
                mR *= aR; mG *= aG; mB *= aB;
                if (tv) tv->albedo_mult = true;
            } else if (material == DFPT_MATERIAL_PHONG) {
                const R u = nextf(), v = nextf();
                const R phi = K<R>::TWO_PI() * u;
                const R cosT = jpow((R)1 - v, (R)1 / (exponent + (R)1));
                if (tv) tv->phong_ct = (double)cosT;
                const R sinT = jsqrt(jmax((R)0, (R)1 - cosT * cosT));
                const R x = jcos(phi) * sinT, y = jsin(phi) * sinT, z = cosT;
                const R rl = jrsqrt(rX * rX + rY * rY + rZ * rZ);
                const R rnX = rX * rl, rnY = rY * rl, rnZ = rZ * rl;
                const bool isY = jabs(rnX) > (R)0.1f;
                const R uX = (isY ? (R)1 : (R)0) * rnZ, uY = -((isY ? (R)0 : (R)1) * rnZ), uZ = (isY ? (R)0 : (R)1) * rnY - (isY ? (R)1 : (R)0) * rnX;
                const R ul = jrsqrt(uX * uX + uY * uY + uZ * uZ);
                const R unX = uX * ul, unY = uY * ul, unZ = uZ * ul;
                const R vnX = rnY * unZ - rnZ * unY, vnY = rnZ * unX - rnX * unZ, vnZ = rnX * unY - rnY * unX;
                const R qX = unX * x + vnX * y + rX * z, qY = unY * x + vnY * y + rY * z, qZ = unZ * x + vnZ * y + rZ * z;
                const R ql = jrsqrt(qX * qX + qY * qY + qZ * qZ);
                oX = sX + rnX * (R)0.01f; oY = sY + rnY * (R)0.01f; oZ = sZ + rnZ * (R)0.01f;
                dX = qX * ql; dY = qY * ql; dZ = qZ * ql;
                mR *= aR; mG *= aG; mB *= aB;
                if (tv) tv->albedo_mult = true;
            } else if (material == DFPT_MATERIAL_GLASS) {
                const R a = (R)1.5f - (R)1, b = (R)1.5f + (R)1, c = (R)1 / (R)1.5f, dd = (R)1.5f / (R)1, e = (a * a) / (b * b);
                const bool in = nX * wX + nY * wY + nZ * wZ > (R)0;
                const R nnt = in ? c : dd;
                const R dw = wX * dX + wY * dY + wZ * dZ;
                const R tir = (R)1 - nnt * nnt * ((R)1 - dw * dw);
                if (tir < (R)0) {
                    oX = sX + wX * (R)0.01f; oY = sY + wY * (R)0.01f; oZ = sZ + wZ * (R)0.01f;
                    dX = rX; dY = rY; dZ = rZ;
                } else {
                    const R st = jsqrt(tir);
                    const R scl = in ? dw * nnt + st : -(dw * nnt + st);
                    const R t0X = dX * nnt - nX * scl, t0Y = dY * nnt - nY * scl, t0Z = dZ * nnt - nZ * scl;
                    const R tl = jrsqrt(t0X * t0X + t0Y * t0Y + t0Z * t0Z);
                    const R tdX = t0X * tl, tdY = t0Y * tl, tdZ = t0Z * tl;
                    const R a1 = in ? -dw : tdX * nX + tdY * nY + tdZ * nZ;
                    const R a2 = (R)1 - a1;
                    const R refl = e + ((R)1 - e) * a2 * a2 * a2 * a2 * a2;
                    const R trans = (R)1 - refl;
                    const R prob = (R)0.25f + (R)0.5f * refl;
                    const R rp = refl / prob, tp = trans / ((R)1 - prob);
                    const bool isR = nextf() < prob;
                    const R m = isR ? rp : tp;
                    mR *= m; mG *= m; mB *= m;
                    const R eps = isR ? (R)0.01f : (R)0.000001f;
                    oX = sX + wX * eps; oY = sY + wY * eps; oZ = sZ + wZ * eps;
                    dX = isR ? rX : tdX; dY = isR ? rY : tdY; dZ = isR ? rZ : tdZ;
                }
            } else if (material == DFPT_MATERIAL_REFLECTION) {
                oX = sX + nX * (R)0.000001f; oY = sY + nY * (R)0.000001f; oZ = sZ + nZ * (R)0.000001f;
                dX = rX; dY = rY; dZ = rZ;
                mR *= aR; mG *= aG; mB *= aB;
                if (tv) tv->albedo_mult = true;
            }
        } while (depth < depthMax);
        const bool hit = intersect(oX, oY, oZ, dX, dY, dZ, true) < K<R>::INF();
        if (!hit) {
            sky_color(dX, dY, dZ);
            pR += mR * color[0] * K<R>::INV_PI(); pG += mG * color[1] * K<R>::INV_PI(); pB += mB * color[2] * K<R>::INV_PI();
            if (tape) {
                tape->esc.push_back({depth, {(double)mR, (double)mG, (double)mB}, {(double)dX, (double)dY, (double)dZ}});
                tape->contrib.push_back({depth, {(double)(mR * color[0] * K<R>::INV_PI()), (double)(mG * color[1] * K<R>::INV_PI()),
                                                 (double)(mB * color[2] * K<R>::INV_PI())}});
            }
        }
        out[0] = pR; out[1] = pG; out[2] = pB;
    }

    void cosine(R wX, R wY, R wZ, R& dX, R& dY, R& dZ) {
        const R u = nextf(), v = nextf();
        const R phi = K<R>::TWO_PI() * u;
        const R cosT = jsqrt(v), sinT = jsqrt((R)1 - v);
        const R x = jcos(phi) * sinT, y = jsin(phi) * sinT, z = cosT;
        const bool isY = jabs(wX) > (R)0.1f;
        const R uX = (isY ? (R)1 : (R)0) * wZ, uY = -((isY ? (R)0 : (R)1) * wZ), uZ = (isY ? (R)0 : (R)1) * wY - (isY ? (R)1 : (R)0) * wX;
        const R ul = jrsqrt(uX * uX + uY * uY + uZ * uZ);
        const R unX = uX * ul, unY = uY * ul, unZ = uZ * ul;
        const R vnX = wY * unZ - wZ * unY, vnY = wZ * unX - wX * unZ, vnZ = wX * unY - wY * unX;
        const R lX = unX * x + vnX * y + wX * z, lY = unY * x + vnY * y + wY * z, lZ = unZ * x + vnZ * y + wZ * z;
        const R ll = jrsqrt(lX * lX + lY * lY + lZ * lZ);
        dX = lX * ll; dY = lY * ll; dZ = lZ * ll;
    }

    // doShaderPhongReflectionModel0 (GRK:1962-2039)
    int phong0(bool test, R pX, R pY, R pZ, R nX, R nY, R nZ, R vX, R vY, R vZ, R aR, R aG, R aB) {
        R r = 0, g = 0, b = 0;
        r += aR * (R)0.2f * (R)1; g += aG * (R)0.2f * (R)1; b += aB * (R)0.2f * (R)1;
        const dfpt_sky* k = S.sky;
        const R lX = (R)k->sun_origin[0] - pX, lY = (R)k->sun_origin[1] - pY, lZ = (R)k->sun_origin[2] - pZ;
        const R l2 = lX * lX + lY * lY + lZ * lZ;
        const R ll = jsqrt(l2);
        const R lr = (R)1 / ll;
        const R lnX = lX * lr, lnY = lY * lr, lnZ = lZ * lr;
        if (test) intersect(pX, pY, pZ, lnX, lnY, lnZ, false);
        const R t = test ? is.distance : K<R>::INF();
        if (t >= K<R>::INF() || t > l2) {
            const R ldn = lnX * nX + lnY * nY + lnZ * nZ;
            r += aR * (R)0.5f * jmax(ldn, (R)0) * (R)1; g += aG * (R)0.5f * jmax(ldn, (R)0) * (R)1; b += aB * (R)0.5f * jmax(ldn, (R)0) * (R)1;
            if (ldn > (R)0) {
                const R rX = (R)2 * ldn * nX - lnX, rY = (R)2 * ldn * nY - lnY, rZ = (R)2 * ldn * nZ - lnZ;
                const R rl = jrsqrt(rX * rX + rY * rY + rZ * rZ);
                const R rdv = rX * rl * vX + rY * rl * vY + rZ * rl * vZ;
                const R sh = jpow(jmax(rdv, (R)0), (R)250);
                r += (R)0.5f * sh * (R)1; g += (R)0.5f * sh * (R)1; b += (R)0.5f * sh * (R)1;
            }
        }
        r = saturate(r, (R)0, (R)1); g = saturate(g, (R)0, (R)1); b = saturate(b, (R)0, (R)1);
        return ((jint(r * (R)255 + (R)0.5f) & 0xFF) << 16) | ((jint(g * (R)255 + (R)0.5f) & 0xFF) << 8) | (jint(b * (R)255 + (R)0.5f) & 0xFF);
    }

    // The non-path-tracing renderers (GRK:2848-2908, 3029-3149, 3707-3996).
    void other(R* out, int gid, int* primitive_offsets) {
        const int mode = S.p->renderer_type;
        const bool skyA = S.sky->is_sky_active == 1;
        (void)skyA;
        R oX = ray[0], oY = ray[1], oZ = ray[2], dX = ray[3], dY = ray[4], dZ = ray[5];
        R pR = 0, pG = 0, pB = 0;
        if (mode == DFPT_RENDERER_RAY_MARCHER) {
            oY = height(oX, oZ) + (R)0.1f;
            const R maxT = jmax(oY, (R)1) * (R)20;
            sky_color(dX, dY, dZ);
            pR = color[0]; pG = color[1]; pB = color[2];
            R delT = (R)0.01f;
            for (R t = (R)0.001f; t < maxT; t += delT) {
                const R sX = oX + dX * t, sY = oY + dY * t, sZ = oZ + dZ * t;
                const R h = height(sX, sZ);
                if (sY < h) {
                    const R e = (R)0.02f;
                    const R nX = height(sX - e, sZ) - height(sX + e, sZ), nY = (R)2 * e, nZ = height(sX, sZ - e) - height(sX, sZ + e);
                    const R nl = (R)1 / jsqrt(nX * nX + nY * nY + nZ * nZ);
                    const R noise = fbm3((R)8, (R)0.5f, (R)0, (R)1, 16, sX, sY, sZ);
                    const R al = saturate(noise * (R)1 + (R)0.1f, (R)0, (R)1);
                    const int c = phong0(false, sX, sY, sZ, nX * nl, nY * nl, nZ * nl, -dX, -dY, -dZ, al, al, al);
                    pR = cr(c); pG = cg(c); pB = cb(c);
                    t = maxT;
                }
                delT = (R)0.01f * t;
            }
            out[0] = pR; out[1] = pG; out[2] = pB;
            return;
        }
        const int depthMax = mode == DFPT_RENDERER_RAY_TRACER ? 5 : 1;
        for (int depth = 0; depth < depthMax; ++depth) {
            intersect(oX, oY, oZ, dX, dY, dZ, false);
            const int po = is.primitive_offset;
            if (depth == 0) primitive_offsets[gid] = po;
            if (is.distance == K<R>::INF() || po == -1) {
                if (mode != DFPT_RENDERER_AMBIENT_OCCLUSION) {
                    sky_color(dX, dY, dZ);
                    pR += color[0]; pG += color[1]; pB += color[2];
                }
                break;
            }
            const R sX = is.px, sY = is.py, sZ = is.pz, nX = is.nx, nY = is.ny, nZ = is.nz;
            if (mode == DFPT_RENDERER_SURFACE_NORMALS) {
                pR = (nX + (R)1) * (R)0.5f; pG = (nY + (R)1) * (R)0.5f; pB = (nZ + (R)1) * (R)0.5f;
                break;
            }
            const R dp = nX * dX + nY * dY + nZ * dZ;
            const bool correct = dp < (R)0;
            const R wX = correct ? nX : -nX, wY = correct ? nY : -nY, wZ = correct ? nZ : -nZ;
            if (mode == DFPT_RENDERER_AMBIENT_OCCLUSION) {
                const R wl = jrsqrt(wX * wX + wY * wY + wZ * wZ);
                const R w1X = wX * wl, w1Y = wY * wl, w1Z = wZ * wl;
                const bool isY = jabs(w1X) > (R)0.1f;
                const R u0X = isY ? (R)0 : (R)1, u0Y = isY ? (R)1 : (R)0;
                const R u1X = u0Y * w1Z, u1Y = -(u0X * w1Z), u1Z = u0X * w1Y - u0Y * w1X;
                const R ul = jrsqrt(u1X * u1X + u1Y * u1Y + u1Z * u1Z);
                const R u2X = u1X * ul, u2Y = u1Y * ul, u2Z = u1Z * ul;
                const R v0X = w1Y * u2Z - w1Z * u2Y, v0Y = w1Z * u2X - w1X * u2Z, v0Z = w1X * u2Y - w1Y * u2X;
                const R xi = nextf(), xj = nextf();
                const R phi = K<R>::TWO_PI() * xi;
                const R cp = jcos(phi), sp = jsin(phi), sth = jsqrt(xj), cth = jsqrt((R)1 - xj);
                const R e0X = cp * sth, e0Y = sp * sth, e0Z = cth;
                const R e1X = e0X * u2X + e0Y * v0X + e0Z * w1X, e1Y = e0X * u2Y + e0Y * v0Y + e0Z * w1Y, e1Z = e0X * u2Z + e0Y * v0Z + e0Z * w1Z;
                const R el = jrsqrt(e1X * e1X + e1Y * e1Y + e1Z * e1Z);
                const R t = intersect(sX + w1X * (R)0.01f, sY + w1Y * (R)0.01f, sZ + w1Z * (R)0.01f, e1X * el, e1Y * el, e1Z * el, false);
                const bool hit = t < (R)S.p->ao_maximum_distance;
                const R v = hit ? (R)1 : (R)0;
                pR += ((R)1 - v) * (R)1 + v * (R)0; pG += ((R)1 - v) * (R)1 + v * (R)0; pB += ((R)1 - v) * (R)1 + v * (R)0;
                break;
            }
            const int so = S.d->primitives[po + 2];
            const int aRGB = texture(jint(S.d->surfaces[so + 1]));
            R aR, aG, aB;
            if (mode == DFPT_RENDERER_RAY_TRACER) {
                aR = ((aRGB >> 16) & 0xFF) / (R)255; aG = ((aRGB >> 8) & 0xFF) / (R)255; aB = (aRGB & 0xFF) / (R)255;
            } else {
                aR = cr(aRGB); aG = cg(aRGB); aB = cb(aRGB);
            }
            // The shadow test below overwrites the intersection record (GRK:1993).
            const int c = phong0(true, sX, sY, sZ, wX, wY, wZ, -dX, -dY, -dZ, aR, aG, aB);
            if (mode == DFPT_RENDERER_RAY_CASTER) {
                pR = cr(c); pG = cg(c); pB = cb(c);
                break;
            }
            pR += cr(c); pG += cg(c); pB += cb(c);
            if (jint(S.d->surfaces[so]) != DFPT_MATERIAL_REFLECTION) break;
            const R dp2 = dp * (R)2;
            oX = sX + nX * (R)0.000001f; oY = sY + nY * (R)0.000001f; oZ = sZ + nZ * (R)0.000001f;
            dX = dX - nX * dp2; dY = dY - nY * dp2; dZ = dZ - nZ * dp2;
        }
        out[0] = pR; out[1] = pG; out[2] = pB;
    }

    // Wireframe overlay (GRK:2910-3027): true when the pixel is set to black.
    bool wireframe() {
        intersect(ray[0], ray[1], ray[2], ray[3], ray[4], ray[5], false);
        const R lineCos = jcos(K<R>::PI() * (R)0.5f / (R)4096);
        if (is.distance != K<R>::INF() && is.primitive_offset != -1 && is.shape_type == DFPT_SHAPE_TRIANGLE) {
            const float* cam = S.d->camera;
            const R uX = cam[7], uY = cam[8], uZ = cam[9], vX = cam[10], vY = cam[11], vZ = cam[12], wX = cam[13], wY = cam[14], wZ = cam[15];
            const R spX = is.px * uX + is.py * uY + is.pz * uZ, spY = is.px * vX + is.py * vY + is.pz * vZ, spZ = is.px * wX + is.py * wY + is.pz * wZ;
            const R spN = jrsqrt(spX * spX + spY * spY + spZ * spZ);
            R P[3][3];
            for (int k = 0; k < 3; ++k) {
                const int o = S.d->triangles[is.shape_offset + k];
                const R x = S.p3(o), y = S.p3(o + 1), z = S.p3(o + 2);
                P[k][0] = x * uX + y * uY + z * uZ; P[k][1] = x * vX + y * vY + z * vZ; P[k][2] = x * wX + y * wY + z * wZ;
            }
            const int from[3] = {0, 1, 2}, to[3] = {2, 0, 1};
            bool edge = false;
            for (int e = 0; e < 3; ++e) {
                const R* F = P[from[e]];
                const R* T = P[to[e]];
                const R ds = ((F[0] - T[0]) * (F[0] - T[0])) + ((F[1] - T[1]) * (F[1] - T[1])) + ((F[2] - T[2]) * (F[2] - T[2]));
                const R t0 = ((spX - F[0]) * (T[0] - F[0])) + ((spY - F[1]) * (T[1] - F[1])) + ((spZ - F[2]) * (T[2] - F[2]));
                const R t1 = t0 / ds;
                const R qX = ((R)1 - t1) * F[0] + t1 * T[0], qY = ((R)1 - t1) * F[1] + t1 * T[1], qZ = ((R)1 - t1) * F[2] + t1 * T[2];
                const R qN = jrsqrt(qX * qX + qY * qY + qZ * qZ);
                const R dpq = qX * spX + qY * spY + qZ * spZ;
                if (dpq * qN * spN >= lineCos) edge = true;
            }
            return edge;
        }
        return false;
    }
};

template <typename R>
struct Film {
    // filmAddColor / filmSetColor (AIK:333-378), the reference's running average.
    static void add(R* f, int* n, R r, R g, R b, bool clear) {
        if (clear || *n == 0) { f[0] = r; f[1] = g; f[2] = b; *n = 1; return; }
        const int nn = *n + 1;
        f[0] = f[0] + ((r - f[0]) / (R)nn);
        f[1] = f[1] + ((g - f[1]) / (R)nn);
        f[2] = f[2] + ((b - f[2]) / (R)nn);
        *n = nn;
    }
};

// Tone map + redo gamma + BGRA8 (GRK:282-307, AIK:410-472, 503-534, 702-774), in R.
template <typename R>
void resolve(const dfpt_params* p, const R* film, int po, uint8_t* bgra) {
    R r = film[0], g = film[1], b = film[2];
    g += (po > -1 && po == p->selected_primitive_offset) ? (R)1 : (R)0;
    const R ex = p->tone_mapper_exposure;
    auto filmic = [&](R v) {
        const R m = jmax(v * ex - (R)0, (R)-3.402823466e+38f);
        const R q = (m * ((R)2.51f * m + (R)0.03f)) / (m * ((R)2.43f * m + (R)0.59f) + (R)0.14f);
        return q < (R)0 ? (R)0 : q > (R)1 ? (R)1 : q;
    };
    if (p->tone_mapper_type == DFPT_TONE_MAPPER_REINHARD) {
        r = (r * ex) / ((R)1 + r * ex); g = (g * ex) / ((R)1 + g * ex); b = (b * ex) / ((R)1 + b * ex);
    } else if (p->tone_mapper_type == DFPT_TONE_MAPPER_REINHARD_MODIFIED_1) {
        r = (R)1 - jexp(-r * ex); g = (R)1 - jexp(-g * ex); b = (R)1 - jexp(-b * ex);
    } else if (p->tone_mapper_type == DFPT_TONE_MAPPER_REINHARD_MODIFIED_2) {
        const R lw = (R)1 / ((R)4 * (R)4);
        const R rm = r * ex, gm = g * ex, bm = b * ex;
        r = rm * ((R)1 + rm * lw) / ((R)1 + rm); g = gm * ((R)1 + gm * lw) / ((R)1 + gm); b = bm * ((R)1 + bm * lw) / ((R)1 + bm);
    } else if (p->tone_mapper_type == DFPT_TONE_MAPPER_FILMIC_CURVE_ACES_MODIFIED) {
        r = filmic(r); g = filmic(g); b = filmic(b);
    }
    // RGBColorSpace.SRGB (image4j RGBColorSpace.java:77, 283-293): breakPoint 0.00304, gamma 2.4.
    const float bp = 0.00304f, gm = 2.4f;
    const float pe = (float)std::pow((double)bp, (double)(1.0f / gm - 1.0f));
    const float slope = 1.0f / (gm / pe - gm * bp + bp);
    const float match = gm * slope / pe;
    const float seg = match * (float)std::pow((double)bp, (double)(1.0f / gm)) - slope * bp;
    auto redo = [&](R v) {
        return v <= (R)0 ? (R)0 : v >= (R)1 ? (R)1 : v <= (R)bp ? v * (R)slope : (R)match * jpow(v, (R)1 / (R)gm) - (R)seg;
    };
    r = redo(r); g = redo(g); b = redo(b);
    auto q = [](R v) { return jint(jmax(jmin(v * (R)255 + (R)0.5f, (R)255), (R)0)); };
    bgra[0] = (uint8_t)q(b); bgra[1] = (uint8_t)q(g); bgra[2] = (uint8_t)q(r); bgra[3] = 255;
}

struct Outputs {
    double* film;  // W*H*3 running average (in R, stored as double)
    double* sum;   // per-pixel sum of pass radiance
    double* sumsq; // per-pixel sum of squares
    int* primitive_offsets;
    uint8_t* bgra;
    int* hit_prim;
    int* hit_type;
    int* hit_off;
    double* hit_dist;
    double* hit_normal;
    uint64_t* rng_state;
    uint64_t* counters;
};

template <typename R>
void render_rows(const Scene& S, int pass_begin, int passes, int row_begin, int row_end, Outputs& o, std::vector<R>& film,
                 std::vector<int>& n, Counters& total) {
    Kernel<R> k(S);
    const dfpt_params* p = S.p;
    const bool pt = !(p->renderer_type >= 1 && p->renderer_type <= 6) || p->renderer_type == DFPT_RENDERER_PATH_TRACER;
    for (int pass = pass_begin; pass < pass_begin + passes; ++pass) {
        for (int y = row_begin; y < row_end; ++y) {
            for (int x = 0; x < S.width; ++x) {
                const int gid = y * S.width + x;
                k.rng.kind = p->rng_kind;
                k.rng.pixel = (uint32_t)gid;
                k.rng.pass = (uint32_t)pass;
                k.rng.seed_lo = (uint32_t)p->seed;
                k.rng.seed_hi = (uint32_t)(p->seed >> 32);
                k.rng.draws = 0;
                k.rng.lcg = o.rng_state ? o.rng_state[gid] : 0;
                R c[3] = {0, 0, 0};
                bool set_black = false;
                if (k.create_primary_ray(gid)) {
                    if (pt) k.path_trace(c, gid, o.primitive_offsets);
                    else k.other(c, gid, o.primitive_offsets);
                    if (pass == pass_begin + passes - 1 && o.hit_prim) {
                        // The primary-hit record of the last pass, re-traced without RNG draws.
                        k.intersect(k.ray[0], k.ray[1], k.ray[2], k.ray[3], k.ray[4], k.ray[5], false);
                        o.hit_prim[gid] = k.is.primitive_offset;
                        o.hit_type[gid] = k.is.primitive_offset >= 0 ? k.is.shape_type : -1;
                        o.hit_off[gid] = k.is.primitive_offset >= 0 ? k.is.shape_offset : -1;
                        o.hit_dist[gid] = (double)k.is.distance;
                        if (k.is.primitive_offset >= 0) {
                            o.hit_normal[3 * gid] = (double)k.is.nx; o.hit_normal[3 * gid + 1] = (double)k.is.ny; o.hit_normal[3 * gid + 2] = (double)k.is.nz;
                        }
                    }
                    if (p->wireframes == 1) set_black = k.wireframe();
                } else {
                    set_black = true;
                }
                if (o.rng_state) o.rng_state[gid] = k.rng.lcg;
                R* f = film.data() + 3 * (size_t)gid;
                if (set_black) { f[0] = f[1] = f[2] = 0; n[gid] = 1; }
                else Film<R>::add(f, &n[gid], c[0], c[1], c[2], pass == pass_begin);
                if (o.sum) {
                    for (int ch = 0; ch < 3; ++ch) {
                        const double v = set_black ? 0.0 : (double)c[ch];
                        o.sum[3 * (size_t)gid + ch] += v;
                        o.sumsq[3 * (size_t)gid + ch] += v * v;
                    }
                }
                if (pass == pass_begin + passes - 1 && o.bgra) resolve<R>(p, f, o.primitive_offsets[gid], o.bgra + 4 * (size_t)gid);
            }
        }
    }
    total.closest += k.cnt.closest;
    total.any += k.cnt.any;
    total.nodes += k.cnt.nodes;
    total.tris += k.cnt.tris;
    total.closest_nodes += k.cnt.closest_nodes;
    total.closest_tris += k.cnt.closest_tris;
}

template <typename R>
int render(const Scene& S, int pass_begin, int passes, int threads, int row_begin, int row_end, Outputs& o) {
    const size_t np = (size_t)S.width * S.height;
    std::vector<R> film(np * 3, (R)0);
    std::vector<int> n(np, 0);
    if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next_row(row_begin);
    std::vector<Counters> counters((size_t)threads);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&, t]() {
            for (;;) {
                const int y = next_row.fetch_add(1);
                if (y >= row_end) break;
                render_rows<R>(S, pass_begin, passes, y, y + 1, o, film, n, counters[t]);
            }
        });
    }
    for (auto& th : pool) th.join();
    for (size_t i = (size_t)row_begin * S.width; i < (size_t)row_end * S.width; ++i)
        for (int c = 0; c < 3; ++c) o.film[3 * i + c] = (double)film[3 * i + c];
    if (o.counters) {
        for (auto& c : counters) {
            o.counters[0] += c.closest; o.counters[1] += c.any; o.counters[2] += c.nodes; o.counters[3] += c.tris;
            o.counters[4] += c.closest_nodes; o.counters[5] += c.closest_tris;
        }
    }
    return 0;
}

// ---- FP64 host adjoint -------------------------------------------------------------------------
// Dual numbers over (turbidity, sun x, sun y, sun z) carry the sky and sun terms' derivatives
// straight from Sky.set's inputs (Sky.java:295-333) through the Perez model and the sun sample.

struct Dual {
    double v, d[4];
};
Dual dc(double v) { return Dual{v, {0, 0, 0, 0}}; }
Dual operator+(Dual a, Dual b) { Dual r{a.v + b.v, {}}; for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] + b.d[j]; return r; }
Dual operator-(Dual a, Dual b) { Dual r{a.v - b.v, {}}; for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] - b.d[j]; return r; }
Dual operator-(Dual a) { Dual r{-a.v, {}}; for (int j = 0; j < 4; ++j) r.d[j] = -a.d[j]; return r; }
Dual operator*(Dual a, Dual b) { Dual r{a.v * b.v, {}}; for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] * b.v + a.v * b.d[j]; return r; }
Dual operator/(Dual a, Dual b) { Dual r{a.v / b.v, {}}; for (int j = 0; j < 4; ++j) r.d[j] = (a.d[j] * b.v - a.v * b.d[j]) / (b.v * b.v); return r; }
Dual operator+(Dual a, double b) { return a + dc(b); }
Dual operator+(double a, Dual b) { return dc(a) + b; }
Dual operator-(Dual a, double b) { return a - dc(b); }
Dual operator-(double a, Dual b) { return dc(a) - b; }
Dual operator*(Dual a, double b) { return a * dc(b); }
Dual operator*(double a, Dual b) { return dc(a) * b; }
Dual operator/(double a, Dual b) { return dc(a) / b; }
Dual operator/(Dual a, double b) { return a / dc(b); }
Dual fn(Dual a, double v, double slope) { Dual r{v, {}}; for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] * slope; return r; }
Dual dexp(Dual a) { const double e = std::exp(a.v); return fn(a, e, e); }
Dual dsqrt(Dual a) { const double s = std::sqrt(std::max(a.v, 0.0)); return fn(a, s, s > 0 ? 0.5 / s : 0.0); }
Dual dtan(Dual a) { const double t = std::tan(a.v); return fn(a, t, 1.0 + t * t); }
Dual dacos(Dual a) {
    const double c = std::max(-1.0, std::min(1.0, a.v));
    const double s = std::sqrt(std::max(0.0, 1.0 - c * c));
    return fn(a, std::acos(c), (a.v > -1.0 && a.v < 1.0 && s > 1e-12) ? -1.0 / s : 0.0);
}
Dual dclamp(Dual a, double lo, double hi) { return a.v < lo ? dc(lo) : a.v > hi ? dc(hi) : a; }

struct SunDual {
    Dual w[3];       // world sun direction (normalised)
    Dual sky[3];     // sky-frame sun direction (u = X, v = Z, w = Y)
    Dual theta, zl, zx, zy, L[5], X[5], Y[5];
};

SunDual sky_set_dual(double turbidity, const double* s) {
    SunDual r;
    Dual t{turbidity, {1, 0, 0, 0}};
    Dual sx{s[0], {0, 1, 0, 0}}, sy{s[1], {0, 0, 1, 0}}, sz{s[2], {0, 0, 0, 1}};
    const Dual len = dsqrt(sx * sx + sy * sy + sz * sz);
    r.w[0] = sx / len; r.w[1] = sy / len; r.w[2] = sz / len;
    const Dual a = r.w[0], b = r.w[2], c = r.w[1];
    const Dual l2 = dsqrt(a * a + b * b + c * c);
    r.sky[0] = a / l2; r.sky[1] = b / l2; r.sky[2] = c / l2;
    r.theta = dacos(dclamp(r.sky[2], -1.0, 1.0));
    const Dual th = r.theta, th2 = th * th, th3 = th2 * th, t2 = t * t;
    const double pi_f = (double)3.14159274101257324219f;
    const Dual chi = (4.0 / 9.0 - t * (1.0 / 120.0)) * (pi_f - 2.0 * th);
    r.zl = ((4.0453 * t - 4.9710) * dtan(chi) - 0.2155 * t + 2.4192) * 1000.0;
    r.zx = (0.00165 * th3 - 0.00374 * th2 + 0.00208 * th) * t2 + (-0.02902 * th3 + 0.06377 * th2 - 0.03202 * th + 0.00394) * t +
           (0.11693 * th3 - 0.21196 * th2 + 0.06052 * th + 0.25885);
    r.zy = (0.00275 * th3 - 0.00610 * th2 + 0.00316 * th) * t2 + (-0.04212 * th3 + 0.08970 * th2 - 0.04153 * th + 0.00515) * t +
           (0.15346 * th3 - 0.26756 * th2 + 0.06669 * th + 0.26688);
    const double Lc[5][2] = {{0.17872, -1.46303}, {-0.35540, 0.42749}, {-0.02266, 5.32505}, {0.12064, -2.57705}, {-0.06696, 0.37027}};
    const double Xc[5][2] = {{-0.01925, -0.25922}, {-0.06651, 0.00081}, {-0.00041, 0.21247}, {-0.06409, -0.89887}, {-0.00325, 0.04517}};
    const double Yc[5][2] = {{-0.01669, -0.26078}, {-0.09495, 0.00921}, {-0.00792, 0.21023}, {-0.04405, -1.65369}, {-0.01092, 0.05291}};
    for (int i = 0; i < 5; ++i) {
        r.L[i] = Lc[i][0] * t + Lc[i][1];
        r.X[i] = Xc[i][0] * t + Xc[i][1];
        r.Y[i] = Yc[i][0] * t + Yc[i][1];
    }
    return r;
}

// The FP64 sky color of a direction (the R = double sky_color above) as duals.
void sky_color_dual(const SunDual& k, bool active, double dX, double dY, double dZ, Dual out[3]) {
    double d0X = dX, d0Y = dZ, d0Z = dY;  // basis u = X, v = Z, w = Y
    out[0] = out[1] = out[2] = dc((double)0.01f);
    if (!(d0Z >= 0.0 && active)) return;
    d0Z = std::max(d0Z, (double)0.001f);
    const double lr = 1.0 / std::sqrt(d0X * d0X + d0Y * d0Y + d0Z * d0Z);
    const double d1X = d0X * lr, d1Y = d0Y * lr, d1Z = d0Z * lr;
    const Dual dp = d1X * k.sky[0] + d1Y * k.sky[1] + d1Z * k.sky[2];
    const double theta1 = std::acos(std::max(std::min(d1Z, 1.0), -1.0));
    const double cos1 = std::cos(theta1), cos1r = 1.0 / (cos1 + 0.01);
    const Dual cos0 = fn(k.theta, std::cos(k.theta.v), -std::sin(k.theta.v));
    const Dual gamma = dacos(dp);
    const Dual cosg = dclamp(dp, -1.0, 1.0);
    const Dual* L = k.L;
    const Dual* X = k.X;
    const Dual* Y = k.Y;
    const Dual den_l = (1.0 + L[0] * dexp(L[1])) * (1.0 + L[2] * dexp(L[3] * k.theta) + L[4] * cos0 * cos0);
    const Dual num_l = (1.0 + L[0] * dexp(L[1] * cos1r)) * (1.0 + L[2] * dexp(L[3] * gamma) + L[4] * cosg * cosg);
    const Dual rel = k.zl * num_l / den_l * 1.0e-4;
    const Dual den_x = (1.0 + X[0] * dexp(X[1])) * (1.0 + X[2] * dexp(X[3] * theta1) + X[4] * cos0 * cos0);
    const Dual num_x = (1.0 + X[0] * dexp(X[1] * cos1r)) * (1.0 + X[2] * dexp(X[3] * gamma) + X[4] * cosg * cosg);
    const Dual x = k.zx * num_x / den_x;
    const Dual den_y = (1.0 + Y[0] * dexp(Y[1])) * (1.0 + Y[2] * dexp(Y[3] * theta1) + Y[4] * cos0 * cos0);
    const Dual num_y = (1.0 + Y[0] * dexp(Y[1] * cos1r)) * (1.0 + Y[2] * dexp(Y[3] * gamma) + Y[4] * cosg * cosg);
    const Dual y = k.zy * num_y / den_y;
    const Dual c0 = 1.0 / ((double)0.0241f + (double)0.2562f * x - (double)0.7341f * y);
    const Dual c1 = ((double)-1.3515f - (double)1.7703f * x + (double)5.9114f * y) * c0;
    const Dual c2 = ((double)0.03f - (double)31.4424f * x + (double)30.0717f * y) * c0;
    const Dual cX = (double)10246.121f + c1 * (double)187.75537f + c2 * (double)213.14803f;
    const Dual cY = (double)10676.695f + c1 * (double)192.59653f + c2 * (double)76.29494f;
    const Dual cZ = (double)12372.504f + c1 * (double)3482.8765f + c2 * (double)-235.71611f;
    const Dual R = cX * rel / cY, G = rel, B = cZ * rel / cY;
    out[0] = (double)3.2410042f * R + (double)-1.5373994f * G + (double)-0.49861607f * B;
    out[1] = (double)-0.9692241f * R + (double)1.8759298f * G + (double)0.041554242f * B;
    out[2] = (double)0.05563942f * R + (double)-0.20401107f * G + (double)1.0571486f * B;
    const int m = out[0].v <= out[1].v && out[0].v <= out[2].v ? 0 : out[1].v <= out[2].v ? 1 : 2;
    if (out[m].v < 0.0) {
        const Dual w = out[m];
        for (int c = 0; c < 3; ++c) out[c] = out[c] - w;
    }
}

// The sun term's derivative over the rim of the sun's cone, visibility included (the estimator of the
// GPU replay, here in FP64 with FP64 shadow rays): the cone of directions towards the sun's disk has
// axis W and half-angle a, sin^2 a = 500^2 / |origin - p|^2 (GRK:2238-2347); for the mean of
// G(w) = c max(w.n, 0) V(w) over it, d/dq = E_phi[(G(w_phi) - k) (w_phi.dW/dq - d cos a/dq) / (1 - cos a)]
// for a rim direction at uniform angle phi and k = the forward sample's G (Reynolds transport over
// the moving cone; k's mean is G's mean). phi: Philox4x32-10 at counter (pass, 2^30 + bounce,
// seed_hi, "RIM!"), key (pixel, seed_lo), its first word.
void sun_rim_dual(Kernel<double>& k, const SunDual& sd, const dfpt_sky* sky, uint32_t pixel, uint32_t pass, uint32_t seed_lo,
                  uint32_t seed_hi, int bounce, const double* p, const double* n, double c, double g_forward, double* gsky) {
    const Dual tX = sd.w[0] * 10000.0 - p[0], tY = sd.w[1] * 10000.0 - p[1], tZ = sd.w[2] * 10000.0 - p[2];
    const double oX = (double)sky->sun_origin[0] - p[0], oY = (double)sky->sun_origin[1] - p[1], oZ = (double)sky->sun_origin[2] - p[2];
    const double sin2 = (500.0 * 500.0) / (oX * oX + oY * oY + oZ * oZ);
    if (!(sin2 > 0.0 && sin2 < 1.0)) return;
    const Dual cosA = dsqrt(1.0 - (500.0 * 500.0) / (tX * tX + tY * tY + tZ * tZ));
    const double cos_a = std::sqrt(1.0 - sin2), sin_a = std::sqrt(sin2), one_m_cos = sin2 / (1.0 + cos_a);
    uint32_t cnt[4] = {pass, 0x40000000u | (uint32_t)bounce, seed_hi, 0x52494D21u};
    philox(cnt, pixel, seed_lo);
    const double phi = (double)(3.14159274101257324219f * 2.0f) * ((double)(cnt[0] >> 8) * (1.0 / 16777216.0));
    const double wX = sky->sun_direction_world[0], wY = sky->sun_direction_world[1], wZ = sky->sun_direction_world[2];
    const double aX = std::fabs(wX), aY = std::fabs(wY), aZ = std::fabs(wZ);
    const double vX = aX < aY && aX < aZ ? 0.0 : aY < aZ ? wZ : wY;
    const double vY = aX < aY && aX < aZ ? wZ : aY < aZ ? 0.0 : -wX;
    const double vZ = aX < aY && aX < aZ ? -wY : aY < aZ ? -wX : 0.0;
    const double vl = 1.0 / std::sqrt(vX * vX + vY * vY + vZ * vZ);
    const double vnX = vX * vl, vnY = vY * vl, vnZ = vZ * vl;
    const double unX = vnY * wZ - vnZ * wY, unY = vnZ * wX - vnX * wZ, unZ = vnX * wY - vnY * wX;
    const double x = std::cos(phi) * sin_a, y = std::sin(phi) * sin_a, z = cos_a;
    double rX = unX * x + vnX * y + wX * z, rY = unY * x + vnY * y + wY * z, rZ = unZ * x + vnZ * y + wZ * z;
    const double rl = 1.0 / std::sqrt(rX * rX + rY * rY + rZ * rZ);
    rX *= rl; rY *= rl; rZ *= rl;
    const double dot0 = rX * wX + rY * wY + rZ * wZ, dot1 = rX * n[0] + rY * n[1] + rZ * n[2];
    double g_rim = 0.0;
    if (dot0 > 0.0 && dot1 > 0.0 && c != 0.0) {
        const double t = k.intersect(p[0], p[1], p[2], rX, rY, rZ, true);
        if (t >= K<double>::INF() - 0.0001) g_rim = c * dot1;
    }
    const double q = (g_rim - g_forward) / one_m_cos;
    for (int j = 0; j < 4; ++j) gsky[j] += q * (rX * sd.w[0].d[j] + rY * sd.w[1].d[j] + rZ * sd.w[2].d[j] - cosA.d[j]);
}

// Renders with the parameters in FP64 and computes d(sum w * image)/d(parameters) by recording
// each path's vertices and sweeping them (explicit sums of the later contributions).
void diff_rows(const Scene& S, const DiffIn& din, const SunDual& sd, int pass_begin, int passes, int row_begin, int row_end,
               const double* dldi, double* image, std::vector<double>& grad) {
    Kernel<double> k(S);
    k.diff = &din;
    Tape tape;
    k.tape = &tape;
    const dfpt_params* p = S.p;
    const int np = (int)(S.d->primitives_count / 3);
    const double inv_pi = (double)(1.0f / 3.14159274101257324219f);
    const bool sky_on = S.sky->is_sky_active == 1;
    for (int y = row_begin; y < row_end; ++y) {
        for (int x = 0; x < S.width; ++x) {
            const int gid = y * S.width + x;
            double acc[3] = {0, 0, 0};
            const double w[3] = {dldi[3 * gid] / passes, dldi[3 * gid + 1] / passes, dldi[3 * gid + 2] / passes};
            for (int pass = pass_begin; pass < pass_begin + passes; ++pass) {
                k.rng.kind = p->rng_kind;
                k.rng.pixel = (uint32_t)gid;
                k.rng.pass = (uint32_t)pass;
                k.rng.seed_lo = (uint32_t)p->seed;
                k.rng.seed_hi = (uint32_t)(p->seed >> 32);
                k.rng.draws = 0;
                k.rng.lcg = 0;
                tape.clear();
                double c[3] = {0, 0, 0};
                if (!k.create_primary_ray(gid)) continue;
                int first_hit = -1;
                k.path_trace(c, 0, &first_hit);
                for (int ch = 0; ch < 3; ++ch) acc[ch] += c[ch];
                // Reverse sweep over the record.
                for (size_t vi = 0; vi < tape.v.size(); ++vi) {
                    const TapeVertex& v = tape.v[vi];
                    double later[3] = {0, 0, 0};
                    for (auto& ct : tape.contrib)
                        if (ct.first > (int)vi)
                            for (int ch = 0; ch < 3; ++ch) later[ch] += ct.second[ch];
                    double* g = grad.data() + (size_t)v.prim * 7;
                    for (int ch = 0; ch < 3; ++ch) g[3 + ch] += w[ch] * v.T[ch];
                    if (v.sun) {
                        const double cw = (w[0] * v.T[0] * v.a0[0] + w[1] * v.T[1] * v.a0[1] + w[2] * v.T[2] * v.a0[2]) * inv_pi;
                        if (v.sun_vis)
                            for (int ch = 0; ch < 3; ++ch) g[ch] += w[ch] * v.T[ch] * v.tex[ch] * v.sun_dot * inv_pi;
                        sun_rim_dual(k, sd, S.sky, (uint32_t)gid, (uint32_t)pass, (uint32_t)p->seed, (uint32_t)(p->seed >> 32), (int)vi,
                                     v.p, v.w, cw, v.sun_vis ? cw * v.sun_dot : 0.0, grad.data() + (size_t)np * 7);
                    }
                    if (v.alive && v.albedo_mult)
                        for (int ch = 0; ch < 3; ++ch)
                            if (v.a0[ch] != 0.0) g[ch] += w[ch] * later[ch] * v.tex[ch] / v.a0[ch];
                    if (v.alive && v.material == DFPT_MATERIAL_PHONG && v.phong_ct > 0.0)
                        g[6] += (w[0] * later[0] + w[1] * later[1] + w[2] * later[2]) * (1.0 / (v.exponent + 1.0) + std::log(v.phong_ct));
                }
                for (const TapeEscape& e : tape.esc) {
                    Dual sc[3];
                    sky_color_dual(sd, sky_on, e.d[0], e.d[1], e.d[2], sc);
                    for (int j = 0; j < 4; ++j)
                        grad[(size_t)np * 7 + j] += (w[0] * e.T[0] * sc[0].d[j] + w[1] * e.T[1] * sc[1].d[j] + w[2] * e.T[2] * sc[2].d[j]) * inv_pi;
                }
            }
            for (int ch = 0; ch < 3; ++ch) image[3 * gid + ch] = acc[ch] / passes;
        }
    }
}

}  // namespace

extern "C" {

// Renders `passes` passes starting at pass index `pass_begin` (the film starts cleared) over rows
// [row_begin, row_end) with `threads` host threads, in FP32 strict (precision 32) or FP64 (64).
// Any output pointer except `film` may be NULL; `rng_state` holds the per-pixel LCG states.
int oracle_render(const dfpt_scene_desc* scene, const dfpt_sky* sky, const dfpt_params* params, int width, int height,
                  int pass_begin, int passes, int precision, int threads, int row_begin, int row_end, double* film,
                  double* sum, double* sumsq, int* primitive_offsets, uint8_t* bgra, int* hit_prim, int* hit_type,
                  int* hit_off, double* hit_dist, double* hit_normal, uint64_t* rng_state, uint64_t* counters) {
    if (!scene || !sky || !params || !film || width <= 0 || height <= 0 || passes < 1) return -1;
    if (scene->primitive_extensions && scene->primitive_extensions_count != scene->primitives_count / 3 * 4) return -2;
    if (row_begin < 0) row_begin = 0;
    if (row_end > height || row_end <= 0) row_end = height;
    Scene S{scene, sky, params, width, height};
    std::vector<int> po_local;
    Outputs o{film, sum, sumsq, primitive_offsets, bgra, hit_prim, hit_type, hit_off, hit_dist, hit_normal, rng_state, counters};
    if (!o.primitive_offsets) {
        po_local.assign((size_t)width * height, -1);
        o.primitive_offsets = po_local.data();
    }
    if (precision == 64) return render<double>(S, pass_begin, passes, threads, row_begin, row_end, o);
    return render<float>(S, pass_begin, passes, threads, row_begin, row_end, o);
}

// Single-ray entry points for known-answer tests (precision 32 or 64).
int oracle_intersect(const dfpt_scene_desc* scene, const dfpt_params* params, const double* ray6, int testing, int precision,
                     double* out_distance, int* out_prim, int* out_type, int* out_off, double* out_point3, double* out_normal3) {
    dfpt_sky sky{};
    Scene S{scene, &sky, params, 1, 1};
    if (precision == 64) {
        Kernel<double> k(S);
        const double t = k.intersect(ray6[0], ray6[1], ray6[2], ray6[3], ray6[4], ray6[5], testing != 0);
        *out_distance = t;
        if (!testing) {
            *out_prim = k.is.primitive_offset; *out_type = k.is.shape_type; *out_off = k.is.shape_offset;
            if (k.is.primitive_offset >= 0) {
                out_point3[0] = k.is.px; out_point3[1] = k.is.py; out_point3[2] = k.is.pz;
                out_normal3[0] = k.is.nx; out_normal3[1] = k.is.ny; out_normal3[2] = k.is.nz;
            }
        }
        return 0;
    }
    Kernel<float> k(S);
    const float t = k.intersect((float)ray6[0], (float)ray6[1], (float)ray6[2], (float)ray6[3], (float)ray6[4], (float)ray6[5], testing != 0);
    *out_distance = t;
    if (!testing) {
        *out_prim = k.is.primitive_offset; *out_type = k.is.shape_type; *out_off = k.is.shape_offset;
        if (k.is.primitive_offset >= 0) {
            out_point3[0] = k.is.px; out_point3[1] = k.is.py; out_point3[2] = k.is.pz;
            out_normal3[0] = k.is.nx; out_normal3[1] = k.is.ny; out_normal3[2] = k.is.nz;
        }
    }
    return 0;
}

int oracle_sky(const dfpt_sky* sky, const double* dir3, int precision, double* out3) {
    dfpt_scene_desc d{};
    dfpt_params p{};
    Scene S{&d, sky, &p, 1, 1};
    if (precision == 64) {
        Kernel<double> k(S);
        k.sky_color(dir3[0], dir3[1], dir3[2]);
        for (int i = 0; i < 3; ++i) out3[i] = k.color[i];
    } else {
        Kernel<float> k(S);
        k.sky_color((float)dir3[0], (float)dir3[1], (float)dir3[2]);
        for (int i = 0; i < 3; ++i) out3[i] = k.color[i];
    }
    return 0;
}

double oracle_simplex3(double x, double y, double z, int precision) {
    if (precision == 64) return Kernel<double>::simplex3(x, y, z);
    return Kernel<float>::simplex3((float)x, (float)y, (float)z);
}

double oracle_fbm3(double frequency, double gain, double minimum, double maximum, int octaves, double x, double y, double z, int precision) {
    if (precision == 64) return Kernel<double>::fbm3(frequency, gain, minimum, maximum, octaves, x, y, z);
    return Kernel<float>::fbm3((float)frequency, (float)gain, (float)minimum, (float)maximum, octaves, (float)x, (float)y, (float)z);
}

// Philox4x32-10 block for known-answer tests.
int oracle_philox(const uint32_t* counter4, const uint32_t* key2, uint32_t* out4) {
    uint32_t c[4] = {counter4[0], counter4[1], counter4[2], counter4[3]};
    philox(c, key2[0], key2[1]);
    for (int i = 0; i < 4; ++i) out4[i] = c[i];
    return 0;
}

// The first `count` numbers of a pixel's stream (LCG from `state`, or the counter stream).
int oracle_random(int kind, uint64_t state, uint32_t pixel, uint32_t pass, uint64_t seed, int count, float* out) {
    Random r{kind, state, pixel, pass, (uint32_t)seed, (uint32_t)(seed >> 32), 0};
    for (int i = 0; i < count; ++i) out[i] = r.next();
    return 0;
}

int oracle_tonemap(const dfpt_params* params, const double* rgb3, int precision, uint8_t* bgra4) {
    if (precision == 64) resolve<double>(params, rgb3, -1, bgra4);
    else {
        const float f[3] = {(float)rgb3[0], (float)rgb3[1], (float)rgb3[2]};
        resolve<float>(params, f, -1, bgra4);
    }
    return 0;
}

// FP64 host adjoint: renders `passes` passes from `pass_begin` with per-primitive parameters
// (albedo multiplier 3, added emission 3, Phong exponent 1 per primitive) under the sky `sky`
// (which must equal Sky.set(sun, turbidity)), writes the mean image, and
// grad[P * 7 + 4] = d(sum dldi * image)/d(albedo 3, emission 3, exponent; per primitive) and
// d/d(turbidity, sun x, y, z).
int oracle_diff(const dfpt_scene_desc* scene, const dfpt_sky* sky, const dfpt_params* params, int width, int height, int pass_begin,
                int passes, int threads, const double* albedo, const double* emission, const double* exponent, double turbidity,
                const double* sun3, const double* dldi, double* image, double* grad) {
    if (!scene || !sky || !params || !albedo || !emission || !exponent || !sun3 || !dldi || !image || !grad) return -1;
    if (width <= 0 || height <= 0 || passes < 1 || params->rng_kind != DFPT_RNG_COUNTER) return -1;
    if (scene->primitive_extensions && scene->primitive_extensions_count != scene->primitives_count / 3 * 4) return -2;
    Scene S{scene, sky, params, width, height};
    const DiffIn din{albedo, emission, exponent};
    const SunDual sd = sky_set_dual(turbidity, sun3);
    const int np = (int)(scene->primitives_count / 3);
    const size_t glen = (size_t)np * 7 + 4;
    if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::vector<double>> g((size_t)threads, std::vector<double>(glen, 0.0));
    std::atomic<int> next_row(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&, t]() {
            for (;;) {
                const int y = next_row.fetch_add(1);
                if (y >= height) break;
                diff_rows(S, din, sd, pass_begin, passes, y, y + 1, dldi, image, g[t]);
            }
        });
    }
    for (auto& th : pool) th.join();
    for (size_t i = 0; i < glen; ++i) {
        double v = 0;
        for (int t = 0; t < threads; ++t) v += g[t][i];
        grad[i] = v;
    }
    return 0;
}

}  // extern "C"
