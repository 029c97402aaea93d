// dfpt_adjoint.cuh - path-replay adjoint of the path tracer (included by dfpt_kernels.cuh).
//
// Gradients of an image loss with respect to per-primitive albedo (a multiplier of the albedo
// texture color), emission (added to the emission texture color), Phong exponent, and the sky's
// turbidity and sun direction. The forward pass (k_shade etc. with DevParams::diff set) keeps per
// sample only the path's total radiance and one sun-visibility bit per bounce; the backward pass
// replays every path from its counter-based RNG key (same pixel, same pass index, same draws),
// accumulating the radiance gathered so far, so that at each vertex the radiance that arrives
// from later vertices is total - gathered (path-replay backpropagation). Per vertex k with
// throughput T_k, loss weight w = dLoss/dImage / spp:
//   emission e_k              dL/de   = T_k
//   albedo a_k = tex * p      dL/dp   = tex * (T_k dot/pi [sun seen]) + (later radiance) / p
//                             (the second term when the vertex multiplied T by the albedo;
//                             Russian roulette's survival probability is held constant)
//   Phong exponent n          dL/dn   = (later radiance) * (1/(n+1) + ln cos)   (score of the
//                             lobe density (n+1) cos^n the cosine was drawn from)
//   sky (turbidity, sun)      forward-mode duals through the sky color of escaping rays; the sun
//                             term's derivative over the rim of the sun's cone (sun_rim_tan),
//                             visibility included
// Tangents of the sky fields with respect to (turbidity, sun direction) come from the host.

// ---- Dual numbers with four tangents: d/d(turbidity, sun x, sun y, sun z) ----

struct D4 {
    float v;
    float d[4];
};

__device__ __forceinline__ D4 d4c(float v) {
    D4 r;
    r.v = v;
    r.d[0] = r.d[1] = r.d[2] = r.d[3] = 0.0f;
    return r;
}
__device__ __forceinline__ D4 d4f(const DevParams& P, int field, float v) {
    D4 r;
    r.v = v;
    const float* t = P.diff_sky_tan + 4 * field;
    r.d[0] = t[0]; r.d[1] = t[1]; r.d[2] = t[2]; r.d[3] = t[3];
    return r;
}
__device__ __forceinline__ D4 operator+(D4 a, D4 b) {
    D4 r; r.v = a.v + b.v;
    for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] + b.d[j];
    return r;
}
__device__ __forceinline__ D4 operator-(D4 a, D4 b) {
    D4 r; r.v = a.v - b.v;
    for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] - b.d[j];
    return r;
}
__device__ __forceinline__ D4 operator-(D4 a) {
    D4 r; r.v = -a.v;
    for (int j = 0; j < 4; ++j) r.d[j] = -a.d[j];
    return r;
}
__device__ __forceinline__ D4 operator*(D4 a, D4 b) {
    D4 r; r.v = a.v * b.v;
    for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] * b.v + a.v * b.d[j];
    return r;
}
__device__ __forceinline__ D4 operator/(D4 a, D4 b) {
    D4 r; r.v = a.v / b.v;
    const float ib = 1.0f / b.v;
    for (int j = 0; j < 4; ++j) r.d[j] = (a.d[j] - r.v * b.d[j]) * ib;
    return r;
}
__device__ __forceinline__ D4 operator+(D4 a, float b) { a.v += b; return a; }
__device__ __forceinline__ D4 operator+(float b, D4 a) { a.v += b; return a; }
__device__ __forceinline__ D4 operator-(D4 a, float b) { a.v -= b; return a; }
__device__ __forceinline__ D4 operator-(float b, D4 a) { return d4c(b) - a; }
__device__ __forceinline__ D4 operator*(D4 a, float b) {
    a.v *= b;
    for (int j = 0; j < 4; ++j) a.d[j] *= b;
    return a;
}
__device__ __forceinline__ D4 operator*(float b, D4 a) { return a * b; }
__device__ __forceinline__ D4 chain(D4 a, float value, float slope) {
    D4 r; r.v = value;
    for (int j = 0; j < 4; ++j) r.d[j] = a.d[j] * slope;
    return r;
}
__device__ __forceinline__ D4 d4exp(D4 a) { const float e = expf(a.v); return chain(a, e, e); }
__device__ __forceinline__ D4 d4sqrt(D4 a) {
    const float s = sqrtf(fmaxf(a.v, 0.0f));
    return chain(a, s, s > 0.0f ? 0.5f / s : 0.0f);
}
__device__ __forceinline__ D4 d4rsqrt(D4 a) { return d4c(1.0f) / d4sqrt(a); }
// acos of the value clamped to [-1, 1]; no slope where the clamp is active.
__device__ __forceinline__ D4 d4acos_clamped(D4 a) {
    const float c = fminf(fmaxf(a.v, -1.0f), 1.0f);
    const float s = sqrtf(fmaxf(1.0f - c * c, 0.0f));
    const bool inside = a.v > -1.0f && a.v < 1.0f && s > 1.0e-6f;
    return chain(a, acosf(c), inside ? -1.0f / s : 0.0f);
}
__device__ __forceinline__ D4 d4clamp(D4 a, float lo, float hi) {
    if (a.v < lo) return d4c(lo);
    if (a.v > hi) return d4c(hi);
    return a;
}
__device__ __forceinline__ D4 d4sel(bool c, D4 a, D4 b) { return c ? a : b; }

// sky_color with the sky fields as duals: the color of an escaping ray and its tangents.
__device__ void sky_color_tan(const DevParams& P, float dx, float dy, float dz, D4& r, D4& g, D4& b) {
    float d0x = dx * P.sky_u[0] + dy * P.sky_u[1] + dz * P.sky_u[2];
    float d0y = dx * P.sky_v[0] + dy * P.sky_v[1] + dz * P.sky_v[2];
    float d0z = dx * P.sky_w[0] + dy * P.sky_w[1] + dz * P.sky_w[2];
    r = g = b = d4c(0.01f);
    if (!(d0z >= 0.0f && P.sky_active == 1)) return;
    d0z = jmax(d0z, 0.001f);
    const float lr = rsqrt_j(d0x * d0x + d0y * d0y + d0z * d0z);
    const float d1x = d0x * lr, d1y = d0y * lr, d1z = d0z * lr;
    const D4 dp = d4f(P, SKY_SUN_DIR, P.sun_dir[0]) * d1x + d4f(P, SKY_SUN_DIR + 1, P.sun_dir[1]) * d1y +
                  d4f(P, SKY_SUN_DIR + 2, P.sun_dir[2]) * d1z;
    const float cos1 = fminf(fmaxf(d1z, -1.0f), 1.0f);
    const float theta1 = acosf(cos1);
    const float cos1r = 1.0f / (cos1 + 0.01f);
    const D4 cosg = d4clamp(dp, -1.0f, 1.0f);
    const D4 gamma = d4acos_clamped(dp);
    const D4 c0 = d4f(P, SKY_COS_THETA0, P.cos_theta0);
    const D4 c0sq = c0 * c0;
    D4 L[5], X[5], Y[5];
    for (int k = 0; k < 5; ++k) {
        L[k] = d4f(P, SKY_PEREZ_L + k, P.perez_l[k]);
        X[k] = d4f(P, SKY_PEREZ_X + k, P.perez_x[k]);
        Y[k] = d4f(P, SKY_PEREZ_Y + k, P.perez_y[k]);
    }
    const D4 num_l = (1.0f + L[0] * d4exp(L[1] * cos1r)) * (1.0f + L[2] * d4exp(L[3] * gamma) + L[4] * cosg * cosg);
    const D4 rel_l = d4f(P, SKY_ZENITH_L, P.zenith_l) * num_l / d4f(P, SKY_DEN_L, P.den_l) * 1.0e-4f;
    const D4 den_x = d4f(P, SKY_DEN_X_A, P.den_x_a) * (1.0f + X[2] * d4exp(X[3] * theta1) + X[4] * c0sq);
    const D4 num_x = (1.0f + X[0] * d4exp(X[1] * cos1r)) * (1.0f + X[2] * d4exp(X[3] * gamma) + X[4] * cosg * cosg);
    const D4 x = d4f(P, SKY_ZENITH_X, P.zenith_x) * num_x / den_x;
    const D4 den_y = d4f(P, SKY_DEN_Y_A, P.den_y_a) * (1.0f + Y[2] * d4exp(Y[3] * theta1) + Y[4] * c0sq);
    const D4 num_y = (1.0f + Y[0] * d4exp(Y[1] * cos1r)) * (1.0f + Y[2] * d4exp(Y[3] * gamma) + Y[4] * cosg * cosg);
    const D4 y = d4f(P, SKY_ZENITH_Y, P.zenith_y) * num_y / den_y;
    const D4 k0 = d4c(1.0f) / (0.0241f + 0.2562f * x - 0.7341f * y);
    const D4 k1 = (-1.3515f - 1.7703f * x + 5.9114f * y) * k0;
    const D4 k2 = (0.03f - 31.4424f * x + 30.0717f * y) * k0;
    const D4 cX = 10246.121f + k1 * 187.75537f + k2 * 213.14803f;
    const D4 cY = 10676.695f + k1 * 192.59653f + k2 * 76.29494f;
    const D4 cZ = 12372.504f + k1 * 3482.8765f + k2 * -235.71611f;
    const D4 Yr = d4c(1.0f) / cY;
    const D4 R = cX * rel_l * Yr, G = rel_l, B = cZ * rel_l * Yr;
    r = 3.2410042f * R + -1.5373994f * G + -0.49861607f * B;
    g = -0.9692241f * R + 1.8759298f * G + 0.041554242f * B;
    b = 0.05563942f * R + -0.20401107f * G + 1.0571486f * B;
    // w = max(0, -min(0, min(r, g, b))) is added to every channel.
    const D4 m = d4sel(r.v <= g.v && r.v <= b.v, r, d4sel(g.v <= b.v, g, b));
    if (m.v < 0.0f) {
        r = r - m;
        g = g - m;
        b = b - m;
    }
}

// The sun term's derivative with respect to (turbidity, sun direction), visibility included. The
// sun sample is uniform over the cone C of directions towards the sun's disk (axis: the world sun
// direction W, half-angle a with sin^2 a = 500^2 / |origin - p|^2), so the vertex's expected sun term
// is the mean of G(w) = c max(w.n, 0) V(w) over C (c: the loss-weighted albedo factor / pi, V: the
// shadow ray's visibility). Under a change of the sun direction C moves rigidly and its angle
// changes with the distance to the sun's origin; the derivative of the mean over a moving domain is
// an integral over its rim (Reynolds transport):
//   d/dq mean_C G = (1 / Omega) * integral over the rim of (G - k) v_n dl,   Omega = 2 pi (1 - cos a),
// with v_n = (w.dW/dq - d cos a/dq) / sin a the rim's outward speed and k any number independent of
// the rim point (the rim integral of v_n is d Omega / dq). One rim direction at angle phi, uniform,
// gives (G(w_phi) - k) (w_phi.dW/dq - d cos a/dq) / (1 - cos a); k = the forward sample's own G
// (whose mean is the mean of G) makes the estimate small where the whole cone is lit or shadowed,
// and leaves the shadow edges that cross the cone - which a derivative with the visibility held
// fixed misses. phi comes from its own counter-based stream (pixel, pass, bounce), so the replay
// draws nothing the forward did not. One extra any-hit ray per sun sample.
__device__ void sun_rim_tan(const DevScene& S, const DevParams& P, uint32_t pixel, uint32_t pass, int bounce, float px, float py,
                            float pz, float nx, float ny, float nz, float c, float g_forward, float gsky[4]) {
    const float sr2 = 500.0f * 500.0f;
    const D4 tx = d4f(P, SKY_SUN_ORIGIN, P.sun_origin[0]) - px;
    const D4 ty = d4f(P, SKY_SUN_ORIGIN + 1, P.sun_origin[1]) - py;
    const D4 tz = d4f(P, SKY_SUN_ORIGIN + 2, P.sun_origin[2]) - pz;
    const D4 sin2 = d4c(sr2) / (tx * tx + ty * ty + tz * tz);
    if (!(sin2.v > 0.0f && sin2.v < 1.0f)) return;
    const D4 cos_a = d4sqrt(1.0f - sin2);
    const float sin_a = sqrtf(sin2.v);
    const float one_m_cos = sin2.v / (1.0f + cos_a.v);  // 1 - cos a without cancellation
    const uint4 rb = philox4x32_10(make_uint4(pass, 0x40000000u | (uint32_t)bounce, P.seed_hi, 0x52494D21u), make_uint2(pixel, P.seed_lo));
    const float phi = TWO_PI * ((float)(rb.x >> 8) * (1.0f / 16777216.0f));
    const float wx = P.sun_dir_world[0], wy = P.sun_dir_world[1], wz = P.sun_dir_world[2];
    const float ax = fabsf(wx), ay = fabsf(wy), az = fabsf(wz);
    const float vx = ax < ay && ax < az ? 0.0f : ay < az ? wz : wy;
    const float vy = ax < ay && ax < az ? wz : ay < az ? 0.0f : -wx;
    const float vz = ax < ay && ax < az ? -wy : ay < az ? -wx : 0.0f;
    const float vr = rsqrtf(vx * vx + vy * vy + vz * vz);
    const float vnx = vx * vr, vny = vy * vr, vnz = vz * vr;
    const float unx = vny * wz - vnz * wy, uny = vnz * wx - vnx * wz, unz = vnx * wy - vny * wx;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float x = cp * sin_a, y = sp * sin_a, z = cos_a.v;
    float rx = unx * x + vnx * y + wx * z, ry = uny * x + vny * y + wy * z, rz = unz * x + vnz * y + wz * z;
    const float rr = rsqrtf(rx * rx + ry * ry + rz * rz);
    rx *= rr; ry *= rr; rz *= rr;
    const float dot0 = rx * wx + ry * wy + rz * wz, dot1 = rx * nx + ry * ny + rz * nz;
    float g_rim = 0.0f;
    if (dot0 > 0.0f && dot1 > 0.0f && c != 0.0f) {
        TraceStats st{0, 0};
        const Hit h = trace_v<true, 1>(S, true, px, py, pz, rx, ry, rz, st);
        if (h.t >= INF - 0.0001f) g_rim = c * dot1;
    }
    const float k = (g_rim - g_forward) / one_m_cos;
    if (k == 0.0f) return;
    const D4 dwx = d4f(P, SKY_SUN_DIR_WORLD, wx), dwy = d4f(P, SKY_SUN_DIR_WORLD + 1, wy), dwz = d4f(P, SKY_SUN_DIR_WORLD + 2, wz);
    for (int j = 0; j < 4; ++j) gsky[j] += k * (rx * dwx.d[j] + ry * dwy.d[j] + rz * dwz.d[j] - cos_a.d[j]);
}

// Per-block gradient accumulation: per-primitive entries in shared memory (float, one launch) when
// they fit, else straight into row 0 with double atomics; the four sky entries in registers.
struct GradAcc {
    float* sh;     // shared [P * 7] or null
    double* row;   // this block's row (shared mode) / row 0 (atomic mode)
    __device__ __forceinline__ void add(int prim, int k, float v) {
        if (v == 0.0f) return;
        if (sh) atomicAdd(sh + prim * DFPT_DIFF_PER_PRIM + k, v);
        else atomicAdd(row + prim * DFPT_DIFF_PER_PRIM + k, (double)v);
    }
};

__device__ __forceinline__ void grad_begin(float* sh, int n) {
    if (sh)
        for (int k = threadIdx.x; k < n; k += blockDim.x) sh[k] = 0.0f;
    __syncthreads();
}

// Block-reduces the sky tangents and adds the block's partials to its row.
__device__ __forceinline__ void grad_end(float* sh, double* row, int n_prim_entries, const float gsky[4], float* red) {
    float v[4] = {gsky[0], gsky[1], gsky[2], gsky[3]};
    for (int off = 16; off > 0; off >>= 1)
        for (int j = 0; j < 4; ++j) v[j] += __shfl_down_sync(0xFFFFFFFFu, v[j], off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    if (lane == 0)
        for (int j = 0; j < 4; ++j) red[warp * 4 + j] = v[j];
    __syncthreads();
    if (threadIdx.x < 4) {
        float t = 0.0f;
        for (int w = 0; w < warps; ++w) t += red[w * 4 + threadIdx.x];
        if (sh) row[n_prim_entries + threadIdx.x] += (double)t;
        else atomicAdd(row + n_prim_entries + threadIdx.x, (double)t);
    }
    if (sh)
        for (int k = threadIdx.x; k < n_prim_entries; k += blockDim.x)
            if (sh[k] != 0.0f) row[k] += (double)sh[k];
}

// One bounce of the replay (the structure of k_shade, GRK:3185-3686). BATCH: the replay runs in
// waves of the handle's passes (path = wave slot; pixel and pass from the slot key); otherwise one
// pass at a time (path = pixel, the pass index from the device counter).
template <bool BATCH, bool SHARED>
__global__ void __launch_bounds__(256) k_shade_adj(DevScene S, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q, int bounce) {
    extern __shared__ float dyn_sh[];
    __shared__ float red[32 * 4];
    const DevParams& P = *Pp;
    const int n = B.counts[bounce];
    const int qi = B.sorted_queues ? 0 : (bounce & 1);
    const uint32_t pass_now = BATCH ? 0u : (uint32_t)*B.pass_index;
    const size_t npix = (size_t)P.width * (size_t)P.height;
    const float inv_spp = 1.0f / (float)P.diff_spp;
    const int n_prim_entries = S.primitive_count * DFPT_DIFF_PER_PRIM;
    GradAcc acc;
    acc.sh = SHARED ? dyn_sh : nullptr;
    acc.row = SHARED ? B.diff_rows + (size_t)blockIdx.x * B.diff_row_len : B.diff_rows;
    grad_begin(acc.sh, n_prim_entries);
    float gsky[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    GRID_STRIDE_UNIFORM(i, n) {
        bool emit_next = false;
        float4 no = make_float4(0, 0, 0, 0), nd = make_float4(0, 0, 0, 0);
        if (i < n) {
            const float4 o4 = B.q_o[qi][i], d4 = B.q_d[qi][i];
            const int path = __float_as_int(o4.w);
            uint32_t pixel = (uint32_t)path, pass = pass_now;
            if constexpr (BATCH) {
                const int4 key = Q.slot_key[path];
                pixel = (uint32_t)key.y;
                pass = (uint32_t)key.z;
            }
            const size_t sample = (size_t)((int)pass - P.diff_pass0);
            const int4 hr = B.q_hit[i];
            Hit h;
            h.t = __int_as_float(hr.x);
            h.prim = hr.y;
            h.shape_type = hr.z;
            h.shape_offset = hr.w;
            float4 T = B.throughput[PSI(path)];
            float4 Lu = B.radiance[PSI(path)];  // radiance gathered so far along the replay
            const float4 Lt = B.diff_L[sample * npix + pixel];
            float4 w = B.diff_dldi[pixel];
            w.x *= inv_spp; w.y *= inv_spp; w.z *= inv_spp;
            if (h.t == INF || h.prim == -1) {
                D4 sr, sg, sb;
                sky_color_tan(P, d4.x, d4.y, d4.z, sr, sg, sb);
                Lu.x += T.x * sr.v * INV_PI; Lu.y += T.y * sg.v * INV_PI; Lu.z += T.z * sb.v * INV_PI;
                for (int j = 0; j < 4; ++j) gsky[j] += (w.x * T.x * sr.d[j] + w.y * T.y * sg.d[j] + w.z * T.z * sb.d[j]) * INV_PI;
                B.radiance[PSI(path)] = Lu;
            } else {
                Rng rng = make_rng(P, pixel, pass, B.rng[path]);
                const Surf s = surface(S, P, o4.x, o4.y, o4.z, d4.x, d4.y, d4.z, h);
                const int so_off = __ldg(S.prim_info + h.prim).z;
                const float dp = s.nx * d4.x + s.ny * d4.y + s.nz * d4.z;
                const float dp2 = dp * 2.0f;
                const bool correct = dp < 0.0f;
                const float wx = correct ? s.nx : -s.nx, wy = correct ? s.ny : -s.ny, wz = correct ? s.nz : -s.nz;
                const int albedo = texture_color(S, f2i(__ldg(S.surfaces + so_off + 1)), s);
                const int emission = texture_color(S, f2i(__ldg(S.surfaces + so_off + 2)), s);
                const float tr = cr(albedo), tg = cg(albedo), tb = cb(albedo);
                float ar = tr, ag = tg, ab = tb;
                float er = cr(emission), eg = cg(emission), eb = cb(emission);
                const int material = f2i(__ldg(S.surfaces + so_off + 0));
                float exponent = 50.0f;
                if (S.prim_ext) primitive_extension(S, h.prim, er, eg, eb, exponent);
                diff_surface(P, h.prim, ar, ag, ab, er, eg, eb, exponent);
                // Emission.
                Lu.x += T.x * er; Lu.y += T.y * eg; Lu.z += T.z * eb;
                acc.add(h.prim, 3, w.x * T.x);
                acc.add(h.prim, 4, w.y * T.y);
                acc.add(h.prim, 5, w.z * T.z);
                // Sun sample (same draws as the forward; visibility from the forward's bits).
                if ((material == DFPT_MATERIAL_CLEAR_COAT || material == DFPT_MATERIAL_LAMBERTIAN || material == DFPT_MATERIAL_PHONG) &&
                    P.sun_active == 1) {
                    const float u = rng.next(), v = rng.next();
                    float lx, ly, lz, dot1;
                    const int seen = (B.diff_vis[sample * npix + pixel] >> bounce) & 1;
                    const float c = (w.x * T.x * ar + w.y * T.y * ag + w.z * T.z * ab) * INV_PI;
                    float g_forward = 0.0f;
                    if (sun_sample(P, s.px, s.py, s.pz, wx, wy, wz, u, v, lx, ly, lz, dot1) && seen) {
                        const float k = dot1 * INV_PI;
                        Lu.x += T.x * (ar * 1.0f * k); Lu.y += T.y * (ag * 1.0f * k); Lu.z += T.z * (ab * 1.0f * k);
                        acc.add(h.prim, 0, w.x * T.x * tr * k);
                        acc.add(h.prim, 1, w.y * T.y * tg * k);
                        acc.add(h.prim, 2, w.z * T.z * tb * k);
                        g_forward = c * dot1;
                    }
                    sun_rim_tan(S, P, pixel, pass, bounce, s.px, s.py, s.pz, wx, wy, wz, c, g_forward, gsky);
                }
                const float a0r = ar, a0g = ag, a0b = ab;  // before Russian roulette's 1/q
                const int depth = bounce + 1;
                bool alive = true;
                if (depth >= P.depth_rr) {
                    const float q = jmax(ar, jmax(ag, ab));
                    const float r = rng.next();
                    if (r >= q) alive = false;
                    else {
                        const float qr = 1.0f / q;
                        ar *= qr; ag *= qr; ab *= qr;
                    }
                }
                if (alive) {
                    const Scatter sct = scatter(s, material, wx, wy, wz, o4, d4, dp2, ar, ag, ab, exponent, rng, T);
                    // Radiance of the later vertices (every term carries this vertex's factors).
                    const float lr = Lt.x - Lu.x, lg = Lt.y - Lu.y, lb = Lt.z - Lu.z;
                    if (sct.albedo) {
                        if (a0r != 0.0f) acc.add(h.prim, 0, w.x * lr * tr / a0r);
                        if (a0g != 0.0f) acc.add(h.prim, 1, w.y * lg * tg / a0g);
                        if (a0b != 0.0f) acc.add(h.prim, 2, w.z * lb * tb / a0b);
                    }
                    if (material == DFPT_MATERIAL_PHONG && sct.phong_ct > 0.0f)
                        acc.add(h.prim, 6, (w.x * lr + w.y * lg + w.z * lb) * (1.0f / (exponent + 1.0f) + logf(sct.phong_ct)));
                    emit_next = true;
                    no = make_float4(sct.o.x, sct.o.y, sct.o.z, __int_as_float(path));
                    nd = make_float4(sct.d.x, sct.d.y, sct.d.z, 0.0f);
                }
                B.throughput[PSI(path)] = T;
                B.radiance[PSI(path)] = Lu;
                B.rng[path] = rng.state;
            }
        }
        const int slot = warp_push(B.counts + bounce + 1, emit_next);
        if (slot >= 0) {
            B.q_o[qi ^ 1][slot] = no;
            B.q_d[qi ^ 1][slot] = nd;
        }
    }
    __syncthreads();
    grad_end(acc.sh, acc.row, n_prim_entries, gsky, red);
}

// After the last bounce: the continuation ray's any-hit test; escaping rays add sky tangents.
template <bool BATCH, int V>
__global__ void __launch_bounds__(256) k_final_adj(DevScene S, const DevParams* __restrict__ Pp, DevPass B, DevBatch Q, int bounce) {
    __shared__ float red[32 * 4];
    const DevParams& P = *Pp;
    const int n = B.counts[bounce];
    const int qi = B.sorted_queues ? 0 : (bounce & 1);
    const int n_prim_entries = S.primitive_count * DFPT_DIFF_PER_PRIM;
    const float inv_spp = 1.0f / (float)P.diff_spp;
    float gsky[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    WARP_DYNAMIC(i, n, B.counts + DFPT_COUNTS_FETCH + bounce) {
        TraceStats st{0, 0};
        const bool valid = i < n;
        float4 o = make_float4(0, 0, 0, 0), d = make_float4(0, 0, 1, 0);
        if (valid) {
            o = B.q_o[qi][i];
            d = B.q_d[qi][i];
        }
        const Hit h = trace_v<true, V>(S, valid, o.x, o.y, o.z, d.x, d.y, d.z, st);
        if (valid && !(h.t < INF)) {
            const int path = __float_as_int(o.w);
            const float4 T = B.throughput[PSI(path)];
            int pixel = path;
            if constexpr (BATCH) pixel = Q.slot_key[path].y;
            float4 w = B.diff_dldi[pixel];
            w.x *= inv_spp; w.y *= inv_spp; w.z *= inv_spp;
            D4 sr, sg, sb;
            sky_color_tan(P, d.x, d.y, d.z, sr, sg, sb);
            for (int j = 0; j < 4; ++j) gsky[j] += (w.x * T.x * sr.d[j] + w.y * T.y * sg.d[j] + w.z * T.z * sb.d[j]) * INV_PI;
        }
    }
    __syncthreads();
    // Only the sky entries: shared-mode rows are per block, atomic mode adds into row 0.
    grad_end(nullptr, B.diff_rows + (size_t)blockIdx.x * B.diff_row_len, n_prim_entries, gsky, red);
}

// Sums the per-block rows into out[row_len].
__global__ void k_diff_reduce(const double* __restrict__ rows, int n_rows, int row_len, double* __restrict__ out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < row_len; k += gridDim.x * blockDim.x) {
        double t = 0.0;
        for (int r = 0; r < n_rows; ++r) t += rows[(size_t)r * row_len + k];
        out[k] = t;
    }
}
