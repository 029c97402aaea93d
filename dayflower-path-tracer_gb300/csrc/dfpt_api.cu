// dfpt_api.cu - the C-ABI: scene validation and upload, pass scheduling (CUDA graphs), readback.
//
// One handle = one compiled scene resident in HBM + one film. dfpt_render replays a captured CUDA
// graph per pass: camera -> [trace closest -> shade -> shadow rays] x depth -> final any-hit ->
// film, the wavefront form of GPURendererKernel.run (GPURendererKernel.java:252-308).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dfpt.h"
#include "dfpt_cull.h"
#include "dfpt_internal.h"
#include "dfpt_launch.h"
#include "dfpt_noise_tables.h"
#include "dfpt_store.h"

namespace {
thread_local std::string g_last_error;
}

int dfpt_fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

namespace {

// ---------------------------------------------------------------------------------------------
// Validation of the compiled scene: every offset the kernels will follow is checked here so no
// device access can leave its array.

bool in_range(int64_t off, int64_t len, int64_t count) { return off >= 0 && len >= 0 && off + len <= count; }

int check_triangle(const HostScene& s, int off) {
    if (!in_range(off, 12, (int64_t)s.triangles.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "triangle offset %d out of range", off);
    for (int k = 0; k < 3; ++k) {
        if (!in_range(s.triangles[off + k], 3, (int64_t)s.point3fs.size()))
            return dfpt_fail(DFPT_ERR_INVALID_SCENE, "triangle %d position offset out of range", off);
        if (!in_range(s.triangles[off + 3 + k], 3, (int64_t)s.vector3fs.size()) || !in_range(s.triangles[off + 9 + k], 3, (int64_t)s.vector3fs.size()))
            return dfpt_fail(DFPT_ERR_INVALID_SCENE, "triangle %d normal/tangent offset out of range", off);
        if (!in_range(s.triangles[off + 6 + k], 2, (int64_t)s.point2fs.size()))
            return dfpt_fail(DFPT_ERR_INVALID_SCENE, "triangle %d texture coordinate offset out of range", off);
    }
    return DFPT_OK;
}

int texture_min_size(int type) {
    switch (type) {
        case DFPT_TEXTURE_BLEND: return 5;
        case DFPT_TEXTURE_BULLSEYE: return 4;
        case DFPT_TEXTURE_CHECKERBOARD: return 8;
        case DFPT_TEXTURE_CONSTANT: return 3;
        case DFPT_TEXTURE_FBM: return 7;
        case DFPT_TEXTURE_IMAGE: return 8;
        case DFPT_TEXTURE_SURFACE_NORMAL: return 3;
        case DFPT_TEXTURE_UV: return 2;
        default: return -1;
    }
}

int check_texture(const HostScene& s, int to, bool allow_blend) {
    const int64_t n = (int64_t)s.textures.size();
    if (!in_range(to, 1, n)) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "texture offset %d out of range", to);
    const int type = (int)s.textures[to];
    const int need = texture_min_size(type);
    if (need < 0) {
        // Unknown types evaluate to black in the reference (GRK:1615-1617); only the type is read.
        return DFPT_OK;
    }
    if (!in_range(to, need, n)) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "texture record at %d truncated", to);
    if (type == DFPT_TEXTURE_IMAGE) {
        const float w = s.textures[to + 4], h = s.textures[to + 5];
        if (!(w >= 1.0f && h >= 1.0f && w * h < 1.0e9f)) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "image texture at %d has bad size", to);
        if (!in_range(to, 8 + (int64_t)((int)(w * h)), n)) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "image texture at %d truncated", to);
    }
    if (type == DFPT_TEXTURE_BLEND) {
        if (!allow_blend) return DFPT_OK;  // nested blends evaluate to black; never followed
        for (int k = 2; k <= 3; ++k) {
            int r = check_texture(s, (int)s.textures[to + k], false);
            if (r) return r;
        }
    }
    return DFPT_OK;
}

int check_surface(const HostScene& s, int so) {
    if (!in_range(so, 6, (int64_t)s.surfaces.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "surface offset %d out of range", so);
    for (int k = 1; k <= 3; ++k) {
        int r = check_texture(s, (int)s.surfaces[so + k], true);
        if (r) return r;
    }
    return DFPT_OK;
}

float int_bits(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

int float_bits_int(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}

// Triangle record: {a, triangle offset}, {b - a, last in its leaf}, {c - a, node index of its leaf}
// (the compact pair walk resumes the threaded order from a leaf it took off its stack; 0 for
// triangle primitives).
int add_tri_record(const HostScene& s, Derived& d, int off, bool last, int leaf_node = 0) {
    const float* P = s.point3fs.data();
    const int a = s.triangles[off], b = s.triangles[off + 1], c = s.triangles[off + 2];
    d.tris.push_back(make_float4(P[a], P[a + 1], P[a + 2], int_bits(off)));
    d.tris.push_back(make_float4(P[b] - P[a], P[b + 1] - P[a + 1], P[b + 2] - P[a + 2], int_bits(last ? 1 : 0)));
    d.tris.push_back(make_float4(P[c] - P[a], P[c + 1] - P[a + 1], P[c + 2] - P[a + 2], int_bits(leaf_node)));
    return (int)(d.tris.size() / 3) - 1;
}

// Converts one flattened BVH (SceneCompiler.java:888-995) rooted at `root` to node records.
int convert_bvh(const HostScene& s, Derived& d, int root, int& first_node) {
    const int64_t nb = (int64_t)s.bvh.size();
    std::vector<int> offs;       // relative offsets in preorder
    int pending = 1, rel = 0;
    while (pending > 0) {
        const int at = root + rel;
        if (!in_range(at, 5, nb)) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "BVH node at %d out of range", at);
        offs.push_back(rel);
        if (offs.size() > (size_t)nb) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "BVH at %d is not a tree", root);
        const int type = s.bvh[at];
        if (type == 1) {
            pending += 1;
            rel += 5;
        } else if (type == 2) {
            const int cnt = s.bvh[at + 4];
            if (cnt < 0 || !in_range(at, 5 + (int64_t)cnt, nb)) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "BVH leaf at %d truncated", at);
            pending -= 1;
            rel += 5 + cnt;
        } else {
            return dfpt_fail(DFPT_ERR_INVALID_SCENE, "BVH node at %d has type %d", at, type);
        }
    }
    std::vector<int> index_of_rel(rel + 1, -1);
    for (size_t i = 0; i < offs.size(); ++i) index_of_rel[offs[i]] = (int)i;
    first_node = (int)(d.nodes.size() / 2);
    for (size_t i = 0; i < offs.size(); ++i) {
        const int at = root + offs[i];
        const int type = s.bvh[at], next = s.bvh[at + 1], mn = s.bvh[at + 2], mx = s.bvh[at + 3];
        int next_index = -1;
        if (next != -1) {
            if (next <= offs[i] || next >= (int)index_of_rel.size() || index_of_rel[next] < 0)
                return dfpt_fail(DFPT_ERR_INVALID_SCENE, "BVH node at %d has a bad next pointer %d", at, next);
            next_index = first_node + index_of_rel[next];
        }
        if (!in_range(mn, 3, (int64_t)s.point3fs.size()) || !in_range(mx, 3, (int64_t)s.point3fs.size()))
            return dfpt_fail(DFPT_ERR_INVALID_SCENE, "BVH node at %d has bounds out of range", at);
        int leaf = -1;
        if (type == 1) {
            if (s.bvh[at + 4] != offs[i] + 5) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "BVH node at %d: left child is not the next node", at);
        } else {
            const int cnt = s.bvh[at + 4];
            if (cnt == 0) {
                leaf = -2;
            } else {
                for (int k = 0; k < cnt; ++k) {
                    const int toff = s.bvh[at + 5 + k];
                    int r = check_triangle(s, toff);
                    if (r) return r;
                    const int rec = add_tri_record(s, d, toff, k == cnt - 1, first_node + (int)i);
                    if (k == 0) leaf = rec;
                }
            }
        }
        const float* P = s.point3fs.data();
        d.nodes.push_back(make_float4(P[mn], P[mn + 1], P[mn + 2], int_bits(next_index)));
        d.nodes.push_back(make_float4(P[mx], P[mx + 1], P[mx + 2], int_bits(leaf)));
    }
    return DFPT_OK;
}

int build_derived(const HostScene& s, Derived& d) {
    const int np = (int)(s.primitives.size() / 3);
    std::vector<std::pair<int, int>> bvh_roots;  // root offset -> first node
    for (int i = 0; i < np; ++i) {
        const int type = s.primitives[3 * i], off = s.primitives[3 * i + 1], so = s.primitives[3 * i + 2];
        int r = check_surface(s, so);
        if (r) return r;
        int rec = 0;
        if (type == DFPT_SHAPE_PLANE) {
            if (!in_range(off, 4, (int64_t)s.planes.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "plane offset %d out of range", off);
            for (int k = 0; k < 3; ++k)
                if (!in_range(s.planes[off + k], 3, (int64_t)s.point3fs.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "plane %d point out of range", off);
            if (!in_range(s.planes[off + 3], 3, (int64_t)s.vector3fs.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "plane %d normal out of range", off);
            const float* A = s.point3fs.data() + s.planes[off];
            const float* N = s.vector3fs.data() + s.planes[off + 3];
            rec = (int)d.plane_a.size();
            d.plane_a.push_back(make_float4(A[0], A[1], A[2], 0.0f));
            d.plane_n.push_back(make_float4(N[0], N[1], N[2], 0.0f));
        } else if (type == DFPT_SHAPE_SPHERE) {
            if (!in_range(off, 2, (int64_t)s.spheres.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "sphere offset %d out of range", off);
            const int po = (int)s.spheres[off];
            if (!in_range(po, 3, (int64_t)s.point3fs.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "sphere %d position out of range", off);
            rec = (int)d.sphere4.size();
            d.sphere4.push_back(make_float4(s.point3fs[po], s.point3fs[po + 1], s.point3fs[po + 2], s.spheres[off + 1]));
        } else if (type == DFPT_SHAPE_TERRAIN) {
            if (!in_range(off, 5, (int64_t)s.terrains.size())) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "terrain offset %d out of range", off);
        } else if (type == DFPT_SHAPE_TRIANGLE) {
            int r2 = check_triangle(s, off);
            if (r2) return r2;
            rec = add_tri_record(s, d, off, true);
        } else if (type == DFPT_SHAPE_TRIANGLE_MESH) {
            rec = -1;
            for (auto& pr : bvh_roots)
                if (pr.first == off) rec = pr.second;
            if (rec < 0) {
                int first = 0;
                int r2 = convert_bvh(s, d, off, first);
                if (r2) return r2;
                bvh_roots.emplace_back(off, first);
                rec = first;
            }
        } else {
            // Unknown shape types never intersect (GRK:1195-1243 has no branch for them).
            rec = 0;
        }
        d.prim_info.push_back(make_int4(type, off, so, rec));
    }
    if (d.nodes.empty()) { d.nodes.push_back(make_float4(0, 0, 0, 0)); d.nodes.push_back(make_float4(0, 0, 0, 0)); }
    if (d.tris.empty()) for (int k = 0; k < 3; ++k) d.tris.push_back(make_float4(0, 0, 0, 0));
    if (d.sphere4.empty()) d.sphere4.push_back(make_float4(0, 0, 0, 0));
    if (d.plane_a.empty()) { d.plane_a.push_back(make_float4(0, 0, 0, 0)); d.plane_n.push_back(make_float4(0, 0, 0, 0)); }
    if (d.prim_info.empty()) d.prim_info.push_back(make_int4(0, 0, 0, 0));
    return DFPT_OK;
}


// ---------------------------------------------------------------------------------------------
// Primitive culling structure. World bounds of each bounded primitive: its object-space bound
// (mesh: the BVH root box; sphere: center +- radius; triangle: its three vertices) mapped by the
// inverse of its world-to-object matrix (the matrix the kernel transforms rays with), in double,
// padded by 1e-4 of the box's extent and magnitude plus 1e-4 and rounded outward to float. Planes,
// terrains, primitives with singular or non-finite matrices go to the unbounded list.

bool invert_affine(const float* m, double* inv) {
    // m: row-major 4x4 with rows 0-2 the affine map [A | t]; inv = [A^-1 | -A^-1 t].
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
    if (!(std::fabs(det) > 1e-300) || !std::isfinite(det)) return false;
    const double r = 1.0 / det;
    double A[9] = {(e * i - f * h) * r, (c * h - b * i) * r, (b * f - c * e) * r,
                   (f * g - d * i) * r, (a * i - c * g) * r, (c * d - a * f) * r,
                   (d * h - e * g) * r, (b * g - a * h) * r, (a * e - b * d) * r};
    const double tx = m[3], ty = m[7], tz = m[11];
    for (int k = 0; k < 3; ++k) {
        inv[4 * k + 0] = A[3 * k]; inv[4 * k + 1] = A[3 * k + 1]; inv[4 * k + 2] = A[3 * k + 2];
        inv[4 * k + 3] = -(A[3 * k] * tx + A[3 * k + 1] * ty + A[3 * k + 2] * tz);
    }
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(inv[k])) return false;
    return true;
}

using dfpt_cull::CullItem;
using dfpt_cull::CullNode;

// Object-space bound per primitive (6 floats: lo, hi; NaN lo.x for unbounded shapes).
void cull_object_bounds(const Derived& d, int np, std::vector<float>& obj) {
    obj.assign((size_t)6 * np, 0.0f);
    for (int i = 0; i < np; ++i) {
        const int4 info = d.prim_info[i];
        float* o = obj.data() + 6 * (size_t)i;
        if (info.x == DFPT_SHAPE_TRIANGLE_MESH) {
            const float4 a = d.nodes[2 * (size_t)info.w], b = d.nodes[2 * (size_t)info.w + 1];
            o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = b.x; o[4] = b.y; o[5] = b.z;
        } else if (info.x == DFPT_SHAPE_SPHERE) {
            const float4 sp = d.sphere4[info.w];
            const float r = std::fabs(sp.w);
            o[0] = sp.x - r; o[1] = sp.y - r; o[2] = sp.z - r; o[3] = sp.x + r; o[4] = sp.y + r; o[5] = sp.z + r;
        } else if (info.x == DFPT_SHAPE_TRIANGLE) {
            const float4 a = d.tris[3 * (size_t)info.w], e0 = d.tris[3 * (size_t)info.w + 1], e1 = d.tris[3 * (size_t)info.w + 2];
            const float v[3][3] = {{a.x, a.y, a.z}, {a.x + e0.x, a.y + e0.y, a.z + e0.z}, {a.x + e1.x, a.y + e1.y, a.z + e1.z}};
            for (int c = 0; c < 3; ++c) {
                o[c] = std::min(v[0][c], std::min(v[1][c], v[2][c]));
                o[3 + c] = std::max(v[0][c], std::max(v[1][c], v[2][c]));
            }
            // The triangle's vertices a + e are rounded sums: widen by their rounding.
            for (int c = 0; c < 3; ++c) {
                const float m = std::max(std::fabs(o[c]), std::fabs(o[3 + c]));
                o[c] -= m * 1e-6f;
                o[3 + c] += m * 1e-6f;
            }
        } else {
            o[0] = NAN;
        }
    }
}

// The culling BVH from object bounds and the world-to-object matrices.
void build_culling(const std::vector<float>& obj, const std::vector<float>& w2o, int np, Derived& d) {
    d.cull_nodes.clear();
    d.cull_prims.clear();
    d.always.clear();
    std::vector<CullItem> items;
    d.prim_box.assign((size_t)2 * std::max(np, 1), make_float4(-INFINITY, -INFINITY, -INFINITY, 0));
    for (int i = 0; i < np; ++i) d.prim_box[2 * i + 1] = make_float4(INFINITY, INFINITY, INFINITY, 0);
    for (int i = 0; i < np; ++i) {
        const float* o = obj.data() + 6 * (size_t)i;
        double inv[12];
        bool ok = !std::isnan(o[0]) && invert_affine(w2o.data() + 16 * (size_t)i, inv);
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = 0; ok && k < 8; ++k) {
            const double p[3] = {(k & 1) ? o[3] : o[0], (k & 2) ? o[4] : o[1], (k & 4) ? o[5] : o[2]};
            for (int a = 0; a < 3; ++a) {
                const double w = inv[4 * a] * p[0] + inv[4 * a + 1] * p[1] + inv[4 * a + 2] * p[2] + inv[4 * a + 3];
                if (!std::isfinite(w)) ok = false;
                lo[a] = std::min(lo[a], w);
                hi[a] = std::max(hi[a], w);
            }
        }
        if (!ok) {
            d.always.push_back(i);
            continue;
        }
        CullItem it;
        it.prim = i;
        double ext = 0, mag = 0;
        for (int a = 0; a < 3; ++a) {
            ext = std::max(ext, hi[a] - lo[a]);
            mag = std::max(mag, std::max(std::fabs(lo[a]), std::fabs(hi[a])));
        }
        const double pad = 1e-4 * (ext + mag) + 1e-4;
        for (int a = 0; a < 3; ++a) {
            it.lo[a] = std::nextafter((float)(lo[a] - pad), -INFINITY);
            it.hi[a] = std::nextafter((float)(hi[a] + pad), INFINITY);
        }
        d.prim_box[2 * i] = make_float4(it.lo[0], it.lo[1], it.lo[2], 0);
        d.prim_box[2 * i + 1] = make_float4(it.hi[0], it.hi[1], it.hi[2], 0);
        items.push_back(it);
    }
    d.bounded = (int)items.size();
    if (!items.empty()) {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (const CullItem& it : items)
            for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], it.lo[a]); hi[a] = std::max(hi[a], it.hi[a]); }
        d.bounds_lo = make_float4(lo[0], lo[1], lo[2], 0);
        d.bounds_hi = make_float4(hi[0], hi[1], hi[2], 0);
        std::vector<CullNode> nodes;
        dfpt_cull::build_cull_node(items, 0, (int)items.size(), nodes, d.cull_prims, 0);
        d.cull_nodes.resize(2 * nodes.size());
        for (size_t k = 0; k < nodes.size(); ++k) {
            float la, ra;
            std::memcpy(&la, &nodes[k].left, 4);
            std::memcpy(&ra, &nodes[k].right, 4);
            d.cull_nodes[2 * k] = make_float4(nodes[k].lo[0], nodes[k].lo[1], nodes[k].lo[2], la);
            d.cull_nodes[2 * k + 1] = make_float4(nodes[k].hi[0], nodes[k].hi[1], nodes[k].hi[2], ra);
        }
    }
    if (d.cull_nodes.empty()) { d.cull_nodes.push_back(make_float4(0, 0, 0, 0)); d.cull_nodes.push_back(make_float4(0, 0, 0, 0)); }
    if (d.cull_prims.empty()) d.cull_prims.push_back(0);
}

template <typename T>
void copy_array(std::vector<T>& dst, const T* src, int64_t n) {
    dst.assign(src, src + n);
    if (dst.empty()) dst.push_back(T());
}

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

float powf_j(float a, float b) { return (float)std::pow((double)a, (double)b); }

}  // namespace

struct dfpt_handle {
    SceneStore sc;  // the compiled scene, host copy + device arrays
    int width = 0, height = 0, n_pixels = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 0;
    KernelSet fast{}, strict{}, wide{};  // wide: the batch stages over this handle's scene
    bool use_strict = false;
    // Parameters.
    dfpt_params params{};
    dfpt_sky sky{};
    DevParams dev_params_host{};
    DevBuf<DevParams> dev_params;
    // Pass buffers.
    DevBuf<float4> q_o0, q_o1, q_d0, q_d1, s_o, s_d, s_c, throughput, primary_o, primary_d, film_sum, film_comp;
    DevBuf<int4> q_hit;
    DevBuf<uint64_t> rng;
    DevBuf<int> pixel_flags, counts, pass_index, film_n, primitive_offsets, hit_prim, hit_type, hit_off;
    DevBuf<float> hit_dist, hit_normal, scratch_rgb;
    DevBuf<uint8_t> bgra;
    DevBuf<unsigned long long> stats;
    DevBuf<double> mean;
    DevPass pass{};
    LaunchCtx ctx{};
    size_t shadow_capacity = 0;  // rays the deferred shadow queue holds (pixels x bounces)
    int host_pass = 0;  // passes issued so far (mirrors the device pass counter)
    int clear_pass = 0;
    bool counting = false;
    bool record_hits = false;
    // Differentiable rendering (dfpt_diff_*): parameters, the forward's per-sample records, the
    // backward's gradient rows.
    bool diff_on = false;     // shading reads the per-primitive parameters
    bool diff_ready = false;  // the last forward's samples are stored for a backward
    int diff_pass0 = 0, diff_spp = 0;
    size_t diff_capacity = 0;  // samples x pixels the per-sample records hold
    DevBuf<float4> diff_albedo, diff_emission, diff_L, diff_dldi;
    DevBuf<float> diff_exponent, diff_sky_tan;
    DevBuf<int> vis, diff_vis;
    DevBuf<double> diff_rows, diff_out;
    // Graph of one pass.
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_valid = false;
    int graph_kernels = 0;
    bool use_graph = true;
    // Wide passes: dfpt_render's passes but the last run `wide_samples` at a time through the
    // batch stages (one scene), so each launch carries k samples per pixel (see render_wide).
    int wide_samples = 8;
    bool pixel_tiles = true;   // plain passes in 8 x 4 pixel-tile slot order (DevParams::pixel_tiles)
    int tail_bounce = -1;      // plain passes: first bounce of the tail launch (-1: a launch per bounce)
    int shadow_config = -1;    // traversal configuration of the sun shadow-ray launches (-1: trace_config's)
    // Plain passes: the deferred shadow rays binned by origin cell before their launch.
    bool pass_shadow_sort = true;
    DevBuf<int> p_sort_bins;                  // offsets, bounce-1 ray counts, shadow counts, chunk sums
    DevBuf<float4> p_s2_o, p_s2_d, p_s2_c;    // the binned copy of the shadow queue
    size_t p_s2_capacity = 0;
    DevPass pass_shadow2{};                   // `pass` reading the binned copy
    // Plain passes: bounce 1's rays binned (direction bin over an origin grid of pass_ray_sort
    // bits; 0 = off) between the shading of bounce 0 and their traversal.
    int pass_ray_sort = 0;
    DevBuf<float4> p_r2_o, p_r2_d;            // the binned copy of bounce 1's queue
    DevPass pass_ray_count{};                 // `pass` with the bin counts (bounce 0's shading)
    DevPass pass_ray_read{};                  // `pass` reading the binned copy (bounce 1)
    int wide_capacity = 0;
    size_t wide_shadow = 0;
    DevBuf<float4> w_q_o0, w_q_o1, w_q_d0, w_q_d1, w_s_o, w_s_d, w_s_c, w_throughput;  // w_throughput: throughput + radiance records (PSI)
    DevBuf<int4> w_q_hit, w_slot_key;
    DevBuf<uint64_t> w_rng;
    DevBuf<int> w_pixel_flags, w_counts, w_wave_entries;
    DevBuf<DevScene> w_scene;
    DevBuf<long long> w_sample_begin, w_film_begin, w_wave_base, w_wave_tab;
    DevPass wpass{};
    DevBatch wq{};
    LaunchCtx wctx{};
    cudaGraphExec_t wide_graph = nullptr;
    bool wide_graph_valid = false;
    int wide_graph_kernels = 0;
    long long wide_range[5] = {0, 0, 0, -1, -1};  // wave base, range end, pass of sample 0, clear sample, selection pass
    int pass_index_host = 0;  // source of pass-index copies (pageable: consumed on return)
    bool ray_sort = true;     // bin rays between bounces in wide passes
    bool shadow_sort = true;  // with ray_sort, also bin the sun shadow rays before their launch
    bool shadow_defer = false;  // wide passes: one shadow launch per wave (queue of slots x depth)
    DevBuf<int> w_sort_bins;
    DevBuf<float4> w_s2_o, w_s2_d, w_s2_c;  // the binned copy of the shadow queue
    DevBuf<int> w_vis;                       // differentiable mode: visibility bits per slot
    DevPass wpass_shadow{};                  // wpass with the shadow queue pointing at the copy
    LaunchCtx wctx_shadow{};
    uint64_t launches = 0;
    // L2 residency of the traversal records (see apply_l2_policy).
    bool l2_persist = true;
    cudaAccessPolicyWindow l2_window{};
    // Per-kernel timing (direct launches with an event between kernels).
    bool profiling = false;
    std::vector<cudaEvent_t> events;
    std::vector<int> event_kind;  // kind of the kernel between events i and i+1
    int events_used = 0;
};

namespace {

void release(dfpt_handle* h) {
    for (cudaEvent_t e : h->events) cudaEventDestroy(e);
    h->events.clear();
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
    if (h->wide_graph) cudaGraphExecDestroy(h->wide_graph);
    h->wide_graph = nullptr;
    {
        DevBuf<float4>* w4[] = {&h->w_q_o0, &h->w_q_o1, &h->w_q_d0, &h->w_q_d1, &h->w_s_o, &h->w_s_d, &h->w_s_c, &h->w_throughput};
        for (auto* b : w4) b->release();
        h->w_q_hit.release(); h->w_slot_key.release(); h->w_rng.release(); h->w_pixel_flags.release(); h->w_counts.release();
        h->w_wave_entries.release(); h->w_scene.release(); h->w_sample_begin.release(); h->w_film_begin.release();
        h->w_wave_base.release(); h->w_wave_tab.release(); h->w_sort_bins.release();
        h->w_s2_o.release(); h->w_s2_d.release(); h->w_s2_c.release(); h->w_vis.release();
    }
    h->sc.release();
    h->diff_albedo.release(); h->diff_emission.release(); h->diff_L.release(); h->diff_dldi.release();
    h->diff_exponent.release(); h->diff_sky_tan.release(); h->vis.release(); h->diff_vis.release();
    h->diff_rows.release(); h->diff_out.release();
    DevBuf<float>* fb[] = {&h->hit_dist, &h->hit_normal, &h->scratch_rgb};
    for (auto* b : fb) b->release();
    DevBuf<int>* ib[] = {&h->pixel_flags, &h->counts, &h->pass_index, &h->film_n, &h->primitive_offsets, &h->hit_prim, &h->hit_type, &h->hit_off};
    for (auto* b : ib) b->release();
    DevBuf<float4>* f4[] = {&h->q_o0, &h->q_o1, &h->q_d0, &h->q_d1, &h->s_o, &h->s_d, &h->s_c, &h->throughput, &h->primary_o, &h->primary_d, &h->film_sum, &h->film_comp};
    for (auto* b : f4) b->release();
    h->rng.release();
    h->bgra.release();
    h->stats.release();
    h->mean.release();
    h->dev_params.release();
    h->p_sort_bins.release(); h->p_s2_o.release(); h->p_s2_d.release(); h->p_s2_c.release();
    h->p_r2_o.release(); h->p_r2_d.release();
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
    // Lines the window marked persisting go back to normal with the records they cached.
    if (h->l2_window.num_bytes > 0) (void)cudaCtxResetPersistingL2Cache();
    h->l2_window = cudaAccessPolicyWindow{};
}

}  // namespace

void dev_params_fill(DevParams& d, const dfpt_params& p, const dfpt_sky& k, const float* cam, int width, int height) {
    std::memset(&d, 0, sizeof(d));
    d.renderer_type = p.renderer_type;
    d.tone_mapper_type = p.tone_mapper_type;
    d.shader_type = p.shader_type;
    d.normal_mapping = p.normal_mapping;
    d.wireframes = p.wireframes;
    d.depth_max = p.pt_ray_depth_maximum;
    d.depth_rr = p.pt_ray_depth_russian_roulette;
    d.exposure = p.tone_mapper_exposure;
    d.ao_max_distance = p.ao_maximum_distance;
    d.g_amplitude = p.global_amplitude;
    d.g_frequency = p.global_frequency;
    d.g_gain = p.global_gain;
    d.g_lacunarity = p.global_lacunarity;
    d.g_octaves = p.global_octaves;
    d.selected_primitive_offset = p.selected_primitive_offset;
    d.rng_kind = p.rng_kind;
    d.seed_lo = (uint32_t)p.seed;
    d.seed_hi = (uint32_t)(p.seed >> 32);
    d.width = width;
    d.height = height;
    for (int i = 0; i < 3; ++i) {
        d.sky_u[i] = k.orthonormal_basis_u[i];
        d.sky_v[i] = k.orthonormal_basis_v[i];
        d.sky_w[i] = k.orthonormal_basis_w[i];
        d.sun_dir[i] = k.sun_direction[i];
        d.sun_dir_world[i] = k.sun_direction_world[i];
        d.sun_origin[i] = k.sun_origin[i];
    }
    d.theta = k.theta;
    d.sky_active = k.is_sky_active;
    d.sun_active = k.is_sun_active;
    for (int i = 0; i < 5; ++i) {
        d.perez_l[i] = (float)k.perez_relative_luminance[i];
        d.perez_x[i] = (float)k.perez_x[i];
        d.perez_y[i] = (float)k.perez_y[i];
    }
    d.zenith_l = (float)k.zenith_relative_luminance;
    d.zenith_x = (float)k.zenith_x;
    d.zenith_y = (float)k.zenith_y;
    const double t0 = (double)k.theta, c0 = std::cos(t0);
    const double* L = k.perez_relative_luminance;
    d.den_l = (float)((1.0 + L[0] * std::exp(L[1])) * (1.0 + L[2] * std::exp(L[3] * t0) + L[4] * c0 * c0));
    d.den_x_a = (float)(1.0 + k.perez_x[0] * std::exp(k.perez_x[1]));
    d.den_y_a = (float)(1.0 + k.perez_y[0] * std::exp(k.perez_y[1]));
    d.cos_theta0 = (float)c0;
    const float pi_f = 3.14159274101257324219f;
    const float pi180 = pi_f / 180.0f;
    d.fov_tan_x = (float)std::tan((double)(cam[4] * 0.5f * pi180));
    d.fov_tan_y = (float)std::tan((double)(-cam[5] * 0.5f * pi180));
    d.wire_cos = (float)std::cos((double)(pi_f * 0.5f / 4096.0f));
    // RGBColorSpace.SRGB (breakPoint 0.00304, gamma 2.4) derived constants, float arithmetic.
    const float bp = 0.00304f, g = 2.4f;
    const float pe = powf_j(bp, 1.0f / g - 1.0f);
    d.cs_break = bp;
    d.cs_gamma = g;
    d.cs_slope = 1.0f / (g / pe - g * bp + bp);
    d.cs_slope_match = g * d.cs_slope / pe;
    d.cs_segment = d.cs_slope_match * powf_j(bp, 1.0f / g) - d.cs_slope * bp;
}

namespace {

bool is_simple_mode(int rt);

void fill_dev_params(dfpt_handle* h) {
    DevParams& d = h->dev_params_host;
    dev_params_fill(d, h->params, h->sky, h->sc.host.camera.data(), h->width, h->height);
    d.record_hits = h->record_hits ? 1 : 0;
    d.counting = h->counting ? 1 : 0;
    d.clear_pass = h->clear_pass;
    // Tile slot order: the counter stream keys samples by pixel, so the order is free; the LCG's
    // per-pixel states, the wireframe overlay's per-pixel rays and the adjoint's per-pixel records
    // keep slot = pixel.
    // The per-pixel modes (k_simple) write their results at slot = pixel.
    d.pixel_tiles = (h->pixel_tiles && h->params.rng_kind == DFPT_RNG_COUNTER && h->params.wireframes != 1 && !h->diff_on &&
                     !is_simple_mode(h->params.renderer_type) && h->width % 8 == 0 && h->height % 4 == 0) ? 1 : 0;
    if (h->diff_on) {
        d.diff = 1;
        d.diff_pass0 = h->diff_pass0;
        d.diff_spp = h->diff_spp;
        d.diff_albedo = h->diff_albedo.p;
        d.diff_emission = h->diff_emission.p;
        d.diff_exponent = h->diff_exponent.p;
        d.diff_sky_tan = h->diff_sky_tan.p;
    }
}

// The sky fields the kernels read (DevParams, SKY_* order) as functions of turbidity and the world
// sun direction: Sky.set (Sky.java:295-333) and the derived Perez denominators, in double without
// the float narrowing, for the tangent table.
void sky_fields(double t, const double* dir, double* f) {
    const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const double wx = dir[0] / len, wy = dir[1] / len, wz = dir[2] / len;
    // Sky basis u = X, v = Z, w = Y: the sky-frame sun direction is (x, z, y), already unit.
    const double sx = wx, sy = wz, sz = wy;
    f[SKY_SUN_DIR] = sx; f[SKY_SUN_DIR + 1] = sy; f[SKY_SUN_DIR + 2] = sz;
    const double theta = std::acos(std::max(-1.0, std::min(1.0, sz)));
    const double th2 = theta * theta, th3 = th2 * theta, t2 = t * t;
    const double pi_f = (double)3.14159274101257324219f;
    const double chi = (4.0 / 9.0 - t / 120.0) * (pi_f - 2.0 * theta);
    const double L[5] = {0.17872 * t - 1.46303, -0.35540 * t + 0.42749, -0.02266 * t + 5.32505, 0.12064 * t - 2.57705, -0.06696 * t + 0.37027};
    const double X[5] = {-0.01925 * t - 0.25922, -0.06651 * t + 0.00081, -0.00041 * t + 0.21247, -0.06409 * t - 0.89887, -0.00325 * t + 0.04517};
    const double Y[5] = {-0.01669 * t - 0.26078, -0.09495 * t + 0.00921, -0.00792 * t + 0.21023, -0.04405 * t - 1.65369, -0.01092 * t + 0.05291};
    for (int i = 0; i < 5; ++i) {
        f[SKY_PEREZ_L + i] = L[i];
        f[SKY_PEREZ_X + i] = X[i];
        f[SKY_PEREZ_Y + i] = Y[i];
    }
    f[SKY_ZENITH_L] = ((4.0453 * t - 4.9710) * std::tan(chi) - 0.2155 * t + 2.4192) * 1000.0;
    f[SKY_ZENITH_X] = (0.00165 * th3 - 0.00374 * th2 + 0.00208 * theta + 0.0) * t2 +
                      (-0.02902 * th3 + 0.06377 * th2 - 0.03202 * theta + 0.00394) * t +
                      (0.11693 * th3 - 0.21196 * th2 + 0.06052 * theta + 0.25885);
    f[SKY_ZENITH_Y] = (0.00275 * th3 - 0.00610 * th2 + 0.00316 * theta + 0.0) * t2 +
                      (-0.04212 * th3 + 0.08970 * th2 - 0.04153 * theta + 0.00515) * t +
                      (0.15346 * th3 - 0.26756 * th2 + 0.06669 * theta + 0.26688);
    const double c0 = std::cos(theta);
    f[SKY_DEN_L] = (1.0 + L[0] * std::exp(L[1])) * (1.0 + L[2] * std::exp(L[3] * theta) + L[4] * c0 * c0);
    f[SKY_DEN_X_A] = 1.0 + X[0] * std::exp(X[1]);
    f[SKY_DEN_Y_A] = 1.0 + Y[0] * std::exp(Y[1]);
    f[SKY_COS_THETA0] = c0;
    for (int i = 0; i < 3; ++i) {
        f[SKY_SUN_ORIGIN + i] = (i == 0 ? wx : i == 1 ? wy : wz) * 10000.0;
        f[SKY_SUN_DIR_WORLD + i] = i == 0 ? wx : i == 1 ? wy : wz;
    }
}

// d(field)/d(turbidity, sun x, sun y, sun z) by central differences of sky_fields in double
// (smooth closed forms: step 1e-6 leaves ~1e-10 relative error).
void sky_tangents(double t, const double* dir, float* out) {
    const double h = 1.0e-6;
    double fp[DFPT_SKY_FIELDS], fm[DFPT_SKY_FIELDS];
    for (int j = 0; j < 4; ++j) {
        double tp = t, tm = t, dp[3] = {dir[0], dir[1], dir[2]}, dm[3] = {dir[0], dir[1], dir[2]};
        if (j == 0) { tp += h; tm -= h; }
        else { dp[j - 1] += h; dm[j - 1] -= h; }
        sky_fields(tp, dp, fp);
        sky_fields(tm, dm, fm);
        for (int k = 0; k < DFPT_SKY_FIELDS; ++k) out[4 * k + j] = (float)((fp[k] - fm[k]) / (2.0 * h));
    }
}


int push_params(dfpt_handle* h) {
    fill_dev_params(h);
    CUDA_TRY(cudaMemcpyAsync(h->dev_params.p, &h->dev_params_host, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    return DFPT_OK;
}

int reset_rng(dfpt_handle* h) {
    std::vector<uint64_t> seeds((size_t)h->n_pixels);
    for (int i = 0; i < h->n_pixels; ++i) seeds[i] = splitmix64(h->params.seed + (uint64_t)i);
    CUDA_TRY(cudaMemcpyAsync(h->rng.p, seeds.data(), seeds.size() * 8, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

// The kernel set of a pass: the strict set when selected, and always for the ray caster, whose hit
// ids are the reference's bit for bit (one rounding per float operation); the fast set otherwise.
const KernelSet& kset(dfpt_handle* h) {
    return (h->use_strict || h->params.renderer_type == DFPT_RENDERER_RAY_CASTER) ? h->strict : h->fast;
}

bool is_simple_mode(int rt) {
    return rt == DFPT_RENDERER_AMBIENT_OCCLUSION || rt == DFPT_RENDERER_RAY_CASTER || rt == DFPT_RENDERER_RAY_MARCHER ||
           rt == DFPT_RENDERER_RAY_TRACER || rt == DFPT_RENDERER_SURFACE_NORMALS;
}

// Kernel kinds reported by dfpt_read_profile.
enum { KIND_CAMERA, KIND_TRACE, KIND_SHADE, KIND_SHADOW, KIND_FINAL, KIND_SIMPLE, KIND_WIREFRAME, KIND_FILM, KIND_END, KIND_SORT, KIND_COUNT };

void mark(dfpt_handle* h, int kind) {
    if (!h->profiling) return;
    if (h->events_used >= (int)h->events.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) { (void)cudaGetLastError(); return; }
        h->events.push_back(e);
    }
    cudaEventRecord(h->events[h->events_used], h->stream);
    if ((int)h->event_kind.size() < h->events_used + 1) h->event_kind.resize(h->events_used + 1);
    h->event_kind[h->events_used] = kind;
    h->events_used++;
}

// Issues one pass on the handle's stream; returns the number of kernels launched.
int issue_pass(dfpt_handle* h) {
    const KernelSet& K = kset(h);
    const LaunchCtx& c = h->ctx;
    int k = 0;
    cudaMemsetAsync(h->counts.p, 0, DFPT_COUNTS_SIZE * sizeof(int), h->stream);
    if (is_simple_mode(h->params.renderer_type)) {
        mark(h, KIND_SIMPLE); K.simple(c); ++k;
    } else {
        const int nb = h->params.pt_ray_depth_maximum < 1 ? 1 : (h->params.pt_ray_depth_maximum > DFPT_MAX_DEPTH ? DFPT_MAX_DEPTH : h->params.pt_ray_depth_maximum);
        // With tail_bounce t, bounces t .. nb - 1 and the final any-hit run in one tail launch (t = 0:
        // the camera rays' traversal and shading too).
        const int tb = (h->tail_bounce >= 0 && h->tail_bounce < nb && K.tail) ? h->tail_bounce : nb;
        mark(h, KIND_CAMERA); K.camera(c); ++k;
        // With pass_ray_sort, bounce 0's shading counts the bins of the rays it queues, and bounce
        // 1 (its traversal and shading, or the tail from there) reads them in bin order.
        const bool sort_rays = h->pass_ray_sort > 0 && K.sort_rays && nb > 1 && h->pass_ray_read.q_o[1];
        LaunchCtx c1 = c;
        for (int b = 0; b < tb; ++b) {
            mark(h, KIND_TRACE); K.trace_closest(c1, b); ++k;
            if (b == 0 && sort_rays) {
                LaunchCtx c0 = c;
                c0.pass = &h->pass_ray_count;
                mark(h, KIND_SHADE); K.shade(c0, b); ++k;
                mark(h, KIND_SORT); k += K.sort_rays(c0, 1, h->pass_ray_read);
                c1.pass = &h->pass_ray_read;
            } else {
                mark(h, KIND_SHADE); K.shade(c1, b); ++k;
                c1.pass = &h->pass;
            }
        }
        if (tb < nb) {
            mark(h, KIND_TRACE); K.tail(c1, tb, nb); ++k;
        } else {
            mark(h, KIND_FINAL); K.final_(c1, nb); ++k;
        }
        // The sun shadow rays of all bounces, traced together (binned by origin cell first when
        // pass_shadow_sort is on: shading and the tail counted the bins).
        if (h->sky.is_sun_active == 1) {
            LaunchCtx cs = c;
            if (h->shadow_config >= 0 && h->shadow_config < K.trace_configs) {
                cs.trace_config = h->shadow_config;
                cs.grid_trace = K.trace_grid(h->shadow_config, h->sms);
            }
            if (h->pass.sort_count_shadow && K.sort_shadow) {
                mark(h, KIND_SORT); k += K.sort_shadow(c, h->pass_shadow2);
                cs.pass = &h->pass_shadow2;
            }
            mark(h, KIND_SHADOW); K.shadow(cs, 0); ++k;
        }
    }
    if (h->params.wireframes == 1) { mark(h, KIND_WIREFRAME); K.wireframe(c); ++k; }
    mark(h, KIND_FILM); K.film(c); ++k;
    mark(h, KIND_END); K.end_pass(c); ++k;
    mark(h, KIND_COUNT);
    return k;
}

// The replay of the last forward's samples (k_shade_adj / k_final_adj) for one pass; returns the
// number of kernels launched.
int issue_replay_pass(dfpt_handle* h) {
    const KernelSet& K = h->fast;
    const LaunchCtx& c = h->ctx;
    int k = 0;
    cudaMemsetAsync(h->counts.p, 0, DFPT_COUNTS_SIZE * sizeof(int), h->stream);
    const int nb = h->params.pt_ray_depth_maximum < 1 ? 1 : (h->params.pt_ray_depth_maximum > DFPT_MAX_DEPTH ? DFPT_MAX_DEPTH : h->params.pt_ray_depth_maximum);
    K.camera(c); ++k;
    for (int b = 0; b < nb; ++b) {
        K.trace_closest(c, b); ++k;
        K.shade_adj(c, b); ++k;
    }
    K.final_adj(c, nb); ++k;
    K.end_pass(c); ++k;
    return k;
}

int bounces_of(const dfpt_handle* h);

// ---- Wide passes -------------------------------------------------------------------------------
// dfpt_render(h, n) renders passes p .. p+n-1. With the path tracer, the counter-based RNG and no
// per-pass outputs in use (wireframes, hit records, differentiable mode, strict kernels), passes
// p .. p+n-2 run through the batch stages as one scene whose samples are (pass, pixel): a wave holds
// `wide_samples` passes of every pixel, so every launch - late bounces included - carries k times
// the rays of a pass. The RNG is keyed by (pixel, pass index) exactly as in a pass, and the film
// takes each pixel's samples in pass order (k_bfilm), so the film equals pass-by-pass rendering.
// The last pass runs as a normal pass: it writes the selection buffer and tone maps the image.

bool wide_eligible(const dfpt_handle* h) {
    return h->wide_samples > 1 && !is_simple_mode(h->params.renderer_type) && h->params.rng_kind == DFPT_RNG_COUNTER &&
           h->params.wireframes != 1 && !h->record_hits && !h->use_strict && h->wide.b_camera != nullptr;
}

int wide_prepare(dfpt_handle* h) {
    const size_t n = (size_t)h->n_pixels;
    const int cap = (int)std::min<size_t>((size_t)h->wide_samples * n, (size_t)1 << 27);
    // One bounce of shadow rays (traced before the next bounce), or every bounce's when deferred.
    const size_t shadow = (size_t)cap * (size_t)(h->shadow_defer ? bounces_of(h) : 1);
    if (cap != h->wide_capacity || shadow != h->wide_shadow) {
        DevBuf<float4>* w4[] = {&h->w_q_o0, &h->w_q_o1, &h->w_q_d0, &h->w_q_d1, &h->w_s_o, &h->w_s_d, &h->w_s_c, &h->w_throughput};
        for (auto* b : w4) b->release();
        h->w_q_hit.release(); h->w_slot_key.release(); h->w_rng.release(); h->w_pixel_flags.release();
        const size_t c = (size_t)cap;
        CUDA_TRY(h->w_q_o0.alloc(c)); CUDA_TRY(h->w_q_o1.alloc(c)); CUDA_TRY(h->w_q_d0.alloc(c)); CUDA_TRY(h->w_q_d1.alloc(c));
        CUDA_TRY(h->w_q_hit.alloc(c)); CUDA_TRY(h->w_slot_key.alloc(c));
        CUDA_TRY(h->w_throughput.alloc(2 * c)); CUDA_TRY(h->w_rng.alloc(c)); CUDA_TRY(h->w_pixel_flags.alloc(c));
        CUDA_TRY(h->w_s_o.alloc(shadow)); CUDA_TRY(h->w_s_d.alloc(shadow)); CUDA_TRY(h->w_s_c.alloc(shadow));
        h->w_s2_o.release(); h->w_s2_d.release(); h->w_s2_c.release(); h->w_vis.release();
        h->wide_capacity = cap;
        h->wide_shadow = shadow;
        h->wide_graph_valid = false;
    }
    if (!h->w_counts.p) {
        CUDA_TRY(h->w_counts.alloc(DFPT_COUNTS_SIZE));
        CUDA_TRY(h->w_wave_entries.alloc(1));
        CUDA_TRY(h->w_scene.alloc(1));
        CUDA_TRY(h->w_wave_base.alloc(5));
        CUDA_TRY(h->w_wave_tab.alloc(8));
        // Offsets, then the ray and the shadow-ray counts (zero at rest).
        CUDA_TRY(h->w_sort_bins.alloc(3 * DFPT_SORT_BINS + DFPT_SORT_CHUNKS));
        CUDA_TRY(cudaMemsetAsync(h->w_sort_bins.p, 0, (3 * DFPT_SORT_BINS + DFPT_SORT_CHUNKS) * sizeof(int), h->stream));
        const std::vector<long long> sb = {0, 1ll << 62}, fb = {0, (long long)n};
        CUDA_TRY(upload(h->w_sample_begin, sb, h->stream));
        CUDA_TRY(upload(h->w_film_begin, fb, h->stream));
    }
    // The scene record (culling mode and pointers may change between calls).
    std::vector<DevScene> one(1, h->sc.scene);
    CUDA_TRY(upload(h->w_scene, one, h->stream));
    DevPass& B = h->wpass;
    B = DevPass{};
    B.n_pixels = h->wide_capacity;
    B.q_o[0] = h->w_q_o0.p; B.q_o[1] = h->w_q_o1.p; B.q_d[0] = h->w_q_d0.p; B.q_d[1] = h->w_q_d1.p;
    B.q_hit = h->w_q_hit.p; B.s_o = h->w_s_o.p; B.s_d = h->w_s_d.p; B.s_c = h->w_s_c.p;
    B.throughput = h->w_throughput.p; B.radiance = h->w_throughput.p + 1; B.rng = h->w_rng.p; B.pixel_flags = h->w_pixel_flags.p;
    B.counts = h->w_counts.p; B.stats = h->stats.p; B.pass_index = h->pass_index.p;
    B.film_sum = h->film_sum.p; B.film_comp = h->film_comp.p; B.film_n = h->film_n.p; B.bgra = h->bgra.p;
    B.sorted_queues = (h->ray_sort && h->wide.b_sort) ? 1 : 0;
    B.sort_bins = h->w_sort_bins.p;
    B.primitive_offsets = h->primitive_offsets.p;  // selection buffer: first hits of the call's last pass
    B.sort_count = h->w_sort_bins.p + DFPT_SORT_BINS;
    B.sort_count_shadow = h->shadow_sort ? h->w_sort_bins.p + 2 * DFPT_SORT_BINS : nullptr;  // null: shadow rays unbinned
    B.sort_partials = h->w_sort_bins.p + 3 * DFPT_SORT_BINS;
    if (h->diff_on) {
        // The differentiable forward / replay: visibility bits per slot, the per-sample records.
        if (!h->w_vis.p) CUDA_TRY(h->w_vis.alloc((size_t)h->wide_capacity));
        B.vis = h->w_vis.p;
        B.diff_L = h->pass.diff_L; B.diff_vis = h->pass.diff_vis; B.diff_dldi = h->pass.diff_dldi;
        B.diff_rows = h->pass.diff_rows; B.diff_row_len = h->pass.diff_row_len;
    }
    if (B.sorted_queues && !h->w_s2_o.p) {
        CUDA_TRY(h->w_s2_o.alloc(h->wide_shadow));
        CUDA_TRY(h->w_s2_d.alloc(h->wide_shadow));
        CUDA_TRY(h->w_s2_c.alloc(h->wide_shadow));
    }
    h->wpass_shadow = B;
    if (B.sorted_queues) {
        h->wpass_shadow.s_o = h->w_s2_o.p;
        h->wpass_shadow.s_d = h->w_s2_d.p;
        h->wpass_shadow.s_c = h->w_s2_c.p;
    }
    DevBatch& Q = h->wq;
    Q.scenes = h->w_scene.p;
    Q.params = h->dev_params.p;
    Q.sample_begin = h->w_sample_begin.p;
    Q.film_begin = h->w_film_begin.p;
    Q.n_scenes = 1;
    Q.capacity = h->wide_capacity;
    Q.total = 1ll << 62;
    Q.wave_base = h->w_wave_base.p;
    Q.slot_key = h->w_slot_key.p;
    Q.wave_tab = h->w_wave_tab.p;
    Q.wave_entries = h->w_wave_entries.p;
    LaunchCtx& c = h->wctx;
    c = h->ctx;
    c.scene = &h->sc.scene;  // the one-scene batch kernels take the scene record as their parameter
    h->wide.occupancy(h->sms, c.grid, c.grid_trace, c.grid_simple);
    c.grid_trace = h->wide.trace_grid(c.trace_config, h->sms);
    c.pass = &h->wpass;
    c.batch = &h->wq;
    h->wctx_shadow = c;
    h->wctx_shadow.pass = &h->wpass_shadow;
    if (h->shadow_config >= 0 && h->shadow_config < h->wide.trace_configs) {
        h->wctx_shadow.trace_config = h->shadow_config;
        h->wctx_shadow.grid_trace = h->wide.trace_grid(h->shadow_config, h->sms);
    }
    return DFPT_OK;
}

// One wave; returns the number of kernels launched.
cudaError_t graph_l2_window(dfpt_handle* h, cudaGraph_t g);

int issue_wide_wave(dfpt_handle* h) {
    const KernelSet& K = h->wide;
    const LaunchCtx& c = h->wctx;
    int k = 0;
    cudaMemsetAsync(h->w_counts.p, 0, DFPT_COUNTS_SIZE * sizeof(int), h->stream);
    K.b_wave(c, 0); ++k;
    mark(h, KIND_CAMERA); K.b_camera(c, 0); ++k;
    const int nb = bounces_of(h);
    // Sun shadow rays: traced right after each bounce's shading (the queue holds one bounce), or,
    // with shadow_defer, all bounces' at once after the last bounce (queue of slots x depth).
    auto shadows = [&]() {
        if (h->sky.is_sun_active != 1) return;
        // h->wctx_shadow: the shadow launches' configuration, reading the binned copy.
        if (h->wpass.sorted_queues && h->wpass.sort_count_shadow) {
            mark(h, KIND_SORT); k += K.b_sort_shadow(c, h->wpass_shadow);
            mark(h, KIND_SHADOW); K.b_shadow(h->wctx_shadow, 0); ++k;
        } else {
            LaunchCtx cs = h->wctx_shadow;
            cs.pass = c.pass;
            mark(h, KIND_SHADOW); K.b_shadow(cs, 0); ++k;
        }
        mark(h, KIND_END); K.b_shadow_reset(c, 0); ++k;
    };
    for (int b = 0; b < nb; ++b) {
        mark(h, KIND_TRACE); K.b_trace_closest(c, b); ++k;
        mark(h, KIND_SHADE); K.b_shade(c, b); ++k;
        if (h->wpass.sorted_queues) { mark(h, KIND_SORT); k += K.b_sort(c, b, true); }
        if (!h->shadow_defer) shadows();
    }
    mark(h, KIND_FINAL); K.b_final(c, nb); ++k;
    if (h->shadow_defer) shadows();
    mark(h, KIND_FILM); K.b_film(c, 0); ++k;
    mark(h, KIND_END); K.b_end(c, 0); ++k;
    mark(h, KIND_COUNT);
    return k;
}

// Passes host_pass .. host_pass + passes - 1 as waves of wide_samples passes.
int render_wide(dfpt_handle* h, int passes) {
    int r = wide_prepare(h);
    if (r) return r;
    const long long n = h->n_pixels;
    // The RNG pass of sample j is host_pass + j; the film restarts at the clear pass if it is here.
    const long long cs = (long long)h->clear_pass - h->host_pass;
    h->wide_range[0] = 0;
    h->wide_range[1] = (long long)passes * n;
    h->wide_range[2] = h->host_pass;
    h->wide_range[3] = (cs >= 0 && cs < passes) ? cs : -1;
    h->wide_range[4] = h->host_pass + passes - 1;  // the selection buffer shows the last pass
    CUDA_TRY(cudaMemcpyAsync(h->w_wave_base.p, h->wide_range, 5 * sizeof(long long), cudaMemcpyHostToDevice, h->stream));
    const long long waves = (h->wide_range[1] + h->wide_capacity - 1) / h->wide_capacity;
    if (h->use_graph && !h->profiling) {
        if (!h->wide_graph_valid) {
            if (h->wide_graph) cudaGraphExecDestroy(h->wide_graph);
            h->wide_graph = nullptr;
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            const int k = issue_wide_wave(h);
            cudaError_t e = cudaStreamEndCapture(h->stream, &g);
            if (e == cudaSuccess) e = graph_l2_window(h, g);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&h->wide_graph, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                h->wide_graph = nullptr;
                return dfpt_fail(DFPT_ERR_CUDA, "wide-pass graph: %s", cudaGetErrorString(e));
            }
            h->wide_graph_kernels = k;
            h->wide_graph_valid = true;
        }
        for (long long w = 0; w < waves; ++w) {
            CUDA_TRY(cudaGraphLaunch(h->wide_graph, h->stream));
            h->launches += (uint64_t)h->wide_graph_kernels;
        }
    } else {
        for (long long w = 0; w < waves; ++w) h->launches += (uint64_t)issue_wide_wave(h);
        CUDA_TRY(cudaGetLastError());
    }
    // The image: the film tone mapped, with the selection highlight of the last pass's first hits.
    mark(h, KIND_FILM);
    h->wide.b_resolve(h->wctx, 0);
    h->launches += 1;
    mark(h, KIND_COUNT);
    CUDA_TRY(cudaGetLastError());
    // The device pass counter follows (the next normal pass reads it).
    h->host_pass += passes;
    h->pass_index_host = h->host_pass;
    CUDA_TRY(cudaMemcpyAsync(h->pass_index.p, &h->pass_index_host, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    return DFPT_OK;
}

int bounces_of(const dfpt_handle* h) {
    const int d = h->params.pt_ray_depth_maximum;
    return d < 1 ? 1 : (d > DFPT_MAX_DEPTH ? DFPT_MAX_DEPTH : d);
}

// Each path emits at most one shadow ray per bounce, so pixels x bounces rays always fit.
int ensure_shadow_capacity(dfpt_handle* h) {
    const size_t need = (size_t)h->n_pixels * (size_t)bounces_of(h);
    if (h->shadow_capacity >= need) return DFPT_OK;
    h->s_o.release(); h->s_d.release(); h->s_c.release();
    CUDA_TRY(h->s_o.alloc(need));
    CUDA_TRY(h->s_d.alloc(need));
    CUDA_TRY(h->s_c.alloc(need));
    h->shadow_capacity = need;
    h->pass.s_o = h->s_o.p; h->pass.s_d = h->s_d.p; h->pass.s_c = h->s_c.p;
    h->graph_valid = false;
    h->wide_graph_valid = false;
    return DFPT_OK;
}

// Plain passes' binning: the bins, the binned copy of the shadow queue (as large as the queue) and
// of bounce 1's queue (a ray per pixel), or none; `pass` gets the bin pointers its shading counts
// the shadow rays into, pass_ray_count those of bounce 1's rays.
int pass_shadow_sort_prepare(dfpt_handle* h) {
    DevPass& B = h->pass;
    if (!h->pass_shadow_sort && h->pass_ray_sort <= 0) {
        if (B.sort_bins) {
            B.sort_bins = B.sort_count = B.sort_count_shadow = B.sort_partials = nullptr;
            h->graph_valid = false;
        }
        h->pass_ray_read = DevPass{};
        return DFPT_OK;
    }
    if (!h->p_sort_bins.p) {
        CUDA_TRY(h->p_sort_bins.alloc(3 * DFPT_SORT_BINS + DFPT_SORT_CHUNKS));
        CUDA_TRY(cudaMemsetAsync(h->p_sort_bins.p, 0, (3 * DFPT_SORT_BINS + DFPT_SORT_CHUNKS) * sizeof(int), h->stream));
    }
    if (h->p_s2_capacity < h->shadow_capacity) {
        h->p_s2_o.release(); h->p_s2_d.release(); h->p_s2_c.release();
        CUDA_TRY(h->p_s2_o.alloc(h->shadow_capacity));
        CUDA_TRY(h->p_s2_d.alloc(h->shadow_capacity));
        CUDA_TRY(h->p_s2_c.alloc(h->shadow_capacity));
        h->p_s2_capacity = h->shadow_capacity;
        h->graph_valid = false;
    }
    if (h->pass_ray_sort > 0 && !h->p_r2_o.p) {
        CUDA_TRY(h->p_r2_o.alloc((size_t)h->n_pixels));
        CUDA_TRY(h->p_r2_d.alloc((size_t)h->n_pixels));
        h->graph_valid = false;
    }
    int* const shadow_counts = h->pass_shadow_sort ? h->p_sort_bins.p + 2 * DFPT_SORT_BINS : nullptr;
    if (B.sort_count_shadow != shadow_counts || B.sort_bins != h->p_sort_bins.p) h->graph_valid = false;
    B.sort_bins = h->p_sort_bins.p;
    B.sort_count = nullptr;  // counted by bounce 0's shading only (pass_ray_count)
    B.sort_count_shadow = shadow_counts;
    B.sort_partials = h->p_sort_bins.p + 3 * DFPT_SORT_BINS;
    B.sort_ray_bits = h->pass_ray_sort;
    h->pass_shadow2 = B;
    h->pass_shadow2.s_o = h->p_s2_o.p;
    h->pass_shadow2.s_d = h->p_s2_d.p;
    h->pass_shadow2.s_c = h->p_s2_c.p;
    h->pass_ray_count = B;
    h->pass_ray_count.sort_count = h->p_sort_bins.p + DFPT_SORT_BINS;
    h->pass_ray_read = DevPass{};
    if (h->pass_ray_sort > 0) {
        h->pass_ray_read = B;
        h->pass_ray_read.q_o[1] = h->p_r2_o.p;
        h->pass_ray_read.q_d[1] = h->p_r2_d.p;
    }
    return DFPT_OK;
}

// L2 residency: the traversal records (BVH nodes + triangles, one allocation) get an access-policy
// window - hits persisting, misses streaming - on every kernel node of the pass and wave graphs,
// and on the handle's stream when the handle created that stream, so the ray queues and path
// state streaming through L2 each bounce do not evict the scene. A stream the caller passed to
// dfpt_set_stream is never given the window: it outlives the handle, and a window left on it
// would keep marking a freed range (or another handle's) as persisting. The persisting carve-out
// is a limit of this process's CUDA context (it ends with it).
int apply_l2_policy(dfpt_handle* h) {
    cudaAccessPolicyWindow w{};
    if (h->l2_persist && h->sc.trav.p) {
        int dev = 0, max_window = 0, max_persist = 0;
        CUDA_TRY(cudaGetDevice(&dev));
        CUDA_TRY(cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev));
        CUDA_TRY(cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev));
        const size_t bytes = std::min(h->sc.trav.n * sizeof(float4), (size_t)std::max(max_window, 0));
        if (bytes > 0 && max_persist > 0) {
            size_t current = 0;
            CUDA_TRY(cudaDeviceGetLimit(&current, cudaLimitPersistingL2CacheSize));
            const size_t want = std::min(bytes, (size_t)max_persist);
            if (current < want) CUDA_TRY(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want));
            w.base_ptr = h->sc.trav.p;
            w.num_bytes = bytes;
            w.hitRatio = (float)std::min(1.0, (double)want / (double)bytes);
            w.hitProp = cudaAccessPropertyPersisting;
            w.missProp = cudaAccessPropertyStreaming;
        }
    }
    h->l2_window = w;
    if (h->own_stream) {
        cudaStreamAttrValue v{};
        v.accessPolicyWindow = w;
        CUDA_TRY(cudaStreamSetAttribute(h->stream, cudaStreamAttributeAccessPolicyWindow, &v));
    }
    return DFPT_OK;
}

// The handle's L2 window on every kernel node of a captured graph (capture does not carry it).
cudaError_t graph_l2_window(dfpt_handle* h, cudaGraph_t g) {
    if (h->l2_window.num_bytes == 0) return cudaSuccess;
    size_t count = 0;
    cudaError_t e = cudaGraphGetNodes(g, nullptr, &count);
    std::vector<cudaGraphNode_t> nodes(count);
    if (e == cudaSuccess && count) e = cudaGraphGetNodes(g, nodes.data(), &count);
    cudaKernelNodeAttrValue kv{};
    kv.accessPolicyWindow = h->l2_window;
    for (size_t i = 0; e == cudaSuccess && i < count; ++i) {
        cudaGraphNodeType type;
        e = cudaGraphNodeGetType(nodes[i], &type);
        if (e == cudaSuccess && type == cudaGraphNodeTypeKernel)
            e = cudaGraphKernelNodeSetAttribute(nodes[i], cudaKernelNodeAttributeAccessPolicyWindow, &kv);
    }
    return e;
}

int build_graph(dfpt_handle* h) {
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
    h->graph_valid = false;
    h->wide_graph_valid = false;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int k = issue_pass(h);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    }
    e = graph_l2_window(h, g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        cudaGraphDestroy(g);
        return dfpt_fail(DFPT_ERR_CUDA, "graph L2 window: %s", cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&h->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        h->graph_exec = nullptr;
        return dfpt_fail(DFPT_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    }
    h->graph_kernels = k;
    h->graph_valid = true;
    return DFPT_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// SceneStore: validation and upload of one compiled scene.

void SceneStore::release() {
    DevBuf<float>* fb[] = {&point2fs, &point3fs, &vector3fs, &spheres, &terrains, &textures, &surfaces, &o2w, &w2o, &camera};
    for (auto* b : fb) b->release();
    DevBuf<int>* ib[] = {&planes, &triangles, &primitives};
    for (auto* b : ib) b->release();
    DevBuf<float4>* f4[] = {&trav, &pairs, &shade_tris, &sphere4, &plane_a, &plane_n, &prim_ext, &cull_nodes, &prim_box};
    for (auto* b : f4) b->release();
    prim_info.release();
    cull_prims.release();
    always.release();
}

int scene_load(const dfpt_scene_desc* sd, SceneStore& st) {
    if (!sd) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL scene");
    if (sd->camera_count < 19 || !sd->camera) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "camera needs 19 floats");
    if (sd->primitives_count % 3 != 0) return dfpt_fail(DFPT_ERR_INVALID_SCENE, "primitives count %lld is not a multiple of 3", (long long)sd->primitives_count);
    const int64_t np = sd->primitives_count / 3;
    if (sd->primitives_object_to_world_count < np * 16 || sd->primitives_world_to_object_count < np * 16)
        return dfpt_fail(DFPT_ERR_INVALID_SCENE, "primitive matrices need 16 floats per primitive");
    HostScene& s = st.host;
    copy_array(s.point2fs, sd->point2fs, sd->point2fs_count);
    copy_array(s.point3fs, sd->point3fs, sd->point3fs_count);
    copy_array(s.vector3fs, sd->vector3fs, sd->vector3fs_count);
    copy_array(s.planes, sd->planes, sd->planes_count);
    copy_array(s.spheres, sd->spheres, sd->spheres_count);
    copy_array(s.terrains, sd->terrains, sd->terrains_count);
    copy_array(s.triangles, sd->triangles, sd->triangles_count);
    copy_array(s.bvh, sd->bounding_volume_hierarchies, sd->bounding_volume_hierarchies_count);
    copy_array(s.textures, sd->textures, sd->textures_count);
    copy_array(s.surfaces, sd->surfaces, sd->surfaces_count);
    s.primitives.assign(sd->primitives, sd->primitives + sd->primitives_count);
    s.o2w.assign(sd->primitives_object_to_world, sd->primitives_object_to_world + np * 16);
    s.w2o.assign(sd->primitives_world_to_object, sd->primitives_world_to_object + np * 16);
    if (s.o2w.empty()) { s.o2w.assign(16, 0.0f); s.w2o.assign(16, 0.0f); }
    s.camera.assign(sd->camera, sd->camera + 19);
    s.prim_ext.clear();
    if (sd->primitive_extensions_count != 0 || sd->primitive_extensions) {
        if (!sd->primitive_extensions || sd->primitive_extensions_count != np * 4)
            return dfpt_fail(DFPT_ERR_INVALID_SCENE, "primitive extensions need 4 floats per primitive (%lld given for %lld primitives)",
                             (long long)sd->primitive_extensions_count, (long long)np);
        for (int64_t i = 0; i < np; ++i) {
            const float* x = sd->primitive_extensions + 4 * i;
            if (!(x[0] >= 0.0f && x[0] <= 1.0e6f) || !std::isfinite(x[1]) || !std::isfinite(x[2]) || !std::isfinite(x[3]) ||
                x[1] < 0.0f || x[2] < 0.0f || x[3] < 0.0f)
                return dfpt_fail(DFPT_ERR_INVALID_SCENE, "primitive %lld: bad extension record {%g, %g, %g, %g}", (long long)i, x[0],
                                 x[1], x[2], x[3]);
            s.prim_ext.push_back(make_float4(x[0], x[1], x[2], x[3]));
        }
    }
    Derived& d = st.derived;
    int r = build_derived(s, d);
    if (r) return r;
    cull_object_bounds(d, (int)np, st.obj_box);
    build_culling(st.obj_box, s.w2o, (int)np, d);
    if (d.nodes.size() / 2 > (size_t)INT32_MAX / 4 || d.tris.size() / 3 > (size_t)INT32_MAX / 4) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "scene too large");
    st.scene.primitive_count = (int)np;
    st.scene.textures_count = (int)s.textures.size();
    return DFPT_OK;
}

int scene_upload(SceneStore& st, cudaStream_t s) {
    const HostScene& h = st.host;
    Derived& d = st.derived;
    CUDA_TRY(upload(st.point2fs, h.point2fs, s));
    CUDA_TRY(upload(st.point3fs, h.point3fs, s));
    CUDA_TRY(upload(st.vector3fs, h.vector3fs, s));
    CUDA_TRY(upload(st.planes, h.planes, s));
    CUDA_TRY(upload(st.spheres, h.spheres, s));
    CUDA_TRY(upload(st.terrains, h.terrains, s));
    CUDA_TRY(upload(st.triangles, h.triangles, s));
    CUDA_TRY(upload(st.textures, h.textures, s));
    CUDA_TRY(upload(st.surfaces, h.surfaces, s));
    CUDA_TRY(upload(st.primitives, h.primitives, s));
    CUDA_TRY(upload(st.o2w, h.o2w, s));
    CUDA_TRY(upload(st.w2o, h.w2o, s));
    CUDA_TRY(upload(st.camera, h.camera, s));
    CUDA_TRY(upload(st.prim_info, d.prim_info, s));
    {
        std::vector<float4> trav(d.nodes);
        trav.insert(trav.end(), d.tris.begin(), d.tris.end());
        st.trav_nodes = d.nodes.size();
        CUDA_TRY(upload(st.trav, trav, s));
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    {
        // Pair records. The walk over them assumes every inner node N has two children: L = N + 1,
        // R = next(L), and R's subtree ends where N's does (next(R) == next(N)); otherwise the
        // scene keeps the threaded walk alone.
        const size_t nn = d.nodes.size() / 2;
        std::vector<float4> pairs(4 * nn, make_float4(0, 0, 0, 0));
        bool full_binary = true, empty_leaf = false;
        auto next_of = [&](size_t n) { return float_bits_int(d.nodes[2 * n].w); };
        auto leaf_of = [&](size_t n) { return float_bits_int(d.nodes[2 * n + 1].w); };
        for (size_t n = 0; n < nn && full_binary; ++n) {
            if (leaf_of(n) == -2) empty_leaf = true;
            if (leaf_of(n) != -1) continue;
            const size_t l = n + 1;
            const int r = l < nn ? next_of(l) : -1;
            if (l >= nn || r < 0 || (size_t)r >= nn || next_of((size_t)r) != next_of(n)) { full_binary = false; break; }
            const float4 lo = d.nodes[2 * l], lh = d.nodes[2 * l + 1], ro = d.nodes[2 * (size_t)r], rh = d.nodes[2 * (size_t)r + 1];
            pairs[4 * n] = make_float4(lo.x, lo.y, lo.z, lh.x);
            pairs[4 * n + 1] = make_float4(lh.y, lh.z, ro.x, ro.y);
            pairs[4 * n + 2] = make_float4(ro.z, rh.x, rh.y, rh.z);
            pairs[4 * n + 3] = make_float4(lh.w, rh.w, int_bits(r), 0.0f);
        }
        st.scene.use_pairs = full_binary ? (empty_leaf ? 1 : 2) : 0;
        st.scene.pair_stack = 8;
        CUDA_TRY(upload(st.pairs, pairs, s));
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    {
        // Shading records: the triangle's vertex values in one 144-byte record, indexed by triangle
        // offset / 12, when every triangle the traversal can report sits at a multiple of 12.
        bool aligned = true;
        for (size_t k = 0; k < d.tris.size(); k += 3)
            if (float_bits_int(d.tris[k].w) % 12 != 0) aligned = false;
        const size_t nt = h.triangles.size() / 12;
        st.shade_tris.release();
        if (aligned && nt > 0) {
            std::vector<float4> rec(9 * nt, make_float4(0, 0, 0, 0));
            auto ok3 = [&](int i, size_t n) { return i >= 0 && (size_t)i + 3 <= n; };
            for (size_t t = 0; t < nt; ++t) {
                const int* T = h.triangles.data() + 12 * t;
                bool valid = true;
                for (int k = 0; k < 3; ++k) valid = valid && ok3(T[k], h.point3fs.size()) && ok3(T[3 + k], h.vector3fs.size()) &&
                                                    ok3(T[9 + k], h.vector3fs.size()) && T[6 + k] >= 0 &&
                                                    (size_t)T[6 + k] + 2 <= h.point2fs.size();
                if (!valid) continue;  // never reported by the traversal (it reports validated triangles only)
                const float* P = h.point3fs.data();
                const float* V = h.vector3fs.data();
                const float* U = h.point2fs.data();
                const float* a = P + T[0]; const float* b = P + T[1]; const float* c = P + T[2];
                const float* na = V + T[3]; const float* nb = V + T[4]; const float* nc = V + T[5];
                const float* ua = U + T[6]; const float* ub = U + T[7]; const float* uc = U + T[8];
                const float* ga = V + T[9]; const float* gb = V + T[10]; const float* gc = V + T[11];
                float4* R = rec.data() + 9 * t;
                R[0] = make_float4(a[0], a[1], a[2], b[0]);
                R[1] = make_float4(b[1], b[2], c[0], c[1]);
                R[2] = make_float4(c[2], ua[0], ua[1], ub[0]);
                R[3] = make_float4(ub[1], uc[0], uc[1], na[0]);
                R[4] = make_float4(na[1], na[2], nb[0], nb[1]);
                R[5] = make_float4(nb[2], nc[0], nc[1], nc[2]);
                R[6] = make_float4(ga[0], ga[1], ga[2], gb[0]);
                R[7] = make_float4(gb[1], gb[2], gc[0], gc[1]);
                R[8] = make_float4(gc[2], 0.0f, 0.0f, 0.0f);
            }
            CUDA_TRY(upload(st.shade_tris, rec, s));
            CUDA_TRY(cudaStreamSynchronize(s));
        }
    }
    CUDA_TRY(upload(st.sphere4, d.sphere4, s));
    CUDA_TRY(upload(st.plane_a, d.plane_a, s));
    CUDA_TRY(upload(st.plane_n, d.plane_n, s));
    st.prim_ext.release();
    if (!h.prim_ext.empty()) CUDA_TRY(upload(st.prim_ext, h.prim_ext, s));
    int rc = culling_upload(st, d, s);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors below are freed
    DevScene& S = st.scene;
    S.point2fs = st.point2fs.p; S.point3fs = st.point3fs.p; S.vector3fs = st.vector3fs.p;
    S.planes = st.planes.p; S.spheres = st.spheres.p; S.terrains = st.terrains.p; S.triangles = st.triangles.p;
    S.textures = st.textures.p; S.surfaces = st.surfaces.p; S.primitives = st.primitives.p;
    S.o2w = st.o2w.p; S.w2o = st.w2o.p; S.camera = st.camera.p;
    S.prim_info = st.prim_info.p; S.nodes = st.trav.p; S.tris = st.trav.p + st.trav_nodes; S.sphere4 = st.sphere4.p;
    S.pairs = st.pairs.p;
    S.shade_tris = st.shade_tris.p;
    S.plane_a = st.plane_a.p; S.plane_n = st.plane_n.p;
    S.prim_ext = h.prim_ext.empty() ? nullptr : st.prim_ext.p;
    st.derived = Derived();
    return DFPT_OK;
}

int culling_upload(SceneStore& st, const Derived& d, cudaStream_t s) {
    CUDA_TRY(upload(st.cull_nodes, d.cull_nodes, s));
    CUDA_TRY(upload(st.prim_box, d.prim_box, s));
    CUDA_TRY(upload(st.cull_prims, d.cull_prims, s));
    std::vector<int> always = d.always;
    if (always.empty()) always.push_back(0);
    CUDA_TRY(upload(st.always, always, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    DevScene& S = st.scene;
    S.cull_nodes = st.cull_nodes.p; S.prim_box = st.prim_box.p; S.cull_prims = st.cull_prims.p;
    S.always = st.always.p;
    S.always_count = (int)d.always.size();
    S.bounds_lo = d.bounds_lo;
    S.bounds_hi = d.bounds_hi;
    // Culling is offered for scenes with 8 or more bounded primitives; the default mode is the
    // per-primitive box test, the autotuner may pick the BVH candidates or none.
    st.culling_available = d.bounded >= 8;
    S.use_culling = st.culling_available ? st.culling_wanted : 0;
    return DFPT_OK;
}

int scene_rebuild_culling(SceneStore& st, cudaStream_t s) {
    Derived d;
    build_culling(st.obj_box, st.host.w2o, st.scene.primitive_count, d);
    return culling_upload(st, d, s);
}

void scene_set_culling(SceneStore& st, int mode) {
    st.culling_wanted = mode;
    st.scene.use_culling = st.culling_available ? mode : 0;
}

int noise_tables_init(const KernelSet& ks, cudaStream_t st) {
    std::vector<int> perm(DFPT_PERMUTATION, DFPT_PERMUTATION + 256);
    std::vector<float> grad(DFPT_GRADIENT3, DFPT_GRADIENT3 + 36);
    DevBuf<int> dperm;
    DevBuf<float> dgrad;
    cudaError_t e = upload(dperm, perm, st);
    if (e == cudaSuccess) e = upload(dgrad, grad, st);
    if (e == cudaSuccess) {
        ks.init_tables(st, dperm.p, dgrad.p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dperm.release();
    dgrad.release();
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "noise tables: %s", cudaGetErrorString(e));
    }
    return DFPT_OK;
}

extern "C" {

const char* dfpt_last_error(void) { return g_last_error.c_str(); }

int dfpt_create(const dfpt_scene_desc* sd, const dfpt_sky* sky, int32_t width, int32_t height, dfpt_handle** out) {
    if (!sd || !sky || !out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (width <= 0 || height <= 0 || (int64_t)width * (int64_t)height > (1ll << 28))
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "resolution %d x %d is not supported", width, height);
    auto h = new dfpt_handle();
    int r = scene_load(sd, h->sc);
    if (r) { delete h; return r; }

    h->width = width;
    h->height = height;
    h->n_pixels = width * height;
    h->fast = dfpt_fast::kernel_set();
    h->strict = dfpt_strict::kernel_set();
    h->wide = dfpt_wide::kernel_set();
    h->sky = *sky;
    dfpt_params_default(&h->params);
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { (void)cudaGetLastError(); delete h; return dfpt_fail(DFPT_ERR_CUDA, "CUDA device unavailable: %s", cudaGetErrorString(ce)); }
    h->own_stream = true;
    cudaStream_t st = h->stream;
    r = scene_upload(h->sc, st);
    if (r) { release(h); delete h; return r; }

#define TRY_R(expr) do { cudaError_t e_ = (expr); if (e_ != cudaSuccess) { (void)cudaGetLastError(); int code = e_ == cudaErrorMemoryAllocation ? DFPT_ERR_OUT_OF_MEMORY : DFPT_ERR_CUDA; dfpt_fail(code, "%s: %s", #expr, cudaGetErrorString(e_)); release(h); delete h; return code; } } while (0)
    const size_t n = (size_t)h->n_pixels;
    TRY_R(h->q_o0.alloc(n)); TRY_R(h->q_o1.alloc(n)); TRY_R(h->q_d0.alloc(n)); TRY_R(h->q_d1.alloc(n));
    TRY_R(h->q_hit.alloc(n));
    TRY_R(h->throughput.alloc(2 * n)); TRY_R(h->rng.alloc(n)); TRY_R(h->pixel_flags.alloc(n));
    TRY_R(h->primary_o.alloc(n)); TRY_R(h->primary_d.alloc(n));
    TRY_R(h->counts.alloc(DFPT_COUNTS_SIZE)); TRY_R(h->stats.alloc(6)); TRY_R(h->pass_index.alloc(1)); TRY_R(h->mean.alloc(3));
    TRY_R(h->film_sum.alloc(n)); TRY_R(h->film_comp.alloc(n)); TRY_R(h->film_n.alloc(n)); TRY_R(h->bgra.alloc(n * 4));
    TRY_R(h->primitive_offsets.alloc(n));
    TRY_R(h->hit_prim.alloc(n)); TRY_R(h->hit_type.alloc(n)); TRY_R(h->hit_off.alloc(n)); TRY_R(h->hit_dist.alloc(n)); TRY_R(h->hit_normal.alloc(3 * n));
    TRY_R(h->scratch_rgb.alloc(3 * n));
    TRY_R(h->dev_params.alloc(1));
    TRY_R(cudaMemsetAsync(h->film_sum.p, 0, n * sizeof(float4), st));
    TRY_R(cudaMemsetAsync(h->film_comp.p, 0, n * sizeof(float4), st));
    TRY_R(cudaMemsetAsync(h->film_n.p, 0, n * sizeof(int), st));
    TRY_R(cudaMemsetAsync(h->primitive_offsets.p, 0xFF, n * sizeof(int), st));  // Arrays.fill(-1) (GRK:421)
    TRY_R(cudaMemsetAsync(h->hit_normal.p, 0, 3 * n * sizeof(float), st));
    TRY_R(cudaMemsetAsync(h->stats.p, 0, 6 * sizeof(unsigned long long), st));
    TRY_R(cudaMemsetAsync(h->pass_index.p, 0, sizeof(int), st));
    TRY_R(cudaMemsetAsync(h->pixel_flags.p, 0, n * sizeof(int), st));
    DevPass& B = h->pass;
    B.n_pixels = h->n_pixels;
    B.q_o[0] = h->q_o0.p; B.q_o[1] = h->q_o1.p; B.q_d[0] = h->q_d0.p; B.q_d[1] = h->q_d1.p;
    B.q_hit = h->q_hit.p; B.s_o = h->s_o.p; B.s_d = h->s_d.p; B.s_c = h->s_c.p;
    B.throughput = h->throughput.p; B.radiance = h->throughput.p + 1; B.rng = h->rng.p; B.pixel_flags = h->pixel_flags.p;
    B.primary_o = h->primary_o.p; B.primary_d = h->primary_d.p; B.counts = h->counts.p; B.stats = h->stats.p;
    B.pass_index = h->pass_index.p; B.film_sum = h->film_sum.p; B.film_comp = h->film_comp.p; B.film_n = h->film_n.p;
    B.bgra = h->bgra.p; B.primitive_offsets = h->primitive_offsets.p;
    B.hit_prim_offset = h->hit_prim.p; B.hit_shape_type = h->hit_type.p; B.hit_shape_offset = h->hit_off.p;
    B.hit_distance = h->hit_dist.p; B.hit_normal = h->hit_normal.p;

    // Noise tables (both kernel sets own a copy).
    r = noise_tables_init(h->fast, st);
    if (!r) r = noise_tables_init(h->strict, st);
    if (!r) r = noise_tables_init(h->wide, st);
    if (r) { release(h); delete h; return r; }
    TRY_R(cudaStreamSynchronize(st));
#undef TRY_R

    h->ctx.scene = &h->sc.scene;
    h->ctx.params = h->dev_params.p;
    h->ctx.pass = &h->pass;
    h->ctx.stream = h->stream;
    h->fast.occupancy(h->sms, h->ctx.grid, h->ctx.grid_trace, h->ctx.grid_simple);
    // The compact pair walk: the autotuner's pick on every workload measured (the same hits as
    // every other configuration).
    h->ctx.trace_config = DFPT_DEFAULT_TRACE_CONFIG < h->fast.trace_configs ? DFPT_DEFAULT_TRACE_CONFIG : 0;
    h->ctx.grid_trace = h->fast.trace_grid(h->ctx.trace_config, h->sms);
    r = push_params(h);
    if (!r) r = reset_rng(h);
    if (!r) r = apply_l2_policy(h);
    if (r) { release(h); delete h; return r; }
    *out = h;
    return DFPT_OK;
}

int dfpt_destroy(dfpt_handle* h) {
    if (!h) return DFPT_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    release(h);
    delete h;
    return DFPT_OK;
}

int dfpt_set_stream(dfpt_handle* h, void* stream) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->own_stream = false;
    h->stream = (cudaStream_t)stream;
    if (!h->stream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    h->ctx.stream = h->stream;
    h->graph_valid = false;
    h->wide_graph_valid = false;
    return apply_l2_policy(h);
}

int dfpt_set_camera(dfpt_handle* h, const float* camera19) {
    if (!h || !camera19) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    h->sc.host.camera.assign(camera19, camera19 + 19);
    CUDA_TRY(cudaMemcpyAsync(h->sc.camera.p, h->sc.host.camera.data(), 19 * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    return push_params(h);  // the field-of-view tangents are derived from the camera
}

int dfpt_set_transforms(dfpt_handle* h, const float* o2w, const float* w2o, int32_t count) {
    if (!h || !o2w || !w2o) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (count != h->sc.scene.primitive_count) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "primitive count %d != %d", count, h->sc.scene.primitive_count);
    h->sc.host.o2w.assign(o2w, o2w + (size_t)count * 16);
    h->sc.host.w2o.assign(w2o, w2o + (size_t)count * 16);
    if (count == 0) return DFPT_OK;
    CUDA_TRY(cudaMemcpyAsync(h->sc.o2w.p, h->sc.host.o2w.data(), (size_t)count * 64, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->sc.w2o.p, h->sc.host.w2o.data(), (size_t)count * 64, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    // World bounds follow the new transforms (the culling arrays may be reallocated).
    int r = scene_rebuild_culling(h->sc, h->stream);
    if (r) return r;
    h->graph_valid = false;
    h->wide_graph_valid = false;
    return DFPT_OK;
}

int dfpt_set_surfaces(dfpt_handle* h, const float* surfaces, int64_t count) {
    if (!h || !surfaces) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (count != (int64_t)h->sc.host.surfaces.size()) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "surfaces count %lld != %zu", (long long)count, h->sc.host.surfaces.size());
    std::vector<float> old = h->sc.host.surfaces;
    h->sc.host.surfaces.assign(surfaces, surfaces + count);
    for (int i = 0; i < h->sc.scene.primitive_count; ++i) {
        int r = check_surface(h->sc.host, h->sc.host.primitives[3 * i + 2]);
        if (r) { h->sc.host.surfaces.swap(old); return r; }
    }
    CUDA_TRY(cudaMemcpyAsync(h->sc.surfaces.p, h->sc.host.surfaces.data(), (size_t)count * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

int dfpt_set_sky(dfpt_handle* h, const dfpt_sky* sky) {
    if (!h || !sky) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    const bool sun_changed = (h->sky.is_sun_active == 1) != (sky->is_sun_active == 1);
    h->sky = *sky;
    if (sun_changed) h->graph_valid = false;
    h->wide_graph_valid = false;
    return push_params(h);
}

int dfpt_set_params(dfpt_handle* h, const dfpt_params* p) {
    if (!h || !p) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (p->rng_kind != DFPT_RNG_COUNTER && p->rng_kind != DFPT_RNG_LCG) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "unknown rng kind %d", p->rng_kind);
    const bool reseed = p->seed != h->params.seed || p->rng_kind != h->params.rng_kind;
    if (p->renderer_type != h->params.renderer_type || p->pt_ray_depth_maximum != h->params.pt_ray_depth_maximum ||
        p->wireframes != h->params.wireframes)
        h->graph_valid = false;
    h->wide_graph_valid = false;
    h->params = *p;
    int r = push_params(h);
    if (r) return r;
    if (reseed) return reset_rng(h);
    return DFPT_OK;
}

// Not part of the public header: switches between the fast and the strict kernel set (the
// strict set reproduces the reference's float arithmetic operation for operation).
int dfpt_set_strict(dfpt_handle* h, int32_t strict) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    h->use_strict = strict != 0;
    if (h->use_strict) h->strict.occupancy(h->sms, h->ctx.grid, h->ctx.grid_trace, h->ctx.grid_simple);
    else h->fast.occupancy(h->sms, h->ctx.grid, h->ctx.grid_trace, h->ctx.grid_simple);
    h->ctx.grid_trace = kset(h).trace_grid(h->ctx.trace_config, h->sms);
    h->graph_valid = false;
    h->wide_graph_valid = false;
    return DFPT_OK;
}

int dfpt_set_tuning(dfpt_handle* h, const char* key, int32_t value) {
    if (!h || !key) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (std::strcmp(key, "trace_config") == 0) {
        if (value < 0 || value >= h->fast.trace_configs) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "trace_config %d out of range", value);
        h->ctx.trace_config = value;
        h->ctx.grid_trace = kset(h).trace_grid(value, h->sms);
        h->graph_valid = false;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "shadow_config") == 0) {
        if (value < -1 || value >= h->fast.trace_configs) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "shadow_config %d out of range", value);
        h->shadow_config = value;
        h->graph_valid = false;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "ray_sort") == 0) {
        h->ray_sort = value != 0;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "shadow_sort") == 0) {
        h->shadow_sort = value != 0;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "shadow_defer") == 0) {
        h->shadow_defer = value != 0;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "wide_samples") == 0) {
        if (value < 1 || value > 64) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "wide_samples %d outside [1, 64]", value);
        h->wide_samples = value;
        return DFPT_OK;
    }
    if (std::strcmp(key, "l2_persist") == 0) {
        h->l2_persist = value != 0;
        h->graph_valid = false;
    h->wide_graph_valid = false;
        return apply_l2_policy(h);
    }
    if (std::strcmp(key, "trace_carveout") == 0) {
        // Shared-memory carveout preference of the current configuration's closest-hit traversal
        // kernels (percent of the maximum; -1 the driver's choice). A process-wide attribute of
        // those kernels: it applies to every handle that uses them.
        if (value < -1 || value > 100) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "trace_carveout %d outside [-1, 100]", value);
        for (const KernelSet* ks : {&h->fast, &h->strict, &h->wide})
            if (ks->trace_carveout) ks->trace_carveout(h->ctx.trace_config, value);
        CUDA_TRY(cudaGetLastError());
        h->ctx.grid_trace = kset(h).trace_grid(h->ctx.trace_config, h->sms);
        h->graph_valid = false;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "pair_stack") == 0) {
        // Stack entries of the compact pair walk (trace configuration 16); fewer entries take its
        // overflow path more often, with the same hits and visits.
        if (value < 1 || value > 8) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "pair_stack %d outside [1, 8]", value);
        h->sc.scene.pair_stack = value;
        h->graph_valid = false;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "pixel_tiles") == 0) {
        h->pixel_tiles = value != 0;
        return push_params(h);
    }
    if (std::strcmp(key, "pass_shadow_sort") == 0) {
        h->pass_shadow_sort = value != 0;
        h->graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "pass_ray_sort") == 0) {
        if (value < 0 || value > 15 || value % 3 != 0)
            return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "pass_ray_sort %d: 0 or origin-grid bits 3, 6, 9, 12, 15", value);
        h->pass_ray_sort = value;
        h->graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "tail_blocks") == 0) {
        if (value < 2 || value > 4) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "tail_blocks %d outside [2, 4]", value);
        h->ctx.tail_blocks = value;
        h->graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "tail_bounce") == 0) {
        if (value < -1 || value > DFPT_MAX_DEPTH) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "tail_bounce %d outside [-1, %d]", value, DFPT_MAX_DEPTH);
        h->tail_bounce = value;
        h->graph_valid = false;
        return DFPT_OK;
    }
    if (std::strcmp(key, "primitive_culling") == 0) {
        if (value < 0 || value > 2) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "primitive_culling %d: 0 none, 1 box test, 2 BVH", value);
        scene_set_culling(h->sc, value);
        h->graph_valid = false;
        h->wide_graph_valid = false;
        return DFPT_OK;
    }
    return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "unknown tuning key '%s'", key);
}

int dfpt_get_tuning(dfpt_handle* h, const char* key, int32_t* value) {
    if (!h || !key || !value) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (std::strcmp(key, "trace_config") == 0) { *value = h->ctx.trace_config; return DFPT_OK; }
    if (std::strcmp(key, "trace_configs") == 0) { *value = h->fast.trace_configs; return DFPT_OK; }
    if (std::strcmp(key, "shadow_config") == 0) { *value = h->shadow_config; return DFPT_OK; }
    if (std::strcmp(key, "primitive_culling") == 0) { *value = h->sc.scene.use_culling; return DFPT_OK; }
    if (std::strcmp(key, "pair_stack") == 0) { *value = h->sc.scene.pair_stack; return DFPT_OK; }
    if (std::strcmp(key, "l2_persist") == 0) { *value = h->l2_window.num_bytes > 0 ? 1 : 0; return DFPT_OK; }
    if (std::strcmp(key, "wide_samples") == 0) { *value = h->wide_samples; return DFPT_OK; }
    if (std::strcmp(key, "pixel_tiles") == 0) { *value = h->pixel_tiles ? 1 : 0; return DFPT_OK; }
    if (std::strcmp(key, "tail_bounce") == 0) { *value = h->tail_bounce; return DFPT_OK; }
    if (std::strcmp(key, "pass_shadow_sort") == 0) { *value = h->pass_shadow_sort ? 1 : 0; return DFPT_OK; }
    if (std::strcmp(key, "pass_ray_sort") == 0) { *value = h->pass_ray_sort; return DFPT_OK; }
    if (std::strcmp(key, "tail_blocks") == 0) { *value = h->ctx.tail_blocks; return DFPT_OK; }
    if (std::strcmp(key, "ray_sort") == 0) { *value = h->ray_sort ? 1 : 0; return DFPT_OK; }
    if (std::strcmp(key, "shadow_defer") == 0) { *value = h->shadow_defer ? 1 : 0; return DFPT_OK; }
    if (std::strcmp(key, "shadow_sort") == 0) { *value = h->shadow_sort ? 1 : 0; return DFPT_OK; }
    return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "unknown tuning key '%s'", key);
}

// ---- Native frame tuner --------------------------------------------------------------------
// The launch structure of one-pass dfpt_render calls, picked by timing them (CUDA events on the
// handle's stream): the primitive culling mode (scenes with enough bounded primitives), the
// traversal configuration (the handle's, 16, 17), the tail launch's first bounce (-1 .. 4) and
// resident blocks (2 .. 4), then the shadow-ray binning on or off. The
// buffers a pass writes that outlive it (film, image, selection buffer, per-pixel RNG states and
// flags, primary-hit records, counters) and the pass counter are saved first and put back after,
// so the call changes only the tuning.
namespace {
struct SavedRegion {
    void* p;
    size_t bytes;
};
#define DFPT_REGION_OF(b) SavedRegion{(void*)(b).p, (b).n * sizeof(*(b).p)}

int tune_frame_sweep(dfpt_handle* h, int frames, float* best_ms) {
    const int nb = bounces_of(h);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        (void)cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        return dfpt_fail(DFPT_ERR_CUDA, "cudaEventCreate failed");
    }
    auto frame_ms = [&](float& ms) -> int {
        int r = dfpt_render(h, 1);  // untimed: builds the pass graph of this structure
        if (!r && cudaEventRecord(e0, h->stream) != cudaSuccess) r = dfpt_fail(DFPT_ERR_CUDA, "cudaEventRecord failed");
        for (int i = 0; !r && i < frames; ++i) r = dfpt_render(h, 1);
        if (!r && cudaEventRecord(e1, h->stream) != cudaSuccess) r = dfpt_fail(DFPT_ERR_CUDA, "cudaEventRecord failed");
        if (!r && cudaEventSynchronize(e1) != cudaSuccess) r = dfpt_fail(DFPT_ERR_CUDA, "frame timing failed");
        if (!r && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) r = dfpt_fail(DFPT_ERR_CUDA, "cudaEventElapsedTime failed");
        if (r) (void)cudaGetLastError();
        ms /= (float)frames;
        return r;
    };
    int r = DFPT_OK;
    // Primitive culling first, where the scene has enough bounded primitives for it (the setter
    // keeps 0 otherwise); every mode gives the same hits.
    {
        const int cull0 = h->sc.scene.use_culling;
        r = dfpt_set_tuning(h, "primitive_culling", 1);
        if (!r && h->sc.scene.use_culling == 1) {
            float best_ms = 3.4e38f;
            int best_mode = cull0;
            for (int mode = 0; mode <= 2 && !r; ++mode) {
                float ms = 0.0f;
                r = dfpt_set_tuning(h, "primitive_culling", mode);
                if (!r) r = frame_ms(ms);
                if (!r && ms < best_ms) { best_ms = ms; best_mode = mode; }
            }
            if (!r) r = dfpt_set_tuning(h, "primitive_culling", best_mode);
        } else if (!r) {
            r = dfpt_set_tuning(h, "primitive_culling", cull0);
        }
    }
    int configs[3] = {h->ctx.trace_config, 16, 17};
    int best_cfg = h->ctx.trace_config, best_blocks = h->ctx.tail_blocks, best_tail = h->tail_bounce;
    float best = 3.4e38f;
    for (int ci = 0; ci < 3 && !r; ++ci) {
        const int cfg = configs[ci];
        if (cfg >= h->fast.trace_configs || (ci > 0 && cfg == configs[0]) || (ci == 2 && cfg == configs[1])) continue;
        r = dfpt_set_tuning(h, "trace_config", cfg);
        for (int blocks = 2; blocks <= 4 && !r; ++blocks) {
            r = dfpt_set_tuning(h, "tail_blocks", blocks);
            for (int tail = -1; tail <= 4 && tail < nb && !r; ++tail) {
                if (tail < 0 && blocks != 2) continue;  // no tail launch: its blocks do not matter
                r = dfpt_set_tuning(h, "tail_bounce", tail);
                float ms = 0.0f;
                if (!r) r = frame_ms(ms);
                if (!r && ms < best) { best = ms; best_cfg = cfg; best_blocks = blocks; best_tail = tail; }
            }
        }
    }
    if (!r) r = dfpt_set_tuning(h, "trace_config", best_cfg);
    if (!r) r = dfpt_set_tuning(h, "tail_blocks", best_blocks);
    if (!r) r = dfpt_set_tuning(h, "tail_bounce", best_tail);
    if (!r) {
        const bool sort = h->pass_shadow_sort;
        float ms = 0.0f;
        r = dfpt_set_tuning(h, "pass_shadow_sort", sort ? 0 : 1);
        if (!r) r = frame_ms(ms);
        if (!r && ms < best) best = ms;
        else if (!r) r = dfpt_set_tuning(h, "pass_shadow_sort", sort ? 1 : 0);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!r && best_ms) *best_ms = best;
    return r;
}
}  // namespace

int dfpt_tune_frame(dfpt_handle* h, int32_t frames, float* ms_per_frame) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    if (frames < 1 || frames > 1024) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "frames %d outside [1, 1024]", frames);
    if (h->diff_on) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "dfpt_tune_frame inside a differentiable forward (call dfpt_diff_end first)");
    if (ms_per_frame) *ms_per_frame = 0.0f;
    // The other renderers run one kernel per pass: nothing to choose.
    if (is_simple_mode(h->params.renderer_type)) return DFPT_OK;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    SavedRegion regions[] = {DFPT_REGION_OF(h->film_sum), DFPT_REGION_OF(h->film_comp), DFPT_REGION_OF(h->film_n),
                             DFPT_REGION_OF(h->bgra), DFPT_REGION_OF(h->primitive_offsets), DFPT_REGION_OF(h->pixel_flags),
                             DFPT_REGION_OF(h->rng), DFPT_REGION_OF(h->stats), DFPT_REGION_OF(h->hit_prim),
                             DFPT_REGION_OF(h->hit_type), DFPT_REGION_OF(h->hit_off), DFPT_REGION_OF(h->hit_dist),
                             DFPT_REGION_OF(h->hit_normal)};
    size_t total = 0;
    for (const SavedRegion& g : regions) total += (g.bytes + 255) & ~(size_t)255;
    DevBuf<uint8_t> saved;
    CUDA_TRY(saved.alloc(total));
    size_t at = 0;
    cudaError_t ce = cudaSuccess;
    for (const SavedRegion& g : regions) {
        if (ce == cudaSuccess && g.bytes) ce = cudaMemcpyAsync(saved.p + at, g.p, g.bytes, cudaMemcpyDeviceToDevice, h->stream);
        at += (g.bytes + 255) & ~(size_t)255;
    }
    if (ce != cudaSuccess) {
        (void)cudaGetLastError();
        saved.release();
        return dfpt_fail(DFPT_ERR_CUDA, "saving the film before tuning: %s", cudaGetErrorString(ce));
    }
    const int host_pass0 = h->host_pass;
    const int r = tune_frame_sweep(h, frames, ms_per_frame);
    // Put back what the timed passes wrote, and the pass counter (the next pass reads it).
    at = 0;
    ce = cudaSuccess;
    for (const SavedRegion& g : regions) {
        if (ce == cudaSuccess && g.bytes) ce = cudaMemcpyAsync(g.p, saved.p + at, g.bytes, cudaMemcpyDeviceToDevice, h->stream);
        at += (g.bytes + 255) & ~(size_t)255;
    }
    h->host_pass = host_pass0;
    h->pass_index_host = host_pass0;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(h->pass_index.p, &h->pass_index_host, sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
    saved.release();
    if (ce != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "restoring the film after tuning: %s", cudaGetErrorString(ce));
    }
    return r;
}

int dfpt_set_record_hits(dfpt_handle* h, int32_t enabled) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    h->record_hits = enabled != 0;
    return push_params(h);
}

int dfpt_set_graphs(dfpt_handle* h, int32_t enabled) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    h->use_graph = enabled != 0;
    return DFPT_OK;
}

int dfpt_set_counting(dfpt_handle* h, int32_t enabled) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    h->counting = enabled != 0;
    return push_params(h);
}

int dfpt_clear(dfpt_handle* h) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    h->clear_pass = h->host_pass;
    return push_params(h);
}

int dfpt_render(dfpt_handle* h, int32_t passes) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    if (passes < 0) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "passes < 0");
    if (h->counting) CUDA_TRY(cudaMemsetAsync(h->stats.p, 0, 6 * sizeof(unsigned long long), h->stream));
    if (passes == 0) return DFPT_OK;
    h->events_used = 0;
    {
        int r = ensure_shadow_capacity(h);
        if (!r) r = pass_shadow_sort_prepare(h);
        if (r) return r;
    }
    if (passes >= 2 && wide_eligible(h)) {
        // Every pass in waves; the selection buffer and the image come from the last one.
        return render_wide(h, passes);
    }
    if (h->use_graph && !h->profiling) {
        if (!h->graph_valid) {
            int r = build_graph(h);
            if (r) return r;
        }
        for (int i = 0; i < passes; ++i) {
            CUDA_TRY(cudaGraphLaunch(h->graph_exec, h->stream));
            h->launches += (uint64_t)h->graph_kernels;
        }
    } else {
        for (int i = 0; i < passes; ++i) h->launches += (uint64_t)issue_pass(h);
        CUDA_TRY(cudaGetLastError());
    }
    h->host_pass += passes;
    return DFPT_OK;
}

int dfpt_synchronize(dfpt_handle* h) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

int dfpt_read_bgra8(dfpt_handle* h, uint8_t* out) {
    if (!h || !out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaMemcpyAsync(out, h->bgra.p, (size_t)h->n_pixels * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

int dfpt_read_film(dfpt_handle* h, float* rgb, int32_t* samples) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    kset(h).film_average(h->ctx, h->scratch_rgb.p, h->film_n.p == nullptr ? nullptr : nullptr);
    h->launches += 1;
    CUDA_TRY(cudaGetLastError());
    if (rgb) CUDA_TRY(cudaMemcpyAsync(rgb, h->scratch_rgb.p, (size_t)h->n_pixels * 12, cudaMemcpyDeviceToHost, h->stream));
    if (samples) CUDA_TRY(cudaMemcpyAsync(samples, h->film_n.p, (size_t)h->n_pixels * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

int dfpt_read_film_mean(dfpt_handle* h, double* mean3) {
    if (!h || !mean3) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaMemsetAsync(h->mean.p, 0, 3 * sizeof(double), h->stream));
    kset(h).film_mean(h->ctx, h->mean.p);
    h->launches += 1;
    CUDA_TRY(cudaGetLastError());
    double sums[3];
    CUDA_TRY(cudaMemcpyAsync(sums, h->mean.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < 3; ++i) mean3[i] = sums[i] / (double)h->n_pixels;
    return DFPT_OK;
}

int dfpt_read_primitive_offsets(dfpt_handle* h, int32_t* out) {
    if (!h || !out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaMemcpyAsync(out, h->primitive_offsets.p, (size_t)h->n_pixels * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

int dfpt_read_hits(dfpt_handle* h, int32_t* prim, int32_t* type, int32_t* off, float* dist, float* normal3) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    if (!h->record_hits) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "hit recording is off (dfpt_set_record_hits)");
    const size_t n = (size_t)h->n_pixels;
    if (prim) CUDA_TRY(cudaMemcpyAsync(prim, h->hit_prim.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (type) CUDA_TRY(cudaMemcpyAsync(type, h->hit_type.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (off) CUDA_TRY(cudaMemcpyAsync(off, h->hit_off.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (dist) CUDA_TRY(cudaMemcpyAsync(dist, h->hit_dist.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (normal3) CUDA_TRY(cudaMemcpyAsync(normal3, h->hit_normal.p, n * 12, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return DFPT_OK;
}

int dfpt_diff_forward(dfpt_handle* h, const dfpt_diff_params* dp, int32_t spp, float* image_rgb) {
    if (!h || !dp) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (spp < 1) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "spp %d < 1", spp);
    if (h->params.renderer_type != DFPT_RENDERER_PATH_TRACER) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "differentiable rendering needs the path tracer");
    if (h->params.rng_kind != DFPT_RNG_COUNTER) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "the replay needs the counter-based RNG");
    if (h->use_strict) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "differentiable rendering runs on the fast kernel set");
    if (!h->fast.shade_adj) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "kernel set has no adjoint");
    if (!(dp->turbidity > 0.0f) || !std::isfinite(dp->turbidity)) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "turbidity must be positive");
    const double sl = (double)dp->sun_direction[0] * dp->sun_direction[0] + (double)dp->sun_direction[1] * dp->sun_direction[1] +
                      (double)dp->sun_direction[2] * dp->sun_direction[2];
    if (!(sl > 0.0) || !std::isfinite(sl)) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "sun direction must be a nonzero finite vector");
    const int np = h->sc.scene.primitive_count;
    const size_t n = (size_t)h->n_pixels;
    // Per-primitive parameters.
    std::vector<float4> alb((size_t)std::max(np, 1), make_float4(1, 1, 1, 0)), emi((size_t)std::max(np, 1), make_float4(0, 0, 0, 0));
    std::vector<float> ex((size_t)std::max(np, 1), 50.0f);
    for (int i = 0; i < np; ++i) {
        if (dp->albedo) alb[i] = make_float4(dp->albedo[3 * i], dp->albedo[3 * i + 1], dp->albedo[3 * i + 2], 0.0f);
        if (dp->emission) emi[i] = make_float4(dp->emission[3 * i], dp->emission[3 * i + 1], dp->emission[3 * i + 2], 0.0f);
        if (dp->phong_exponent) {
            ex[i] = dp->phong_exponent[i];
            if (!(ex[i] > -1.0f) || !std::isfinite(ex[i])) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "Phong exponent %g of primitive %d must exceed -1", ex[i], i);
        }
    }
    CUDA_TRY(h->stream ? cudaStreamSynchronize(h->stream) : cudaSuccess);
    CUDA_TRY(upload(h->diff_albedo, alb, h->stream));
    CUDA_TRY(upload(h->diff_emission, emi, h->stream));
    CUDA_TRY(upload(h->diff_exponent, ex, h->stream));
    // Sky from (turbidity, sun direction), keeping the sky/sun switches.
    dfpt_sky sky;
    const int sky_on = h->sky.is_sky_active, sun_on = h->sky.is_sun_active;
    int r = dfpt_sky_set(&sky, dp->sun_direction, dp->turbidity);
    if (r) return r;
    sky.is_sky_active = sky_on;
    sky.is_sun_active = sun_on;
    if ((h->sky.is_sun_active == 1) != (sky.is_sun_active == 1)) h->graph_valid = false;
    h->wide_graph_valid = false;
    h->sky = sky;
    std::vector<float> tan(4 * DFPT_SKY_FIELDS);
    const double dir[3] = {dp->sun_direction[0], dp->sun_direction[1], dp->sun_direction[2]};
    sky_tangents((double)dp->turbidity, dir, tan.data());
    CUDA_TRY(upload(h->diff_sky_tan, tan, h->stream));
    // Per-sample records of this forward.
    if (!h->vis.p) {
        CUDA_TRY(h->vis.alloc(n));
        CUDA_TRY(cudaMemsetAsync(h->vis.p, 0, n * sizeof(int), h->stream));
    }
    if (h->diff_capacity < (size_t)spp * n) {
        h->diff_L.release();
        h->diff_vis.release();
        CUDA_TRY(h->diff_L.alloc((size_t)spp * n));
        CUDA_TRY(h->diff_vis.alloc((size_t)spp * n));
        h->diff_capacity = (size_t)spp * n;
    }
    if (!h->diff_dldi.p) CUDA_TRY(h->diff_dldi.alloc(n));
    const int rows = std::max(h->ctx.grid, 1), row_len = np * DFPT_DIFF_PER_PRIM + DFPT_DIFF_GLOBAL;
    if (h->diff_rows.n != (size_t)rows * row_len) {
        h->diff_rows.release();
        h->diff_out.release();
        CUDA_TRY(h->diff_rows.alloc((size_t)rows * row_len));
        CUDA_TRY(h->diff_out.alloc((size_t)row_len));
    }
    DevPass& B = h->pass;
    B.vis = h->vis.p; B.diff_L = h->diff_L.p; B.diff_vis = h->diff_vis.p; B.diff_dldi = h->diff_dldi.p;
    B.diff_rows = h->diff_rows.p; B.diff_row_len = row_len;
    h->graph_valid = false;
    h->wide_graph_valid = false;  // the pass record changed
    h->diff_on = true;
    h->diff_pass0 = h->host_pass;
    h->diff_spp = spp;
    h->clear_pass = h->host_pass;  // the forward starts a fresh film
    r = push_params(h);
    if (!r) r = dfpt_render(h, spp);
    if (r) return r;
    h->diff_ready = true;
    if (image_rgb) return dfpt_read_film(h, image_rgb, nullptr);
    return DFPT_OK;
}

int dfpt_diff_backward(dfpt_handle* h, const float* dloss_dimage, double* grad_albedo, double* grad_emission,
                       double* grad_phong_exponent, double* grad_sky) {
    if (!h || !dloss_dimage) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!h->diff_ready) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "dfpt_diff_backward needs a dfpt_diff_forward first");
    const size_t n = (size_t)h->n_pixels;
    const int np = h->sc.scene.primitive_count;
    const int row_len = np * DFPT_DIFF_PER_PRIM + DFPT_DIFF_GLOBAL;
    const int rows = (int)(h->diff_rows.n / (size_t)row_len);
    std::vector<float4> w(n);
    for (size_t i = 0; i < n; ++i) w[i] = make_float4(dloss_dimage[3 * i], dloss_dimage[3 * i + 1], dloss_dimage[3 * i + 2], 0.0f);
    CUDA_TRY(upload(h->diff_dldi, w, h->stream));
    CUDA_TRY(cudaMemsetAsync(h->diff_rows.p, 0, h->diff_rows.n * sizeof(double), h->stream));
    // Replay the forward's passes: same pass indices, so the same RNG streams.
    const int pass0 = h->diff_pass0;
    if (h->diff_spp >= 2 && wide_eligible(h) && h->wide.b_shade_adj) {
        // In waves of wide_samples passes through the batch stages (slot keys give pixel and pass).
        int r = wide_prepare(h);
        if (r) return r;
        h->wide_range[0] = 0;
        h->wide_range[1] = (long long)h->diff_spp * h->n_pixels;
        h->wide_range[2] = pass0;
        h->wide_range[3] = -1;
        h->wide_range[4] = -1;
        CUDA_TRY(cudaMemcpyAsync(h->w_wave_base.p, h->wide_range, 5 * sizeof(long long), cudaMemcpyHostToDevice, h->stream));
        const long long waves = (h->wide_range[1] + h->wide_capacity - 1) / h->wide_capacity;
        const KernelSet& K = h->wide;
        const LaunchCtx& c = h->wctx;
        const int nb = bounces_of(h);
        for (long long wv = 0; wv < waves; ++wv) {
            cudaMemsetAsync(h->w_counts.p, 0, DFPT_COUNTS_SIZE * sizeof(int), h->stream);
            K.b_wave(c, 0);
            K.b_camera(c, 0);
            for (int b = 0; b < nb; ++b) {
                K.b_trace_closest(c, b);
                K.b_shade_adj(c, b);
                if (h->wpass.sorted_queues) h->launches += (uint64_t)K.b_sort(c, b, false);
            }
            K.b_final_adj(c, nb);
            K.b_end(c, 0);
            h->launches += (uint64_t)(2 * nb + 4);
        }
    } else {
        CUDA_TRY(cudaMemcpyAsync(h->pass_index.p, &pass0, sizeof(int), cudaMemcpyHostToDevice, h->stream));
        for (int j = 0; j < h->diff_spp; ++j) h->launches += (uint64_t)issue_replay_pass(h);
    }
    h->fast.diff_reduce(h->ctx, h->diff_rows.p, rows, row_len, h->diff_out.p);
    h->launches += 1;
    CUDA_TRY(cudaGetLastError());
    std::vector<double> out((size_t)row_len);
    CUDA_TRY(cudaMemcpyAsync(out.data(), h->diff_out.p, (size_t)row_len * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));  // also keeps pass0 alive for its copy
    for (int i = 0; i < np; ++i) {
        const double* g = out.data() + (size_t)i * DFPT_DIFF_PER_PRIM;
        if (grad_albedo) for (int c = 0; c < 3; ++c) grad_albedo[3 * i + c] = g[c];
        if (grad_emission) for (int c = 0; c < 3; ++c) grad_emission[3 * i + c] = g[3 + c];
        if (grad_phong_exponent) grad_phong_exponent[i] = g[6];
    }
    if (grad_sky) for (int j = 0; j < DFPT_DIFF_GLOBAL; ++j) grad_sky[j] = out[(size_t)np * DFPT_DIFF_PER_PRIM + j];
    return DFPT_OK;
}

int dfpt_diff_end(dfpt_handle* h) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->diff_on = false;
    h->diff_ready = false;
    h->diff_L.release(); h->diff_vis.release(); h->diff_capacity = 0;
    h->diff_rows.release(); h->diff_out.release();
    DevPass& B = h->pass;
    B.diff_L = nullptr; B.diff_vis = nullptr; B.diff_rows = nullptr;
    h->graph_valid = false;
    h->wide_graph_valid = false;
    return push_params(h);
}

int dfpt_l2_reset(void) {
    CUDA_TRY(cudaCtxResetPersistingL2Cache());
    return DFPT_OK;
}

int dfpt_read_counters(dfpt_handle* h, uint64_t* c6) {
    if (!h || !c6) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    unsigned long long v[6];
    CUDA_TRY(cudaMemcpyAsync(v, h->stats.p, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < 6; ++i) c6[i] = v[i];
    return DFPT_OK;
}

int dfpt_set_profiling(dfpt_handle* h, int32_t enabled) {
    if (!h) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "handle == NULL");
    h->profiling = enabled != 0;
    h->events_used = 0;
    return DFPT_OK;
}

int dfpt_read_profile(dfpt_handle* h, double* ms_by_kind, int32_t* launches_by_kind) {
    if (!h || !ms_by_kind || !launches_by_kind) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int i = 0; i < KIND_COUNT; ++i) { ms_by_kind[i] = 0.0; launches_by_kind[i] = 0; }
    if (!h->profiling || h->events_used < 2) return DFPT_OK;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (int i = 0; i + 1 < h->events_used; ++i) {
        float ms = 0.0f;
        CUDA_TRY(cudaEventElapsedTime(&ms, h->events[i], h->events[i + 1]));
        const int kind = h->event_kind[i];
        if (kind >= 0 && kind < KIND_COUNT) { ms_by_kind[kind] += ms; launches_by_kind[kind] += 1; }
    }
    return DFPT_OK;
}

int dfpt_launch_count(dfpt_handle* h, uint64_t* launches) {
    if (!h || !launches) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    *launches = h->launches;
    return DFPT_OK;
}

}  // extern "C"
