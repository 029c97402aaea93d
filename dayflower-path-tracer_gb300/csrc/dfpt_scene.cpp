// dfpt_scene.cpp - host-side scene compiler, BVH builder, camera and sky set-up.
//
// This is the producer side of the renderer's data contract. It restates, for callers without
// a JVM, what the reference does before the first Kernel.execute:
//   - SceneCompiler.compile            src/main/java/org/dayflower/pathtracer/scene/compiler/SceneCompiler.java:79-188
//   - BVH flattening                   SceneCompiler.java:888-995
//   - BVH builder (binned SAH sweep)   src/main/java/org/dayflower/pathtracer/scene/bvh/BoundingVolumeHierarchy.java:118-157,805-986
//   - Camera ONB / field of view       src/main/java/org/dayflower/pathtracer/scene/Camera.java:743-760,877-946
//   - Transform matrices               src/main/java/org/dayflower/pathtracer/scene/Transform.java:184-193 (Matrix44F)
//   - Sky.set Perez coefficients       src/main/java/org/dayflower/pathtracer/scene/Sky.java:295-333
// All float arithmetic is single precision, one rounding per operation (built with
// -ffp-contract=off), so the arrays are the same on x86-64 and aarch64 hosts.
#include "dfpt.h"
#include "dfpt_internal.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------------------------------------
// Value types with Java Float.compare equality (NaN == NaN, -0.0 != 0.0).

inline uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x007fffffu) != 0u) u = 0x7fc00000u;
    return u;
}

struct Key {
    std::vector<uint32_t> w;
    bool operator==(const Key& o) const { return w == o.w; }
};
struct KeyHash {
    size_t operator()(const Key& k) const {
        uint64_t h = 1469598103934665603ull;
        for (uint32_t x : k.w) { h ^= x; h *= 1099511628211ull; }
        return (size_t)h;
    }
};

// First-occurrence-ordered set of value keys: the stream().distinct() of the reference.
struct Distinct {
    std::unordered_map<Key, int, KeyHash> index;
    std::vector<Key> order;
    int add(const Key& k) {
        auto it = index.find(k);
        if (it != index.end()) return it->second;
        int i = (int)order.size();
        index.emplace(k, i);
        order.push_back(k);
        return i;
    }
    int find(const Key& k) const {
        auto it = index.find(k);
        return it == index.end() ? -1 : it->second;
    }
};

// Fixed-size keys for the large sets (points, vectors, triangles): no allocation per key.
template <size_t N>
struct KeyN {
    std::array<uint32_t, N> w;
    bool operator==(const KeyN& o) const { return w == o.w; }
};
template <size_t N>
struct KeyNHash {
    size_t operator()(const KeyN<N>& k) const {
        uint64_t h = 1469598103934665603ull;
        for (uint32_t x : k.w) { h ^= x; h *= 1099511628211ull; }
        h ^= h >> 29;
        h *= 0xbf58476d1ce4e5b9ull;
        return (size_t)(h ^ (h >> 32));
    }
};
// First-occurrence-ordered set over fixed-size keys: open addressing, linear probing.
template <size_t N>
struct DistinctN {
    std::vector<KeyN<N>> order;
    std::vector<int32_t> slot;  // -1 empty, else index into order
    size_t mask = 0;
    void grow() {
        const size_t cap = slot.empty() ? 1024 : slot.size() * 2;
        slot.assign(cap, -1);
        mask = cap - 1;
        for (size_t i = 0; i < order.size(); ++i) {
            size_t h = KeyNHash<N>()(order[i]) & mask;
            while (slot[h] >= 0) h = (h + 1) & mask;
            slot[h] = (int32_t)i;
        }
    }
    int add(const KeyN<N>& k) {
        if ((order.size() + 1) * 2 > slot.size()) grow();
        size_t h = KeyNHash<N>()(k) & mask;
        for (;;) {
            const int32_t s = slot[h];
            if (s < 0) {
                slot[h] = (int32_t)order.size();
                order.push_back(k);
                return slot[h];
            }
            if (order[s] == k) return s;
            h = (h + 1) & mask;
        }
    }
    int find(const KeyN<N>& k) const {
        if (slot.empty()) return -1;
        size_t h = KeyNHash<N>()(k) & mask;
        for (;;) {
            const int32_t s = slot[h];
            if (s < 0) return -1;
            if (order[s] == k) return s;
            h = (h + 1) & mask;
        }
    }
};

KeyN<3> key3(float x, float y, float z) { return KeyN<3>{{fbits(x), fbits(y), fbits(z)}}; }
KeyN<2> key2(float x, float y) { return KeyN<2>{{fbits(x), fbits(y)}}; }

struct V3 { float x, y, z; };

struct Vertex { float p[3], n[3], uv[2], t[3]; };

struct Tri { Vertex v[3]; };

KeyN<33> tri_key(const Tri& t) {
    KeyN<33> k;
    int n = 0;
    for (int i = 0; i < 3; ++i) {
        const Vertex& v = t.v[i];
        // Vertex.equals compares texture coordinates, position, normal, tangent.
        for (float f : v.uv) k.w[n++] = fbits(f);
        for (float f : v.p) k.w[n++] = fbits(f);
        for (float f : v.n) k.w[n++] = fbits(f);
        for (float f : v.t) k.w[n++] = fbits(f);
    }
    return k;
}

struct Shape {
    int type = 0;
    float params[9] = {0};  // plane a,b,c | sphere pos, radius | terrain 5
    V3 plane_normal{0, 0, 0};
    std::vector<Tri> tris;  // mesh or single triangle
};

struct Surface {
    int material, albedo, emission, normal;
    float noise_amount, noise_scale;
};

struct Primitive {
    int shape, surface;
    float o2w[16], w2o[16];
};

// ---------------------------------------------------------------------------------------------
// BoundingVolumeHierarchy.createBoundingVolumeHierarchy restated.

struct BvhItem {  // the per-triangle LeafNode of the builder
    float mx, my, mz, nx, ny, nz;  // maximum, minimum
    int tri;                       // index into the mesh triangle list
    float cx() const { return (mx + nx) * 0.5f; }
    float cy() const { return (my + ny) * 0.5f; }
    float cz() const { return (mz + nz) * 0.5f; }
};

struct BvhNode {
    bool leaf = false;
    int depth = 0;
    float mx = 0, my = 0, mz = 0, nx = 0, ny = 0, nz = 0;
    std::vector<int> tris;
    std::unique_ptr<BvhNode> left, right;
};

inline float jmax(float a, float b) { return (a != a) ? a : (b != b) ? b : (a >= b ? a : b); }
inline float jmin(float a, float b) { return (a != a) ? a : (b != b) ? b : (a <= b ? a : b); }

struct SplitResult { float cost; float split; int axis; long order; };

// Evaluates one split candidate exactly as the inner loop at BoundingVolumeHierarchy.java:843-920.
SplitResult eval_split(const std::vector<BvhItem>& items, int axis, float split) {
    float mlx = -FLT_MAX_F, mly = -FLT_MAX_F, mlz = -FLT_MAX_F, nlx = FLT_MAX_F, nly = FLT_MAX_F, nlz = FLT_MAX_F;
    float mrx = -FLT_MAX_F, mry = -FLT_MAX_F, mrz = -FLT_MAX_F, nrx = FLT_MAX_F, nry = FLT_MAX_F, nrz = FLT_MAX_F;
    int cl = 0, cr = 0;
    for (const BvhItem& it : items) {
        const float value = axis == 0 ? it.cx() : axis == 1 ? it.cy() : it.cz();
        if (value < split) {
            mlx = jmax(mlx, it.mx); mly = jmax(mly, it.my); mlz = jmax(mlz, it.mz);
            nlx = jmin(nlx, it.nx); nly = jmin(nly, it.ny); nlz = jmin(nlz, it.nz);
            cl++;
        } else {
            mrx = jmax(mrx, it.mx); mry = jmax(mry, it.my); mrz = jmax(mrz, it.mz);
            nrx = jmin(nrx, it.nx); nry = jmin(nry, it.ny); nrz = jmin(nrz, it.nz);
            cr++;
        }
    }
    SplitResult r{0.0f, split, axis, 0};
    if (cl <= 1 || cr <= 1) { r.axis = -1; return r; }
    const float slx = mlx - nlx, sly = mly - nly, slz = mlz - nlz;
    const float srx = mrx - nrx, sry = mry - nry, srz = mrz - nrz;
    const float sl = slx * sly + sly * slz + slz * slx;
    const float sr = srx * sry + sry * srz + srz * srx;
    r.cost = sl * (float)cl + sr * (float)cr;
    return r;
}

// The same search restated with per-axis sorted item lists, O(n log n) per tree level instead of
// O(candidates x n) per node. For a candidate split s on an axis, the left group is every item
// whose centroid is < s: a prefix of the items sorted by that centroid, so its bounds are a prefix
// max/min and its count a position in the sorted list. Max/min of non-NaN floats do not depend on
// the order they are taken in (a NaN makes the cost NaN in either order), so every candidate's
// count and cost - and with it the chosen split - are the ones the reference's item loop gives.
// The chosen partition and the child bounds are still computed by the item loop in list order.
struct SortedSweep {
    const std::vector<BvhItem>* items = nullptr;  // all items of the mesh, by id
    const std::vector<float>* cen[3] = {nullptr, nullptr, nullptr};
    // prefix (k items) and suffix (items k..n-1) bounds: mx, my, mz, nx, ny, nz
    std::vector<float> pre, suf;

    void bounds_scan(const std::vector<int>& order) {
        const size_t n = order.size();
        pre.resize((n + 1) * 6);
        suf.resize((n + 1) * 6);
        float* P = pre.data();
        P[0] = P[1] = P[2] = -FLT_MAX_F;
        P[3] = P[4] = P[5] = FLT_MAX_F;
        for (size_t k = 0; k < n; ++k) {
            const BvhItem& it = (*items)[order[k]];
            const float* a = P + k * 6;
            float* b = P + (k + 1) * 6;
            b[0] = jmax(a[0], it.mx); b[1] = jmax(a[1], it.my); b[2] = jmax(a[2], it.mz);
            b[3] = jmin(a[3], it.nx); b[4] = jmin(a[4], it.ny); b[5] = jmin(a[5], it.nz);
        }
        float* S = suf.data();
        float* e = S + n * 6;
        e[0] = e[1] = e[2] = -FLT_MAX_F;
        e[3] = e[4] = e[5] = FLT_MAX_F;
        for (size_t k = n; k-- > 0;) {
            const BvhItem& it = (*items)[order[k]];
            const float* a = S + (k + 1) * 6;
            float* b = S + k * 6;
            b[0] = jmax(a[0], it.mx); b[1] = jmax(a[1], it.my); b[2] = jmax(a[2], it.mz);
            b[3] = jmin(a[3], it.nx); b[4] = jmin(a[4], it.ny); b[5] = jmin(a[5], it.nz);
        }
    }

    static float cost_of(const float* l, int cl, const float* r, int cr) {
        const float slx = l[0] - l[3], sly = l[1] - l[4], slz = l[2] - l[5];
        const float srx = r[0] - r[3], sry = r[1] - r[4], srz = r[2] - r[5];
        const float sl = slx * sly + sly * slz + slz * slx;
        const float sr = srx * sry + sry * srz + srz * srx;
        return sl * (float)cl + sr * (float)cr;
    }
};

// Orders item ids by one centroid coordinate, NaN last (a NaN centroid is never < a split).
struct CentroidLess {
    const float* v;
    bool operator()(int a, int b) const {
        const float x = v[a], y = v[b];
        if (y != y) return x == x;
        return x < y;
    }
};

struct BvhBuilder {
    int threads = 1;
    bool exhaustive = false;  // evaluate every candidate with the item loop (test cross-check)
    std::atomic<int> spawned{0};

    std::unique_ptr<BvhNode> make_leaf(const std::vector<BvhItem>& items, int depth) {
        auto leaf = std::make_unique<BvhNode>();
        leaf->leaf = true;
        leaf->depth = depth;
        for (const BvhItem& it : items) leaf->tris.push_back(it.tri);
        return leaf;
    }

    // The candidate list in loop order; float stepping exactly as the reference's for-loop.
    static void candidates(int depth, float mx, float my, float mz, float nx, float ny, float nz,
                           std::vector<std::pair<int, float>>& cands) {
        cands.clear();
        for (int axis = 0; axis < 3; ++axis) {
            const float start = axis == 0 ? nx : axis == 1 ? ny : nz;
            const float stop = axis == 0 ? mx : axis == 1 ? my : mz;
            if (std::fabs(stop - start) < 1.0e-4f) continue;
            const float step = (stop - start) / (1024.0f / ((float)depth + 1.0f));
            for (float split = start + step; split < stop - step; split += step) cands.emplace_back(axis, split);
        }
    }

    std::unique_ptr<BvhNode> build(std::vector<BvhItem>& items, int depth, float mx, float my, float mz,
                                   float nx, float ny, float nz) {
        const int size0 = (int)items.size();
        if (size0 < 4) return make_leaf(items, depth);
        const float sx = mx - nx, sy = my - ny, sz = mz - nz;
        float minimum_cost = (float)size0 * (sx * sy + sy * sz + sz * sx);
        float best_split = FLT_MAX_F;
        int best_axis = -1;
        std::vector<std::pair<int, float>> cands;
        candidates(depth, mx, my, mz, nx, ny, nz, cands);
        const size_t nc = cands.size();
        std::vector<SplitResult> res(nc);
        const long work = (long)nc * (long)size0;
        int nt = (threads > 1 && work > 4000000L) ? threads : 1;
        if (nt > 1) {
            std::vector<std::thread> pool;
            std::atomic<size_t> next{0};
            for (int t = 0; t < nt; ++t) {
                pool.emplace_back([&]() {
                    for (;;) {
                        size_t i = next.fetch_add(1);
                        if (i >= nc) break;
                        res[i] = eval_split(items, cands[i].first, cands[i].second);
                    }
                });
            }
            for (auto& th : pool) th.join();
        } else {
            for (size_t i = 0; i < nc; ++i) res[i] = eval_split(items, cands[i].first, cands[i].second);
        }
        // Sequential reduction keeps the reference's "first strictly cheaper candidate" rule.
        for (size_t i = 0; i < nc; ++i) {
            if (res[i].axis < 0) continue;
            if (res[i].cost < minimum_cost) {
                minimum_cost = res[i].cost;
                best_split = res[i].split;
                best_axis = res[i].axis;
            }
        }
        if (best_axis == -1) return make_leaf(items, depth);
        std::vector<BvhItem> left, right;
        left.reserve(size0 / 2);
        right.reserve(size0 / 2);
        float mlx = -FLT_MAX_F, mly = -FLT_MAX_F, mlz = -FLT_MAX_F, nlx = FLT_MAX_F, nly = FLT_MAX_F, nlz = FLT_MAX_F;
        float mrx = -FLT_MAX_F, mry = -FLT_MAX_F, mrz = -FLT_MAX_F, nrx = FLT_MAX_F, nry = FLT_MAX_F, nrz = FLT_MAX_F;
        for (const BvhItem& it : items) {
            const float value = best_axis == 0 ? it.cx() : best_axis == 1 ? it.cy() : it.cz();
            if (value < best_split) {
                left.push_back(it);
                mlx = jmax(mlx, it.mx); mly = jmax(mly, it.my); mlz = jmax(mlz, it.mz);
                nlx = jmin(nlx, it.nx); nly = jmin(nly, it.ny); nlz = jmin(nlz, it.nz);
            } else {
                right.push_back(it);
                mrx = jmax(mrx, it.mx); mry = jmax(mry, it.my); mrz = jmax(mrz, it.mz);
                nrx = jmin(nrx, it.nx); nry = jmin(nry, it.ny); nrz = jmin(nrz, it.nz);
            }
        }
        std::vector<BvhItem>().swap(items);
        auto node_left = build(left, depth + 1, mlx, mly, mlz, nlx, nly, nlz);
        node_left->mx = mlx; node_left->my = mly; node_left->mz = mlz;
        node_left->nx = nlx; node_left->ny = nly; node_left->nz = nlz;
        auto node_right = build(right, depth + 1, mrx, mry, mrz, nrx, nry, nrz);
        node_right->mx = mrx; node_right->my = mry; node_right->mz = mrz;
        node_right->nx = nrx; node_right->ny = nry; node_right->nz = nrz;
        auto tree = std::make_unique<BvhNode>();
        tree->depth = depth;
        tree->left = std::move(node_left);
        tree->right = std::move(node_right);
        return tree;
    }

    // The sorted-list form of build(). `ids` is the node's item list in the reference's order;
    // `by[a]` the same ids sorted by centroid a. Children get stable partitions of all four lists,
    // which stay sorted, so the mesh is sorted once.
    std::unique_ptr<BvhNode> build_sorted(const std::vector<BvhItem>& all, const std::vector<float>* cen,
                                          std::vector<int>& ids, std::vector<int>* by, int depth,
                                          float mx, float my, float mz, float nx, float ny, float nz) {
        const int size0 = (int)ids.size();
        if (size0 < 4) {
            auto leaf = std::make_unique<BvhNode>();
            leaf->leaf = true;
            leaf->depth = depth;
            for (int id : ids) leaf->tris.push_back(all[id].tri);
            return leaf;
        }
        const float sx = mx - nx, sy = my - ny, sz = mz - nz;
        float minimum_cost = (float)size0 * (sx * sy + sy * sz + sz * sx);
        float best_split = FLT_MAX_F;
        int best_axis = -1;
        std::vector<std::pair<int, float>> cands;
        candidates(depth, mx, my, mz, nx, ny, nz, cands);
        SortedSweep sw;
        sw.items = &all;
        size_t ci = 0;
        for (int axis = 0; axis < 3 && ci < cands.size(); ++axis) {
            if (cands[ci].first != axis) continue;
            const std::vector<int>& order = by[axis];
            const float* v = cen[axis].data();
            sw.bounds_scan(order);
            int k = 0;  // items with centroid < split, in sorted order
            for (; ci < cands.size() && cands[ci].first == axis; ++ci) {
                const float split = cands[ci].second;
                while (k < size0 && v[order[k]] < split) ++k;
                const int cl = k, cr = size0 - k;
                if (cl <= 1 || cr <= 1) continue;
                const float cost = SortedSweep::cost_of(sw.pre.data() + (size_t)k * 6, cl, sw.suf.data() + (size_t)k * 6, cr);
                if (cost < minimum_cost) {
                    minimum_cost = cost;
                    best_split = split;
                    best_axis = axis;
                }
            }
        }
        if (best_axis == -1) {
            auto leaf = std::make_unique<BvhNode>();
            leaf->leaf = true;
            leaf->depth = depth;
            for (int id : ids) leaf->tris.push_back(all[id].tri);
            return leaf;
        }
        float mlx = -FLT_MAX_F, mly = -FLT_MAX_F, mlz = -FLT_MAX_F, nlx = FLT_MAX_F, nly = FLT_MAX_F, nlz = FLT_MAX_F;
        float mrx = -FLT_MAX_F, mry = -FLT_MAX_F, mrz = -FLT_MAX_F, nrx = FLT_MAX_F, nry = FLT_MAX_F, nrz = FLT_MAX_F;
        const float* vb = cen[best_axis].data();
        std::vector<int> lid, rid;
        lid.reserve(size0);
        rid.reserve(size0);
        for (int id : ids) {
            const BvhItem& it = all[id];
            if (vb[id] < best_split) {
                lid.push_back(id);
                mlx = jmax(mlx, it.mx); mly = jmax(mly, it.my); mlz = jmax(mlz, it.mz);
                nlx = jmin(nlx, it.nx); nly = jmin(nly, it.ny); nlz = jmin(nlz, it.nz);
            } else {
                rid.push_back(id);
                mrx = jmax(mrx, it.mx); mry = jmax(mry, it.my); mrz = jmax(mrz, it.mz);
                nrx = jmin(nrx, it.nx); nry = jmin(nry, it.ny); nrz = jmin(nrz, it.nz);
            }
        }
        std::vector<int> lby[3], rby[3];
        for (int a = 0; a < 3; ++a) {
            lby[a].reserve(lid.size());
            rby[a].reserve(rid.size());
            for (int id : by[a]) (vb[id] < best_split ? lby[a] : rby[a]).push_back(id);
            std::vector<int>().swap(by[a]);
        }
        std::vector<int>().swap(ids);
        std::unique_ptr<BvhNode> node_left, node_right;
        auto run_left = [&]() { node_left = build_sorted(all, cen, lid, lby, depth + 1, mlx, mly, mlz, nlx, nly, nlz); };
        // Large subtrees build on their own thread (the tree does not depend on the schedule).
        if (size0 > 20000 && spawned.fetch_add(1) < threads - 1) {
            std::thread t(run_left);
            node_right = build_sorted(all, cen, rid, rby, depth + 1, mrx, mry, mrz, nrx, nry, nrz);
            t.join();
        } else {
            run_left();
            node_right = build_sorted(all, cen, rid, rby, depth + 1, mrx, mry, mrz, nrx, nry, nrz);
        }
        node_left->mx = mlx; node_left->my = mly; node_left->mz = mlz;
        node_left->nx = nlx; node_left->ny = nly; node_left->nz = nlz;
        node_right->mx = mrx; node_right->my = mry; node_right->mz = mrz;
        node_right->nx = nrx; node_right->ny = nry; node_right->nz = nrz;
        auto tree = std::make_unique<BvhNode>();
        tree->depth = depth;
        tree->left = std::move(node_left);
        tree->right = std::move(node_right);
        return tree;
    }

    std::unique_ptr<BvhNode> create(const std::vector<Tri>& tris) {
        std::vector<BvhItem> items;
        items.reserve(tris.size());
        float mx = -FLT_MAX_F, my = -FLT_MAX_F, mz = -FLT_MAX_F, nx = FLT_MAX_F, ny = FLT_MAX_F, nz = FLT_MAX_F;
        for (size_t i = 0; i < tris.size(); ++i) {
            const float* p0 = tris[i].v[0].p;
            const float* p1 = tris[i].v[1].p;
            const float* p2 = tris[i].v[2].p;
            BvhItem it;
            it.mx = jmax(jmax(p0[0], p1[0]), p2[0]);
            it.my = jmax(jmax(p0[1], p1[1]), p2[1]);
            it.mz = jmax(jmax(p0[2], p1[2]), p2[2]);
            it.nx = jmin(jmin(p0[0], p1[0]), p2[0]);
            it.ny = jmin(jmin(p0[1], p1[1]), p2[1]);
            it.nz = jmin(jmin(p0[2], p1[2]), p2[2]);
            it.tri = (int)i;
            items.push_back(it);
            mx = jmax(mx, it.mx); my = jmax(my, it.my); mz = jmax(mz, it.mz);
            nx = jmin(nx, it.nx); ny = jmin(ny, it.ny); nz = jmin(nz, it.nz);
        }
        std::unique_ptr<BvhNode> root;
        if (exhaustive) {
            std::vector<BvhItem> work = items;
            root = build(work, 0, mx, my, mz, nx, ny, nz);
        } else {
            const int n = (int)items.size();
            std::vector<float> cen[3];
            std::vector<int> ids(n), by[3];
            for (int a = 0; a < 3; ++a) cen[a].resize(n);
            for (int i = 0; i < n; ++i) {
                ids[i] = i;
                cen[0][i] = items[i].cx();
                cen[1][i] = items[i].cy();
                cen[2][i] = items[i].cz();
            }
            std::thread sorters[3];
            for (int a = 0; a < 3; ++a) {
                by[a] = ids;
                sorters[a] = std::thread([&, a]() { std::sort(by[a].begin(), by[a].end(), CentroidLess{cen[a].data()}); });
            }
            for (auto& t : sorters) t.join();
            spawned = 0;
            root = build_sorted(items, cen, ids, by, 0, mx, my, mz, nx, ny, nz);
        }
        root->mx = mx; root->my = my; root->mz = mz;
        root->nx = nx; root->ny = ny; root->nz = nz;
        return root;
    }
};

int bvh_size(const BvhNode* n) {
    if (n->leaf) return 5 + (int)n->tris.size();
    return 5 + bvh_size(n->left.get()) + bvh_size(n->right.get());
}

// Node.addBounds: maximum, minimum, then the left and right subtrees (preorder).
void bvh_add_bounds(const BvhNode* n, DistinctN<3>& points) {
    points.add(key3(n->mx, n->my, n->mz));
    points.add(key3(n->nx, n->ny, n->nz));
    if (!n->leaf) {
        bvh_add_bounds(n->left.get(), points);
        bvh_add_bounds(n->right.get(), points);
    }
}

// Structural equality of two BVH trees (TreeNode/LeafNode.equals), used for distinct().
bool bvh_equal(const BvhNode* a, const BvhNode* b, const std::vector<Tri>& ta, const std::vector<Tri>& tb) {
    if (a->leaf != b->leaf) return false;
    if (fbits(a->mx) != fbits(b->mx) || fbits(a->my) != fbits(b->my) || fbits(a->mz) != fbits(b->mz)) return false;
    if (fbits(a->nx) != fbits(b->nx) || fbits(a->ny) != fbits(b->ny) || fbits(a->nz) != fbits(b->nz)) return false;
    if (a->leaf) {
        if (a->tris.size() != b->tris.size()) return false;
        for (size_t i = 0; i < a->tris.size(); ++i)
            if (!(tri_key(ta[a->tris[i]]) == tri_key(tb[b->tris[i]]))) return false;
        return true;
    }
    return bvh_equal(a->left.get(), b->left.get(), ta, tb) && bvh_equal(a->right.get(), b->right.get(), ta, tb);
}

// doCompileBoundingVolumeHierarchy: preorder list, relative offsets, skip ("next") pointers.
void bvh_flatten(const BvhNode* n, int next_after, std::vector<int32_t>& out, int base,
                 const std::vector<int>& tri_offsets, const DistinctN<3>& points, const std::vector<int>& point_index) {
    const int here = (int)out.size() - base;
    (void)here;
    const int max_off = point_index[points.find(key3(n->mx, n->my, n->mz))] * 3;
    const int min_off = point_index[points.find(key3(n->nx, n->ny, n->nz))] * 3;
    if (n->leaf) {
        out.push_back(2);
        out.push_back(next_after);
        out.push_back(min_off);
        out.push_back(max_off);
        out.push_back((int32_t)n->tris.size());
        for (int t : n->tris) out.push_back(tri_offsets[t]);
        return;
    }
    const size_t head = out.size();
    out.push_back(1);
    out.push_back(next_after);
    out.push_back(min_off);
    out.push_back(max_off);
    out.push_back(0);  // left, patched below
    const int left_off = (int)out.size() - base;
    out[head + 4] = left_off;
    const int right_off = left_off + bvh_size(n->left.get());
    bvh_flatten(n->left.get(), right_off, out, base, tri_offsets, points, point_index);
    bvh_flatten(n->right.get(), next_after, out, base, tri_offsets, points, point_index);
}

// Matrix44F arithmetic (Matrix44F.java: multiply 238-257, inverse 185-225, rotation 673-736).
struct M44 { float e[16]; };

M44 m_mul(const M44& a, const M44& b) {
    M44 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float s = a.e[i * 4 + 0] * b.e[0 * 4 + j];
            s = s + a.e[i * 4 + 1] * b.e[1 * 4 + j];
            s = s + a.e[i * 4 + 2] * b.e[2 * 4 + j];
            s = s + a.e[i * 4 + 3] * b.e[3 * 4 + j];
            r.e[i * 4 + j] = s;
        }
    return r;
}

bool m_inverse(const M44& m, M44& out) {
    const float* e = m.e;
    const float e11 = e[0], e12 = e[1], e13 = e[2], e14 = e[3];
    const float e21 = e[4], e22 = e[5], e23 = e[6], e24 = e[7];
    const float e31 = e[8], e32 = e[9], e33 = e[10], e34 = e[11];
    const float e41 = e[12], e42 = e[13], e43 = e[14], e44 = e[15];
    const float a = e11 * e22 - e12 * e21, b = e11 * e23 - e13 * e21, c = e11 * e24 - e14 * e21;
    const float d = e12 * e23 - e13 * e22, ee = e12 * e24 - e14 * e22, f = e13 * e24 - e14 * e23;
    const float g = e31 * e42 - e32 * e41, h = e31 * e43 - e33 * e41, i = e31 * e44 - e34 * e41;
    const float j = e32 * e43 - e33 * e42, k = e32 * e44 - e34 * e42, l = e33 * e44 - e34 * e43;
    const float det = a * l - b * k + c * j + d * i - ee * h + f * g;
    if (std::fabs(det) < 1.0e-12f) return false;
    const float r = 1.0f / det;
    float* o = out.e;
    o[0] = (+e22 * l - e23 * k + e24 * j) * r;
    o[1] = (-e12 * l + e13 * k - e14 * j) * r;
    o[2] = (+e42 * f - e43 * ee + e44 * d) * r;
    o[3] = (-e32 * f + e33 * ee - e34 * d) * r;
    o[4] = (-e21 * l + e23 * i - e24 * h) * r;
    o[5] = (+e11 * l - e13 * i + e14 * h) * r;
    o[6] = (-e41 * f + e43 * c - e44 * b) * r;
    o[7] = (+e31 * f - e33 * c + e34 * b) * r;
    o[8] = (+e21 * k - e22 * i + e24 * g) * r;
    o[9] = (-e11 * k + e12 * i - e14 * g) * r;
    o[10] = (+e41 * ee - e42 * c + e44 * a) * r;
    o[11] = (-e31 * ee + e32 * c - e34 * a) * r;
    o[12] = (-e21 * j + e22 * h - e23 * g) * r;
    o[13] = (+e11 * j - e12 * h + e13 * g) * r;
    o[14] = (-e41 * d + e42 * b - e43 * a) * r;
    o[15] = (+e31 * d - e32 * b + e33 * a) * r;
    return true;
}

bool transform_matrices(const float* t10, float* o2w, float* w2o) {
    const float px = t10[0], py = t10[1], pz = t10[2];
    const float qx = t10[3], qy = t10[4], qz = t10[5], qw = t10[6];
    const float sx = t10[7], sy = t10[8], sz = t10[9];
    M44 T = {{1, 0, 0, px, 0, 1, 0, py, 0, 0, 1, pz, 0, 0, 0, 1}};
    // Matrix44F.rotation(QuaternionF): rows u, v, w.
    const float wx = 2.0f * (qx * qz - qw * qy), wy = 2.0f * (qy * qz + qw * qx), wz = 1.0f - 2.0f * (qx * qx + qy * qy);
    const float vx = 2.0f * (qx * qy + qw * qz), vy = 1.0f - 2.0f * (qx * qx + qz * qz), vz = 2.0f * (qy * qz - qw * qx);
    const float ux = 1.0f - 2.0f * (qy * qy + qz * qz), uy = 2.0f * (qx * qy - qw * qz), uz = 2.0f * (qx * qz + qw * qy);
    M44 R = {{ux, uy, uz, 0, vx, vy, vz, 0, wx, wy, wz, 0, 0, 0, 0, 1}};
    M44 S = {{sx, 0, 0, 0, 0, sy, 0, 0, 0, 0, sz, 0, 0, 0, 0, 1}};
    M44 O = m_mul(m_mul(T, R), S);
    M44 W;
    if (!m_inverse(O, W)) return false;
    std::memcpy(o2w, O.e, 64);
    std::memcpy(w2o, W.e, 64);
    return true;
}

V3 normal_normalized(const float* a, const float* b, const float* c) {
    // Vector3F.normalNormalized: cross(b - a, c - a), divided by its length.
    const float abx = b[0] - a[0], aby = b[1] - a[1], abz = b[2] - a[2];
    const float acx = c[0] - a[0], acy = c[1] - a[1], acz = c[2] - a[2];
    const float nx = aby * acz - abz * acy;
    const float ny = abz * acx - abx * acz;
    const float nz = abx * acy - aby * acx;
    const float len = std::sqrt(nx * nx + ny * ny + nz * nz);
    return V3{nx / len, ny / len, nz / len};
}

}  // namespace

struct dfpt_scene_builder {
    std::vector<std::vector<float>> textures;
    std::vector<Surface> surfaces;
    std::vector<Shape> shapes;
    std::vector<Primitive> primitives;
    float camera[19];
    bool camera_set = false;
    bool exhaustive_bvh = false;
};

struct dfpt_compiled {
    std::vector<float> point2fs, point3fs, vector3fs, spheres, terrains, textures, surfaces, o2w, w2o, camera;
    std::vector<int32_t> planes, triangles, bvh, primitives;
};

extern "C" {

int dfpt_builder_create(dfpt_scene_builder** out) {
    if (!out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "out_builder == NULL");
    *out = new dfpt_scene_builder();
    return DFPT_OK;
}

int dfpt_builder_destroy(dfpt_scene_builder* b) {
    delete b;
    return DFPT_OK;
}

int dfpt_builder_add_texture(dfpt_scene_builder* b, const float* record, int32_t count) {
    if (!b || !record || count < 2) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad texture record");
    const int type = (int)record[0];
    if (type < 1 || type > 8) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "unknown texture type %d", type);
    if ((int)record[1] != count) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "texture size field %d != count %d", (int)record[1], count);
    if (type == DFPT_TEXTURE_BLEND) {
        const int ta = (int)record[2], tb = (int)record[3];
        if (ta < 0 || tb < 0 || ta >= (int)b->textures.size() || tb >= (int)b->textures.size())
            return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "blend texture refers to unknown textures");
    }
    b->textures.emplace_back(record, record + count);
    return (int)b->textures.size() - 1;
}

int dfpt_builder_add_surface(dfpt_scene_builder* b, int32_t material, int32_t albedo, int32_t emission,
                             int32_t normal, float noise_amount, float noise_scale) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "builder == NULL");
    const int nt = (int)b->textures.size();
    if (material < 1 || material > 5 || albedo < 0 || albedo >= nt || emission < 0 || emission >= nt || normal < 0 || normal >= nt)
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad surface");
    b->surfaces.push_back(Surface{material, albedo, emission, normal, noise_amount, noise_scale});
    return (int)b->surfaces.size() - 1;
}

int dfpt_builder_add_shape(dfpt_scene_builder* b, int32_t type, const float* params) {
    if (!b || !params) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad shape");
    Shape s;
    s.type = type;
    if (type == DFPT_SHAPE_PLANE) {
        std::memcpy(s.params, params, 9 * sizeof(float));
        s.plane_normal = normal_normalized(params, params + 3, params + 6);
    } else if (type == DFPT_SHAPE_SPHERE) {
        std::memcpy(s.params, params, 4 * sizeof(float));
    } else if (type == DFPT_SHAPE_TERRAIN) {
        std::memcpy(s.params, params, 5 * sizeof(float));
    } else {
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "use dfpt_builder_add_mesh for triangles");
    }
    b->shapes.push_back(std::move(s));
    return (int)b->shapes.size() - 1;
}

int dfpt_builder_add_mesh(dfpt_scene_builder* b, const float* v11, int64_t nv, const int32_t* idx, int64_t nt, int32_t as_mesh) {
    if (!b || !v11 || !idx || nv <= 0 || nt <= 0) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad mesh");
    if (!as_mesh && nt != 1) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "a single triangle needs triangle_count == 1");
    Shape s;
    s.type = as_mesh ? DFPT_SHAPE_TRIANGLE_MESH : DFPT_SHAPE_TRIANGLE;
    s.tris.resize((size_t)nt);
    for (int64_t t = 0; t < nt; ++t) {
        for (int k = 0; k < 3; ++k) {
            const int32_t vi = idx[t * 3 + k];
            if (vi < 0 || vi >= nv) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "mesh index %d out of range", vi);
            const float* src = v11 + (int64_t)vi * 11;
            Vertex& v = s.tris[t].v[k];
            std::memcpy(v.p, src, 12);
            std::memcpy(v.n, src + 3, 12);
            std::memcpy(v.uv, src + 6, 8);
            std::memcpy(v.t, src + 8, 12);
        }
    }
    b->shapes.push_back(std::move(s));
    return (int)b->shapes.size() - 1;
}

int dfpt_builder_add_primitive(dfpt_scene_builder* b, int32_t shape, int32_t surface, const float* t10) {
    if (!b || shape < 0 || shape >= (int)b->shapes.size() || surface < 0 || surface >= (int)b->surfaces.size())
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad primitive");
    Primitive p;
    p.shape = shape;
    p.surface = surface;
    static const float identity[10] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 1};
    if (!transform_matrices(t10 ? t10 : identity, p.o2w, p.w2o))
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "transform cannot be inverted");
    b->primitives.push_back(p);
    return (int)b->primitives.size() - 1;
}

int dfpt_builder_set_camera(dfpt_scene_builder* b, const float* eye, const float* look_at, float fov_x, float res_x,
                            float res_y, float aperture, float focal, int32_t lens) {
    if (!b || !eye || !look_at || res_x < 1.0f || res_y < 1.0f) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad camera");
    float* c = b->camera;
    std::memset(c, 0, sizeof(b->camera));
    c[0] = aperture;
    c[1] = eye[0]; c[2] = eye[1]; c[3] = eye[2];
    c[16] = res_x; c[17] = res_y;
    // setFieldOfViewX (Camera.java:743-748), with MathF's float-rounded trig.
    const float rad = (float)((double)fov_x * (3.14159265358979323846 / 180.0));
    const float tn = (float)std::tan((double)(rad * 0.5f));
    const float at = (float)std::atan((double)(tn * (res_y / res_x)));
    c[4] = fov_x;
    c[5] = (float)((double)(2.0f * at) * (180.0 / 3.14159265358979323846));
    c[6] = focal;
    // W from the viewing direction (doSetOrthoNormalBasisW), then U = up x W, V = W x U.
    const float w0x = look_at[0] - eye[0], w0y = look_at[1] - eye[1], w0z = look_at[2] - eye[2];
    const float wr = 1.0f / std::sqrt(w0x * w0x + w0y * w0y + w0z * w0z);
    const float wx = w0x * wr, wy = w0y * wr, wz = w0z * wr;
    const float upx = 0.0f, upy = 1.0f, upz = 0.0f;
    const float u0x = upy * wz - upz * wy, u0y = upz * wx - upx * wz, u0z = upx * wy - upy * wx;
    const float ur = 1.0f / std::sqrt(u0x * u0x + u0y * u0y + u0z * u0z);
    const float ux = u0x * ur, uy = u0y * ur, uz = u0z * ur;
    const float v0x = wy * uz - wz * uy, v0y = wz * ux - wx * uz, v0z = wx * uy - wy * ux;
    const float vr = 1.0f / std::sqrt(v0x * v0x + v0y * v0y + v0z * v0z);
    c[7] = ux; c[8] = uy; c[9] = uz;
    c[10] = v0x * vr; c[11] = v0y * vr; c[12] = v0z * vr;
    c[13] = wx; c[14] = wy; c[15] = wz;
    c[18] = (float)lens;
    b->camera_set = true;
    return DFPT_OK;
}

// Selects the builder's split search: 0 = sorted sweep (default), 1 = the reference's loop over
// every item for every candidate. Both give the same tree; the second is kept to check that.
int dfpt_builder_set_exhaustive(dfpt_scene_builder* b, int32_t on) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "null builder");
    b->exhaustive_bvh = on != 0;
    return DFPT_OK;
}

int dfpt_builder_compile(dfpt_scene_builder* b, int32_t threads, dfpt_compiled** out) {
    if (!b || !out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad compile arguments");
    if (!b->camera_set) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "camera not set");
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    auto cs = std::make_unique<dfpt_compiled>();

    // doFindAll*: lists in primitive order.
    std::vector<int> mesh_prims;  // primitive indices whose shape is a mesh
    for (size_t i = 0; i < b->primitives.size(); ++i)
        if (b->shapes[b->primitives[i].shape].type == DFPT_SHAPE_TRIANGLE_MESH) mesh_prims.push_back((int)i);

    // One BVH per mesh primitive (doFindAllBoundingVolumeHierarchyRootNodes); meshes shared by
    // several primitives are built once since the builder is deterministic.
    BvhBuilder builder;
    builder.threads = threads;
    builder.exhaustive = b->exhaustive_bvh;
    std::unordered_map<int, std::shared_ptr<BvhNode>> bvh_of_shape;
    std::vector<int> mesh_shapes_in_order;
    for (int pi : mesh_prims) {
        const int si = b->primitives[pi].shape;
        mesh_shapes_in_order.push_back(si);
        if (!bvh_of_shape.count(si)) bvh_of_shape[si] = std::shared_ptr<BvhNode>(builder.create(b->shapes[si].tris).release());
    }

    // Unique triangle meshes (TriangleMesh.equals compares the triangle lists).
    std::vector<int> unique_mesh_shapes;
    {
        auto same_mesh = [&](int a, int c) {
            const auto& ta = b->shapes[a].tris;
            const auto& tc = b->shapes[c].tris;
            if (ta.size() != tc.size()) return false;
            for (size_t i = 0; i < ta.size(); ++i)
                if (!(tri_key(ta[i]) == tri_key(tc[i]))) return false;
            return true;
        };
        for (int si : mesh_shapes_in_order) {
            bool dup = false;
            for (int u : unique_mesh_shapes)
                if (u == si || same_mesh(u, si)) { dup = true; break; }
            if (!dup) unique_mesh_shapes.push_back(si);
        }
    }
    // Unique BVH roots (distinct over Node.equals), aligned with the unique meshes.
    std::vector<int> unique_bvh_shapes;
    for (int si : mesh_shapes_in_order) {
        bool dup = false;
        for (int u : unique_bvh_shapes)
            if (u == si || bvh_equal(bvh_of_shape[u].get(), bvh_of_shape[si].get(), b->shapes[u].tris, b->shapes[si].tris)) { dup = true; break; }
        if (!dup) unique_bvh_shapes.push_back(si);
    }

    // Surfaces and textures.
    Distinct dsurf;
    std::vector<int> surface_rep;  // builder surface index of each unique surface
    // Canonical texture ids: textures equal by value share an id (blend records use child ids).
    std::vector<int> tex_canon(b->textures.size());
    Distinct dtexval;
    for (size_t i = 0; i < b->textures.size(); ++i) {
        std::vector<float> rec = b->textures[i];
        if ((int)rec[0] == DFPT_TEXTURE_BLEND) {
            rec[2] = (float)tex_canon[(int)rec[2]];
            rec[3] = (float)tex_canon[(int)rec[3]];
        }
        Key k;
        for (float f : rec) k.w.push_back(fbits(f));
        tex_canon[i] = dtexval.add(k);
    }
    auto surf_key = [&](const Surface& s) {
        return Key{{(uint32_t)s.material, (uint32_t)tex_canon[s.albedo], (uint32_t)tex_canon[s.emission],
                    (uint32_t)tex_canon[s.normal], fbits(s.noise_amount), fbits(s.noise_scale)}};
    };
    // doFindAllTextures: per surface (primitive order, duplicates included) albedo, emission,
    // normal, then the children of whichever of those are blend textures.
    Distinct dtex;
    std::vector<int> tex_rep;  // builder index of each unique texture
    auto add_tex = [&](int ti) {
        const size_t before = dtex.order.size();
        dtex.add(Key{{(uint32_t)tex_canon[ti]}});
        if (dtex.order.size() != before) tex_rep.push_back(ti);
    };
    for (const Primitive& p : b->primitives) {
        const Surface& s = b->surfaces[p.surface];
        const size_t before = dsurf.order.size();
        dsurf.add(surf_key(s));
        if (dsurf.order.size() != before) surface_rep.push_back(p.surface);
        add_tex(s.albedo);
        add_tex(s.emission);
        add_tex(s.normal);
        for (int ti : {s.albedo, s.emission, s.normal}) {
            if ((int)b->textures[ti][0] == DFPT_TEXTURE_BLEND) {
                add_tex((int)b->textures[ti][2]);
                add_tex((int)b->textures[ti][3]);
            }
        }
    }
    std::vector<int> tex_offset_of_canon(dtexval.order.size(), -1);
    {
        int off = 0;
        for (int ti : tex_rep) {
            tex_offset_of_canon[tex_canon[ti]] = off;
            off += (int)b->textures[ti][1];
        }
    }
    for (int ti : tex_rep) {
        std::vector<float> rec = b->textures[ti];
        if ((int)rec[0] == DFPT_TEXTURE_BLEND) {
            rec[2] = (float)tex_offset_of_canon[tex_canon[(int)rec[2]]];
            rec[3] = (float)tex_offset_of_canon[tex_canon[(int)rec[3]]];
        }
        cs->textures.insert(cs->textures.end(), rec.begin(), rec.end());
    }
    for (int si : surface_rep) {
        const Surface& s = b->surfaces[si];
        cs->surfaces.push_back((float)s.material);
        cs->surfaces.push_back((float)tex_offset_of_canon[tex_canon[s.albedo]]);
        cs->surfaces.push_back((float)tex_offset_of_canon[tex_canon[s.emission]]);
        cs->surfaces.push_back((float)tex_offset_of_canon[tex_canon[s.normal]]);
        cs->surfaces.push_back(s.noise_amount);
        cs->surfaces.push_back(s.noise_scale);
    }

    // Points (BVH bounds first), texture coordinates, vectors.
    DistinctN<3> p3, v3;
    DistinctN<2> p2;
    for (int si : mesh_shapes_in_order) bvh_add_bounds(bvh_of_shape[si].get(), p3);
    auto add_tri_points = [&](const Tri& t) {
        for (int k = 0; k < 3; ++k) p3.add(key3(t.v[k].p[0], t.v[k].p[1], t.v[k].p[2]));
    };
    for (const Primitive& p : b->primitives) {
        const Shape& s = b->shapes[p.shape];
        if (s.type == DFPT_SHAPE_PLANE) {
            for (int k = 0; k < 3; ++k) p3.add(key3(s.params[3 * k], s.params[3 * k + 1], s.params[3 * k + 2]));
        } else if (s.type == DFPT_SHAPE_SPHERE) {
            p3.add(key3(s.params[0], s.params[1], s.params[2]));
        } else if (s.type == DFPT_SHAPE_TRIANGLE || s.type == DFPT_SHAPE_TRIANGLE_MESH) {
            for (const Tri& t : s.tris) add_tri_points(t);
        }
    }
    for (const Primitive& p : b->primitives) {
        const Shape& s = b->shapes[p.shape];
        if (s.type == DFPT_SHAPE_TRIANGLE || s.type == DFPT_SHAPE_TRIANGLE_MESH)
            for (const Tri& t : s.tris)
                for (int k = 0; k < 3; ++k) p2.add(key2(t.v[k].uv[0], t.v[k].uv[1]));
    }
    for (const Primitive& p : b->primitives) {
        const Shape& s = b->shapes[p.shape];
        if (s.type == DFPT_SHAPE_PLANE) {
            v3.add(key3(s.plane_normal.x, s.plane_normal.y, s.plane_normal.z));
        } else if (s.type == DFPT_SHAPE_TRIANGLE || s.type == DFPT_SHAPE_TRIANGLE_MESH) {
            for (const Tri& t : s.tris) {
                for (int k = 0; k < 3; ++k) v3.add(key3(t.v[k].n[0], t.v[k].n[1], t.v[k].n[2]));
                for (int k = 0; k < 3; ++k) v3.add(key3(t.v[k].t[0], t.v[k].t[1], t.v[k].t[2]));
            }
        }
    }
    auto unpack = [](const auto& d, std::vector<float>& out) {
        for (const auto& k : d.order)
            for (uint32_t w : k.w) {
                float f;
                std::memcpy(&f, &w, 4);
                out.push_back(f);
            }
        if (out.empty()) out.push_back(0.0f);
    };
    unpack(p2, cs->point2fs);
    unpack(p3, cs->point3fs);
    unpack(v3, cs->vector3fs);
    std::vector<int> identity_index(p3.order.size());
    for (size_t i = 0; i < identity_index.size(); ++i) identity_index[i] = (int)i;

    // Shapes: unique planes, spheres, terrains, triangles (primitive order).
    Distinct dplane, dsphere, dterrain;
    DistinctN<33> dtri;
    std::vector<int> plane_off(b->shapes.size(), -1), sphere_off(b->shapes.size(), -1), terrain_off(b->shapes.size(), -1);
    std::vector<std::vector<int>> tri_off(b->shapes.size());
    for (const Primitive& p : b->primitives) {
        const Shape& s = b->shapes[p.shape];
        const int si = p.shape;
        if (s.type == DFPT_SHAPE_PLANE) {
            Key k{{}};
            for (int i = 0; i < 9; ++i) k.w.push_back(fbits(s.params[i]));
            k.w.push_back(fbits(s.plane_normal.x)); k.w.push_back(fbits(s.plane_normal.y)); k.w.push_back(fbits(s.plane_normal.z));
            const size_t before = dplane.order.size();
            const int u = dplane.add(k);
            plane_off[si] = u * 4;
            if (dplane.order.size() != before) {
                for (int q = 0; q < 3; ++q) cs->planes.push_back(p3.find(key3(s.params[3 * q], s.params[3 * q + 1], s.params[3 * q + 2])) * 3);
                cs->planes.push_back(v3.find(key3(s.plane_normal.x, s.plane_normal.y, s.plane_normal.z)) * 3);
            }
        } else if (s.type == DFPT_SHAPE_SPHERE) {
            Key k{{fbits(s.params[0]), fbits(s.params[1]), fbits(s.params[2]), fbits(s.params[3])}};
            const size_t before = dsphere.order.size();
            const int u = dsphere.add(k);
            sphere_off[si] = u * 2;
            if (dsphere.order.size() != before) {
                cs->spheres.push_back((float)(p3.find(key3(s.params[0], s.params[1], s.params[2])) * 3));
                cs->spheres.push_back(s.params[3]);
            }
        } else if (s.type == DFPT_SHAPE_TERRAIN) {
            Key k{{}};
            for (int i = 0; i < 4; ++i) k.w.push_back(fbits(s.params[i]));
            k.w.push_back((uint32_t)(int)s.params[4]);
            const size_t before = dterrain.order.size();
            const int u = dterrain.add(k);
            terrain_off[si] = u * 5;
            if (dterrain.order.size() != before) {
                for (int i = 0; i < 4; ++i) cs->terrains.push_back(s.params[i]);
                cs->terrains.push_back((float)(int)s.params[4]);
            }
        } else {
            std::vector<int>& offs = tri_off[si];
            const bool fill = offs.empty();
            for (const Tri& t : s.tris) {
                const size_t before = dtri.order.size();
                const int u = dtri.add(tri_key(t));
                if (fill) offs.push_back(u * 12);
                if (dtri.order.size() != before) {
                    for (int k = 0; k < 3; ++k) cs->triangles.push_back(p3.find(key3(t.v[k].p[0], t.v[k].p[1], t.v[k].p[2])) * 3);
                    for (int k = 0; k < 3; ++k) cs->triangles.push_back(v3.find(key3(t.v[k].n[0], t.v[k].n[1], t.v[k].n[2])) * 3);
                    for (int k = 0; k < 3; ++k) cs->triangles.push_back(p2.find(key2(t.v[k].uv[0], t.v[k].uv[1])) * 2);
                    for (int k = 0; k < 3; ++k) cs->triangles.push_back(v3.find(key3(t.v[k].t[0], t.v[k].t[1], t.v[k].t[2])) * 3);
                }
            }
        }
    }

    // BVH arrays for the unique roots, concatenated; root offsets per unique mesh.
    std::unordered_map<int, int> bvh_root_offset;
    for (size_t u = 0; u < unique_bvh_shapes.size(); ++u) {
        const int si = unique_bvh_shapes[u];
        const int base = (int)cs->bvh.size();
        bvh_root_offset[si] = base;
        bvh_flatten(bvh_of_shape[si].get(), -1, cs->bvh, base, tri_off[si], p3, identity_index);
    }
    // Meshes equal to a unique one share its root offset.
    for (int si : mesh_shapes_in_order) {
        if (bvh_root_offset.count(si)) continue;
        for (int u : unique_bvh_shapes)
            if (bvh_equal(bvh_of_shape[u].get(), bvh_of_shape[si].get(), b->shapes[u].tris, b->shapes[si].tris)) {
                bvh_root_offset[si] = bvh_root_offset[u];
                break;
            }
    }

    // Primitives (every Primitive is unique: Transform has identity equality).
    for (const Primitive& p : b->primitives) {
        const Shape& s = b->shapes[p.shape];
        int shape_offset = 0;
        switch (s.type) {
            case DFPT_SHAPE_PLANE: shape_offset = plane_off[p.shape]; break;
            case DFPT_SHAPE_SPHERE: shape_offset = sphere_off[p.shape]; break;
            case DFPT_SHAPE_TERRAIN: shape_offset = terrain_off[p.shape]; break;
            case DFPT_SHAPE_TRIANGLE: shape_offset = tri_off[p.shape][0]; break;
            default: shape_offset = bvh_root_offset[p.shape]; break;
        }
        cs->primitives.push_back(s.type);
        cs->primitives.push_back(shape_offset);
        cs->primitives.push_back(dsurf.find(surf_key(b->surfaces[p.surface])) * 6);
        cs->o2w.insert(cs->o2w.end(), p.o2w, p.o2w + 16);
        cs->w2o.insert(cs->w2o.end(), p.w2o, p.w2o + 16);
    }
    if (cs->planes.empty()) cs->planes.push_back(0);
    if (cs->spheres.empty()) cs->spheres.push_back(0.0f);
    if (cs->terrains.empty()) cs->terrains.push_back(0.0f);
    if (cs->triangles.empty()) cs->triangles.push_back(0);
    if (cs->bvh.empty()) cs->bvh.push_back(0);
    if (cs->textures.empty()) cs->textures.push_back(0.0f);
    if (cs->surfaces.empty()) cs->surfaces.push_back(0.0f);
    if (cs->primitives.empty()) cs->primitives.push_back(0);
    cs->camera.assign(b->camera, b->camera + 19);
    *out = cs.release();
    return DFPT_OK;
}

int dfpt_compiled_destroy(dfpt_compiled* c) {
    delete c;
    return DFPT_OK;
}

int dfpt_compiled_describe(const dfpt_compiled* c, dfpt_scene_desc* d) {
    if (!c || !d) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad describe arguments");
    d->point2fs = c->point2fs.data(); d->point2fs_count = (int64_t)c->point2fs.size();
    d->point3fs = c->point3fs.data(); d->point3fs_count = (int64_t)c->point3fs.size();
    d->vector3fs = c->vector3fs.data(); d->vector3fs_count = (int64_t)c->vector3fs.size();
    d->planes = c->planes.data(); d->planes_count = (int64_t)c->planes.size();
    d->spheres = c->spheres.data(); d->spheres_count = (int64_t)c->spheres.size();
    d->terrains = c->terrains.data(); d->terrains_count = (int64_t)c->terrains.size();
    d->triangles = c->triangles.data(); d->triangles_count = (int64_t)c->triangles.size();
    d->bounding_volume_hierarchies = c->bvh.data(); d->bounding_volume_hierarchies_count = (int64_t)c->bvh.size();
    d->textures = c->textures.data(); d->textures_count = (int64_t)c->textures.size();
    d->surfaces = c->surfaces.data(); d->surfaces_count = (int64_t)c->surfaces.size();
    d->primitives = c->primitives.data(); d->primitives_count = (int64_t)c->primitives.size();
    d->primitives_object_to_world = c->o2w.data(); d->primitives_object_to_world_count = (int64_t)c->o2w.size();
    d->primitives_world_to_object = c->w2o.data(); d->primitives_world_to_object_count = (int64_t)c->w2o.size();
    d->camera = c->camera.data(); d->camera_count = (int64_t)c->camera.size();
    d->primitive_extensions = nullptr; d->primitive_extensions_count = 0;  // not among the compiled arrays
    return DFPT_OK;
}

int dfpt_sky_set(dfpt_sky* sky, const float* dir, float turbidity) {
    if (!sky || !dir) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "bad sky arguments");
    std::memset(sky, 0, sizeof(*sky));
    // Vector3F.normalize divides by the float length.
    const float len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const float dwx = dir[0] / len, dwy = dir[1] / len, dwz = dir[2] / len;
    // The sky basis: u = X, v = Z, w = Y (Sky.java:61), transformReverse = dot with u, v, w.
    const float u[3] = {1, 0, 0}, v[3] = {0, 0, 1}, w[3] = {0, 1, 0};
    const float sx0 = dwx * u[0] + dwy * u[1] + dwz * u[2];
    const float sy0 = dwx * v[0] + dwy * v[1] + dwz * v[2];
    const float sz0 = dwx * w[0] + dwy * w[1] + dwz * w[2];
    const float sl = std::sqrt(sx0 * sx0 + sy0 * sy0 + sz0 * sz0);
    const float sdx = sx0 / sl, sdy = sy0 / sl, sdz = sz0 / sl;
    for (int i = 0; i < 3; ++i) {
        sky->orthonormal_basis_u[i] = u[i];
        sky->orthonormal_basis_v[i] = v[i];
        sky->orthonormal_basis_w[i] = w[i];
    }
    sky->sun_direction_world[0] = dwx; sky->sun_direction_world[1] = dwy; sky->sun_direction_world[2] = dwz;
    sky->sun_direction[0] = sdx; sky->sun_direction[1] = sdy; sky->sun_direction[2] = sdz;
    sky->sun_origin[0] = 0.0f + dwx * 10000.0f;
    sky->sun_origin[1] = 0.0f + dwy * 10000.0f;
    sky->sun_origin[2] = 0.0f + dwz * 10000.0f;
    const float zc = sdz < -1.0f ? -1.0f : sdz > 1.0f ? 1.0f : sdz;
    sky->theta = (float)std::acos((double)zc);
    const double theta = sky->theta, theta2 = theta * theta, theta3 = theta * theta * theta;
    const double t = turbidity, t2 = t * t;
    const double pi_f = (double)3.14159274101257324219f;  // MathF.PI, a float
    const double chi = (4.0 / 9.0 - t / 120.0) * (pi_f - 2.0 * theta);
    sky->zenith_relative_luminance = ((4.0453 * t - 4.9710) * std::tan(chi) - 0.2155 * t + 2.4192) * 1000.0;
    sky->zenith_x = (0.00165 * theta3 - 0.00374 * theta2 + 0.00208 * theta + 0.0) * t2 +
                    (-0.02902 * theta3 + 0.06377 * theta2 - 0.03202 * theta + 0.00394) * t +
                    (0.11693 * theta3 - 0.21196 * theta2 + 0.06052 * theta + 0.25885);
    sky->zenith_y = (0.00275 * theta3 - 0.00610 * theta2 + 0.00316 * theta + 0.0) * t2 +
                    (-0.04212 * theta3 + 0.08970 * theta2 - 0.04153 * theta + 0.00515) * t +
                    (0.15346 * theta3 - 0.26756 * theta2 + 0.06669 * theta + 0.26688);
    const double pl[5] = {0.17872 * t - 1.46303, -0.35540 * t + 0.42749, -0.02266 * t + 5.32505, 0.12064 * t - 2.57705, -0.06696 * t + 0.37027};
    const double px[5] = {-0.01925 * t - 0.25922, -0.06651 * t + 0.00081, -0.00041 * t + 0.21247, -0.06409 * t - 0.89887, -0.00325 * t + 0.04517};
    const double py[5] = {-0.01669 * t - 0.26078, -0.09495 * t + 0.00921, -0.00792 * t + 0.21023, -0.04405 * t - 1.65369, -0.01092 * t + 0.05291};
    for (int i = 0; i < 5; ++i) {
        sky->perez_relative_luminance[i] = pl[i];
        sky->perez_x[i] = px[i];
        sky->perez_y[i] = py[i];
    }
    sky->is_sky_active = 1;
    sky->is_sun_active = 1;
    return DFPT_OK;
}

void dfpt_params_default(dfpt_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->renderer_type = DFPT_RENDERER_PATH_TRACER;
    p->tone_mapper_type = DFPT_TONE_MAPPER_FILMIC_CURVE_ACES_MODIFIED;
    p->shader_type = DFPT_SHADER_GOURAUD;
    p->normal_mapping = 1;
    p->wireframes = 0;
    p->pt_ray_depth_maximum = 5;
    p->pt_ray_depth_russian_roulette = 5;
    p->tone_mapper_exposure = 1.0f;
    p->ao_maximum_distance = 200.0f;
    p->global_amplitude = 0.5f;
    p->global_frequency = 0.2f;
    p->global_lacunarity = 2.0f;
    p->global_gain = 1.0f / 2.0f;
    p->global_octaves = 2;
    p->selected_primitive_offset = -1;
    p->rng_kind = DFPT_RNG_COUNTER;
    p->seed = 0x9E3779B97F4A7C15ull;
}

}  // extern "C"
