// dfpt_cull.h - the host builder of the primitive-culling BVH (a BVH over the world boxes of a
// scene's bounded primitives). Header-only, without CUDA types, so that the CPU tests build it with
// the host compiler alone.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace dfpt_cull {

struct CullItem { float lo[3], hi[3]; int prim; };

// A node of the culling BVH: its box, and either two child nodes (left, right >= 0) or a leaf
// (left = -(first + 1), right = count) whose primitives are prims[first .. first + count - 1], in
// index order. The device walk reads it as two float4s {lo, left bits}, {hi, right bits}.
struct CullNode { float lo[3]; int left; float hi[3]; int right; };

// Surface area of a box (the SAH's hit probability up to a common factor).
inline double cull_area(const float lo[3], const float hi[3]) {
    const double x = std::max(0.0, (double)hi[0] - lo[0]), y = std::max(0.0, (double)hi[1] - lo[1]), z = std::max(0.0, (double)hi[2] - lo[2]);
    return 2.0 * (x * y + y * z + z * x);
}

// One node of the culling BVH over items [begin, end). Splits by the surface-area heuristic (each
// axis's centroid order swept for the cheapest split, a node test costing as much as a primitive's
// box test), so that a ray's walk collects few candidates besides the primitives whose boxes it
// crosses; leaves hold at most 4 primitives (in index order). Nodes with very many items, and every
// node past depth 16, split at the median of the longest centroid axis, which bounds the depth (the
// walk keeps a 32-entry stack). The tree only decides which primitives a ray box-tests: hits do not
// depend on it.
inline int build_cull_node(std::vector<CullItem>& items, int begin, int end, std::vector<CullNode>& nodes, std::vector<int>& prims,
                           int depth) {
    const int node = (int)nodes.size();
    nodes.push_back(CullNode{});
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = begin; k < end; ++k)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], items[k].lo[a]);
            hi[a] = std::max(hi[a], items[k].hi[a]);
            const float c = 0.5f * (items[k].lo[a] + items[k].hi[a]);
            clo[a] = std::min(clo[a], c);
            chi[a] = std::max(chi[a], c);
        }
    const int n = end - begin;
    int split = -1;  // items [begin, split) go left
    if (n > 2 && n <= 65536 && depth < 16) {
        const double area = cull_area(lo, hi);
        double best = INFINITY;
        int best_axis = 0, best_i = 0;
        std::vector<double> left((size_t)n);
        for (int a = 0; a < 3; ++a) {
            std::sort(items.begin() + begin, items.begin() + end, [a](const CullItem& x, const CullItem& y) {
                const float cx = x.lo[a] + x.hi[a], cy = y.lo[a] + y.hi[a];
                return cx < cy || (cx == cy && x.prim < y.prim);
            });
            float bl[3] = {INFINITY, INFINITY, INFINITY}, bh[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int i = 0; i < n; ++i) {
                for (int c = 0; c < 3; ++c) { bl[c] = std::min(bl[c], items[begin + i].lo[c]); bh[c] = std::max(bh[c], items[begin + i].hi[c]); }
                left[(size_t)i] = cull_area(bl, bh);  // box of items 0..i
            }
            float rl[3] = {INFINITY, INFINITY, INFINITY}, rh[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int i = n - 1; i >= 1; --i) {
                for (int c = 0; c < 3; ++c) { rl[c] = std::min(rl[c], items[begin + i].lo[c]); rh[c] = std::max(rh[c], items[begin + i].hi[c]); }
                // Items [0, i) left, [i, n) right.
                const double cost = left[(size_t)i - 1] * i + cull_area(rl, rh) * (n - i);
                if (cost < best) { best = cost; best_axis = a; best_i = i; }
            }
        }
        // A leaf of up to 4 costs its boxes' tests; a split costs the node test plus the children's.
        const bool leaf = n <= 4 && !(area > 0.0 && 1.0 + best / area < (double)n);
        if (!leaf) {
            const int a = best_axis;
            std::sort(items.begin() + begin, items.begin() + end, [a](const CullItem& x, const CullItem& y) {
                const float cx = x.lo[a] + x.hi[a], cy = y.lo[a] + y.hi[a];
                return cx < cy || (cx == cy && x.prim < y.prim);
            });
            split = begin + best_i;
        }
    } else if (n > 4) {
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        split = (begin + end) / 2;
        std::nth_element(items.begin() + begin, items.begin() + split, items.begin() + end, [axis](const CullItem& x, const CullItem& y) {
            const float cx = x.lo[axis] + x.hi[axis], cy = y.lo[axis] + y.hi[axis];
            return cx < cy || (cx == cy && x.prim < y.prim);
        });
    }
    int l, r;
    if (split < 0) {
        std::vector<int> ps;
        for (int k = begin; k < end; ++k) ps.push_back(items[k].prim);
        std::sort(ps.begin(), ps.end());
        l = -((int)prims.size() + 1);
        r = end - begin;
        prims.insert(prims.end(), ps.begin(), ps.end());
    } else {
        l = build_cull_node(items, begin, split, nodes, prims, depth + 1);
        r = build_cull_node(items, split, end, nodes, prims, depth + 1);
    }
    CullNode& out = nodes[(size_t)node];
    for (int a = 0; a < 3; ++a) { out.lo[a] = lo[a]; out.hi[a] = hi[a]; }
    out.left = l;
    out.right = r;
    return node;
}

}  // namespace dfpt_cull
