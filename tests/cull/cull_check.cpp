// Checks the primitive-culling BVH that dfpt_cull.h builds (test harness, host only).
// Input (stdin): n, then n boxes (lo xyz, hi xyz); m, then m rays (origin xyz, direction xyz).
// Output (one line): nodes depth candidates_mean missed overflow16 errors
//   - every node's box holds its children's boxes (or its leaf's primitive boxes), children follow
//     their parent in preorder, leaves hold 1-4 primitives in index order, every primitive is in
//     exactly one leaf;
//   - a walk of the tree collects every primitive whose own box the ray's half line crosses
//     (`missed` counts those it would not collect), and `candidates_mean` / `overflow16` give the
//     mean candidate count and the fraction of rays with more than 16 candidates.
#include <cmath>
#include <cstdio>
#include <vector>

#include "dfpt_cull.h"

using dfpt_cull::CullItem;
using dfpt_cull::CullNode;

static bool crosses(const float lo[3], const float hi[3], const double o[3], const double d[3]) {
    double tn = 0.0, tf = INFINITY;
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0) {
            if (o[a] < lo[a] || o[a] > hi[a]) return false;
            continue;
        }
        double t0 = (lo[a] - o[a]) / d[a], t1 = (hi[a] - o[a]) / d[a];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::max(tn, t0);
        tf = std::min(tf, t1);
    }
    return tn <= tf;
}

int main() {
    int n = 0;
    if (std::scanf("%d", &n) != 1) return 2;
    std::vector<CullItem> items((size_t)n);
    for (int i = 0; i < n; ++i) {
        CullItem& it = items[(size_t)i];
        if (std::scanf("%f %f %f %f %f %f", &it.lo[0], &it.lo[1], &it.lo[2], &it.hi[0], &it.hi[1], &it.hi[2]) != 6) return 2;
        it.prim = i;
    }
    const std::vector<CullItem> orig = items;
    std::vector<CullNode> nodes;
    std::vector<int> prims;
    if (n > 0) dfpt_cull::build_cull_node(items, 0, n, nodes, prims, 0);
    long errors = 0;
    int depth = 0;
    std::vector<int> seen((size_t)n, 0);
    std::vector<std::pair<int, int>> stack;
    if (n > 0) stack.push_back({0, 0});
    const int nn = (int)nodes.size();
    while (!stack.empty()) {
        const int k = stack.back().first, dep = stack.back().second;
        stack.pop_back();
        depth = std::max(depth, dep);
        const CullNode& nd = nodes[(size_t)k];
        if (nd.left < 0) {
            const int first = -nd.left - 1, count = nd.right;
            if (count < 1 || count > 4 || first < 0 || first + count > (int)prims.size()) { ++errors; continue; }
            for (int j = first; j < first + count; ++j) {
                const int p = prims[(size_t)j];
                if (p < 0 || p >= n) { ++errors; continue; }
                ++seen[(size_t)p];
                if (j > first && prims[(size_t)j - 1] >= p) ++errors;
                for (int a = 0; a < 3; ++a)
                    if (orig[(size_t)p].lo[a] < nd.lo[a] || orig[(size_t)p].hi[a] > nd.hi[a]) ++errors;
            }
        } else {
            if (nd.left <= k || nd.right <= k || nd.left >= nn || nd.right >= nn) { ++errors; continue; }
            for (int c : {nd.left, nd.right})
                for (int a = 0; a < 3; ++a)
                    if (nodes[(size_t)c].lo[a] < nd.lo[a] || nodes[(size_t)c].hi[a] > nd.hi[a]) ++errors;
            stack.push_back({nd.right, dep + 1});
            stack.push_back({nd.left, dep + 1});
        }
    }
    for (int s : seen)
        if (s != 1) ++errors;
    int m = 0;
    if (std::scanf("%d", &m) != 1) m = 0;
    long missed = 0, overflow = 0;
    double cand_sum = 0.0;
    for (int r = 0; r < m; ++r) {
        double o[3], d[3];
        if (std::scanf("%lf %lf %lf %lf %lf %lf", &o[0], &o[1], &o[2], &d[0], &d[1], &d[2]) != 6) return 2;
        std::vector<char> cand((size_t)n, 0);
        int nc = 0;
        std::vector<int> st;
        if (n > 0) st.push_back(0);
        while (!st.empty()) {
            const CullNode& nd = nodes[(size_t)st.back()];
            st.pop_back();
            if (!crosses(nd.lo, nd.hi, o, d)) continue;
            if (nd.left < 0) {
                for (int j = -nd.left - 1; j < -nd.left - 1 + nd.right; ++j) { cand[(size_t)prims[(size_t)j]] = 1; ++nc; }
            } else {
                st.push_back(nd.right);
                st.push_back(nd.left);
            }
        }
        for (int i = 0; i < n; ++i)
            if (!cand[(size_t)i] && crosses(orig[(size_t)i].lo, orig[(size_t)i].hi, o, d)) ++missed;
        cand_sum += nc;
        if (nc > 16) ++overflow;
    }
    std::printf("%d %d %.4f %ld %.5f %ld\n", nn, depth, m ? cand_sum / m : 0.0, missed, m ? (double)overflow / m : 0.0, errors);
    return errors ? 1 : 0;
}
