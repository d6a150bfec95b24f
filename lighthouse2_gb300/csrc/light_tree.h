/* light_tree.h - the binary light tree of the stochastic-lightcuts light selection (host code).
 *
 * Follows RenderCore::UpdateLightTree / FindBestMatch / UpdateLightTreeNormals
 * (lib/rendercore_optix7/rendercore.cpp:571-680) and the LightCluster constructors and cost
 * (lib/RenderSystem/common_classes.h:487-527):
 *   - leaves: area light i at record i + 1, point light i at 1 + ntri + i, spot light i at 1 + ntri + npt + i; a
 *     leaf's box holds the triangle's vertices or the light's position +- 0.001, its intensity is the light's
 *     energy (the radiance sum for a spot light), its light word the index with bit 30 (point) or 29 (spot);
 *   - agglomerative build: the list of open clusters, a cluster A and its best match B (the lowest intensity x
 *     squared box diagonal of the merged pair, first index on ties); while more than one cluster is open, if B's
 *     best match is A the two merge into a new record (a copy of A grown by B, children A and B) that joins the end of
 *     the list and becomes the next A, else A, B move on to B and B's match;
 *   - the last open cluster is copied to record 0 (the root);
 *   - normals: a triangle leaf takes the light's normal, point and spot leaves none (0); an interior node the
 *     normalised sum of its children's normals when their dot product exceeds 0.9, else none; each child records
 *     its parent, in the normal's w (the root's children name record 0).
 * One deviation: the reference's leaf constructors grow a box that nothing initialised (indeterminate contents);
 * here every leaf box starts empty (min +1e34, max -1e34, aabb::Reset), which the constructors evidently assume.
 *
 * Record layout (16 32-bit words, the device's LightCluster, common_classes.h:522-527): light, left, right (ints,
 * -1 for none), intensity; box minimum xyz, 0; box maximum xyz, 0; normal xyz, parent (int, -1 for none). */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "lh2g_types.h"

namespace lh2g {

struct LightTreeNode {
    int32_t light, left, right;
    float intensity;
    float bmin[4], bmax[4];
    float N[3];
    int32_t parent;
};
static_assert(sizeof(LightTreeNode) == 64, "one record is 4 float4");

namespace lighttree_detail {
/* aabb::Grow's _mm_min_ps / _mm_max_ps lane rule: the first operand where it is smaller (larger), else the second */
inline float lane_min(float a, float b) { return a < b ? a : b; }
inline float lane_max(float a, float b) { return a > b ? a : b; }
inline void grow_point(LightTreeNode& c, float x, float y, float z) {
    const float p[4] = {x, y, z, 0.0f};
    for (int k = 0; k < 4; k++) c.bmin[k] = lane_min(c.bmin[k], p[k]), c.bmax[k] = lane_max(c.bmax[k], p[k]);
}
inline void grow_box(LightTreeNode& c, const LightTreeNode& o) {
    for (int k = 0; k < 4; k++) c.bmin[k] = lane_min(c.bmin[k], o.bmin[k]), c.bmax[k] = lane_max(c.bmax[k], o.bmax[k]);
}
inline LightTreeNode empty_leaf(int32_t light, float intensity) {
    LightTreeNode c;
    c.light = light, c.left = c.right = -1, c.intensity = intensity;
    for (int k = 0; k < 4; k++) c.bmin[k] = 1e34f, c.bmax[k] = -1e34f;
    c.N[0] = c.N[1] = c.N[2] = 0.0f;
    c.parent = -1;
    return c;
}
/* LightCluster::Cost: intensity times the squared diagonal of the box */
inline float cost(const LightTreeNode& c) {
    const float dx = c.bmax[0] - c.bmin[0], dy = c.bmax[1] - c.bmin[1], dz = c.bmax[2] - c.bmin[2];
    return c.intensity * (dx * dx + dy * dy + dz * dz);
}
inline int best_match(const std::vector<LightTreeNode>& t, const std::vector<int>& open, int a, int n) {
    float bestCost = 1e34f;
    int best = 0;
    for (int i = 0; i < n; i++) {
        if (i == a) continue;
        LightTreeNode m = t[open[a]];
        grow_box(m, t[open[i]]);
        m.intensity += t[open[i]].intensity;
        const float c = cost(m);
        if (c < bestCost) bestCost = c, best = i;
    }
    return best;
}
}  // namespace lighttree_detail

/* The tree of the given lights: 2 * (ntri + npt + nspot) records (record 0 the root; none for no lights). */
inline std::vector<LightTreeNode> build_light_tree(const lh2g_light_tri* tri, int ntri, const lh2g_point_light* pt, int npt,
                                                   const lh2g_spot_light* spot, int nspot) {
    using namespace lighttree_detail;
    const int L = ntri + npt + nspot;
    std::vector<LightTreeNode> t((size_t)2 * L);
    if (L == 0) return t;
    for (LightTreeNode& c : t) c = empty_leaf(-1, 0.0f);
    std::vector<int> open((size_t)L);
    for (int i = 0; i < ntri; i++) {
        LightTreeNode c = empty_leaf(i, tri[i].energy);
        grow_point(c, tri[i].vertex0[0], tri[i].vertex0[1], tri[i].vertex0[2]);
        grow_point(c, tri[i].vertex1[0], tri[i].vertex1[1], tri[i].vertex1[2]);
        grow_point(c, tri[i].vertex2[0], tri[i].vertex2[1], tri[i].vertex2[2]);
        t[(size_t)i + 1] = c, open[(size_t)i] = i + 1;
    }
    for (int i = 0; i < npt; i++) {
        LightTreeNode c = empty_leaf(i | (1 << 30), pt[i].energy);
        const float* p = pt[i].position;
        grow_point(c, p[0] - 0.001f, p[1] - 0.001f, p[2] - 0.001f);
        grow_point(c, p[0] + 0.001f, p[1] + 0.001f, p[2] + 0.001f);
        t[(size_t)i + 1 + ntri] = c, open[(size_t)i + ntri] = i + 1 + ntri;
    }
    for (int i = 0; i < nspot; i++) {
        LightTreeNode c = empty_leaf(i | (1 << 29), spot[i].radiance[0] + spot[i].radiance[1] + spot[i].radiance[2]);
        const float* p = spot[i].position;
        grow_point(c, p[0] - 0.001f, p[1] - 0.001f, p[2] - 0.001f);
        grow_point(c, p[0] + 0.001f, p[1] + 0.001f, p[2] + 0.001f);
        t[(size_t)i + 1 + ntri + npt] = c, open[(size_t)i + ntri + npt] = i + 1 + ntri + npt;
    }
    int n = L, last = L, a = 0, b = best_match(t, open, a, n);
    while (n > 1) {
        const int c = best_match(t, open, b, n);
        if (a == c) {
            LightTreeNode m = t[(size_t)open[(size_t)a]];
            grow_box(m, t[(size_t)open[(size_t)b]]);
            m.intensity += t[(size_t)open[(size_t)b]].intensity;
            m.left = open[(size_t)a], m.right = open[(size_t)b];
            t[(size_t)last + 1] = m;
            open.erase(open.begin() + a);   /* A leaves the list, then B (one place earlier if it followed A) */
            if (b > a) b--;
            open.erase(open.begin() + b);
            n -= 2;
            open.insert(open.begin() + n, ++last);
            a = n++;
            b = best_match(t, open, a, n);
        } else {
            a = b, b = c;
        }
    }
    t[0] = t[(size_t)open[0]];
    /* normals and parents, children before their parent (an explicit post-order walk from the root) */
    std::vector<std::pair<int, bool>> stack{{0, false}};
    while (!stack.empty()) {
        const int node = stack.back().first;
        const bool childrenDone = stack.back().second;
        stack.pop_back();
        LightTreeNode& c = t[(size_t)node];
        if (c.left < 0) {
            if (c.light & ((1 << 30) + (1 << 29))) c.N[0] = c.N[1] = c.N[2] = 0.0f;
            else std::memcpy(c.N, tri[c.light].N, sizeof c.N);
            continue;
        }
        if (!childrenDone) {
            stack.push_back({node, true});
            stack.push_back({c.right, false});
            stack.push_back({c.left, false});
            continue;
        }
        const float* nl = t[(size_t)c.left].N;
        const float* nr = t[(size_t)c.right].N;
        if (nl[0] * nr[0] + nl[1] * nr[1] + nl[2] * nr[2] > 0.9f) {
            const float s[3] = {nl[0] + nr[0], nl[1] + nr[1], nl[2] + nr[2]};
            const float inv = 1.0f / std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
            c.N[0] = s[0] * inv, c.N[1] = s[1] * inv, c.N[2] = s[2] * inv;
        } else {
            c.N[0] = c.N[1] = c.N[2] = 0.0f;
        }
        t[(size_t)c.left].parent = t[(size_t)c.right].parent = node;
    }
    return t;
}

}  // namespace lh2g
