// bvh_build.cpp -- host construction of one surface mesh's BVH.
//
// Binned SAH as SimBVH.buildBVH / subdivide / findBestSplitPlaneBinned (reference
// FF_SRL/FF_SRL/bvh.py:281-518), reproducing the reference's number types so that the
// topology (child ids, triangle order, levels) is identical:
//   - centroids are float32 ((a + b) + c) / 3 (calculateCentroids, bvh.py:6-21);
//   - the root box is the float32 min/max of all points (bvh.py:479-480) and its area
//     is formed in float32; every other box is grown in double from float vertices;
//   - costs, the bin scale, the bin index, the split position and the partition test
//     are double, as NumPy 1.x computed a float32 scalar with a Python number;
//   - children are numbered in creation order from 1 (nodesUsed starts at 1) and the
//     recursion visits the left child first;
//   - a node whose best binned cost is >= its own cost, or whose partition leaves one
//     side empty, stays a leaf; the root is created with leftNode = 0 and, if it is never
//     split, marked a leaf (-1) instead of keeping the reference's dangling child id.
// Compiled without fused multiply-add so float and double expressions round as written.
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include "ffsrl_internal.h"

namespace {

struct Node {
    double lo[3], hi[3];
    int32_t left = -1, first = 0, count = 0, level = -1;
};

struct Builder {
    const float* pts;
    const int32_t* faces;
    int bins;
    std::vector<float> cent;  // [3F]
    std::vector<int32_t> tri;
    std::vector<Node> nodes;
    int used = 1;
    float root_lo[3], root_hi[3];

    double area(const double* lo, const double* hi) const {
        double e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
        return e0 * e1 + e1 * e2 + e2 * e0;
    }

    double node_cost(int n) const {
        if (n == 0) {
            float e0 = root_hi[0] - root_lo[0], e1 = root_hi[1] - root_lo[1], e2 = root_hi[2] - root_lo[2];
            float a = e0 * e1 + e1 * e2;
            a = a + e2 * e0;
            return double(nodes[n].count) * double(a);
        }
        return double(nodes[n].count) * area(nodes[n].lo, nodes[n].hi);
    }

    void grow(double* lo, double* hi, int32_t f) const {
        for (int c = 0; c < 3; ++c) {
            const float* p = pts + 3 * (int64_t)faces[3 * (int64_t)f + c];
            for (int d = 0; d < 3; ++d) {
                double v = p[d];
                if (v < lo[d]) lo[d] = v;
                if (v > hi[d]) hi[d] = v;
            }
        }
    }

    void update_bounds(int n) {
        Node& nd = nodes[n];
        for (int d = 0; d < 3; ++d) { nd.lo[d] = 1e30; nd.hi[d] = -1e30; }
        for (int i = nd.first; i < nd.first + nd.count; ++i) grow(nd.lo, nd.hi, tri[i]);
    }

    void best_split(int n, double* best_cost, int* best_axis, double* best_pos) {
        const Node& nd = nodes[n];
        *best_cost = 1e30; *best_axis = -1; *best_pos = 0.0;
        std::vector<double> blo(3 * bins), bhi(3 * bins);
        std::vector<int64_t> bcnt(bins);
        std::vector<double> larea(bins), rarea(bins);
        std::vector<int64_t> lcnt(bins), rcnt(bins);
        for (int axis = 0; axis < 3; ++axis) {
            double bmin = 1e30, bmax = -1e30;
            for (int j = 0; j < nd.count; ++j) {
                double c = cent[3 * (int64_t)tri[nd.first + j] + axis];
                bmin = c < bmin ? c : bmin;
                bmax = c > bmax ? c : bmax;
            }
            if (bmax == bmin) continue;
            for (int b = 0; b < bins; ++b) {
                bcnt[b] = 0;
                for (int d = 0; d < 3; ++d) { blo[3 * b + d] = 1e30; bhi[3 * b + d] = -1e30; }
            }
            double scale = double(bins) / (bmax - bmin);
            for (int j = 0; j < nd.count; ++j) {
                int32_t f = tri[nd.first + j];
                double c = cent[3 * (int64_t)f + axis];
                int64_t b = (int64_t)((c - bmin) * scale);
                if (b > bins - 1) b = bins - 1;
                bcnt[b] += 1;
                grow(&blo[3 * b], &bhi[3 * b], f);
            }
            double llo[3] = {1e30, 1e30, 1e30}, lhi[3] = {-1e30, -1e30, -1e30};
            double rlo[3] = {1e30, 1e30, 1e30}, rhi[3] = {-1e30, -1e30, -1e30};
            int64_t ls = 0, rs = 0;
            for (int j = 0; j < bins - 1; ++j) {
                ls += bcnt[j];
                lcnt[j] = ls;
                for (int d = 0; d < 3; ++d) {
                    llo[d] = std::min(llo[d], blo[3 * j + d]);
                    lhi[d] = std::max(lhi[d], bhi[3 * j + d]);
                }
                larea[j] = area(llo, lhi);
                int k = bins - 1 - j;
                rs += bcnt[k];
                rcnt[bins - 2 - j] = rs;
                for (int d = 0; d < 3; ++d) {
                    rlo[d] = std::min(rlo[d], blo[3 * k + d]);
                    rhi[d] = std::max(rhi[d], bhi[3 * k + d]);
                }
                rarea[bins - 2 - j] = area(rlo, rhi);
            }
            double step = (bmax - bmin) / double(bins);
            for (int j = 0; j < bins - 1; ++j) {
                double cost = double(lcnt[j]) * larea[j] + double(rcnt[j]) * rarea[j];
                if (cost < *best_cost) {
                    *best_axis = axis;
                    *best_pos = bmin + step * double(j + 1);
                    *best_cost = cost;
                }
            }
        }
    }

    void subdivide(int n, int level) {
        double cost, pos;
        int axis;
        best_split(n, &cost, &axis, &pos);
        if (cost >= node_cost(n)) return;
        int i = nodes[n].first;
        int j = i + nodes[n].count - 1;
        while (i <= j) {
            if (double(cent[3 * (int64_t)tri[i] + axis]) < pos) {
                ++i;
            } else {
                std::swap(tri[i], tri[j]);
                --j;
            }
        }
        int lc = i - nodes[n].first;
        if (lc == 0 || lc == nodes[n].count) return;
        int l = used, r = used + 1;
        used += 2;
        nodes[l].first = nodes[n].first; nodes[l].count = lc; nodes[l].level = level + 1;
        nodes[r].first = i; nodes[r].count = nodes[n].count - lc; nodes[r].level = level + 1;
        nodes[n].left = l;
        nodes[n].count = 0;
        update_bounds(l);
        update_bounds(r);
        subdivide(l, level + 1);
        subdivide(r, level + 1);
    }
};

}  // namespace

extern "C" int32_t ffsrl_bvh_build_host(const float* points, const int32_t* faces, int32_t num_points,
                                        int32_t num_faces, int32_t bins, int32_t* left_node, int32_t* first_tri_id,
                                        int32_t* tri_count, int32_t* level, int32_t* tri_id, float* aabb_min,
                                        float* aabb_max, int32_t* num_nodes, int32_t* max_level) {
    if (!points || !faces || num_points <= 0 || num_faces <= 0 || bins < 2 || !left_node || !first_tri_id ||
        !tri_count || !level || !tri_id || !num_nodes || !max_level)
        return ffsrl::fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh_build_host: null pointer or empty mesh");
    for (int64_t i = 0; i < 3 * (int64_t)num_faces; ++i)
        if (faces[i] < 0 || faces[i] >= num_points)
            return ffsrl::fail(FFSRL_ERR_INVALID_ARGUMENT, "ffsrl_bvh_build_host: face index out of range");
    Builder b;
    b.pts = points;
    b.faces = faces;
    b.bins = bins;
    b.cent.resize(3 * (size_t)num_faces);
    for (int64_t f = 0; f < num_faces; ++f) {
        const float* A = points + 3 * (int64_t)faces[3 * f];
        const float* B = points + 3 * (int64_t)faces[3 * f + 1];
        const float* C = points + 3 * (int64_t)faces[3 * f + 2];
        for (int d = 0; d < 3; ++d) {
            float s = A[d] + B[d];
            s = s + C[d];
            b.cent[3 * f + d] = s / 3.0f;
        }
    }
    b.tri.resize(num_faces);
    for (int32_t f = 0; f < num_faces; ++f) b.tri[f] = f;
    b.nodes.resize(2 * (size_t)num_faces);
    for (int d = 0; d < 3; ++d) { b.root_lo[d] = points[d]; b.root_hi[d] = points[d]; }
    for (int64_t i = 1; i < num_points; ++i)
        for (int d = 0; d < 3; ++d) {
            float v = points[3 * i + d];
            if (v < b.root_lo[d]) b.root_lo[d] = v;
            if (v > b.root_hi[d]) b.root_hi[d] = v;
        }
    Node& root = b.nodes[0];
    root.left = 0; root.first = 0; root.count = num_faces; root.level = 0;
    for (int d = 0; d < 3; ++d) { root.lo[d] = b.root_lo[d]; root.hi[d] = b.root_hi[d]; }
    b.subdivide(0, 0);
    // The reference creates the root with leftNode = 0 (bvh.py:480); when the root is never
    // split that makes refit and traversal treat nodes 0 and 1 as its children, and node 1
    // does not exist.  An unsplit root is marked as the leaf it is.
    if (b.used == 1) b.nodes[0].left = -1;
    int ml = 0;
    for (int n = 0; n < b.used; ++n) {
        const Node& nd = b.nodes[n];
        left_node[n] = nd.left;
        first_tri_id[n] = nd.first;
        tri_count[n] = nd.count;
        level[n] = nd.level;
        if (aabb_min) for (int d = 0; d < 3; ++d) aabb_min[3 * n + d] = float(nd.lo[d]);
        if (aabb_max) for (int d = 0; d < 3; ++d) aabb_max[3 * n + d] = float(nd.hi[d]);
        ml = std::max(ml, nd.level);
    }
    for (int32_t f = 0; f < num_faces; ++f) tri_id[f] = b.tri[f];
    *num_nodes = b.used;
    *max_level = ml;
    return FFSRL_OK;
}
