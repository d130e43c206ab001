"""TEST INFRASTRUCTURE ONLY: numpy restatement of the reference's host BVH build.

Follows ``SimBVH.buildBVH`` / ``subdivide`` / ``findBestSplitPlaneBinned`` /
``updateNodeBounds`` / ``calculateNodeCost`` (``FF_SRL/FF_SRL/bvh.py:281-518``) and the
device centroid kernel ``calculateCentroids`` (``bvh.py:6-21``).  The reference ran
under NumPy 1.x promotion (it predates NumPy 2): an ``np.float32`` scalar combined with a
Python float or int is computed in float64.  This module makes each of those promotions
explicit so it gives the same answers under NumPy 2:

* centroids: float32, ``((a + b) + c) / 3``;
* bin bounds and node bounds grow a float64 box from float32 vertices (exact values);
* the root's bounds are the float32 min/max of all points, so its parent area is
  formed in float32 and then multiplied by the triangle count in float64;
* ``scale``, bin index, split position and the partition test are float64.

The product's C++ builder (``ffsrl_bvh_build_host``) is checked against this for
bit-identical topology (left child, first triangle, count, level, triangle order).
"""

from __future__ import annotations

import numpy as np


def _area64(lo: np.ndarray, hi: np.ndarray) -> float:
    e = hi - lo
    return float(e[0] * e[1] + e[1] * e[2] + e[2] * e[0])


def build_bvh(points: np.ndarray, faces: np.ndarray, bins: int = 8) -> dict:
    points = np.ascontiguousarray(points, dtype=np.float32)
    faces = np.ascontiguousarray(faces, dtype=np.int64).reshape(-1, 3)
    F = len(faces)
    A, B, C = points[faces[:, 0]], points[faces[:, 1]], points[faces[:, 2]]
    cent = ((A + B) + C) / np.float32(3.0)
    tri = np.arange(F, dtype=np.int64)
    corner = np.stack([A, B, C], axis=1).astype(np.float64)  # [F,3,3]

    cap = 2 * F
    left = -np.ones(cap, dtype=np.int64)
    first = np.zeros(cap, dtype=np.int64)
    count = np.zeros(cap, dtype=np.int64)
    level = -np.ones(cap, dtype=np.int64)
    lo = np.zeros((cap, 3))
    hi = np.zeros((cap, 3))

    left[0], first[0], count[0], level[0] = 0, 0, F, 0
    lo32, hi32 = points.min(axis=0), points.max(axis=0)
    lo[0], hi[0] = lo32, hi32
    used = [1]

    def node_cost(n: int) -> float:
        if n == 0:
            e = hi32 - lo32  # float32
            area = np.float32(np.float32(e[0] * e[1]) + np.float32(e[1] * e[2])) + np.float32(e[2] * e[0])
            return float(count[n]) * float(area)
        return float(count[n]) * _area64(lo[n], hi[n])

    def update_bounds(n: int) -> None:
        ids = tri[first[n]:first[n] + count[n]]
        pts = corner[ids].reshape(-1, 3)
        lo[n] = np.minimum(pts.min(axis=0), 1e30)
        hi[n] = np.maximum(pts.max(axis=0), -1e30)

    def best_split(n: int):
        best_cost, best_axis, best_pos = 1e30, -1, 0.0
        ids = tri[first[n]:first[n] + count[n]]
        for axis in range(3):
            cs = cent[ids, axis]
            bmin, bmax = float(cs.min()), float(cs.max())
            if bmax == bmin:
                continue
            scale = bins / (bmax - bmin)
            bid = np.minimum(bins - 1, ((cs.astype(np.float64) - bmin) * scale).astype(np.int64))
            blo = np.full((bins, 3), 1e30)
            bhi = np.full((bins, 3), -1e30)
            bcnt = np.bincount(bid, minlength=bins)
            pts = corner[ids]  # [n,3,3]
            np.minimum.at(blo, bid, pts.min(axis=1))
            np.maximum.at(bhi, bid, pts.max(axis=1))
            lcnt, rcnt = [0] * (bins - 1), [0] * (bins - 1)
            larea, rarea = [0.0] * (bins - 1), [0.0] * (bins - 1)
            llo, lhi = np.full(3, 1e30), np.full(3, -1e30)
            rlo, rhi = np.full(3, 1e30), np.full(3, -1e30)
            ls = rs = 0
            for j in range(bins - 1):
                ls += int(bcnt[j])
                lcnt[j] = ls
                llo, lhi = np.minimum(llo, blo[j]), np.maximum(lhi, bhi[j])
                larea[j] = _area64(llo, lhi)
                k = bins - 1 - j
                rs += int(bcnt[k])
                rcnt[bins - 2 - j] = rs
                rlo, rhi = np.minimum(rlo, blo[k]), np.maximum(rhi, bhi[k])
                rarea[bins - 2 - j] = _area64(rlo, rhi)
            step = (bmax - bmin) / bins
            for j in range(bins - 1):
                cost = lcnt[j] * larea[j] + rcnt[j] * rarea[j]
                if cost < best_cost:
                    best_axis, best_pos, best_cost = axis, bmin + step * (j + 1), cost
        return best_cost, best_axis, best_pos

    def subdivide(n: int, lev: int) -> None:
        best_cost, axis, pos = best_split(n)
        if best_cost >= node_cost(n):
            return
        i = int(first[n])
        j = i + int(count[n]) - 1
        while i <= j:
            if float(cent[tri[i], axis]) < pos:
                i += 1
            else:
                tri[i], tri[j] = tri[j], tri[i]
                j -= 1
        lc = i - int(first[n])
        if lc == 0 or lc == count[n]:
            return
        l, r = used[0], used[0] + 1
        used[0] += 2
        first[l], count[l], level[l] = first[n], lc, lev + 1
        first[r], count[r], level[r] = i, count[n] - lc, lev + 1
        left[n] = l
        count[n] = 0
        update_bounds(l)
        update_bounds(r)
        subdivide(l, lev + 1)
        subdivide(r, lev + 1)

    subdivide(0, 0)
    n = used[0]
    if n == 1:  # unsplit root: a leaf, not the reference's dangling leftNode = 0
        left[0] = -1
    return {
        "left_node": left[:n].astype(np.int32),
        "first_tri_id": first[:n].astype(np.int32),
        "tri_count": count[:n].astype(np.int32),
        "level": level[:n].astype(np.int32),
        "tri_id": tri.astype(np.int32),
        "aabb_min": lo[:n].astype(np.float32),
        "aabb_max": hi[:n].astype(np.float32),
        "num_nodes": n,
        "max_level": int(level[:n].max()),
    }
