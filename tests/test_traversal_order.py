"""The fused ray-cast's visiting order keeps the reference's hit (CPU restatement).

The reference traverses the BVH in a fixed pre-order, right child first, prunes a node
whose box entry is not nearer than the best hit so far, and keeps the first of equally
near hits (meshQueryRayManyEnvs, render.py:411-498).  The fused kernel (query_packed in
render.cu) visits the nearer child first, by the ray's sign along the split axis the
refit stores, and keeps equal hits by the reference's pre-order rank.  Its node test forms
the slab distances with a fused multiply-add and falls back to the reference's divisions
when a decision is within rounding of its threshold.

This test restates both traversals in float32 numpy, on a host-built BVH, and checks that
they return the same face and the same distance for rays from cameras outside, close to
and inside a mesh.
"""

import math

import numpy as np

from ffsrl import meshgen as mg
from ffsrl.bvh import build_topology
from ffsrl.render import look_at_rotation

f32 = np.float32
U = 2.0 ** -24


def qrot(q, v):
    u = np.asarray(q[:3], dtype=f32)
    w = f32(q[3])
    c = f32(2) * w * w - f32(1)
    d = f32(2) * (u[0] * v[0] + u[1] * v[1] + u[2] * v[2])
    cr = np.array([u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]], dtype=f32)
    return (v * c + u * d + cr * (w * f32(2))).astype(f32)


def slab(ro, rd, lo, hi):
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = (lo - ro) / rd
        t2 = (hi - ro) / rd

    def fmin(a, b):
        return a if a < b else b

    def fmax(a, b):
        return a if a > b else b

    tmin = fmax(fmax(fmin(t1[0], t2[0]), fmin(t1[1], t2[1])), fmin(t1[2], t2[2]))
    tmax = fmin(fmin(fmax(t1[0], t2[0]), fmax(t1[1], t2[1])), fmax(t1[2], t2[2]))
    return (tmax >= 0 and tmax >= tmin), tmin


def node_hit_fused(ro, rd, inv, roinv, g0, lo, hi, tmin_best):
    with np.errstate(over="ignore", invalid="ignore"):
        tl = (lo.astype(np.float64) * inv - roinv).astype(f32)
        th = (hi.astype(np.float64) * inv - roinv).astype(f32)
    m = f32(np.abs(tl).sum() + np.abs(th).sum())
    if m < 3e37 and g0 < 3e37:
        tmin = max(min(tl[0], th[0]), min(tl[1], th[1]), min(tl[2], th[2]))
        tmax = min(max(tl[0], th[0]), max(tl[1], th[1]), max(tl[2], th[2]))
        g = f32(m * 8 * U + g0)
        if tmax < -g or tmax - tmin < -2 * g or tmin > tmin_best + g:
            return False
        if tmax > g and tmax - tmin > 2 * g and tmin < tmin_best - g:
            return True
    h, tn = slab(ro, rd, lo, hi)
    return h and tn < tmin_best


def moller_trumbore(a, b, c, ro, rd):
    ab, ac = b - a, c - a
    pvec = np.array([rd[1] * ac[2] - rd[2] * ac[1], rd[2] * ac[0] - rd[0] * ac[2], rd[0] * ac[1] - rd[1] * ac[0]],
                    dtype=f32)
    det = f32(ab[0] * pvec[0] + ab[1] * pvec[1]) + ab[2] * pvec[2]
    if abs(det) < 1e-4:
        return -1.0
    inv = f32(1) / det
    tv = ro - a
    u = (f32(tv[0] * pvec[0] + tv[1] * pvec[1]) + tv[2] * pvec[2]) * inv
    if u < 0 or u > 1:
        return -1.0
    q = np.array([tv[1] * ab[2] - tv[2] * ab[1], tv[2] * ab[0] - tv[0] * ab[2], tv[0] * ab[1] - tv[1] * ab[0]],
                 dtype=f32)
    v = (f32(rd[0] * q[0] + rd[1] * q[1]) + rd[2] * q[2]) * inv
    if v < 0 or u + v > 1:
        return -1.0
    return float((f32(ac[0] * q[0] + ac[1] * q[1]) + ac[2] * q[2]) * inv)


def reference_query(T, tri, ro, rd):
    left, first, cnt, lo, hi = T["left_node"], T["first_tri_id"], T["tri_count"], T["aabb_min"], T["aabb_max"]
    stack, t_best, best = [0], 1e6, -1
    while stack:
        n = stack.pop()
        h, tn = slab(ro, rd, lo[n], hi[n])
        if h and tn < t_best:
            if left[n] == -1:
                for k in range(cnt[n]):
                    f = T["tri_id"][first[n] + k]
                    t = moller_trumbore(*tri[f], ro, rd)
                    if 0 < t < t_best:
                        t_best, best = t, f
            else:
                stack.append(left[n])
                stack.append(left[n] + 1)  # the right child is popped first
    return (best, t_best) if t_best < 1e6 else (-1, 1e6)


def fused_query(T, tri, ro, rd):
    left, first, cnt, lo, hi = T["left_node"], T["first_tri_id"], T["tri_count"], T["aabb_min"], T["aabb_max"]
    inv = (f32(1) / rd).astype(np.float64)
    roinv = (ro * inv.astype(f32)).astype(f32).astype(np.float64)
    g0 = f32(4 * U * np.abs(roinv).sum())
    stack, t_best, best, bf, bk = [0], 1e6, -1, -1, 0
    while stack:
        n = stack.pop()
        if not node_hit_fused(ro, rd, inv, roinv, g0, lo[n], hi[n], t_best):
            continue
        if left[n] == -1:
            fi = first[n]
            for k in range(cnt[n]):
                f = T["tri_id"][fi + k]
                t = moller_trumbore(*tri[f], ro, rd)
                if t > 0 and (t < t_best or (t == t_best and best >= 0 and (fi > bf or (fi == bf and k < bk)))):
                    t_best, best, bf, bk = t, f, fi, k
        else:
            l = left[n]
            # the refit's split code: the axis along which the children's centres lie
            # farthest apart, and whether the right child's centre is the higher one
            d = (lo[l + 1] + hi[l + 1]) - (lo[l] + hi[l])
            ad = np.abs(d)
            axis = 0 if (ad[0] >= ad[1] and ad[0] >= ad[2]) else (1 if ad[1] >= ad[2] else 2)
            left_near = (rd[axis] > 0) == (d[axis] > 0)
            stack.append(l + 1 if left_near else l)
            stack.append(l if left_near else l + 1)
    return (best, t_best) if t_best < 1e6 else (-1, 1e6)


def test_nearer_child_first_keeps_the_reference_hit():
    mesh = mg.ellipsoid_for_tets(600, seed=4)
    pts = mesh["vertex"].astype(f32)
    faces = np.asarray(mesh["triangle"]).reshape(-1, 3)
    T = build_topology(pts, faces)
    tri = [(pts[a], pts[b], pts[c]) for a, b, c in faces]
    rng = np.random.default_rng(5)
    c = pts.mean(axis=0).astype(np.float64)
    rad = float(np.linalg.norm(pts - c, axis=1).max())
    tan = f32(math.tan(math.radians(30)))
    total = hits = 0
    for dist in (2.5, 1.1, 0.4):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        p = (c + d * dist * rad).astype(f32)
        q = np.asarray(look_at_rotation(p, c), dtype=f32)
        W = 20
        for y in range(1, W + 1):
            for x in range(W):
                sx = f32(2) * f32(x) / f32(W) - f32(1)
                sy = f32(2) * f32(y) / f32(W) - f32(1)
                v = qrot(q, np.array([sx * tan, sy * tan, -1], dtype=f32))
                rd = (v / f32(math.sqrt(float(v @ v)))).astype(f32)
                ref = reference_query(T, tri, p, rd)
                got = fused_query(T, tri, p, rd)
                assert got == ref, (dist, x, y, ref, got)
                total += 1
                hits += ref[0] >= 0
    print(f"[traversal] {total} rays, {hits} hits, the same face and distance in both orders")
    assert hits > total // 4
