"""SimBVH: per-environment bounding-volume hierarchies over the visual surface
(reference ``FF_SRL/FF_SRL/bvh.py:144-518``).

The build is the reference's host binned-SAH build (``ffsrl_bvh_build_host``, same
topology bit for bit).  The reference stores one topology for all environments and one
AABB set per environment (``bvh.py:190-196, 506-514``); here each distinct mesh gets its
own topology, shared by every environment that uses it, so environments may differ.

``refitBVH`` updates the boxes from the current visual points: by default with one
launch (a block per environment walking its tree bottom-up); ``fused=False`` runs the
reference's one launch per tree level (``refitBVHLoop``, ``bvh.py:419-440``).
"""

from __future__ import annotations

import contextlib
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr


def build_topology(points: np.ndarray, faces: np.ndarray, bins: int = 8) -> dict:
    """Host BVH build of one mesh (points [P,3] float32, faces [F,3] local ids)."""
    points = np.ascontiguousarray(points, dtype=np.float32)
    faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
    F = len(faces)
    cap = 2 * F
    out = {k: np.zeros(cap, dtype=np.int32) for k in ("left_node", "first_tri_id", "tri_count", "level")}
    out["tri_id"] = np.zeros(F, dtype=np.int32)
    out["aabb_min"] = np.zeros((cap, 3), dtype=np.float32)
    out["aabb_max"] = np.zeros((cap, 3), dtype=np.float32)
    nn, ml = C.c_int32(), C.c_int32()
    check(lib().ffsrl_bvh_build_host(points.ctypes.data, faces.ctypes.data, len(points), F, int(bins),
                                     out["left_node"].ctypes.data, out["first_tri_id"].ctypes.data,
                                     out["tri_count"].ctypes.data, out["level"].ctypes.data,
                                     out["tri_id"].ctypes.data, out["aabb_min"].ctypes.data,
                                     out["aabb_max"].ctypes.data, C.byref(nn), C.byref(ml)))
    n = nn.value
    for k in ("left_node", "first_tri_id", "tri_count", "level", "aabb_min", "aabb_max"):
        out[k] = out[k][:n].copy()
    out["num_nodes"], out["max_level"] = n, ml.value
    return out


def reference_refit_source(simModel) -> np.ndarray | None:
    """The face whose box the reference's refit takes for each visual face, or None where
    it takes the face itself everywhere.

    The reference orders the visual faces object by object over all envs (soft meshes,
    then rigid meshes, then instruments; M, Rg and Lf faces per env) and its refit shifts
    an env-local face id to that order testing ``>`` (``bvh.py:66-74``) where the traversal
    tests ``>=`` (``render.py:462-470``).  So env e's local face M (its first rigid or
    instrument face) is boxed from env e+1's face 0, and with both rigids and an
    instrument its local face M + Rg from env e+1's face M; the last env wraps to env 0's
    faces M and M + Rg.  Defined when every env has the same object face counts (the
    reference's only layout) and more than one env."""
    m = simModel
    N, M = m.numEnvs, m.numEnvMeshesVisFaces
    Rg, Lf = m.numEnvRigidsVisFaces, m.numEnvLaparoscopeVisFaces
    if Rg + Lf == 0 or N < 2 or not m.uniformVisLayout:
        return None
    efo = m.envVisFaceStart[:-1].astype(np.int64)
    src = np.arange(int(m.envVisFaceStart[-1]), dtype=np.int64)
    last = np.arange(N) == N - 1
    nxt = np.roll(efo, -1)
    src[efo + M] = np.where(last, efo[0] + M, nxt)
    if Rg > 0 and Lf > 0:
        src[efo + M + Rg] = np.where(last, efo[0] + M + Rg, nxt + M)
    return src.astype(np.int32)


class SimBVH:
    def __init__(self, device, simModel, binsNumber: int = 8, save: bool = False, load: bool = False,
                 path: str = "bvh.npz", referenceRefitShift: bool = True) -> None:
        """``referenceRefitShift``: box the leaves as the reference's refit does at the
        object boundaries (``reference_refit_source``); False boxes every face itself."""
        self.device = torch.device(device)
        self.simModel = simModel
        self.referenceRefitShift = bool(referenceRefitShift)
        self.binsNumber = int(binsNumber)
        self.numEnvs = simModel.numEnvs
        self.refitGraph = None
        if load:
            topos = self.loadBVH(path)
        else:
            topos = self._build()
        self.topologies = topos
        self._assemble()
        if save:
            self.saveBVH(path)
        if self.device.type == "cuda" and simModel.device.type == "cuda":
            # boxes from the current visual points, as the build computed them, and the
            # packed traversal copies that only the refit writes
            self.refitBVH()

    # ------------------------------------------------------------------ build
    def _build(self) -> list[dict]:
        m = self.simModel
        vis = m.allVisPoint.detach().cpu().numpy()
        faces = m.host["allVisFace"].reshape(-1, 3)
        topos = []
        for k in range(len(m.meshes)):
            e = m.envMesh.index(k)  # first env using mesh k
            p0, p1 = int(m.envVisPointStart[e]), int(m.envVisPointStart[e + 1])
            f0, f1 = int(m.envVisFaceStart[e]), int(m.envVisFaceStart[e + 1])
            topos.append(build_topology(vis[p0:p1], faces[f0:f1] - p0, self.binsNumber))
        return topos

    @staticmethod
    def validate(t: dict, num_faces: int) -> None:
        """Checks a topology before it reaches a kernel: child ids in range, leaf
        triangle ranges inside the triangle map, levels consistent."""
        n = t["num_nodes"]
        left, first, cnt, lev = t["left_node"], t["first_tri_id"], t["tri_count"], t["level"]
        if n < 1 or len(left) != n or len(t["tri_id"]) != num_faces:
            raise ValueError("BVH topology: node or triangle count mismatch")
        inner = left != -1
        if np.any(inner & ((left < 1) | (left + 1 >= n))):
            raise ValueError("BVH topology: child id out of range")
        if np.any(inner & ((lev[np.clip(left, 0, n - 1)] != lev + 1) | (lev[np.clip(left + 1, 0, n - 1)] != lev + 1))):
            raise ValueError("BVH topology: child level is not parent level + 1")
        if np.any(~inner & ((first < 0) | (cnt < 0) | (first + cnt > num_faces))):
            raise ValueError("BVH topology: leaf triangle range out of bounds")
        if np.any((t["tri_id"] < 0) | (t["tri_id"] >= num_faces)):
            raise ValueError("BVH topology: triangle id out of range")
        if lev[0] != 0 or np.any(lev < 0) or t["max_level"] != int(lev.max()):
            raise ValueError("BVH topology: bad levels")

    def _assemble(self) -> None:
        m = self.simModel
        topos = self.topologies
        for k, t in enumerate(topos):
            e = m.envMesh.index(k)
            self.validate(t, int(m.envVisFaceStart[e + 1] - m.envVisFaceStart[e]))
        M = len(topos)
        nn = np.array([t["num_nodes"] for t in topos], dtype=np.int64)
        nt = np.array([len(t["tri_id"]) for t in topos], dtype=np.int64)
        z = np.zeros(1, dtype=np.int64)
        topo_node = np.concatenate([z, np.cumsum(nn)]).astype(np.int32)
        topo_tri = np.concatenate([z, np.cumsum(nt)]).astype(np.int32)
        env_topo = np.asarray(m.envMesh, dtype=np.int32)
        env_nodes = nn[env_topo]
        env_node_off = np.concatenate([z, np.cumsum(env_nodes)])[:-1].astype(np.int32)
        # level groups, deepest level first
        level_node, level_start, topo_level_off = [], [], [0]
        base = 0
        for t in topos:
            lv = t["level"]
            order = np.argsort(-lv, kind="stable")
            level_node.append(order.astype(np.int32))
            counts = np.bincount(t["max_level"] - lv, minlength=t["max_level"] + 1)
            level_start.append((base + np.concatenate([[0], np.cumsum(counts)])).astype(np.int32))
            topo_level_off.append(topo_level_off[-1] + t["max_level"] + 2)
            base += t["num_nodes"]
        dev = self.device
        i32 = dict(dtype=torch.int32, device=dev)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), **i32).clone()
        self.leftNode = T(np.concatenate([t["left_node"] for t in topos]))
        self.firstTriId = T(np.concatenate([t["first_tri_id"] for t in topos]))
        self.triCount = T(np.concatenate([t["tri_count"] for t in topos]))
        self.level = T(np.concatenate([t["level"] for t in topos]))
        self.triId = T(np.concatenate([t["tri_id"] for t in topos]))
        self.envTopology = T(env_topo)
        self.envNodeOffset = T(env_node_off)
        self.envFaceOffset = T(m.envVisFaceStart[:-1])
        self.topoNodeOffset = T(topo_node)
        self.topoTriOffset = T(topo_tri)
        self.topoMaxLevel = T([t["max_level"] for t in topos])
        self.levelNode = T(np.concatenate(level_node))
        self.levelStart = T(np.concatenate(level_start))
        self.topoLevelOffset = T(topo_level_off)
        amin = np.concatenate([topos[k]["aabb_min"] for k in env_topo])
        amax = np.concatenate([topos[k]["aabb_max"] for k in env_topo])
        self.aabbMin = torch.as_tensor(amin, dtype=torch.float32, device=dev).clone()
        self.aabbMax = torch.as_tensor(amax, dtype=torch.float32, device=dev).clone()
        # traversal copies the refit writes: packed node boxes and leaf triangles in tri-map order
        self.nodeBox = torch.zeros((len(amin), 8), dtype=torch.float32, device=dev)
        self.triPos = torch.zeros((m.numAllVisFaces, 12), dtype=torch.float32, device=dev)
        self.numNodes = int(nn[0])
        self.numAllNodes = int(env_nodes.sum())
        self.maxLevel = int(max(t["max_level"] for t in topos))
        self.desc = _lib.Bvh()
        d = self.desc
        d.num_envs, d.num_topologies = m.numEnvs, M
        for name, t in (("env_topology", self.envTopology), ("env_node_offset", self.envNodeOffset),
                        ("env_face_offset", self.envFaceOffset), ("topo_node_offset", self.topoNodeOffset),
                        ("topo_tri_offset", self.topoTriOffset), ("topo_max_level", self.topoMaxLevel),
                        ("left_node", self.leftNode), ("first_tri_id", self.firstTriId),
                        ("tri_count", self.triCount), ("level", self.level), ("tri_id", self.triId),
                        ("aabb_min", self.aabbMin), ("aabb_max", self.aabbMax), ("level_node", self.levelNode),
                        ("level_start", self.levelStart), ("topo_level_offset", self.topoLevelOffset),
                        ("node_box", self.nodeBox), ("tri_pos", self.triPos)):
            setattr(d, name, ptr(t))
        d.total_env_nodes = self.numAllNodes
        d.total_topology_nodes = int(nn.sum())
        d.max_level = self.maxLevel
        src = reference_refit_source(m) if self.referenceRefitShift else None
        self.refitSource = None if src is None else T(src)
        d.refit_source = None if src is None else ptr(self.refitSource)

    # ------------------------------------------------------------- npz files
    def saveBVH(self, path: str) -> None:
        """npz as the reference writes it (bvh.py:165-174): arr_0..arr_6 = triId, aabbMin,
        aabbMax, leftNode, firstTriId, triCount, level of the first topology; further
        topologies follow as arr_7.. in groups of seven."""
        arrs = []
        for t in self.topologies:
            arrs += [t["tri_id"], t["aabb_min"], t["aabb_max"], t["left_node"], t["first_tri_id"], t["tri_count"],
                     t["level"]]
        np.savez(path, *arrs)

    def loadBVH(self, path: str) -> list[dict]:
        z = np.load(path)
        n = len(z.files) // 7
        topos = []
        for k in range(n):
            g = [z[f"arr_{7 * k + j}"] for j in range(7)]
            t = {"tri_id": g[0].astype(np.int32), "aabb_min": g[1].astype(np.float32),
                 "aabb_max": g[2].astype(np.float32), "left_node": g[3].astype(np.int32),
                 "first_tri_id": g[4].astype(np.int32), "tri_count": g[5].astype(np.int32),
                 "level": g[6].astype(np.int32)}
            t["num_nodes"] = len(t["aabb_min"])
            t["max_level"] = int(t["level"].max())
            topos.append(t)
        if len(topos) != len(self.simModel.meshes):
            raise ValueError(f"{path} holds {len(topos)} topologies, the model has {len(self.simModel.meshes)} meshes")
        return topos

    # ------------------------------------------------------------------ refit
    def refitBVH(self, useGraph: bool = False, fused: bool = True, stream=None) -> None:
        """Boxes from the current visual points (bvh.py:442-451).  ``useGraph`` captures the
        refit into a CUDA graph on the first call and replays it afterwards, as the
        reference's ``refitGraph``."""
        m = self.simModel
        m.require_cuda()
        if useGraph:
            from .graphs import Graph
            if self.refitGraph is None or self.refitGraph[0] != fused:
                self.refitGraph = (fused, Graph(lambda: self.refitBVH(fused=fused)))
            with torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext():
                self.refitGraph[1]()
            return
        s = _lib.stream_handle(stream)
        fn = lib().ffsrl_bvh_refit_fused if fused else lib().ffsrl_bvh_refit_levels
        check(fn(C.byref(self.desc), ptr(m.allVisPoint), ptr(m.allVisFace), s))
