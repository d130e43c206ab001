"""SimModelDO: the multi-environment state arrays (reference ``FF_SRL/FF_SRL/modelDO.py:772-1645``).

Every quantity is one flat array over all environments, in the reference's layout
(``modelDO.py:1141-1246``): vec3 arrays are float32 ``[n, 3]``, index arrays int32 holding
global ids.  The arrays are torch tensors on the model's device, so RL code reads them
without copies (the reference's ``wp.to_torch`` getters, ``modelDO.py:1483-1518``).

The reference builds the arrays from a USD stage (``modelDO.py:774-1266``).  USD cannot be
read here; ``stage`` is instead an array-based scene: one mesh dict (as produced by
``ffsrl.meshgen``) replicated over ``numEnvs`` environments, as the reference does, or a
list of ``numEnvs`` mesh dicts for environments with different meshes.
"""

from __future__ import annotations

import contextlib

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr

_MESH_KEYS = ("vertex", "inverse_mass", "tetrahedron", "tetrahedron_rest_volume", "edge", "edge_rest_length",
              "triangle", "vis_face", "point_to_vertex", "vis_point_color")


def _cat(parts, dtype):
    if not parts:
        return np.zeros(0, dtype=dtype)
    return np.ascontiguousarray(np.concatenate(parts), dtype=dtype)


class SimModelDO:
    """Multi-environment soft-body model.

    Keyword arguments and their defaults are the reference's (``modelDO.py:774-802``);
    the instrument-kinematics ones (workspace boxes) are accepted and stored.  Added:

    * ``constraints``: ffsrl flag set of constraint kernels run per iteration (default:
      the reference DO step's volume, distance, drag, connectors and contact);
    * ``distanceCompliance`` / ``volumeComplianceXPBD``: XPBD alphas for the compliant
      variants (``integrator.py:191-240, 507-576``);
    * ``toolRadius``: capsule radii of the synthetic instrument (rod, clamps);
    * ``instrumentMesh``: the instrument's visual mesh, shared by every env (the reference
      reads it from USD or generates capsules, ``laparoscope.py:388-496``): ``points`` [Lp, 3]
      in the frames of their transform slots, ``faces`` [Lf, 3], ``slot`` [Lp] (6 rod, 4/5
      clamp pivots, ``modelDO.py:1031-1033``) and ``color`` [Lp, 3]
      (``meshgen.instrument_mesh`` builds one).  Its points follow the transforms
      (``transformSimLaparoscopeMeshData``) and it is rendered with the env.

    A mesh dict may list static rigid meshes under ``"rigids"`` (``vertex`` [Q, 3],
    ``triangle`` [G, 3], optional ``color`` and texture keys): visual-only objects of the
    env, as the reference's ``SimRigidDO`` (``modelDO.py:642-770, 996-1008``).
    """

    def __init__(self, stage, numEnvs, device="cuda:0",
                 simSubsteps=8, simFrameRate=60, simConstraintsSteps=1,
                 environmentGravity=(0.0, -9.8, 0.0), environmentVelocityDampening=0.1, environmentGroundLevel=0.0,
                 globalKsDistance=1.0, globalKsVolume=1.0, globalKsContact=1.0, globalKsDrag=1.0,
                 globalVolumeCompliance=1.0, globalDeviatoricCompliance=1.0,
                 globalBreakFactor=1.0, globalBreakThreshold=1.0, globalHeatLoss=1.0, globalHeatConduction=1.0,
                 globalHeatTransfer=1.0, globalHeatLimit=1.0, globalHeatSphereRadius=1.0, globalHeatQuantum=1.0,
                 globalLaparoscopeDragLookupRadius=0.15, globalConnectorMassWeightRatio=0.75, globalConnectorKs=0.125,
                 globalConnectorRestLengthMul=0.02,
                 workspaceLow=(-1e5, -1e5, -1e5), workspaceHigh=(1e5, 1e5, 1e5),
                 startingBoxLow=(-1e5, -1e5, -1e5), startingBoxHigh=(1e5, 1e5, 1e5),
                 constraints=None, distanceCompliance=0.0, volumeComplianceXPBD=0.0,
                 toolRadius=(0.004, 0.002, 0.002), instrumentMesh=None):
        if hasattr(stage, "GetPrimAtPath"):
            raise _lib.FFSRLError(_lib.ERR_UNSUPPORTED,
                                  "USD stages are not supported; pass ffsrl.meshgen mesh dicts or an array scene file")
        scenes = self._load_scenes(stage, int(numEnvs))
        if scenes is not None:
            stage = [sc_.mesh for sc_ in scenes]
            if instrumentMesh is None:
                ims = [sc_.instrument["mesh"] for sc_ in scenes if sc_.instrument and "mesh" in sc_.instrument]
                instrumentMesh = ims[0] if ims else None
        meshes = stage if isinstance(stage, (list, tuple)) else [stage] * int(numEnvs)
        if len(meshes) != int(numEnvs):
            raise ValueError(f"got {len(meshes)} meshes for {numEnvs} environments")
        self.device = torch.device(device)
        self.numEnvs = int(numEnvs)
        self.cartesianActions = 3
        self.simSubsteps = int(simSubsteps)
        self.simFrameRate = simFrameRate
        self.simConstraints = int(simConstraintsSteps)
        self.simDt = (1.0 / self.simFrameRate) / self.simSubsteps
        self.gravity = tuple(float(g) for g in environmentGravity)
        self.velocityDampening = float(environmentVelocityDampening)
        self.groundLevel = float(environmentGroundLevel)
        self.globalKsDistance = float(globalKsDistance)
        self.globalDistanceCompliance = globalKsDistance / (self.simDt * self.simDt)
        self.globalKsVolume = float(globalKsVolume)
        self.globalVolumeCompliance = globalKsVolume / (self.simDt * self.simDt)
        self.globalKsContact = float(globalKsContact)
        self.globalKsDrag = float(globalKsDrag)
        self.globalVolumeComplianceNeoHookean = float(globalVolumeCompliance)
        self.gloabalDeviatoricComplianceNeoHookean = float(globalDeviatoricCompliance)
        self.globalLaparoscopeDragLookupRadius = float(globalLaparoscopeDragLookupRadius)
        self.globalBreakFactor, self.globalBreakThreshold = globalBreakFactor, globalBreakThreshold
        self.globalHeatLoss, self.globalHeatConduction = globalHeatLoss, globalHeatConduction
        self.globalHeatTransfer, self.globalHeatLimit = globalHeatTransfer, globalHeatLimit
        self.globalHeatSphereRadius, self.globalHeatQuantum = globalHeatSphereRadius, globalHeatQuantum
        self.globalConnectorMassWeightRatio = float(globalConnectorMassWeightRatio)
        self.globalConnectorKs = float(globalConnectorKs)
        self.globalConnectorRestLengthMul = float(globalConnectorRestLengthMul)
        self.workspaceLow, self.workspaceHigh = tuple(workspaceLow), tuple(workspaceHigh)
        self.startingBoxLow, self.startingBoxHigh = tuple(startingBoxLow), tuple(startingBoxHigh)
        self.constraintFlags = _lib.REFERENCE_STEP if constraints is None else int(constraints)
        self.distanceComplianceXPBD = float(distanceCompliance)
        self.volumeComplianceXPBD = float(volumeComplianceXPBD)
        self.reduce = False

        self.instrumentMesh = self._check_instrument_mesh(instrumentMesh)

        # distinct meshes (topologies) and the env -> mesh map
        uniq, self.envMesh = [], []
        for m in meshes:
            for k, u in enumerate(uniq):
                if u is m:
                    self.envMesh.append(k)
                    break
            else:
                uniq.append(m)
                self.envMesh.append(len(uniq) - 1)
        self.meshes = uniq
        self._concatenate(meshes, toolRadius)
        self._upload()
        self._batch = None
        # bumped by calls that change active values or holes (cutting, heating): the
        # batched step's plan packs those and is rebuilt when this changes
        self.topologyVersion = 0
        if scenes is not None and all(sc_.instrument is not None for sc_ in scenes):
            ins = [sc_.instrument for sc_ in scenes]
            base = np.concatenate([i["bases"] for i in ins]).astype(np.float32)
            tip = np.concatenate([i["tips"] for i in ins]).astype(np.float32)
            rad = np.concatenate([i["radii"] for i in ins]).astype(np.float32)
            xf = np.stack([i["transforms"].reshape(-1) for i in ins]).astype(np.float32)
            hts = np.stack([i["heights"] for i in ins]).astype(np.float32)
            self.setTool(base, tip, rad)
            self.setInstrument(xf, hts)
            self.toolHost = {"base": base, "tip": tip, "radius": rad, "xform": xf, "height": hts}
            self.setEffectorInitialPosition()

    @staticmethod
    def _load_scenes(stage, numEnvs):
        """Array scene files (``ffsrl.scene``) for ``stage`` given as a path or a per-env list
        holding paths; None when the stage is mesh dicts only.  A file shared by several
        envs is read once, so they share its mesh."""
        from . import scene as scene_io
        items = [stage] * numEnvs if scene_io.is_scene_path(stage) else stage
        if not isinstance(items, (list, tuple)) or not any(scene_io.is_scene_path(it) for it in items):
            return None
        cache, out = {}, []
        for it in items:
            if scene_io.is_scene_path(it):
                key = str(it)
                if key not in cache:
                    cache[key] = scene_io.read_scene(key)
                out.append(cache[key])
            else:
                out.append(scene_io.Scene(mesh=it))
        return out

    # ------------------------------------------------------------------ build
    @staticmethod
    def _check_instrument_mesh(im):
        if im is None:
            return None
        out = dict(im)
        out["points"] = np.ascontiguousarray(np.asarray(im["points"], dtype=np.float32).reshape(-1, 3))
        out["faces"] = np.ascontiguousarray(np.asarray(im["faces"], dtype=np.int32).reshape(-1, 3))
        out["slot"] = np.ascontiguousarray(np.asarray(im["slot"], dtype=np.int32).reshape(-1))
        Lp = len(out["points"])
        out["color"] = np.ascontiguousarray(np.asarray(im.get("color", np.full((Lp, 3), 0.6)),
                                                       dtype=np.float32).reshape(-1, 3))
        if len(out["slot"]) != Lp or len(out["color"]) != Lp:
            raise ValueError("instrumentMesh: slot and color need one entry per point")
        if Lp and (out["slot"].min() < 0 or out["slot"].max() > 6):
            raise ValueError("instrumentMesh: slots are 0..6")
        if len(out["faces"]) and (out["faces"].min() < 0 or out["faces"].max() >= Lp):
            raise ValueError("instrumentMesh: face index out of range")
        return out

    def _concatenate(self, meshes, toolRadius):
        """Concatenate the envs' arrays.  Each env's visual points and faces are its objects'
        one after another -- the soft mesh's (``vis_face`` over its surface points), the
        static rigid meshes' (``mesh["rigids"]``) and the instrument's visual mesh
        (``instrumentMesh``) -- so an env's local face ids are the reference's
        (``modelDO.py:1231-1246, 1279-1326``); envs follow one another (env-major)."""
        N = self.numEnvs
        nv = np.array([len(m["vertex"]) for m in meshes], dtype=np.int64)
        nt = np.array([len(m["tetrahedron"]) for m in meshes], dtype=np.int64)
        ne = np.array([len(m["edge"]) for m in meshes], dtype=np.int64)
        nf = np.array([len(m["triangle"]) for m in meshes], dtype=np.int64)
        npnt = np.array([len(m["point_to_vertex"]) for m in meshes], dtype=np.int64)
        nvf = np.array([len(m["vis_face"]) for m in meshes], dtype=np.int64)
        rigids = [list(m.get("rigids", ())) for m in meshes]
        for rs in rigids:
            for r in rs:
                q = np.asarray(r["vertex"]).reshape(-1, 3)
                g = np.asarray(r["triangle"]).reshape(-1, 3)
                if len(g) and (g.min() < 0 or g.max() >= len(q)):
                    raise ValueError("rigid mesh: triangle index out of range")
        nq = np.array([sum(len(np.asarray(r["vertex"]).reshape(-1, 3)) for r in rs) for rs in rigids], dtype=np.int64)
        ng = np.array([sum(len(np.asarray(r["triangle"]).reshape(-1, 3)) for r in rs) for rs in rigids],
                      dtype=np.int64)
        inst = self.instrumentMesh
        Lp = len(inst["points"]) if inst is not None else 0
        Lf = len(inst["faces"]) if inst is not None else 0
        z = np.zeros(1, dtype=np.int64)
        if int(nv.sum()) >= 2**31 or 4 * int(nt.sum()) >= 2**31 or 3 * int(nf.sum()) >= 2**31 or \
                3 * int((nvf + ng).sum() + N * Lf) >= 2**31:
            raise ValueError("model exceeds int32 indexing")
        self.envVertexStart = np.concatenate([z, np.cumsum(nv)]).astype(np.int32)
        self.envTetStart = np.concatenate([z, np.cumsum(nt)]).astype(np.int32)
        self.envEdgeStart = np.concatenate([z, np.cumsum(ne)]).astype(np.int32)
        self.envTriStart = np.concatenate([z, np.cumsum(nf)]).astype(np.int32)
        self.envVisPointStart = np.concatenate([z, np.cumsum(npnt + nq + Lp)]).astype(np.int32)
        self.envVisFaceStart = np.concatenate([z, np.cumsum(nvf + ng + Lf)]).astype(np.int32)
        # remap pairs: the soft mesh's points only, env after env
        self.envMapStart = np.concatenate([z, np.cumsum(npnt)]).astype(np.int32)
        vo, po = self.envVertexStart[:-1].astype(np.int64), self.envVisPointStart[:-1].astype(np.int64)
        self.envInstrumentPointStart = (po + npnt + nq).astype(np.int32)
        h = {}
        h["vertex"] = _cat([m["vertex"] for m in meshes], np.float32).reshape(-1, 3)
        h["inverseMass"] = _cat([m["inverse_mass"] for m in meshes], np.float32)
        h["tetrahedron"] = _cat([m["tetrahedron"].reshape(-1) + vo[e] for e, m in enumerate(meshes)], np.int32)
        h["tetrahedronRestVolume"] = _cat([m["tetrahedron_rest_volume"] for m in meshes], np.float32)
        h["tetrahedronRestVolumeSigned"] = _cat(
            [m.get("tetrahedron_rest_volume_signed", -m["tetrahedron_rest_volume"]) for m in meshes], np.float32)
        h["tetrahedronDmInv"] = _cat([m["tetrahedron_dm_inv"].reshape(-1) for m in meshes], np.float32)
        h["edge"] = _cat([m["edge"].reshape(-1) + vo[e] for e, m in enumerate(meshes)], np.int32)
        h["edgeRestLength"] = _cat([m["edge_rest_length"] for m in meshes], np.float32)
        h["triangle"] = _cat([m["triangle"].reshape(-1) + vo[e] for e, m in enumerate(meshes)], np.int32)
        h["triToEnv"] = np.repeat(np.arange(N, dtype=np.int32), nf)
        h["vertexToEnv"] = np.repeat(np.arange(N, dtype=np.int32), nv)
        faces, colors, static = [], [], []
        grey = np.array([0.6, 0.6, 0.6], dtype=np.float32)
        for e, m in enumerate(meshes):
            faces.append(np.asarray(m["vis_face"]).reshape(-1) + po[e])
            colors.append(np.asarray(m["vis_point_color"], dtype=np.float32).reshape(-1, 3))
            off = po[e] + npnt[e]
            for r in rigids[e]:
                q = np.asarray(r["vertex"], dtype=np.float32).reshape(-1, 3)
                faces.append(np.asarray(r["triangle"]).reshape(-1) + off)
                colors.append(np.asarray(r.get("color", np.broadcast_to(grey, q.shape)), dtype=np.float32).reshape(-1, 3))
                static.append((off, q))
                off += len(q)
            if inst is not None:
                faces.append(np.asarray(inst["faces"]).reshape(-1) + off)
                colors.append(np.asarray(inst["color"], dtype=np.float32).reshape(-1, 3))
        h["allVisFace"] = _cat(faces, np.int32)
        h["allVisPointColor"] = _cat(colors, np.float32).reshape(-1, 3)
        self._staticVisPoints = static
        ptv = []
        for e, m in enumerate(meshes):
            pv = m["point_to_vertex"].astype(np.int64).copy()
            pv[:, 0] += po[e]
            pv[:, 1] += vo[e]
            ptv.append(pv.reshape(-1))
        h["pointToVertex"] = _cat(ptv, np.int32)
        # grasp candidates: the surface (visual) vertices of each env's soft mesh
        self.graspCandStart = self.envMapStart.copy()
        h["graspCand"] = h["pointToVertex"][1::2].copy()
        self._concatenate_connectors(h, meshes, nv, vo)
        self._concatenate_textures(h, rigids, nvf, ng, Lf)
        self.host = h

        self.numVertices = int(self.envVertexStart[-1])
        self.numTetrahedrons = int(self.envTetStart[-1])
        self.numEdges = int(self.envEdgeStart[-1])
        self.numTriangles = int(self.envTriStart[-1])
        self.numVisPoints = int(self.envMapStart[-1])         # soft-mesh visual points (remapped)
        self.numAllVisPoints = int(self.envVisPointStart[-1])
        self.numVisFaces = int(nvf.sum())
        self.numAllVisFaces = int(self.envVisFaceStart[-1])
        self.numRigidVisPoints, self.numRigidVisFaces = int(nq.sum()), int(ng.sum())
        self.numLaparoscopeVisPoints, self.numLaparoscopeVisFaces = N * Lp, N * Lf
        self.simConnectors = int(len(h["connectorVertexId"]))
        # per-env sizes (the reference assumes identical envs; these hold env 0's)
        self.environmentNumVertices = int(nv[0])
        self.numEnvAllVertices = int(nv[0])
        self.numEnvMeshesVisPoints = int(npnt[0])
        self.numEnvMeshesVisFaces = int(nvf[0])
        self.numEnvRigidsVisPoints = int(nq[0])
        self.numEnvRigidsVisFaces = int(ng[0])
        self.numEnvLaparoscopeVisPoints = Lp
        self.numEnvLaparoscopeVisFaces = Lf
        self.numEnvAllVisFaces = int(nvf[0] + ng[0] + Lf)
        # all envs alike in their object face counts: the reference's layout assumption
        self.uniformVisLayout = bool(np.all(nvf == nvf[0]) and np.all(ng == ng[0]))

        # synthetic instrument: 3 capsules + drag point per env, parked far above the
        # scene (out of reach of any mesh until a caller places it)
        r = np.asarray(toolRadius, dtype=np.float32)
        base = np.zeros((4 * N, 3), dtype=np.float32)
        tip = np.zeros((4 * N, 3), dtype=np.float32)
        tip[:, 1] = 1000.0
        base[:, 1] = 1000.1
        rad = np.tile(np.array([r[0], r[1], r[2], 0.0], dtype=np.float32), N)
        self.toolHost = {"base": base, "tip": tip, "radius": rad}

    @staticmethod
    def _concatenate_connectors(h, meshes, nv, vo):
        """Connectors (``SimConnectorDO``, ``modelDO.py:723-770, 977-1015``): a point of one body
        held at a rest distance from a barycentric point of a triangle of another body of
        the same env.  A mesh dict lists them in its own vertex ids: ``connector_vertex_id``
        [C], ``connector_triangle_id`` [C, 3], ``connector_tri_bar`` [C, 3],
        ``connector_rest_dist`` [C]; here they become global ids, env after env."""
        cv, ct, cb, cr = [], [], [], []
        for e, m in enumerate(meshes):
            if m.get("connector_vertex_id") is None:
                continue
            v = np.asarray(m["connector_vertex_id"], dtype=np.int64).reshape(-1)
            t = np.asarray(m["connector_triangle_id"], dtype=np.int64).reshape(-1, 3)
            b = np.asarray(m["connector_tri_bar"], dtype=np.float32).reshape(-1, 3)
            r = np.asarray(m["connector_rest_dist"], dtype=np.float32).reshape(-1)
            if not (len(v) == len(t) == len(b) == len(r)):
                raise ValueError("connectors: vertex ids, triangles, barycentrics and rest distances differ in count")
            if len(v) and (min(v.min(), t.min()) < 0 or max(v.max(), t.max()) >= nv[e]):
                raise ValueError("connectors: vertex id out of range")
            cv.append(v + vo[e])
            ct.append((t + vo[e]).reshape(-1))
            cb.append(b)
            cr.append(r)
        h["connectorVertexId"] = _cat(cv, np.int32)
        h["connectorTriangleId"] = _cat(ct, np.int32)
        h["connectorTriBar"] = _cat(cb, np.float32).reshape(-1, 3)
        h["connectorRestDist"] = _cat(cr, np.float32)

    @staticmethod
    def _texture_entry(obj, num_faces, tables):
        """Append one object's texture (modelDO.py:1056-1125) to ``tables`` once (objects are
        deduplicated by identity) and return (first texel, S, first tex coord, first tex
        index), or zeros for an object without ``texture``."""
        if obj is None or obj.get("texture") is None:
            return (0, 0, 0, 0)
        for o, ent in tables["seen"]:
            if o is obj:
                return ent
        t = np.asarray(obj["texture"], dtype=np.float32)
        if t.ndim != 3 or t.shape[0] != t.shape[1] or t.shape[2] != 3 or t.shape[0] < 1:
            raise ValueError("texture must be a square [S, S, 3] array")
        c = np.asarray(obj["tex_coords"], dtype=np.float32).reshape(-1, 2)
        default = obj.get("vis_face", obj.get("triangle", obj.get("faces")))
        i = np.asarray(obj.get("tex_indices", default), dtype=np.int64).reshape(-1)
        if len(i) != 3 * num_faces or (len(i) and (i.min() < 0 or i.max() >= len(c))):
            raise ValueError("tex_indices must hold 3 tex-coord ids per visual face")
        S = t.shape[0]
        ent = (tables["nt"], S, tables["nc"], tables["ni"])
        tables["tex"].append(t.reshape(-1))
        tables["coords"].append(c.reshape(-1))
        tables["idx"].append(i)
        tables["nt"] += S * S
        tables["nc"] += len(c)
        tables["ni"] += len(i)
        tables["seen"].append((obj, ent))
        return ent

    def _concatenate_textures(self, h, rigids, nvf, ng, Lf):
        """Object and texture tables of the renderer's texture mode.  Per env, its objects
        in face order -- soft mesh, rigids, instrument -- each as (first env-local face, first
        texel, S, first tex coord, first tex index); S = 0 for an object without a texture
        (rendered with its vertex colours).  A texture is ``texture`` [S, S, 3] in [0, 1],
        ``tex_coords`` [T, 2] and ``tex_indices`` (3 per face, default the faces themselves,
        as modelDO.py:636-640)."""
        tables = {"tex": [], "coords": [], "idx": [], "nt": 0, "nc": 0, "ni": 0, "seen": []}
        objects, env_objects, per_mesh = [], [], {}
        inst = self.instrumentMesh
        for e, k in enumerate(self.envMesh):
            if k not in per_mesh:
                m = self.meshes[k]
                ents = [(0,) + self._texture_entry(m, len(m["vis_face"]), tables)]
                f0 = int(nvf[e])
                for r in rigids[e]:
                    g = len(np.asarray(r["triangle"]).reshape(-1, 3))
                    ents.append((f0,) + self._texture_entry(r, g, tables))
                    f0 += g
                if inst is not None:
                    ents.append((f0,) + self._texture_entry(inst, Lf, tables))
                per_mesh[k] = (len(objects), len(ents))
                objects += ents
            env_objects.append(per_mesh[k])
        self.hasTextures = bool(tables["tex"])
        if tables["nt"] >= 2**31 or tables["ni"] >= 2**31:
            raise ValueError("textures exceed int32 indexing")
        h["texture"] = _cat(tables["tex"], np.float32)
        h["texCoords"] = _cat(tables["coords"], np.float32)
        h["texIndices"] = _cat(tables["idx"], np.int32)
        h["objectTexture"] = np.asarray(objects, dtype=np.int32).reshape(-1)
        h["envObjects"] = np.asarray(env_objects, dtype=np.int32).reshape(-1)

    def _upload(self):
        d = self.device
        h = self.host
        f32 = dict(dtype=torch.float32, device=d)
        i32 = dict(dtype=torch.int32, device=d)

        def T(a, **kw):
            return torch.as_tensor(np.ascontiguousarray(a), **kw).clone()

        self.vertex = T(h["vertex"], **f32)
        self.initialVertex = self.vertex.clone()
        self.predictedVertex = torch.zeros_like(self.vertex)
        self.velocity = torch.zeros_like(self.vertex)
        self.initialVelocity = torch.zeros_like(self.vertex)
        self.dP = torch.zeros_like(self.vertex)
        self.collisionDP = torch.zeros_like(self.vertex)
        self.constraintsNumber = torch.zeros(self.numVertices, **i32)
        self.inverseMass = T(h["inverseMass"], **f32)
        self.tetrahedron = T(h["tetrahedron"], **i32)
        self.tetrahedronRestVolume = T(h["tetrahedronRestVolume"], **f32)
        self.tetrahedronRestVolumeSigned = T(h["tetrahedronRestVolumeSigned"], **f32)
        self.activeTetrahedron = torch.ones(self.numTetrahedrons, **f32)
        self.tetrahedronDmInv = T(h["tetrahedronDmInv"], **f32)
        self.tetrahedronLambda = torch.zeros(self.numTetrahedrons, **f32)
        self.edge = T(h["edge"], **i32)
        self.edgeRestLength = T(h["edgeRestLength"], **f32)
        self.activeEdge = torch.ones(self.numEdges, **f32)
        self.edgeLambda = torch.zeros(self.numEdges, **f32)
        self.triangle = T(h["triangle"], **i32)
        self.hole = torch.zeros(self.numTriangles, **i32)
        self.triToEnv = T(h["triToEnv"], **i32)
        self.vertexToEnv = T(h["vertexToEnv"], **i32)
        self.activeDragConstraint = torch.zeros(self.numVertices, **f32)
        ptv = h["pointToVertex"].reshape(-1, 2)
        vis0 = np.zeros((self.numAllVisPoints, 3), dtype=np.float32)
        vis0[ptv[:, 0]] = h["vertex"][ptv[:, 1]]
        for off, q in self._staticVisPoints:  # rigid meshes: visual points that never move
            vis0[off:off + len(q)] = q
        inst = self.instrumentMesh
        if inst is not None:  # local shape until the instrument's transforms are set
            for e in range(self.numEnvs):
                o = int(self.envInstrumentPointStart[e])
                vis0[o:o + len(inst["points"])] = inst["points"]
        self.allVisPoint = T(vis0, **f32)
        self.visPoint = self.allVisPoint
        self.allVisFace = T(h["allVisFace"], **i32)
        self.visFace = self.allVisFace
        self.allVisPointColor = T(h["allVisPointColor"], **f32)
        self.textureT = T(h["texture"], **f32)
        self.texCoordsT = T(h["texCoords"], **f32)
        self.texIndicesT = T(h["texIndices"], **i32)
        self.objectTextureT = T(h["objectTexture"], **i32)
        self.envObjectsT = T(h["envObjects"], **i32)
        self.envMapStartT = T(self.envMapStart, **i32)
        self.envInstrumentPointStartT = T(self.envInstrumentPointStart, **i32)
        # the instrument's visual mesh: local points and their transform slots (the
        # reference's laparoscopeVertex / laparoscopeVertexToXForm, modelDO.py:1217-1221)
        self.laparoscopeVertex = T(inst["points"] if inst is not None else np.zeros((0, 3), np.float32), **f32)
        self.laparoscopeVertexToXForm = T(inst["slot"] if inst is not None else np.zeros(0, np.int32), **i32)
        self.pointToVertex = T(h["pointToVertex"], **i32)
        self.graspCand = T(h["graspCand"], **i32)
        self.graspCandStartT = T(self.graspCandStart, **i32)
        self.laparoscopeBase = T(self.toolHost["base"], **f32)
        self.laparoscopeTip = T(self.toolHost["tip"], **f32)
        self.laparoscopeRadius = T(self.toolHost["radius"], **f32)
        self.laparoscopeInitialBase = self.laparoscopeBase.clone()
        self.laparoscopeInitialTip = self.laparoscopeTip.clone()
        self.laparoscopeInCollision = torch.zeros(self.numEnvs, **i32)
        self.laparoscopeDragCutHeat = torch.zeros(3 * self.numEnvs, **i32)
        self.laparoscopeDragCutHeatUpdate = torch.zeros(3 * self.numEnvs, **i32)
        # instrument kinematics (setInstrument): 7 transforms per env in the reference's
        # storage (row-major transposes), capsule heights, workspace violation flags
        self.laparoscopeXForm = torch.zeros(112 * self.numEnvs, **f32)
        self.laparoscopeInitialXForm = torch.zeros(112 * self.numEnvs, **f32)
        self.laparoscopeHeight = torch.zeros(4 * self.numEnvs, **f32)
        self.laparoscopeWorkspaceViolation = torch.zeros(self.numEnvs, **i32)
        self.hasInstrumentKinematics = False
        self.envStatus = torch.zeros(self.numEnvs, **i32)
        self.envVertexStartT = T(self.envVertexStart, **i32)
        self.envTetStartT = T(self.envTetStart, **i32)
        self.envEdgeStartT = T(self.envEdgeStart, **i32)
        self.envTriStartT = T(self.envTriStart, **i32)
        self.envVisPointStartT = T(self.envVisPointStart, **i32)
        self.connectorVertexId = T(h["connectorVertexId"], **i32)
        self.connectorTriangleId = T(h["connectorTriangleId"], **i32)
        self.connectorTriBar = T(h["connectorTriBar"], **f32)
        self.connectorRestDist = T(h["connectorRestDist"], **f32)

    # ------------------------------------------------------------ descriptors
    def require_cuda(self) -> None:
        """Every GPU entry point checks this: a host pointer given to a kernel would fault."""
        if self.device.type != "cuda":
            raise _lib.FFSRLError(_lib.ERR_INVALID_ARGUMENT,
                                  f"model arrays live on {self.device}; GPU entry points need a CUDA device")

    def params(self) -> _lib.Params:
        p = _lib.Params()
        p.substeps, p.iterations, p.flags = self.simSubsteps, self.simConstraints, self.constraintFlags
        p.dt = self.simDt
        p.gravity[:] = self.gravity
        p.velocity_dampening, p.ground_level = self.velocityDampening, self.groundLevel
        p.ks_distance, p.ks_volume = self.globalKsDistance, self.globalKsVolume
        p.ks_contact, p.ks_drag = self.globalKsContact, self.globalKsDrag
        p.volume_compliance = self.globalVolumeComplianceNeoHookean
        p.deviatoric_compliance = self.gloabalDeviatoricComplianceNeoHookean
        p.distance_compliance, p.volume_compliance_xpbd = self.distanceComplianceXPBD, self.volumeComplianceXPBD
        p.connector_mass_weight_ratio = self.globalConnectorMassWeightRatio
        p.connector_ks, p.connector_rest_length_mul = self.globalConnectorKs, self.globalConnectorRestLengthMul
        return p

    def _fill(self, m: _lib.Model, src: dict) -> _lib.Model:
        m.num_vertices, m.num_tetrahedrons = self.numVertices, self.numTetrahedrons
        m.num_edges, m.num_triangles = self.numEdges, self.numTriangles
        m.num_connectors, m.num_envs = self.simConnectors, self.numEnvs
        for k, v in src.items():
            setattr(m, k, ptr(v))
        return m

    def device_model(self) -> _lib.Model:
        self.require_cuda()
        return self._fill(_lib.Model(), {
            "vertex": self.vertex, "predicted_vertex": self.predictedVertex, "velocity": self.velocity,
            "dp": self.dP, "constraints_number": self.constraintsNumber, "collision_dp": self.collisionDP,
            "inverse_mass": self.inverseMass, "tetrahedron": self.tetrahedron,
            "tetrahedron_rest_volume": self.tetrahedronRestVolume, "active_tetrahedron": self.activeTetrahedron,
            "tetrahedron_dm_inv": self.tetrahedronDmInv, "tetrahedron_lambda": self.tetrahedronLambda,
            "xpbd_rest_volume": self.tetrahedronRestVolumeSigned, "edge": self.edge,
            "edge_rest_length": self.edgeRestLength, "active_edge": self.activeEdge, "edge_lambda": self.edgeLambda,
            "triangle": self.triangle, "tri_to_env": self.triToEnv, "hole": self.hole,
            "vertex_to_env": self.vertexToEnv, "active_drag_constraint": self.activeDragConstraint,
            "laparoscope_base": self.laparoscopeBase, "laparoscope_tip": self.laparoscopeTip,
            "laparoscope_radius": self.laparoscopeRadius, "laparoscope_in_collision": self.laparoscopeInCollision,
            "connector_triangle_id": self.connectorTriangleId, "connector_tri_bar": self.connectorTriBar,
            "connector_vertex_id": self.connectorVertexId, "connector_rest_dist": self.connectorRestDist,
            "env_vertex_start": self.envVertexStartT, "env_tet_start": self.envTetStartT,
            "env_edge_start": self.envEdgeStartT, "env_tri_start": self.envTriStartT,
        })

    def host_model(self) -> tuple[_lib.Model, dict]:
        """Descriptor over host copies of the constant arrays (and the current state).

        Returns the descriptor and the dict of numpy arrays it points into (keep it alive).
        """
        h = self.host
        arrs = {
            "vertex": self.vertex.detach().cpu().numpy().copy(),
            "predicted_vertex": self.predictedVertex.detach().cpu().numpy().copy(),
            "velocity": self.velocity.detach().cpu().numpy().copy(),
            "inverse_mass": h["inverseMass"], "tetrahedron": h["tetrahedron"],
            "tetrahedron_rest_volume": h["tetrahedronRestVolume"],
            "active_tetrahedron": self.activeTetrahedron.cpu().numpy().copy(),
            "tetrahedron_dm_inv": h["tetrahedronDmInv"], "xpbd_rest_volume": h["tetrahedronRestVolumeSigned"],
            "edge": h["edge"], "edge_rest_length": h["edgeRestLength"],
            "active_edge": self.activeEdge.cpu().numpy().copy(), "triangle": h["triangle"],
            "tri_to_env": h["triToEnv"], "hole": self.hole.cpu().numpy().copy(), "vertex_to_env": h["vertexToEnv"],
            "active_drag_constraint": self.activeDragConstraint.cpu().numpy().copy(),
            "laparoscope_base": self.laparoscopeBase.cpu().numpy().copy(),
            "laparoscope_tip": self.laparoscopeTip.cpu().numpy().copy(),
            "laparoscope_radius": self.laparoscopeRadius.cpu().numpy().copy(),
            "laparoscope_in_collision": self.laparoscopeInCollision.cpu().numpy().copy(),
            "env_vertex_start": self.envVertexStart, "env_tet_start": self.envTetStart,
            "env_edge_start": self.envEdgeStart, "env_tri_start": self.envTriStart,
            "connector_triangle_id": h["connectorTriangleId"], "connector_tri_bar": h["connectorTriBar"],
            "connector_vertex_id": h["connectorVertexId"], "connector_rest_dist": h["connectorRestDist"],
        }
        return self._fill(_lib.Model(), arrs), arrs

    # ----------------------------------------------------- reference methods
    def transformSimMeshData(self, stream=None):
        """remapAToB of the simulated vertices onto the visual points (modelDO.py:1441-1444)."""
        self.require_cuda()
        check(lib().ffsrl_remap(ptr(self.allVisPoint), ptr(self.vertex), ptr(self.pointToVertex),
                                self.numVisPoints, _lib.stream_handle(stream)))

    def transformSimLaparoscopeMeshData(self, stream=None, env_ids=None):
        """updateLaparoscopeMeshKernel (modelDO.py:1446-1473): the instrument's visual points
        of every env (or of the envs in the int32 device tensor ``env_ids``) from its
        transforms.  Nothing to do without an instrument mesh or transforms."""
        if self.instrumentMesh is None or not self.hasInstrumentKinematics:
            return
        self.require_cuda()
        n = self.numEnvs if env_ids is None else int(env_ids.numel())
        check(lib().ffsrl_instrument_visual_update(ptr(self.laparoscopeXForm), ptr(self.laparoscopeVertex),
                                                   ptr(self.laparoscopeVertexToXForm),
                                                   int(self.laparoscopeVertexToXForm.numel()), ptr(self.allVisPoint),
                                                   ptr(self.envInstrumentPointStartT),
                                                   None if env_ids is None else ptr(env_ids), n, self.numEnvs,
                                                   _lib.stream_handle(stream)))

    def getVertexPositionsTensor(self, vertexId):
        return self.vertex[vertexId]

    def getVertexPositionsTensorMultiEnvs(self, vertexIds):
        idx = torch.as_tensor(self.envVertexStart[:-1], device=self.device, dtype=torch.long) + \
            torch.as_tensor(vertexIds, device=self.device, dtype=torch.long)
        return self.vertex[idx]

    def getLaparoscopePositionsTensor(self):
        return self.laparoscopeTip[3::4]

    def getLaparoscopeClampVertex(self, vertexId):
        return self.activeDragConstraint[vertexId]

    def getLaparoscopeInCollision(self):
        return self.laparoscopeInCollision

    def resetCollisionInfo(self):
        """Zero the per-env contact counters in place (the reference reallocates the array,
        ``modelDO.py:1520-1522``, which a captured graph would not see)."""
        self.laparoscopeInCollision.zero_()

    def forceLaparoscopeClampVertex(self, vertexId: int, envs, on: float = 1.0, animate: bool = True):
        """forceClampsDragKernel (modelDO.py:281-289) for the envs where ``envs`` is nonzero.
        The clamp animation of the instrument model is not part of this model."""
        self.require_cuda()
        env_ids = torch.nonzero(torch.as_tensor(envs, device=self.device)).to(torch.int32).flatten().contiguous()
        check(lib().ffsrl_force_clamps_drag(ptr(self.activeDragConstraint), int(vertexId), ptr(env_ids),
                                            int(env_ids.numel()), float(on), self.environmentNumVertices,
                                            _lib.stream_handle()))

    def updateClampsDrag(self, state, update, lookupRadius=None):
        """updateClampsDragKernel (modelDO.py:247-279): state/update are int32 [3N] tensors."""
        self.require_cuda()
        r = self.globalLaparoscopeDragLookupRadius if lookupRadius is None else float(lookupRadius)
        check(lib().ffsrl_update_clamps_drag(ptr(self.predictedVertex), ptr(self.vertexToEnv),
                                             ptr(self.laparoscopeTip), ptr(self.activeDragConstraint), r,
                                             ptr(state), ptr(update), self.numVertices, _lib.stream_handle()))

    def graspNearest(self, clamp, radius=None, stream=None):
        """Per env, grasp the surface vertex nearest the drag point within ``radius`` when
        ``clamp[e]`` is nonzero, release the env's grasp when it is zero."""
        self.require_cuda()
        r = self.globalLaparoscopeDragLookupRadius if radius is None else float(radius)
        clamp = torch.as_tensor(clamp, device=self.device, dtype=torch.int32).contiguous()
        check(lib().ffsrl_grasp_nearest(ptr(self.vertex), ptr(self.graspCandStartT), ptr(self.graspCand),
                                        ptr(self.laparoscopeTip), ptr(clamp), r, ptr(self.activeDragConstraint),
                                        self.numEnvs, _lib.stream_handle(stream)))

    def moveTool(self, disp, stream=None):
        """Translate every env's instrument by ``disp`` [N, 3] (device tensor): the capsule
        ends, and the kinematic transforms when the model has them."""
        self.require_cuda()
        disp = disp.contiguous()
        check(lib().ffsrl_move_tool(ptr(self.laparoscopeBase), ptr(self.laparoscopeTip), ptr(disp), self.numEnvs,
                                    _lib.stream_handle(stream)))
        if self.hasInstrumentKinematics:
            with torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext():
                # the translation of a stored transpose is its bottom row
                self.laparoscopeXForm.view(self.numEnvs, 7, 16)[:, :, 12:15] += disp.view(self.numEnvs, 1, 3)

    # ------------------------------------------------- instrument kinematics
    def setInstrument(self, xform, heights):
        """Kinematic instrument (laparoscope.py:370-383): 7 transforms per env, [N, 112] in
        the reference's storage (row-major transposes of column-vector transforms; slots 0
        rod capsule, 1/2 clamps, 3 rotation centre, 4/5 clamp pivots, 6 rod), and capsule
        heights [N, 4].  The capsule ends stay as set by ``setTool`` until an action
        recomputes them from the transforms."""
        self.laparoscopeXForm.copy_(torch.as_tensor(np.asarray(xform, dtype=np.float32).reshape(-1)))
        self.laparoscopeInitialXForm.copy_(self.laparoscopeXForm)
        self.laparoscopeHeight.copy_(torch.as_tensor(np.asarray(heights, dtype=np.float32).reshape(-1)))
        self.hasInstrumentKinematics = True
        if self.device.type == "cuda":
            self.transformSimLaparoscopeMeshData()

    def _require_kinematics(self):
        self.require_cuda()
        if not self.hasInstrumentKinematics:
            raise _lib.FFSRLError(_lib.ERR_INVALID_ARGUMENT, "the model has no instrument transforms (setInstrument)")

    def _flat(self, a, n):
        a = torch.as_tensor(a, dtype=torch.float32, device=self.device).reshape(-1).contiguous()
        if a.numel() != n:
            raise ValueError(f"expected {n} values, got {a.numel()}")
        return a

    def applyActions(self, actions, stream=None):
        """applyActions (modelDO.py:1331-1362): per env, rod forward, rod roll, rotation-
        centre x and y rotation, clamp opening ([N, 5]); then the clamps' grasp update
        (updateClampsDragKernel) and the visual points."""
        self._require_kinematics()
        a = self._flat(actions, 5 * self.numEnvs)
        check(lib().ffsrl_instrument_apply_actions(ptr(self.laparoscopeXForm), ptr(a), ptr(self.laparoscopeDragCutHeat),
                                                   ptr(self.laparoscopeDragCutHeatUpdate), ptr(self.laparoscopeBase),
                                                   ptr(self.laparoscopeTip), ptr(self.laparoscopeHeight), self.numEnvs,
                                                   _lib.stream_handle(stream)))
        self.updateClampsDrag(self.laparoscopeDragCutHeat, self.laparoscopeDragCutHeatUpdate)
        self.transformSimMeshData(stream)
        self.transformSimLaparoscopeMeshData(stream)

    def applyCartesianActions(self, cartesianActions, stream=None):
        """applyCartesianActions (modelDO.py:1364-1383): move each effector by [N, 3]."""
        self._require_kinematics()
        a = self._flat(cartesianActions, 3 * self.numEnvs)
        check(lib().ffsrl_instrument_cartesian(ptr(self.laparoscopeXForm), ptr(a), None, None,
                                               ptr(self.laparoscopeBase), ptr(self.laparoscopeTip),
                                               ptr(self.laparoscopeHeight), self.numEnvs, _lib.stream_handle(stream)))
        self.transformSimMeshData(stream)
        self.transformSimLaparoscopeMeshData(stream)

    def applyCartesianActionsInWorkspace(self, cartesianActions, stream=None):
        """applyCartesianActionsInWorkspace (modelDO.py:1385-1404): components that would take
        the effector out of [workspaceLow, workspaceHigh] are dropped;
        ``laparoscopeWorkspaceViolation`` flags those envs."""
        self._require_kinematics()
        a = self._flat(cartesianActions, 3 * self.numEnvs)
        ws = np.asarray(list(self.workspaceLow) + list(self.workspaceHigh), dtype=np.float32)
        check(lib().ffsrl_instrument_cartesian(ptr(self.laparoscopeXForm), ptr(a), ws.ctypes.data,
                                               ptr(self.laparoscopeWorkspaceViolation), ptr(self.laparoscopeBase),
                                               ptr(self.laparoscopeTip), ptr(self.laparoscopeHeight), self.numEnvs,
                                               _lib.stream_handle(stream)))

    def setRotationCenter(self, translation, rotation, stream=None):
        """setRotationCenter (modelDO.py:1570-1587): the rotation centre of env e takes the
        pose T(translation[e]) Rx Ry Rz(rotation[e]) and carries the instrument with it."""
        self._require_kinematics()
        t = self._flat(translation, 3 * self.numEnvs)
        r = self._flat(rotation, 3 * self.numEnvs)
        check(lib().ffsrl_instrument_set_rotation_center(ptr(self.laparoscopeXForm), ptr(t), ptr(r),
                                                         ptr(self.laparoscopeBase), ptr(self.laparoscopeTip),
                                                         ptr(self.laparoscopeHeight), self.numEnvs,
                                                         _lib.stream_handle(stream)))

    def forceLaparoscopeClamp(self, envs):
        """forceLaparoscopeClamp (modelDO.py:1524-1531): a closing clamp action (-1 rad) for
        the envs where ``envs`` is nonzero."""
        e = torch.clamp(torch.as_tensor(envs, dtype=torch.float32, device=self.device), 0.0, 1.0)
        actions = torch.zeros((self.numEnvs, 5), dtype=torch.float32, device=self.device)
        actions[:, 4] = -e
        self.applyActions(actions)

    def getLaparoscopePositionsTensor(self):
        """Each env's effector (drag point) [N, 3], a view of the capsule-end array."""
        return self.laparoscopeTip.view(self.numEnvs, 4, 3)[:, 3]

    def setTool(self, base, tip, radius=None):
        """Set the instrument's capsule ends [4N, 3] (and radii [4N])."""
        self.laparoscopeBase.copy_(torch.as_tensor(base, dtype=torch.float32))
        self.laparoscopeTip.copy_(torch.as_tensor(tip, dtype=torch.float32))
        if radius is not None:
            self.laparoscopeRadius.copy_(torch.as_tensor(radius, dtype=torch.float32))

    def setEffectorInitialPosition(self):
        self.laparoscopeInitialBase.copy_(self.laparoscopeBase)
        self.laparoscopeInitialTip.copy_(self.laparoscopeTip)
        self.laparoscopeInitialXForm.copy_(self.laparoscopeXForm)

    def resetFixedModel(self, envNums):
        """Restore the listed envs' vertices and instrument, zero their velocity,
        predicted positions and grasp (modelDO.py:1589-1622).  Whole-array copies when
        every env is listed, masked copies otherwise."""
        ids = sorted({int(e) for e in envNums})
        if not ids:
            return
        if ids[0] < 0 or ids[-1] >= self.numEnvs:
            raise ValueError("resetFixedModel: env id out of range")
        if len(ids) == self.numEnvs:
            self.vertex.copy_(self.initialVertex)
            self.predictedVertex.zero_()
            self.velocity.zero_()
            self.activeDragConstraint.zero_()
            self.laparoscopeBase.copy_(self.laparoscopeInitialBase)
            self.laparoscopeTip.copy_(self.laparoscopeInitialTip)
            self.laparoscopeXForm.copy_(self.laparoscopeInitialXForm)
            self.laparoscopeDragCutHeat.zero_()
            self.laparoscopeDragCutHeatUpdate.zero_()
        else:
            self.require_cuda()
            idt = torch.as_tensor(ids, dtype=torch.int32, device=self.device)
            check(lib().ffsrl_reset_envs(ptr(self.vertex), ptr(self.velocity), ptr(self.activeDragConstraint),
                                         ptr(self.initialVertex), ptr(self.laparoscopeBase), ptr(self.laparoscopeTip),
                                         ptr(self.laparoscopeInitialBase), ptr(self.laparoscopeInitialTip),
                                         ptr(self.laparoscopeInCollision), ptr(self.laparoscopeXForm),
                                         ptr(self.laparoscopeInitialXForm), ptr(self.envVertexStartT), ptr(idt),
                                         len(ids), self.numEnvs, _lib.stream_handle(None)))
            sel = torch.zeros(self.numEnvs, dtype=torch.bool, device=self.device)
            sel[idt.long()] = True
            self.predictedVertex.masked_fill_(sel[self.vertexToEnv.long()].unsqueeze(1), 0.0)
            hm = sel.repeat_interleave(3)
            self.laparoscopeDragCutHeat.masked_fill_(hm, 0)
            self.laparoscopeDragCutHeatUpdate.masked_fill_(hm, 0)
        self.transformSimLaparoscopeMeshData()
        self.transformSimMeshData()

    def resetStochasticModel(self, laparoscopeTranslation=None, laparoscopeRotation=None):
        """Restore every env (modelDO.py:1624-1645); the instrument returns to its initial
        pose, then, given a translation and rotation [N, 3], its rotation centre takes that
        pose (``setRotationCenter``)."""
        self.vertex.copy_(self.initialVertex)
        self.laparoscopeBase.copy_(self.laparoscopeInitialBase)
        self.laparoscopeTip.copy_(self.laparoscopeInitialTip)
        self.laparoscopeXForm.copy_(self.laparoscopeInitialXForm)
        self.laparoscopeDragCutHeat.zero_()
        self.laparoscopeDragCutHeatUpdate.zero_()
        if laparoscopeTranslation is not None and laparoscopeRotation is not None:
            self.setRotationCenter(laparoscopeTranslation, laparoscopeRotation)
        self.transformSimLaparoscopeMeshData()
        self.transformSimMeshData()

    def envSlice(self, e: int) -> slice:
        return slice(int(self.envVertexStart[e]), int(self.envVertexStart[e + 1]))
