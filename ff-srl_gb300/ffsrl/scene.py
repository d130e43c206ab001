"""Array scene files: the reference's USD prims and attributes in an npz archive.

The reference builds its model from a USD stage (``FF_SRL/FF_SRL/modelDO.py:1646-1690``):
Mesh prims flagged ``simMesh`` are soft bodies (``SimMeshDO``, ``modelDO.py:545-640``),
Mesh prims flagged ``simRigid`` are static visual objects (``SimRigidDO``,
``modelDO.py:642-700``), and an Xform flagged ``simLaparoscope`` is the instrument
(``laparoscope.py``).  USD cannot be read here (``pxr`` is not installed), so a scene is an
``.npz`` archive whose keys are USD property paths, ``<prim path>.<attribute name>``, e.g.
``/World/Liver.extMesh:vertex``, holding the same attributes:

=============================  ===========================================================
simMesh prim                   ``simMesh`` (1), ``extMesh:vertex`` (local), ``extMesh:elem``,
                               ``extMesh:edge``, ``extMesh:edgeRestLength``,
                               ``extMesh:triangle``, ``extMesh:inverseMass``,
                               ``extMesh:tetrahedronRestVolume``,
                               ``extMesh:inverseRestPosition`` (Dm^-1, [T, 3, 3]),
                               ``points``, ``faceVertexIndices``, ``primvars:displayColor``,
                               ``mapping:pointToVertex``, ``param:*`` scalars,
                               ``xformOp:transform`` (optional); the cutting maps
                               ``mapping:edgeToTriangles``, ``triangleToTetrahedron``,
                               ``tetrahedronToTriangles``, ``tetrahedronNeighbors``
                               (optional, mesh-local ids, -1 for none)
simRigid prim                  ``simRigid`` (1), ``points`` (local), ``faceVertexIndices``,
                               ``primvars:displayColor``, ``xformOp:transform`` (optional)
material (either prim)         ``material:diffuse_texture`` [S, S, 3] in [0, 1] (the
                               reference holds an image path), ``primvars:st``,
                               ``primvars:st:indices`` (default: the faces,
                               ``modelDO.py:636-640``)
simConnector prim              ``simConnector`` (1), ``pointBody`` / ``triBody`` (the
                               bodies' prim paths), ``pointId``, ``triIds``, ``triBar``,
                               ``restDist`` (``modelDO.py:751-770``)
simLaparoscope prim            ``simLaparoscope`` (1), ``laparoscope:transforms`` [7, 16]
                               (the reference's storage), ``laparoscope:heights`` [4],
                               ``laparoscope:radii`` [4], ``laparoscope:bases`` /
                               ``laparoscope:tips`` [4, 3]; its visual mesh as ``points``,
                               ``faceVertexIndices``, ``laparoscope:pointSlot``,
                               ``primvars:displayColor``
=============================  ===========================================================

``xformOp:transform`` is the prim's local-to-world matrix in USD's convention (row
vectors, translation in the last row; ``utils.py:77-82`` applies it with
``Gf.Matrix4d.Transform``).  World positions are formed in float64 and stored as float32.
Attributes this library adds are under ``ffsrl:`` (signed rest volumes, the rest shape,
fixed flags); a file without them loads, with the signed volumes taken as the negated
rest volumes, as ``SimModelDO`` does.  The reference's reduce mappings
(``mapping:vertexTo*``) are read by its non-DO model only and are not written.

Several simMesh prims in one scene are merged into one soft body per env (the
reference concatenates an env's meshes, ``modelDO.py:915-960``); rigid prims attach to it.
"""

from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

PARAMS = ("density", "ksDistance", "ksVolume", "ksContact", "ksDrag", "volumeCompliance", "deviatoricCompliance",
          "breakFactor", "breakThreshold", "heatLoss", "heatConduction", "heatTransfer", "heatLimit",
          "heatSphereRadius", "heatQuantum")

# mesh-dict key <-> USD attribute of a simMesh prim
MESH_ATTRS = (("vertex", "extMesh:vertex"), ("tetrahedron", "extMesh:elem"), ("edge", "extMesh:edge"),
              ("edge_rest_length", "extMesh:edgeRestLength"), ("triangle", "extMesh:triangle"),
              ("inverse_mass", "extMesh:inverseMass"), ("tetrahedron_rest_volume", "extMesh:tetrahedronRestVolume"),
              ("tetrahedron_dm_inv", "extMesh:inverseRestPosition"), ("vis_face", "faceVertexIndices"),
              ("vis_point_color", "primvars:displayColor"), ("point_to_vertex", "mapping:pointToVertex"))
# element maps of the cutting and heating kernels (model.py:207-255), optional
MAP_ATTRS = (("edge_to_triangles", "mapping:edgeToTriangles"), ("triangle_to_tetrahedron", "mapping:triangleToTetrahedron"),
             ("tetrahedron_to_triangles", "mapping:tetrahedronToTriangles"),
             ("tetrahedron_neighbors", "mapping:tetrahedronNeighbors"))
EXTRA_ATTRS = MAP_ATTRS + (("tetrahedron_rest_volume_signed", "ffsrl:tetrahedronRestVolumeSigned"),
               ("rest_vertex", "ffsrl:restVertex"), ("fixed", "ffsrl:fixed"))
# connector prim (modelDO.py:751-770): ids local to its bodies
CONNECTOR_ATTRS = (("connector_vertex_id", "pointId"), ("connector_triangle_id", "triIds"),
                   ("connector_tri_bar", "triBar"), ("connector_rest_dist", "restDist"))
TEXTURE_ATTRS = (("texture", "material:diffuse_texture"), ("tex_coords", "primvars:st"),
                 ("tex_indices", "primvars:st:indices"))
SHAPES = {"vertex": (-1, 3), "tetrahedron": (-1, 4), "edge": (-1, 2), "triangle": (-1, 3), "vis_face": (-1, 3),
          "vis_point_color": (-1, 3), "point_to_vertex": (-1, 2), "tetrahedron_dm_inv": (-1, 9),
          "rest_vertex": (-1, 3), "tex_coords": (-1, 2), "edge_to_triangles": (-1, 2),
          "tetrahedron_to_triangles": (-1, 4), "tetrahedron_neighbors": (-1, 4)}
INT_KEYS = {"tetrahedron", "edge", "triangle", "vis_face", "point_to_vertex", "tex_indices", "edge_to_triangles",
            "triangle_to_tetrahedron", "tetrahedron_to_triangles", "tetrahedron_neighbors"}


@dataclass
class Scene:
    """A loaded scene: the env's soft body (rigids attached under ``"rigids"``), the
    instrument (``None`` without one) and each simMesh prim's ``param:*`` values."""
    mesh: dict
    instrument: dict | None = None
    params: dict = field(default_factory=dict)


def _world(points, xform) -> np.ndarray:
    p = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    if xform is None:
        return p.astype(np.float32)
    M = np.asarray(xform, dtype=np.float64).reshape(4, 4)
    return (p @ M[:3, :3] + M[3, :3]).astype(np.float32)


def _shape(key, a):
    a = np.asarray(a)
    a = a.astype(np.int32) if key in INT_KEYS else a
    return a.reshape(SHAPES[key]) if key in SHAPES else a


def _put_texture(out, prim, obj):
    if obj.get("texture") is not None:
        for key, attr in TEXTURE_ATTRS:
            if key in obj:
                out[f"{prim}.{attr}"] = np.asarray(obj[key])


def _get_texture(z, prim, obj):
    if f"{prim}.material:diffuse_texture" in z:
        for key, attr in TEXTURE_ATTRS:
            if f"{prim}.{attr}" in z:
                obj[key] = _shape(key, z[f"{prim}.{attr}"])


def write_scene(path, meshes, rigids=(), instrument=None, params=None, names=None) -> None:
    """Write soft-body mesh dicts (``ffsrl.meshgen`` form), rigid dicts (``vertex``,
    ``triangle``, ``color``, optional texture) and an instrument (``transforms`` [7, 16],
    ``heights`` [4], ``radii`` [4], ``bases`` / ``tips`` [4, 3] and optionally the visual
    mesh ``points``, ``faces``, ``slot``, ``color``) as a scene archive.  Positions are
    written in world coordinates (no ``xformOp:transform``)."""
    meshes = [meshes] if isinstance(meshes, dict) else list(meshes)
    names = names or [f"Mesh{k}" for k in range(len(meshes))]
    out = {}
    for name, m in zip(names, meshes):
        prim = f"/World/{name}"
        out[f"{prim}.simMesh"] = np.int32(1)
        for key, attr in MESH_ATTRS + EXTRA_ATTRS:
            if key in m:
                out[f"{prim}.{attr}"] = np.asarray(m[key])
        ptv = np.asarray(m["point_to_vertex"]).reshape(-1, 2)
        out[f"{prim}.points"] = np.asarray(m.get("rest_vertex", m["vertex"]), dtype=np.float32)[ptv[:, 1]]
        for p, v in (params or {}).items():
            out[f"{prim}.param:{p}"] = np.float64(v)
        _put_texture(out, prim, m)
        if m.get("connector_vertex_id") is not None and len(m["connector_vertex_id"]):
            cp = f"/World/{name}Connector"
            out[f"{cp}.simConnector"] = np.int32(1)
            out[f"{cp}.pointBody"] = np.asarray(prim)
            out[f"{cp}.triBody"] = np.asarray(prim)
            for key, attr in CONNECTOR_ATTRS:
                out[f"{cp}.{attr}"] = np.asarray(m[key])
    for k, r in enumerate(rigids):
        prim = f"/World/Rigid{k}"
        out[f"{prim}.simRigid"] = np.int32(1)
        out[f"{prim}.points"] = np.asarray(r["vertex"], dtype=np.float32)
        out[f"{prim}.faceVertexIndices"] = np.asarray(r["triangle"], dtype=np.int32)
        if "color" in r:
            out[f"{prim}.primvars:displayColor"] = np.asarray(r["color"], dtype=np.float32)
        _put_texture(out, prim, r)
    if instrument is not None:
        prim = "/World/Laparoscope"
        out[f"{prim}.simLaparoscope"] = np.int32(1)
        for key in ("transforms", "heights", "radii", "bases", "tips"):
            out[f"{prim}.laparoscope:{key}"] = np.asarray(instrument[key], dtype=np.float32)
        if "points" in instrument:
            out[f"{prim}.points"] = np.asarray(instrument["points"], dtype=np.float32)
            out[f"{prim}.faceVertexIndices"] = np.asarray(instrument["faces"], dtype=np.int32)
            out[f"{prim}.laparoscope:pointSlot"] = np.asarray(instrument["slot"], dtype=np.int32)
            out[f"{prim}.primvars:displayColor"] = np.asarray(instrument["color"], dtype=np.float32)
    np.savez_compressed(path, **out)


def _prims(z, flag):
    return sorted({k.rsplit(".", 1)[0] for k in z.files if k.endswith("." + flag) and int(z[k]) == 1})


def merge_meshes(meshes) -> dict:
    """One soft body from several (disjoint) mesh dicts: ids offset, arrays concatenated
    in order, as the reference concatenates an env's meshes.  The cutting maps are not
    carried over (they are rebuilt from the merged topology when needed)."""
    if len(meshes) == 1:
        return meshes[0]
    out = {}
    nv = np.cumsum([0] + [len(m["vertex"]) for m in meshes])
    npnt = np.cumsum([0] + [len(m["point_to_vertex"]) for m in meshes])
    for key in ("vertex", "rest_vertex", "inverse_mass", "tetrahedron_rest_volume", "tetrahedron_rest_volume_signed",
                "tetrahedron_dm_inv", "edge_rest_length", "vis_point_color", "fixed"):
        if all(key in m for m in meshes):
            out[key] = np.concatenate([np.asarray(m[key]) for m in meshes])
    for key in ("tetrahedron", "edge", "triangle"):
        out[key] = np.concatenate([np.asarray(m[key]) + nv[k] for k, m in enumerate(meshes)]).astype(np.int32)
    out["vis_face"] = np.concatenate([np.asarray(m["vis_face"]) + npnt[k] for k, m in enumerate(meshes)]).astype(np.int32)
    out["point_to_vertex"] = np.concatenate(
        [np.asarray(m["point_to_vertex"]) + np.array([npnt[k], nv[k]]) for k, m in enumerate(meshes)]).astype(np.int32)
    if any(m.get("texture") is not None for m in meshes):
        raise ValueError("merge_meshes: textured soft bodies must be the only simMesh prim of a scene")
    return out


def read_scene(path) -> Scene:
    """Load a scene archive written by ``write_scene`` or by an exporter of the same schema."""
    with np.load(path) as z:
        meshes, params = [], {}
        for prim in _prims(z, "simMesh"):
            g = lambda attr: z[f"{prim}.{attr}"] if f"{prim}.{attr}" in z else None
            xf = g("xformOp:transform")
            m = {}
            for key, attr in MESH_ATTRS + EXTRA_ATTRS:
                a = g(attr)
                if a is not None:
                    m[key] = _shape(key, a)
            m["vertex"] = _world(m["vertex"], xf)
            if "rest_vertex" in m:
                m["rest_vertex"] = _world(m["rest_vertex"], xf)
            if "fixed" not in m:
                m["fixed"] = np.asarray(m["inverse_mass"]) == 0
            m["tetrahedron_dm_inv"] = np.asarray(m["tetrahedron_dm_inv"], dtype=np.float32).reshape(-1, 9)
            _get_texture(z, prim, m)
            params[prim] = {p: float(z[f"{prim}.param:{p}"]) for p in PARAMS if f"{prim}.param:{p}" in z}
            meshes.append(m)
        if not meshes:
            raise ValueError(f"{path}: no simMesh prim")
        mesh = dict(merge_meshes(meshes))
        prims = _prims(z, "simMesh")
        offset = dict(zip(prims, np.cumsum([0] + [len(m["vertex"]) for m in meshes])[:-1].tolist()))
        cv, ct, cb, cr = [], [], [], []
        for cp in _prims(z, "simConnector"):
            pb, tb = str(z[f"{cp}.pointBody"]), str(z[f"{cp}.triBody"])
            if pb not in offset or tb not in offset:
                raise ValueError(f"{path}: connector {cp} names a body that is not a simMesh prim")
            cv.append(np.asarray(z[f"{cp}.pointId"], dtype=np.int64).reshape(-1) + offset[pb])
            ct.append(np.asarray(z[f"{cp}.triIds"], dtype=np.int64).reshape(-1, 3) + offset[tb])
            cb.append(np.asarray(z[f"{cp}.triBar"], dtype=np.float32).reshape(-1, 3))
            cr.append(np.asarray(z[f"{cp}.restDist"], dtype=np.float32).reshape(-1))
        if cv:
            mesh["connector_vertex_id"] = np.concatenate(cv).astype(np.int32)
            mesh["connector_triangle_id"] = np.concatenate(ct).astype(np.int32)
            mesh["connector_tri_bar"] = np.concatenate(cb)
            mesh["connector_rest_dist"] = np.concatenate(cr)
        rigids = []
        for prim in _prims(z, "simRigid"):
            q = _world(z[f"{prim}.points"], z[f"{prim}.xformOp:transform"] if f"{prim}.xformOp:transform" in z
                       else None)
            r = {"vertex": q, "triangle": np.asarray(z[f"{prim}.faceVertexIndices"], dtype=np.int32).reshape(-1, 3)}
            if f"{prim}.primvars:displayColor" in z:
                r["color"] = np.asarray(z[f"{prim}.primvars:displayColor"], dtype=np.float32).reshape(-1, 3)
            _get_texture(z, prim, r)
            rigids.append(r)
        if rigids:
            mesh = dict(mesh)
            mesh["rigids"] = rigids
        inst = None
        lap = _prims(z, "simLaparoscope")
        if len(lap) > 1:
            raise ValueError(f"{path}: one simLaparoscope prim per scene")
        if lap:
            prim = lap[0]
            inst = {key: np.asarray(z[f"{prim}.laparoscope:{key}"], dtype=np.float32)
                    for key in ("transforms", "heights", "radii", "bases", "tips")}
            inst["transforms"] = inst["transforms"].reshape(7, 16)
            inst["bases"], inst["tips"] = inst["bases"].reshape(4, 3), inst["tips"].reshape(4, 3)
            if f"{prim}.points" in z:
                inst["mesh"] = {"points": np.asarray(z[f"{prim}.points"], dtype=np.float32).reshape(-1, 3),
                                "faces": np.asarray(z[f"{prim}.faceVertexIndices"], dtype=np.int32).reshape(-1, 3),
                                "slot": np.asarray(z[f"{prim}.laparoscope:pointSlot"], dtype=np.int32),
                                "color": np.asarray(z[f"{prim}.primvars:displayColor"], dtype=np.float32).reshape(-1, 3)}
    return Scene(mesh=mesh, instrument=inst, params=params)


def is_scene_path(stage) -> bool:
    return isinstance(stage, (str, os.PathLike))
