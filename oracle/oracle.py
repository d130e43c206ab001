"""TEST INFRASTRUCTURE ONLY: Python harness of the CPU oracle (ffsrl_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module,
as the checker or the timed CPU baseline.  It restates the reference's kernels
(FF_SRL/FF_SRL/integrator.py, bvh.py, render.py, utils.py) serially in launch and
thread order.  Parity is unpinned: the reference (warp-lang 0.10.1, pxr) cannot run
here and ships no golden vectors; the restatement is pinned by analytic known-answer
tests (tests/test_oracle_kat.py) instead.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "ffsrl_oracle.cpp"
SO = HERE / "_build" / "libffsrl_oracle.so"
ROOT = HERE.parent
sys.path.insert(0, str(ROOT / "ff-srl_gb300"))
from ffsrl import _lib as L  # noqa: E402  (struct layouts of include/ffsrl.h)


def build(force: bool = False) -> Path:
    SO.parent.mkdir(parents=True, exist_ok=True)
    hdr = ROOT / "include" / "ffsrl.h"
    if force or not SO.exists() or SO.stat().st_mtime < max(SRC.stat().st_mtime, hdr.stat().st_mtime):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-fno-fast-math", "-o", str(SO), str(SRC)]
        subprocess.run(cmd, check=True)
    return SO


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(SO))
        P = C.c_void_p
        _lib.oracle_step_f32.argtypes = [C.POINTER(L.Model), C.POINTER(L.Params), C.c_int, C.c_int]
        _lib.oracle_step_f64.argtypes = [C.POINTER(L.Model), C.POINTER(L.Params), C.c_int, C.c_int, P, P, P]
        _lib.oracle_remap.argtypes = [P, P, P, C.c_int32]
        _lib.oracle_refit.argtypes = [C.POINTER(L.Bvh), P, P]
        _lib.oracle_render.argtypes = [C.POINTER(L.Render), C.POINTER(L.Bvh), C.c_int]
        _lib.oracle_refit_mt.argtypes = [C.POINTER(L.Bvh), P, P, C.c_int]
        _lib.oracle_render_mt.argtypes = [C.POINTER(L.Render), C.POINTER(L.Bvh), C.c_int, C.c_int]
        _lib.oracle_reference_refit_source.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, P, P]
        for f in ("oracle_step_f32", "oracle_step_f64", "oracle_render", "oracle_render_mt"):
            getattr(_lib, f).restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleSim:
    """Host copy of a SimModelDO's arrays stepped by the oracle."""

    def __init__(self, model, state=None):
        h = model.host
        V = model.numVertices
        self.model = model
        self.params = model.params()
        src = state or {}
        self.a = {
            "vertex": np.array(src.get("vertex", h["vertex"]), dtype=np.float32).reshape(-1, 3).copy(),
            "predicted_vertex": np.array(src.get("predicted_vertex", np.zeros((V, 3))), dtype=np.float32).reshape(-1, 3).copy(),
            "velocity": np.array(src.get("velocity", np.zeros((V, 3))), dtype=np.float32).reshape(-1, 3).copy(),
            "dp": np.zeros((V, 3), dtype=np.float32),
            "constraints_number": np.zeros(V, dtype=np.int32),
            "inverse_mass": h["inverseMass"],
            "tetrahedron": h["tetrahedron"],
            "tetrahedron_rest_volume": h["tetrahedronRestVolume"],
            "active_tetrahedron": np.array(src.get("active_tetrahedron", np.ones(model.numTetrahedrons)), dtype=np.float32),
            "tetrahedron_dm_inv": h["tetrahedronDmInv"],
            "tetrahedron_lambda": np.zeros(max(model.numTetrahedrons, 1), dtype=np.float32),
            "xpbd_rest_volume": h["tetrahedronRestVolumeSigned"],
            "edge": h["edge"], "edge_rest_length": h["edgeRestLength"],
            "active_edge": np.array(src.get("active_edge", np.ones(model.numEdges)), dtype=np.float32),
            "edge_lambda": np.zeros(max(model.numEdges, 1), dtype=np.float32),
            "triangle": h["triangle"], "tri_to_env": h["triToEnv"],
            "hole": np.array(src.get("hole", np.zeros(model.numTriangles)), dtype=np.int32),
            "vertex_to_env": h["vertexToEnv"],
            "active_drag_constraint": np.array(src.get("active_drag_constraint", np.zeros(V)), dtype=np.float32),
            "laparoscope_base": np.array(src.get("laparoscope_base", model.toolHost["base"]), dtype=np.float32).copy(),
            "laparoscope_tip": np.array(src.get("laparoscope_tip", model.toolHost["tip"]), dtype=np.float32).copy(),
            "laparoscope_radius": np.array(src.get("laparoscope_radius", model.toolHost["radius"]), dtype=np.float32).copy(),
            "laparoscope_in_collision": np.zeros(model.numEnvs, dtype=np.int32),
            "env_vertex_start": model.envVertexStart, "env_tet_start": model.envTetStart,
            "env_edge_start": model.envEdgeStart, "env_tri_start": model.envTriStart,
            "connector_triangle_id": h["connectorTriangleId"], "connector_tri_bar": h["connectorTriBar"],
            "connector_vertex_id": h["connectorVertexId"], "connector_rest_dist": h["connectorRestDist"],
        }
        self.a = {k: np.ascontiguousarray(v) for k, v in self.a.items()}
        m = L.Model()
        m.num_vertices, m.num_tetrahedrons, m.num_edges = V, model.numTetrahedrons, model.numEdges
        m.num_triangles, m.num_connectors, m.num_envs = model.numTriangles, model.simConnectors, model.numEnvs
        for k, v in self.a.items():
            setattr(m, k, _p(v))
        self.desc = m

    def step(self, n: int = 1, threads: int = 1) -> None:
        rc = lib().oracle_step_f32(C.byref(self.desc), C.byref(self.params), int(n), int(threads))
        if rc:
            raise RuntimeError(f"oracle step failed: {rc}")

    def step_f64(self, n: int, x64: np.ndarray, xp64: np.ndarray, v64: np.ndarray, threads: int = 1) -> None:
        rc = lib().oracle_step_f64(C.byref(self.desc), C.byref(self.params), int(n), int(threads),
                                   x64.ctypes.data, xp64.ctypes.data, v64.ctypes.data)
        if rc:
            raise RuntimeError(f"oracle f64 step failed: {rc}")

    def vis_points(self, instrument=None) -> np.ndarray:
        """Every visual point: the soft meshes' remapped from the vertices, the rigid meshes'
        as built, the instrument's from ``instrument`` (an OracleInstrument; without one,
        the model's current host copy of those points)."""
        m = self.model
        out = np.ascontiguousarray(m.allVisPoint.detach().cpu().numpy(), dtype=np.float32).copy()
        ptv = np.ascontiguousarray(m.host["pointToVertex"])
        lib().oracle_remap(out.ctypes.data, self.a["vertex"].ctypes.data, ptv.ctypes.data, m.numVisPoints)
        if instrument is not None and m.instrumentMesh is not None:
            instrument.visual(m.instrumentMesh["points"], m.instrumentMesh["slot"], out, m.envInstrumentPointStart)
        return out


def bvh_desc(bvh, arrays: dict) -> L.Bvh:
    """Host ffsrl_bvh over numpy copies of a SimBVH's arrays (filled into ``arrays``)."""
    names = {"env_topology": bvh.envTopology, "env_node_offset": bvh.envNodeOffset,
             "env_face_offset": bvh.envFaceOffset, "topo_node_offset": bvh.topoNodeOffset,
             "topo_tri_offset": bvh.topoTriOffset, "topo_max_level": bvh.topoMaxLevel, "left_node": bvh.leftNode,
             "first_tri_id": bvh.firstTriId, "tri_count": bvh.triCount, "level": bvh.level, "tri_id": bvh.triId,
             "aabb_min": bvh.aabbMin, "aabb_max": bvh.aabbMax}
    if getattr(bvh, "refitSource", None) is not None:
        names["refit_source"] = bvh.refitSource
    for k, t in names.items():
        arrays[k] = np.ascontiguousarray(t.detach().cpu().numpy())
    d = L.Bvh()
    d.num_envs, d.num_topologies = bvh.desc.num_envs, bvh.desc.num_topologies
    for k, v in arrays.items():
        setattr(d, k, _p(v))
    d.total_env_nodes, d.total_topology_nodes, d.max_level = (bvh.desc.total_env_nodes, bvh.desc.total_topology_nodes,
                                                              bvh.desc.max_level)
    return d


def reference_refit_source(num_envs: int, M: int, Rg: int, Lf: int, env_face_offset) -> np.ndarray:
    """The face each (env, local face) is boxed from by the reference's refit
    (bvh.py:66-74), as env-major global face ids."""
    efo = np.ascontiguousarray(np.asarray(env_face_offset, dtype=np.int32))
    out = np.zeros(num_envs * (M + Rg + Lf), dtype=np.int32)
    lib().oracle_reference_refit_source(num_envs, M, Rg, Lf, _p(efo), _p(out))
    return out


def refit(bvh, vis_points: np.ndarray, vis_face: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    arrays = {}
    d = bvh_desc(bvh, arrays)
    vp = np.ascontiguousarray(vis_points, dtype=np.float32)
    vf = np.ascontiguousarray(vis_face, dtype=np.int32)
    lib().oracle_refit(C.byref(d), vp.ctypes.data, vf.ctypes.data)
    return arrays["aabb_min"], arrays["aabb_max"]


def _render_desc(renderer, vis_points: np.ndarray):
    m = renderer.simModel
    N, R = renderer.numEnvs, renderer.width
    a = {
        "vis_point": np.ascontiguousarray(vis_points, dtype=np.float32),
        "vis_face": np.ascontiguousarray(m.host["allVisFace"], dtype=np.int32),
        "vis_point_color": np.ascontiguousarray(m.host["allVisPointColor"], dtype=np.float32),
        "vertex_normal": np.zeros((m.numAllVisPoints, 3), dtype=np.float32),
        "camera_pos": np.ascontiguousarray(renderer.cameraPosT.cpu().numpy()),
        "camera_rot": np.ascontiguousarray(renderer.cameraRotT.cpu().numpy()),
        "light_dir": np.ascontiguousarray(renderer.lightDir.cpu().numpy()),
        "light_intensity": np.ascontiguousarray(renderer.lightIntensity.cpu().numpy()),
        "color": np.zeros((N * R * R, 3), dtype=np.float32),
        "depth": np.zeros(N * R * R, dtype=np.float32),
    }
    r = L.Render()
    r.num_envs, r.resolution = N, R
    r.num_vis_points, r.num_vis_faces = m.numAllVisPoints, m.numAllVisFaces
    for k, v in a.items():
        setattr(r, k, _p(v))
    r.num_cameras = a["camera_pos"].shape[0]
    r.camera_tan, r.camera_aspect = renderer.camera_tan, renderer.camera_aspect
    r.num_lights = a["light_dir"].shape[0]
    r.render_mode = int(renderer.render_mode)
    if m.hasTextures:
        for k, src in (("texture", m.host["texture"]), ("env_objects", m.host["envObjects"]),
                       ("object_texture", m.host["objectTexture"]), ("tex_coords", m.host["texCoords"]),
                       ("tex_indices", m.host["texIndices"])):
            a[k] = np.ascontiguousarray(src)
            setattr(r, k, _p(a[k]))
    return r, a


def render(renderer, bvh, vis_points: np.ndarray, aabb: tuple | None = None, stack_cap: int = 64):
    """Oracle images (colour [N,R,R,3], depth [N,R,R]) for a WarpRaycastRendererDO's settings."""
    arrays = {}
    d = bvh_desc(bvh, arrays)
    if aabb is not None:
        arrays["aabb_min"][:] = aabb[0]
        arrays["aabb_max"][:] = aabb[1]
    N, R = renderer.numEnvs, renderer.width
    r, a = _render_desc(renderer, vis_points)
    rc = lib().oracle_render(C.byref(r), C.byref(d), int(stack_cap))
    if rc:
        raise RuntimeError(f"oracle render failed: {rc}")
    return a["color"].reshape(N, R, R, 3), a["depth"].reshape(N, R, R), a["vertex_normal"]


class OracleScene:
    """One full env-step on the host, the reference's order: the solve (8 substeps x I
    iterations), visual-point remap, BVH refit and ray-cast. All four run in the C++
    restatement on host-side copies; ``threads`` spreads envs over OpenMP threads. Used
    to time the CPU baseline; the images match ``render``'s."""

    def __init__(self, model, bvh, renderer, stack_cap: int = 64):
        self.sim = OracleSim(model)
        self.model = model
        self.ptv = np.ascontiguousarray(model.host["pointToVertex"], dtype=np.int32)
        self.faces = np.ascontiguousarray(model.host["allVisFace"], dtype=np.int32)
        self.bvh_arrays = {}
        self.bvh = bvh_desc(bvh, self.bvh_arrays)
        self.inst = None
        if model.instrumentMesh is not None and model.hasInstrumentKinematics:
            self.inst = OracleInstrument.from_model(model)
        self.r, self.a = _render_desc(renderer, self.sim.vis_points(self.inst))
        self.stack_cap = stack_cap

    def step(self, threads: int = 1) -> None:
        lib_ = lib()
        self.sim.step(1, threads=threads)
        vp = self.a["vis_point"]
        lib_.oracle_remap(vp.ctypes.data, self.sim.a["vertex"].ctypes.data, self.ptv.ctypes.data,
                          self.model.numVisPoints)
        if self.inst is not None:  # transformSimLaparoscopeMeshData, the end of stepModel
            im = self.model.instrumentMesh
            self.inst.visual(im["points"], im["slot"], vp, self.model.envInstrumentPointStart)
        lib_.oracle_refit_mt(C.byref(self.bvh), vp.ctypes.data, self.faces.ctypes.data, int(threads))
        rc = lib_.oracle_render_mt(C.byref(self.r), C.byref(self.bvh), int(self.stack_cap), int(threads))
        if rc:
            raise RuntimeError(f"oracle render failed: {rc}")


# ---------------------------------------------------------------- instrument kinematics
def _kin_lib():
    lb = lib()
    if not getattr(lb, "_kin_ready", False):
        P = C.c_void_p
        lb.oracle_instrument_update.argtypes = [P, P, P, P, C.c_int]
        lb.oracle_instrument_apply_actions.argtypes = [P, P, P, P, P, P, P, C.c_int]
        lb.oracle_instrument_cartesian.argtypes = [P, P, P, P, P, P, P, C.c_int]
        lb.oracle_instrument_set_rotation_center.argtypes = [P, P, P, P, P, P, C.c_int]
        lb.oracle_instrument_visual.argtypes = [P, P, P, C.c_int, P, P, C.c_int]
        lb._kin_ready = True
    return lb


class OracleInstrument:
    """Host copy of a model's kinematic instrument (transforms, heights, capsule ends,
    clamp state) advanced by the C++ restatement."""

    def __init__(self, xform, height, base, tip, dch=None, dchu=None):
        f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1)).copy()
        self.xform, self.height, self.base, self.tip = f(xform), f(height), f(base), f(tip)
        self.n = len(self.height) // 4
        i = lambda a: np.ascontiguousarray(np.zeros(3 * self.n, np.int32) if a is None else
                                           np.asarray(a, dtype=np.int32).reshape(-1)).copy()
        self.dch, self.dchu = i(dch), i(dchu)
        self.violation = np.zeros(self.n, dtype=np.int32)

    @classmethod
    def from_model(cls, model):
        """Host copy of a SimModelDO's instrument state."""
        c = lambda t: t.detach().cpu().numpy()
        return cls(c(model.laparoscopeXForm), c(model.laparoscopeHeight), c(model.laparoscopeBase),
                   c(model.laparoscopeTip), c(model.laparoscopeDragCutHeat), c(model.laparoscopeDragCutHeatUpdate))

    def update(self):
        _kin_lib().oracle_instrument_update(_p(self.xform), _p(self.base), _p(self.tip), _p(self.height), self.n)

    def apply_actions(self, actions):
        a = np.ascontiguousarray(np.asarray(actions, dtype=np.float32).reshape(-1))
        _kin_lib().oracle_instrument_apply_actions(_p(self.xform), _p(a), _p(self.dch), _p(self.dchu), _p(self.base),
                                                   _p(self.tip), _p(self.height), self.n)

    def cartesian(self, actions, workspace=None):
        a = np.ascontiguousarray(np.asarray(actions, dtype=np.float32).reshape(-1))
        ws = None if workspace is None else np.ascontiguousarray(np.asarray(workspace, dtype=np.float32).reshape(6))
        _kin_lib().oracle_instrument_cartesian(_p(self.xform), _p(a), None if ws is None else _p(ws),
                                               _p(self.violation), _p(self.base), _p(self.tip), _p(self.height), self.n)

    def set_rotation_center(self, translation, rotation):
        t = np.ascontiguousarray(np.asarray(translation, dtype=np.float32).reshape(-1))
        r = np.ascontiguousarray(np.asarray(rotation, dtype=np.float32).reshape(-1))
        _kin_lib().oracle_instrument_set_rotation_center(_p(self.xform), _p(t), _p(r), _p(self.base), _p(self.tip),
                                                         _p(self.height), self.n)

    def visual(self, local_points, point_slot, vis_points, env_first_point):
        """Instrument visual points of every env written into ``vis_points`` (in place)."""
        lp = np.ascontiguousarray(np.asarray(local_points, dtype=np.float32).reshape(-1))
        sl = np.ascontiguousarray(np.asarray(point_slot, dtype=np.int32).reshape(-1))
        fp = np.ascontiguousarray(np.asarray(env_first_point, dtype=np.int32).reshape(-1))
        assert vis_points.dtype == np.float32 and vis_points.flags["C_CONTIGUOUS"]
        _kin_lib().oracle_instrument_visual(_p(self.xform), _p(lp), _p(sl), len(sl), _p(vis_points), _p(fp), self.n)
        return vis_points


# ---------------------------------------------------------------- cutting and heating
def _cut_lib():
    lb = lib()
    if not getattr(lb, "_cut_ready", False):
        P, I, F = C.c_void_p, C.c_int, C.c_float
        lb.oracle_edge_breaker.argtypes = [P, P, P, P, P, I, F, F]
        lb.oracle_check_edge_breaker.argtypes = [P, P, P, P, I, P, I, P, P, P, P, F]
        lb.oracle_tetrahedron_breaker.argtypes = [P, P, P, P, P, I, F]
        lb.oracle_heat_propagation.argtypes = [P, P, P, P, I, F, F, F]
        lb.oracle_heat_update.argtypes = [P, P, P, P, P, I]
        lb.oracle_check_heat.argtypes = [P, P, P, P, P, F, I]
        lb.oracle_heat_laparoscope.argtypes = [P, P, P, P, P, P, P, F, F, I]
        lb.oracle_segment_triangle.argtypes = [P, P, P, P, P]
        lb.oracle_segment_triangle.restype = C.c_int
        lb.oracle_cut_edges.argtypes = [P, P, P, P, P, I, P, I, P, P, P, P, P]
        lb.oracle_update_active_values.argtypes = [P, P, P, I, I]
        lb._cut_ready = True
    return lb


def segment_triangle(pA, pB, pC, sA, sB) -> int:
    """checkSegmentTriangleIntersection (integrator.py:1471-1518) on float32 points."""
    f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(3))
    a = [f(x) for x in (pA, pB, pC, sA, sB)]
    return int(_cut_lib().oracle_segment_triangle(*[_p(x) for x in a]))


class OracleCutting:
    """Host restatement of ffsrl.cutting.SimCutting: the same state and calls over numpy
    copies, each call a serial loop in thread order (integrator.py:700-918, 1153-1185,
    1406-1518, 1583-1605).  ``a`` holds every array by the SimCutting / SimModelDO name."""

    ARRAYS = ("edgeBreaker", "tetrahedronBreaker", "flipEdge", "flipTetrahedron", "tetrahedronHeat",
              "tetrahedronNewHeat", "vertexHeat", "edgesToTriangles", "tetrahedronNeighbors",
              "tetrahedronToTriangle", "triangleToTetrahedron", "sqrtValues")
    MODEL = ("vertex", "predictedVertex", "edge", "edgeRestLength", "activeEdge", "tetrahedron",
             "tetrahedronRestVolume", "activeTetrahedron", "triangle", "triToEnv", "hole", "laparoscopeTip")

    GLOBALS = ("globalBreakFactor", "globalBreakThreshold", "globalHeatConduction", "globalHeatTransfer",
               "globalHeatLoss", "globalHeatLimit", "globalHeatSphereRadius", "globalHeatQuantum")
    DTYPES = {"flipEdge": np.int32, "flipTetrahedron": np.int32, "edgesToTriangles": np.int32,
              "tetrahedronNeighbors": np.int32, "tetrahedronToTriangle": np.int32, "triangleToTetrahedron": np.int32,
              "edge": np.int32, "tetrahedron": np.int32, "triangle": np.int32, "triToEnv": np.int32,
              "hole": np.int32, "edgeToEnv": np.int32}

    def __init__(self, arrays: dict, params: dict | None = None):
        """``arrays`` by name (see ARRAYS, MODEL and ``edgeToEnv``), copied as flat
        float32 / int32; ``params`` the model's global factors (default 1.0)."""
        self.a = {k: np.ascontiguousarray(np.asarray(v, dtype=self.DTYPES.get(k, np.float32)).reshape(-1)).copy()
                  for k, v in arrays.items()}
        self.g = {k: 1.0 for k in self.GLOBALS}
        self.g.update(params or {})
        self.E, self.T, self.F = len(self.a["edgeRestLength"]), len(self.a["tetrahedronRestVolume"]), \
            len(self.a["triToEnv"])

    @classmethod
    def from_cutting(cls, cutting):
        """Host copy of a SimCutting's state and its model's arrays."""
        c = lambda t: t.detach().cpu().numpy()
        m = cutting.model
        arrays = {k: c(getattr(cutting, k)) for k in cls.ARRAYS}
        arrays.update({k: c(getattr(m, k)) for k in cls.MODEL})
        arrays["edgeToEnv"] = c(cutting.edgeToEnv)
        return cls(arrays, {k: getattr(m, k) for k in cls.GLOBALS})

    def _q(self, k):
        return _p(self.a[k])

    def checkEdgeBreaking(self, breakFactor=None, breakThreshold=None, breakLimit=1.0):
        bf = self.g["globalBreakFactor"] if breakFactor is None else breakFactor
        bt = self.g["globalBreakThreshold"] if breakThreshold is None else breakThreshold
        lb, q = _cut_lib(), self._q
        lb.oracle_edge_breaker(q("predictedVertex"), q("edge"), q("edgeRestLength"), q("activeEdge"), q("edgeBreaker"),
                               self.E, float(bf), float(bt))
        lb.oracle_check_edge_breaker(q("edgeBreaker"), q("edge"), q("activeEdge"), q("flipEdge"), self.E,
                                     q("tetrahedron"), self.T, q("activeTetrahedron"), q("flipTetrahedron"),
                                     q("edgesToTriangles"), q("hole"), float(breakLimit))

    def checkTetrahedronBreaking(self, breakFactor=None):
        bf = self.g["globalBreakFactor"] if breakFactor is None else breakFactor
        q = self._q
        _cut_lib().oracle_tetrahedron_breaker(q("predictedVertex"), q("tetrahedron"), q("tetrahedronRestVolume"),
                                              q("activeTetrahedron"), q("tetrahedronBreaker"), self.T, float(bf))

    def propagateHeat(self, heatConduction=None, heatTransfer=None, heatLoss=None):
        c = self.g["globalHeatConduction"] if heatConduction is None else heatConduction
        t = self.g["globalHeatTransfer"] if heatTransfer is None else heatTransfer
        lo = self.g["globalHeatLoss"] if heatLoss is None else heatLoss
        lb, q = _cut_lib(), self._q
        lb.oracle_heat_propagation(q("activeTetrahedron"), q("tetrahedronNeighbors"), q("tetrahedronHeat"),
                                   q("tetrahedronNewHeat"), self.T, float(c), float(t), float(lo))
        lb.oracle_heat_update(q("tetrahedronHeat"), q("tetrahedronNewHeat"), q("activeTetrahedron"), q("tetrahedron"),
                              q("vertexHeat"), self.T)

    def checkHeat(self, heatLimit=None, volumeProportional=False):
        hl = self.g["globalHeatLimit"] if heatLimit is None else heatLimit
        q = self._q
        _cut_lib().oracle_check_heat(q("tetrahedronHeat"), q("flipTetrahedron"),
                                     q("tetrahedronRestVolume") if volumeProportional else None,
                                     q("tetrahedronToTriangle"), q("hole"), float(hl), self.T)

    def heatLaparoscope(self, heatSphereRadius=None, heatQuantum=None):
        r = self.g["globalHeatSphereRadius"] if heatSphereRadius is None else heatSphereRadius
        qn = self.g["globalHeatQuantum"] if heatQuantum is None else heatQuantum
        q = self._q
        _cut_lib().oracle_heat_laparoscope(q("triangle"), q("vertex"), q("activeTetrahedron"),
                                           q("tetrahedronHeat"), q("triangleToTetrahedron"), q("laparoscopeTip"),
                                           q("triToEnv"), float(r), float(qn), self.F)

    def cutLaparoscope(self):
        q = self._q
        _cut_lib().oracle_cut_edges(q("vertex"), q("laparoscopeTip"), q("edge"), q("activeEdge"), q("flipEdge"),
                                    self.E, q("tetrahedron"), self.T, q("activeTetrahedron"), q("flipTetrahedron"),
                                    q("edgesToTriangles"), q("hole"), q("edgeToEnv"))

    def updateActiveValues(self, steps=5):
        lb, q = _cut_lib(), self._q
        lb.oracle_update_active_values(q("flipEdge"), q("activeEdge"), q("sqrtValues"), int(steps), self.E)
        lb.oracle_update_active_values(q("flipTetrahedron"), q("activeTetrahedron"), q("sqrtValues"), int(steps),
                                       self.T)
