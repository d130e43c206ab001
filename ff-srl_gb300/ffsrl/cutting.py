"""Tissue cutting and heating of a SimModelDO (reference ``FF_SRL/FF_SRL/integrator.py:700-918,
1153-1185, 1406-1518, 1583-1605``; state ``model.py:332-348``; maps ``model.py:207-255``).

The reference allocates the state per simMesh and keeps the kernels' launches commented
out of its legacy step (``integrator.py:2182-2230``).  ``SimCutting`` holds that state for
every env of a model (env-major, like the model's own arrays) and launches the library's
kernels on it:

* ``checkEdgeBreaking`` -- ``edgeBreakerKernel`` then ``checkEdgeBreakerKernel``;
* ``checkTetrahedronBreaking`` -- ``tetrahedronBreaker``;
* ``propagateHeat`` -- ``tetrahedronHeatPropagation`` then ``tetrahedronHeatUpdate``;
* ``checkHeat`` -- ``checkTetrahedronHeat`` (or the volume-proportional form);
* ``heatLaparoscope`` -- ``heatLaparoscope`` with each env's own instrument;
* ``cutLaparoscope`` -- ``findIntersectingEdges`` with each env's clamp triangle;
* ``updateActiveValues`` -- ``inDeCreaseActiveValues`` on the edges and the tets.

They write the model's ``activeEdge``, ``activeTetrahedron`` and ``hole`` arrays, which the
reference-shaped step reads live.  The batched step packs them into its plan, so a call
that changes them bumps ``model.topologyVersion`` and the integrator rebuilds its plan; a
call that changes nothing (no edge broke, no tet overheated) leaves the plan as it is.

The element maps the reference reads from its USD assets (``mapping:edgeToTriangles``,
``triangleToTetrahedron``, ``tetrahedronToTriangles``, ``tetrahedronNeighbors``) are taken
from a mesh dict when it carries them (``edge_to_triangles`` [E, 2],
``triangle_to_tetrahedron`` [F], ``tetrahedron_to_triangles`` [T, 4],
``tetrahedron_neighbors`` [T, 4], mesh-local ids) and built by ``topology_maps`` otherwise.
"""

from __future__ import annotations

import contextlib

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr

IN_DE_CREASE_STEPS = 5  # integrator.py:9


def fade_table(steps: int = IN_DE_CREASE_STEPS) -> np.ndarray:
    """sqrt(k / steps), k = 0..steps, as float32 (model.py:765-766)."""
    return np.sqrt(np.array([k * (1.0 / steps) for k in range(steps + 1)], dtype=np.float64)).astype(np.float32)


def _classes(rows: np.ndarray) -> np.ndarray:
    """Class id per row; rows holding the same vertex set share one."""
    if not len(rows):
        return np.zeros(0, dtype=np.int64)
    return np.unique(np.sort(rows, axis=1), axis=0, return_inverse=True)[1].reshape(-1)


def _first_two(cls: np.ndarray, ids: np.ndarray, num: int) -> tuple[np.ndarray, np.ndarray]:
    """For each class c < num, the lowest and second-lowest id among rows of class c
    (-1 where there are fewer)."""
    first = np.full(num, -1, dtype=np.int64)
    second = np.full(num, -1, dtype=np.int64)
    if not len(cls):
        return first, second
    o = np.lexsort((ids, cls))
    c, i = cls[o], ids[o]
    start = np.ones(len(c), dtype=bool)
    start[1:] = c[1:] != c[:-1]
    first[c[start]] = i[start]
    nxt = np.zeros(len(c), dtype=bool)
    nxt[1:] = start[:-1] & ~start[1:]                          # the second row of a class
    second[c[nxt]] = i[nxt]
    return first, second


def topology_maps(tetrahedron, triangle, edge) -> dict:
    """The reference's element maps of one mesh (mesh-local ids, -1 for none):

    * ``tetrahedron_neighbors`` [T, 4]: entry i is the tet sharing the face opposite vertex
      i (the face of the other three vertices);
    * ``tetrahedron_to_triangles`` [T, 4]: the surface triangle that is that face;
    * ``triangle_to_tetrahedron`` [F]: the tet one of whose faces the triangle is;
    * ``edge_to_triangles`` [E, 2]: the surface triangles holding both of the edge's
      vertices, in ascending id order.

    Where a face or an edge has more partners than the map holds (a non-manifold mesh),
    the lowest ids are kept."""
    tet = np.asarray(tetrahedron, dtype=np.int64).reshape(-1, 4)
    tri = np.asarray(triangle, dtype=np.int64).reshape(-1, 3)
    edg = np.asarray(edge, dtype=np.int64).reshape(-1, 2)
    T, F, E = len(tet), len(tri), len(edg)
    opp = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
    faces = tet[:, opp].reshape(-1, 3)                          # face 4t+i: opposite vertex i
    cls = _classes(np.concatenate([faces, tri]))
    fc, tc = cls[:4 * T], cls[4 * T:]
    K = int(cls.max()) + 1 if len(cls) else 0
    f1, f2 = _first_two(fc, np.arange(4 * T), K)               # tet faces per class
    g1, _ = _first_two(tc, np.arange(F), K)                    # surface triangles per class
    fid = np.arange(4 * T)
    other = np.where(f1[fc] == fid, f2[fc], f1[fc]) if T else np.zeros(0, np.int64)
    nbr = np.where(other > -1, other // 4, -1).reshape(T, 4)
    t2f = g1[fc].reshape(T, 4) if T else np.zeros((0, 4), np.int64)
    f2t = np.where(f1[tc] > -1, f1[tc] // 4, -1) if F else np.zeros(0, np.int64)
    e2f = np.full((E, 2), -1, dtype=np.int64)
    if E and F:
        tri_edges = tri[:, [[0, 1], [1, 2], [2, 0]]].reshape(-1, 2)
        ec = _classes(np.concatenate([edg, tri_edges]))
        K2 = int(ec.max()) + 1
        h1, h2 = _first_two(ec[E:], np.repeat(np.arange(F), 3), K2)
        e2f[:, 0], e2f[:, 1] = h1[ec[:E]], h2[ec[:E]]
    return {"tetrahedron_neighbors": nbr.astype(np.int32), "tetrahedron_to_triangles": t2f.astype(np.int32),
            "triangle_to_tetrahedron": f2t.astype(np.int32), "edge_to_triangles": e2f.astype(np.int32)}


MAP_KEYS = ("tetrahedron_neighbors", "tetrahedron_to_triangles", "triangle_to_tetrahedron", "edge_to_triangles")


def mesh_maps(mesh: dict) -> dict:
    """A mesh dict's own maps where it carries all four, else ``topology_maps`` of it."""
    if all(mesh.get(k) is not None for k in MAP_KEYS):
        return {k: np.asarray(mesh[k], dtype=np.int32) for k in MAP_KEYS}
    return topology_maps(mesh["tetrahedron"], mesh["triangle"], mesh["edge"])


def model_maps(model) -> dict:
    """The four maps over a model's env-major arrays (global ids): each distinct mesh's
    maps once, offset per env by the env's first tet and triangle; -1 stays -1."""
    per_mesh = [mesh_maps(m) for m in model.meshes]
    t0 = model.envTetStart[:-1].astype(np.int64)
    f0 = model.envTriStart[:-1].astype(np.int64)
    out = {k: [] for k in MAP_KEYS}
    for e, k in enumerate(model.envMesh):
        m = per_mesh[k]
        for key, base in (("tetrahedron_neighbors", t0[e]), ("tetrahedron_to_triangles", f0[e]),
                          ("triangle_to_tetrahedron", t0[e]), ("edge_to_triangles", f0[e])):
            a = m[key].astype(np.int64)
            out[key].append(np.where(a > -1, a + base, -1).reshape(-1))
    return {k: (np.concatenate(v) if v else np.zeros(0, np.int64)).astype(np.int32) for k, v in out.items()}


class SimCutting:
    """Cutting and heating state of every env of ``simModel`` and the reference's kernels
    over it.  Arrays (torch, on the model's device): ``edgeBreaker`` [E],
    ``tetrahedronBreaker`` [T], ``flipEdge`` [E], ``flipTetrahedron`` [T],
    ``tetrahedronHeat`` / ``tetrahedronNewHeat`` [T], ``vertexHeat`` [V], the maps
    ``edgesToTriangles`` [2E], ``tetrahedronNeighbors`` [4T], ``tetrahedronToTriangle`` [4T],
    ``triangleToTetrahedron`` [F], and the fade table ``sqrtValues``.  The model's
    ``hole`` array is the reference's ``holes``."""

    def __init__(self, simModel, maps: dict | None = None) -> None:
        simModel.require_cuda()
        m = simModel
        self.model = m
        dev = m.device
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        T, E, V = m.numTetrahedrons, m.numEdges, m.numVertices
        self.edgeBreaker = torch.zeros(E, **f32)
        self.tetrahedronBreaker = torch.zeros(T, **f32)
        self.flipEdge = torch.zeros(E, **i32)
        self.flipTetrahedron = torch.zeros(T, **i32)
        self.tetrahedronHeat = torch.zeros(T, **f32)
        self.tetrahedronNewHeat = torch.zeros(T, **f32)
        self.vertexHeat = torch.zeros(V, **f32)
        self._owner = torch.zeros(max(V, 1), **i32)
        mp = maps if maps is not None else model_maps(m)
        self.edgesToTriangles = torch.as_tensor(np.asarray(mp["edge_to_triangles"], np.int32).reshape(-1), **i32)
        self.tetrahedronNeighbors = torch.as_tensor(np.asarray(mp["tetrahedron_neighbors"], np.int32).reshape(-1), **i32)
        self.tetrahedronToTriangle = torch.as_tensor(np.asarray(mp["tetrahedron_to_triangles"], np.int32).reshape(-1),
                                                     **i32)
        self.triangleToTetrahedron = torch.as_tensor(np.asarray(mp["triangle_to_tetrahedron"], np.int32).reshape(-1),
                                                     **i32)
        if (self.edgesToTriangles.numel() != 2 * E or self.tetrahedronNeighbors.numel() != 4 * T or
                self.tetrahedronToTriangle.numel() != 4 * T or self.triangleToTetrahedron.numel() != m.numTriangles):
            raise ValueError("cutting maps do not match the model's element counts")
        self.sqrtValues = torch.as_tensor(fade_table(), **f32)
        self.edgeToEnv = torch.as_tensor(np.repeat(np.arange(m.numEnvs, dtype=np.int32), np.diff(m.envEdgeStart)),
                                         **i32)

    @property
    def flipEdges(self):
        """The name the reference's launches use for ``flipEdge`` (integrator.py:2200)."""
        return self.flipEdge

    @contextlib.contextmanager
    def _topology_guard(self, stream=None):
        """Bump ``model.topologyVersion`` when the enclosed calls (on ``stream``) change the
        model's active values or holes, so the batched step rebuilds its plan only then.

        The arrays are copied on the device before the calls and compared after them on
        the device, reduced to one flag that is read back once: each guarded call waits for
        its stream once, so it cannot be recorded into a CUDA graph."""
        m = self.model
        on = torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext()
        with on:
            before = [t.clone() for t in (m.activeEdge, m.activeTetrahedron, m.hole)]
        yield
        with on:
            changed = torch.zeros((), dtype=torch.bool, device=m.activeEdge.device)
            for a, b in zip(before, (m.activeEdge, m.activeTetrahedron, m.hole)):
                if a.numel():
                    changed |= (a != b).any()
            if bool(changed):
                m.topologyVersion += 1

    # ------------------------------------------------------------------ breaking
    def checkEdgeBreaking(self, breakFactor=None, breakThreshold=None, breakLimit: float = 1.0, stream=None):
        """edgeBreakerKernel then checkEdgeBreakerKernel with limit 1.0, as the legacy step
        launches them (integrator.py:2182-2208).  Factor and threshold default to the
        model's global values."""
        m, s = self.model, _lib.stream_handle(stream)
        bf = m.globalBreakFactor if breakFactor is None else breakFactor
        bt = m.globalBreakThreshold if breakThreshold is None else breakThreshold
        with self._topology_guard(stream):
            self._edge_breaking(m, s, bf, bt, breakLimit)

    def _edge_breaking(self, m, s, bf, bt, breakLimit):
        check(lib().ffsrl_edge_breaker(ptr(m.predictedVertex), ptr(m.edge), ptr(m.edgeRestLength), ptr(m.activeEdge),
                                       ptr(self.edgeBreaker), m.numEdges, float(bf), float(bt), s))
        check(lib().ffsrl_check_edge_breaker(ptr(self.edgeBreaker), ptr(m.edge), ptr(m.activeEdge),
                                             ptr(self.flipEdge), m.numEdges, ptr(m.tetrahedron), m.numTetrahedrons,
                                             ptr(m.activeTetrahedron), ptr(self.flipTetrahedron),
                                             ptr(self.edgesToTriangles), ptr(m.hole), float(breakLimit),
                                             ptr(self.edgeToEnv), ptr(m.envTetStartT), s))

    def checkTetrahedronBreaking(self, breakFactor=None, stream=None):
        """tetrahedronBreaker (integrator.py:777-818): accumulate each tet's overexpansion."""
        m = self.model
        bf = m.globalBreakFactor if breakFactor is None else breakFactor
        check(lib().ffsrl_tetrahedron_breaker(ptr(m.predictedVertex), ptr(m.tetrahedron),
                                              ptr(m.tetrahedronRestVolume), ptr(m.activeTetrahedron),
                                              ptr(self.tetrahedronBreaker), m.numTetrahedrons, float(bf),
                                              _lib.stream_handle(stream)))

    # ------------------------------------------------------------------ heat
    def propagateHeat(self, heatConduction=None, heatTransfer=None, heatLoss=None, stream=None):
        """tetrahedronHeatPropagation then tetrahedronHeatUpdate (integrator.py:2210-2230)."""
        m, s = self.model, _lib.stream_handle(stream)
        c = m.globalHeatConduction if heatConduction is None else heatConduction
        t = m.globalHeatTransfer if heatTransfer is None else heatTransfer
        lo = m.globalHeatLoss if heatLoss is None else heatLoss
        check(lib().ffsrl_heat_propagation(ptr(m.activeTetrahedron), ptr(self.tetrahedronNeighbors),
                                           ptr(self.tetrahedronHeat), ptr(self.tetrahedronNewHeat), m.numTetrahedrons,
                                           float(c), float(t), float(lo), s))
        check(lib().ffsrl_heat_update(ptr(self.tetrahedronHeat), ptr(self.tetrahedronNewHeat),
                                      ptr(m.activeTetrahedron), ptr(m.tetrahedron), ptr(self.vertexHeat),
                                      ptr(self._owner), m.numTetrahedrons, m.numVertices, s))

    def checkHeat(self, heatLimit=None, volumeProportional: bool = False, stream=None):
        """checkTetrahedronHeat, or checkTetrahedronHeatVolumeProportional
        (integrator.py:874-918): overheated tets are flipped and open their surface."""
        m = self.model
        hl = m.globalHeatLimit if heatLimit is None else heatLimit
        with self._topology_guard(stream):
            check(lib().ffsrl_check_heat(ptr(self.tetrahedronHeat), ptr(self.flipTetrahedron),
                                         ptr(m.tetrahedronRestVolume) if volumeProportional else None,
                                         ptr(self.tetrahedronToTriangle), ptr(m.hole), float(hl), m.numTetrahedrons,
                                         _lib.stream_handle(stream)))

    def heatLaparoscope(self, heatSphereRadius=None, heatQuantum=None, positions=None, stream=None):
        """heatLaparoscope (integrator.py:1153-1185): surface triangles near the midpoint of
        each env's clamp tips heat their tets.  Positions default to the model's current
        vertices (the reference has no call site that fixes the array)."""
        m = self.model
        r = m.globalHeatSphereRadius if heatSphereRadius is None else heatSphereRadius
        q = m.globalHeatQuantum if heatQuantum is None else heatQuantum
        x = m.vertex if positions is None else positions
        check(lib().ffsrl_heat_laparoscope(ptr(m.triangle), ptr(x), ptr(m.activeTetrahedron),
                                           ptr(self.tetrahedronHeat), ptr(self.triangleToTetrahedron),
                                           ptr(m.laparoscopeTip), ptr(m.triToEnv), float(r), float(q),
                                           m.numTriangles, _lib.stream_handle(stream)))

    # ------------------------------------------------------------------ cutting
    def cutLaparoscope(self, positions=None, stream=None):
        """findIntersectingEdges (integrator.py:1406-1458): edges crossing each env's clamp
        triangle are cut.  Positions default to the model's current vertices."""
        m = self.model
        x = m.vertex if positions is None else positions
        with self._topology_guard(stream):
            check(lib().ffsrl_cut_edges(ptr(x), ptr(m.laparoscopeTip), ptr(m.edge), ptr(m.activeEdge),
                                        ptr(self.flipEdge), m.numEdges, ptr(m.tetrahedron), m.numTetrahedrons,
                                        ptr(m.activeTetrahedron), ptr(self.flipTetrahedron), ptr(self.edgesToTriangles),
                                        ptr(m.hole), ptr(self.edgeToEnv), ptr(m.envTetStartT),
                                        _lib.stream_handle(stream)))

    def updateActiveValues(self, stream=None):
        """inDeCreaseActiveValues (integrator.py:1583-1605) on the edges and the tets: flipped
        elements fade out (or in) over IN_DE_CREASE_STEPS calls."""
        m, s = self.model, _lib.stream_handle(stream)
        with self._topology_guard(stream):
            check(lib().ffsrl_update_active_values(ptr(self.flipEdge), ptr(m.activeEdge), ptr(self.sqrtValues),
                                                   IN_DE_CREASE_STEPS, m.numEdges, s))
            check(lib().ffsrl_update_active_values(ptr(self.flipTetrahedron), ptr(m.activeTetrahedron),
                                                   ptr(self.sqrtValues), IN_DE_CREASE_STEPS, m.numTetrahedrons, s))
