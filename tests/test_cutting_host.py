"""Cutting and heating on the host: the element maps built from a mesh's topology, and the
CPU restatement of the reference's kernels (integrator.py:700-918, 1153-1185, 1406-1518,
1583-1605) against hand-worked answers."""

import math

import numpy as np
import pytest

import oracle
from ffsrl import cutting as cu, meshgen as mg

TWO_TETS = np.array([[0, 1, 2, 3], [1, 2, 3, 4]])


def test_two_tets_share_the_face_opposite_their_odd_vertex():
    # tet 0 = (0,1,2,3), tet 1 = (1,2,3,4): face (1,2,3) is opposite vertex 0 of tet 0
    # and opposite vertex 4 (slot 3) of tet 1
    surface = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]])
    edges = np.array([[0, 1], [1, 2], [1, 3], [2, 3], [0, 4]])
    m = cu.topology_maps(TWO_TETS, surface, edges)
    assert m["tetrahedron_neighbors"].tolist() == [[1, -1, -1, -1], [-1, -1, -1, 0]]
    # tet 0: faces opposite 1, 2, 3 are (0,2,3), (0,1,3), (0,1,2) = triangles 2, 1, 0
    assert m["tetrahedron_to_triangles"].tolist() == [[-1, 2, 1, 0], [5, 4, 3, -1]]
    assert m["triangle_to_tetrahedron"].tolist() == [0, 0, 0, 1, 1, 1]
    # (0,1) in triangles 0 and 1; (1,2) in 0 and 3; (1,3) in 1 and 4; (2,3) in 2 and 5;
    # (0,4) in none
    assert m["edge_to_triangles"].tolist() == [[0, 1], [0, 3], [1, 4], [2, 5], [-1, -1]]


def test_beam_maps_are_consistent():
    b = mg.beam(4, 3, 2)
    tet, tri, edge = b["tetrahedron"].reshape(-1, 4), b["triangle"].reshape(-1, 3), b["edge"].reshape(-1, 2)
    m = cu.topology_maps(tet, tri, edge)
    nbr, t2f, f2t, e2f = (m[k] for k in ("tetrahedron_neighbors", "tetrahedron_to_triangles",
                                         "triangle_to_tetrahedron", "edge_to_triangles"))
    opp = [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]
    for t in range(len(tet)):
        for i in range(4):
            face = set(tet[t][opp[i]].tolist())
            u = nbr[t, i]
            if u > -1:  # the neighbour holds the same face and points back
                assert face <= set(tet[u].tolist())
                assert t in nbr[u].tolist()
                assert t2f[t, i] == -1
            else:       # a boundary face is a surface triangle
                f = t2f[t, i]
                assert f > -1 and set(tri[f].tolist()) == face
    # every surface triangle belongs to exactly one tet face
    assert (f2t > -1).all()
    for f in range(len(tri)):
        assert f in t2f[f2t[f]].tolist()
    # a closed surface: each surface edge in two triangles, an interior edge in none
    for e, (a, c) in enumerate(edge):
        holders = [f for f in range(len(tri)) if a in tri[f] and c in tri[f]]
        want = (holders + [-1, -1])[:2]
        assert e2f[e].tolist() == want


def test_maps_of_a_mesh_dict_are_used_as_given():
    b = mg.beam(2, 1, 1)
    own = cu.topology_maps(b["tetrahedron"], b["triangle"], b["edge"])
    marked = dict(b, **{k: v.copy() for k, v in own.items()})
    marked["edge_to_triangles"][0] = [-1, -1]
    assert cu.mesh_maps(marked)["edge_to_triangles"][0].tolist() == [-1, -1]
    assert cu.mesh_maps(b)["edge_to_triangles"][0].tolist() == own["edge_to_triangles"][0].tolist()


def test_fade_table():
    t = cu.fade_table()
    assert t.dtype == np.float32 and len(t) == 6
    assert np.allclose(t, np.sqrt(np.arange(6) / 5.0))


def _two_tet_state(**over):
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], dtype=np.float32)
    surface = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]])
    edges = np.array([[0, 1], [1, 2], [1, 3], [2, 3], [0, 4]])
    m = cu.topology_maps(TWO_TETS, surface, edges)
    L0 = np.linalg.norm(x[edges[:, 1]] - x[edges[:, 0]], axis=1)
    a = {"vertex": x, "predictedVertex": x.copy(), "edge": edges, "edgeRestLength": L0,
         "activeEdge": np.ones(5), "tetrahedron": TWO_TETS, "tetrahedronRestVolume": np.array([1 / 6, 1 / 3]),
         "activeTetrahedron": np.ones(2), "triangle": surface, "triToEnv": np.zeros(6), "hole": np.zeros(6),
         "laparoscopeTip": np.zeros((4, 3)), "edgeBreaker": np.zeros(5), "tetrahedronBreaker": np.zeros(2),
         "flipEdge": np.zeros(5), "flipTetrahedron": np.zeros(2), "tetrahedronHeat": np.zeros(2),
         "tetrahedronNewHeat": np.zeros(2), "vertexHeat": np.zeros(5),
         "edgesToTriangles": m["edge_to_triangles"], "tetrahedronNeighbors": m["tetrahedron_neighbors"],
         "tetrahedronToTriangle": m["tetrahedron_to_triangles"],
         "triangleToTetrahedron": m["triangle_to_tetrahedron"], "sqrtValues": cu.fade_table(),
         "edgeToEnv": np.zeros(5)}
    a.update(over)
    return oracle.OracleCutting(a)


def test_edge_breaker_accumulates_overstretch(oracle_lib):
    o = _two_tet_state()
    o.a["predictedVertex"].reshape(-1, 3)[1] = [1.5, 0.0, 0.0]        # edge (0,1): 1 -> 1.5, C = 0.5
    o.checkEdgeBreaking(breakFactor=2.0, breakThreshold=0.2, breakLimit=1.0)
    assert o.a["edgeBreaker"][0] == pytest.approx((0.5 - 0.2) * 2.0, rel=1e-6)
    assert o.a["flipEdge"][0] == 0 and o.a["hole"].sum() == 0    # 0.6 is not beyond the limit
    o.checkEdgeBreaking(breakFactor=2.0, breakThreshold=0.2, breakLimit=1.0)
    assert o.a["edgeBreaker"][0] == pytest.approx(1.2, rel=1e-6)
    assert o.a["flipEdge"][0] == -1
    assert sorted(np.nonzero(o.a["hole"])[0].tolist()) == [0, 1]  # the edge's two surface triangles
    # the reference flips the tet flag at the edge's id (edge 0 -> tet 0): tet 0 holds (0,1)
    assert o.a["flipTetrahedron"].tolist() == [-1, 0]


def test_edge_breaker_flips_the_tet_at_the_edge_id(oracle_lib):
    o = _two_tet_state()
    o.a["predictedVertex"].reshape(-1, 3)[4] = [3.0, 3.0, 3.0]        # stretches (0,4) only: edge 4, in no tet
    o.checkEdgeBreaking(breakFactor=10.0, breakThreshold=0.0, breakLimit=1.0)
    assert o.a["flipEdge"][4] == -1
    assert o.a["flipTetrahedron"].tolist() == [0, 0]   # edge 4 >= 2 tets: the tet part is skipped
    o2 = _two_tet_state()
    o2.a["predictedVertex"].reshape(-1, 3)[2] = [0.0, 3.0, 0.0]       # stretches (1,2) = edge 1 and (2,3) = edge 3
    o2.checkEdgeBreaking(breakFactor=10.0, breakThreshold=0.0, breakLimit=1.0)
    assert o2.a["flipEdge"].tolist() == [0, -1, 0, -1, 0]
    # edge 1 flips tet 1 (its id), edge 3 has no tet of that id
    assert o2.a["flipTetrahedron"].tolist() == [0, -1]


def test_tet_breaker_counts_expansion_only(oracle_lib):
    o = _two_tet_state()
    o.a["predictedVertex"].reshape(-1, 3)[3] = [0.0, 0.0, 2.0]        # tet 0: volume 1/6 -> 2/6
    o.checkTetrahedronBreaking(breakFactor=3.0)
    assert o.a["tetrahedronBreaker"][0] == pytest.approx((2 / 6 - 1 / 6) * 3.0, rel=1e-5)
    # tet 1 = (1,2,3,4): signed volume dot(cross(p2-p1, p3-p1), p4-p1)/6 against 1/3
    x = o.a["predictedVertex"].reshape(-1, 3).astype(np.float64)
    v = np.dot(np.cross(x[2] - x[1], x[3] - x[1]), x[4] - x[1]) / 6.0
    assert o.a["tetrahedronBreaker"][1] == pytest.approx(max(v - 1 / 3, 0.0) * 3.0, abs=1e-6)


def test_heat_conducts_between_neighbours(oracle_lib):
    o = _two_tet_state()
    o.a["tetrahedronHeat"][:] = [10.0, 0.0]
    o.propagateHeat(heatConduction=0.5, heatTransfer=0.4, heatLoss=0.1)
    # tet 0: 10 * 0.9 + (0 - 10) * 0.5 * 0.4 = 7; tet 1: 0 + (10 - 0) * 0.5 * 0.4 = 2
    assert o.a["tetrahedronHeat"].tolist() == pytest.approx([7.0, 2.0])
    # vertices 1, 2, 3 are in both tets: the later tet (1) writes last
    assert o.a["vertexHeat"].tolist() == pytest.approx([7 / 4, 2 / 4, 2 / 4, 2 / 4, 2 / 4])
    o.a["activeTetrahedron"][1] = 0.0
    o.propagateHeat(heatConduction=0.5, heatTransfer=0.4, heatLoss=0.1)
    assert o.a["tetrahedronHeat"].tolist() == pytest.approx([6.3, 0.0])  # no exchange with an inactive tet


def test_check_heat_opens_the_surface(oracle_lib):
    o = _two_tet_state()
    o.a["tetrahedronHeat"][:] = [5.0, 1.0]
    o.checkHeat(heatLimit=2.0)
    assert o.a["flipTetrahedron"].tolist() == [-1, 0]
    assert sorted(np.nonzero(o.a["hole"])[0].tolist()) == [0, 1, 2]  # tet 0's three surface faces
    # volume-proportional: limit * rest volume = 6 * (1/6, 1/3) = (1, 2) -> both exceed
    o2 = _two_tet_state()
    o2.a["tetrahedronHeat"][:] = [1.5, 2.5]
    o2.a["flipTetrahedron"][:] = [3, 0]
    o2.checkHeat(heatLimit=6.0, volumeProportional=True)
    assert o2.a["flipTetrahedron"].tolist() == [-1, -1]              # set whatever it was
    assert o2.a["hole"].tolist() == [1] * 6


def test_heat_laparoscope_heats_triangles_in_reach(oracle_lib):
    o = _two_tet_state()
    tips = np.zeros((4, 3), dtype=np.float32)
    tips[1], tips[2] = [0.2, 0.2, -0.1], [0.2, 0.2, -0.3]   # centre (0.2, 0.2, -0.2) below face (0,1,2)
    o.a["laparoscopeTip"] = tips.reshape(-1)
    o.heatLaparoscope(heatSphereRadius=0.25, heatQuantum=1.5)
    # within 0.25: only triangle 0 (z = 0 plane, distance 0.2) -> tet 0
    assert o.a["tetrahedronHeat"].tolist() == [1.5, 0.0]
    o.heatLaparoscope(heatSphereRadius=10.0, heatQuantum=1.0)      # every triangle: 3 per tet
    assert o.a["tetrahedronHeat"].tolist() == [4.5, 3.0]


def test_segment_triangle_cases(oracle_lib):
    A, B, C = [0, 0, 0], [1, 0, 0], [0, 1, 0]
    assert oracle.segment_triangle(A, B, C, [0.2, 0.2, -1], [0.2, 0.2, 1]) == 1
    assert oracle.segment_triangle(A, B, C, [0.8, 0.8, -1], [0.8, 0.8, 1]) == 0   # outside (s + t > 1)
    assert oracle.segment_triangle(A, B, C, [0.2, 0.2, 0.5], [0.2, 0.2, 1]) == 0  # r > 1: short of the plane
    assert oracle.segment_triangle(A, B, C, [0.1, 0.1, 0], [0.3, 0.1, 0]) == 2    # in the plane
    assert oracle.segment_triangle(A, B, C, [0.1, 0.1, 1], [0.3, 0.1, 1]) == 0    # parallel, off the plane
    assert oracle.segment_triangle(A, B, [2, 0, 0], [0, 0, -1], [0, 0, 1]) == -1  # degenerate triangle


def test_cut_edges_crossing_the_clamps(oracle_lib):
    o = _two_tet_state()
    # clamp triangle (rod tip, right, left) = tips 0, 2, 1 in the plane x = 0.5, bounded by
    # y, z >= -0.5 and y + z <= 0.3: edge (0,1) crosses it at y = z = 0; (1,2), (1,3) and
    # (0,4) cross the plane at y + z = 0.5, 0.5 and 1, outside it; (2,3) lies in x = 0
    tips = np.zeros((4, 3), dtype=np.float32)
    tips[0], tips[1], tips[2] = [0.5, -0.5, -0.5], [0.5, 0.8, -0.5], [0.5, -0.5, 0.8]
    o.a["laparoscopeTip"] = tips.reshape(-1)
    o.cutLaparoscope()
    assert o.a["flipEdge"].tolist() == [-1, 0, 0, 0, 0]
    assert sorted(np.nonzero(o.a["hole"])[0].tolist()) == [0, 1]
    assert o.a["flipTetrahedron"].tolist() == [-1, 0]   # tet 0 holds (0,1); tet 1 does not


def test_active_values_fade_out_and_in(oracle_lib):
    o = _two_tet_state()
    o.a["flipEdge"][:] = [-1, 1, 0, 7, -5]
    seen = []
    for _ in range(6):
        o.updateActiveValues()
        seen.append(o.a["activeEdge"].copy())
    s = np.array(seen)
    r = lambda k: math.sqrt(k / 5)
    assert s[:, 0] == pytest.approx([r(4), r(3), r(2), r(1), r(0), r(0)], abs=1e-7)  # out over five calls
    assert s[:, 1] == pytest.approx([r(1), r(2), r(3), r(4), r(5), r(5)], abs=1e-7)  # in over five calls
    assert (s[:, 2] == 1.0).all()          # never flipped
    assert (s[:, 3] == 1.0).all()          # a counter beyond the table is left alone
    assert s[0, 4] == 0.0                  # -5: the last step down, then done
    assert o.a["flipEdge"].tolist() == [0, 0, 0, 7, 0]


def test_scene_files_carry_the_maps(tmp_path):
    from ffsrl import scene
    b = dict(mg.beam(3, 2, 2))
    b.update(cu.topology_maps(b["tetrahedron"], b["triangle"], b["edge"]))
    p = tmp_path / "cut.npz"
    scene.write_scene(p, b)
    m = scene.read_scene(p).mesh
    for k in cu.MAP_KEYS:
        assert np.array_equal(np.asarray(m[k]), b[k]), k
    assert cu.mesh_maps(m)["edge_to_triangles"].shape == (len(b["edge"]), 2)
