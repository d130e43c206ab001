"""The library's host BVH build against the numpy restatement: identical topology."""

import numpy as np
import pytest

from bvh_oracle import build_bvh
from ffsrl import SimBVH, SimModelDO, meshgen as mg
from ffsrl.bvh import build_topology

KEYS = ("left_node", "first_tri_id", "tri_count", "level", "tri_id")


def _surface(mesh):
    pts = mesh["vertex"][mesh["point_to_vertex"][:, 1]]
    return pts, mesh["vis_face"]


def _check_same(points, faces, bins=8):
    a = build_topology(points, faces, bins)
    b = build_bvh(points, faces, bins)
    assert a["num_nodes"] == b["num_nodes"]
    assert a["max_level"] == b["max_level"]
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    np.testing.assert_array_equal(a["aabb_min"], b["aabb_min"])
    np.testing.assert_array_equal(a["aabb_max"], b["aabb_max"])
    return a


def test_beam_topology_bit_exact(built_lib):
    t = _check_same(*_surface(mg.beam()))
    assert t["num_nodes"] > 100


@pytest.mark.parametrize("target", [500, 3000])
def test_ellipsoid_topology_bit_exact(built_lib, target):
    _check_same(*_surface(mg.ellipsoid_for_tets(target, seed=3)))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_soup_topology_bit_exact(built_lib, seed):
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(300, 3)).astype(np.float32) * np.array([3.0, 1.0, 0.2], dtype=np.float32)
    faces = rng.integers(0, 300, size=(200, 3))
    _check_same(pts, faces, bins=8)


def test_bins_parameter(built_lib):
    _check_same(*_surface(mg.ellipsoid_for_tets(800, seed=5)), bins=4)


def test_single_triangle_root_is_leaf(built_lib):
    t = _check_same(np.eye(3, dtype=np.float32), np.array([[0, 1, 2]]))
    assert t["left_node"].tolist() == [-1]
    assert t["tri_count"].tolist() == [1]


def test_topology_covers_every_triangle_once(built_lib):
    pts, faces = _surface(mg.ellipsoid_for_tets(2000, seed=1))
    t = build_topology(pts, faces)
    leaf = t["left_node"] == -1
    covered = np.concatenate([t["tri_id"][f:f + c] for f, c in zip(t["first_tri_id"][leaf], t["tri_count"][leaf])])
    assert sorted(covered.tolist()) == list(range(len(faces)))
    SimBVH.validate(t, len(faces))


def test_npz_round_trip(built_lib, tmp_path):
    pool = [mg.ellipsoid_for_tets(600, seed=1), mg.ellipsoid_for_tets(900, seed=2)]
    m = SimModelDO([pool[0], pool[1], pool[0]], 3, "cpu")
    b = SimBVH("cpu", m, save=True, path=str(tmp_path / "b.npz"))
    c = SimBVH("cpu", m, load=True, path=str(tmp_path / "b.npz"))
    for k in ("leftNode", "firstTriId", "triCount", "level", "triId", "aabbMin", "aabbMax", "envNodeOffset"):
        assert np.array_equal(getattr(b, k).numpy(), getattr(c, k).numpy()), k
    assert b.numAllNodes == c.numAllNodes


def test_validate_rejects_bad_child(built_lib):
    pts, faces = _surface(mg.beam())
    t = build_topology(pts, faces)
    t["left_node"] = t["left_node"].copy()
    t["left_node"][0] = t["num_nodes"] - 1
    with pytest.raises(ValueError):
        SimBVH.validate(t, len(faces))


def test_npz_reference_layout(built_lib, tmp_path):
    # bvh.py:165-197: arr_0 triId, arr_1/arr_2 the boxes of the first env [numNodes, 3],
    # arr_3..arr_6 leftNode, firstTriId, triCount, level -- a file written that way loads
    mesh = mg.ellipsoid_for_tets(500, seed=4)
    m = SimModelDO(mesh, 2, "cpu")
    pts, faces = _surface(mesh)
    t = build_topology(pts, faces)
    np.savez(tmp_path / "ref.npz", t["tri_id"], t["aabb_min"], t["aabb_max"], t["left_node"], t["first_tri_id"],
             t["tri_count"], t["level"])
    b = SimBVH("cpu", m, load=True, path=str(tmp_path / "ref.npz"))
    for k in ("left_node", "first_tri_id", "tri_count", "level", "tri_id"):
        assert np.array_equal(b.topologies[0][k], t[k]), k
    assert b.numNodes == t["num_nodes"] and b.maxLevel == t["max_level"]
    b.saveBVH(str(tmp_path / "out.npz"))
    z = np.load(tmp_path / "out.npz")
    assert z.files == [f"arr_{k}" for k in range(7)]
    assert z["arr_1"].shape == (t["num_nodes"], 3) and np.array_equal(z["arr_3"], t["left_node"])
    # a file with fewer topologies than the model's distinct meshes is refused
    two = SimModelDO([mesh, mg.ellipsoid_for_tets(700, seed=5)], 2, "cpu")
    with pytest.raises(ValueError):
        SimBVH("cpu", two, load=True, path=str(tmp_path / "ref.npz"))
