"""Multi-object visual layout (modelDO.py:996-1127, 1231-1246, 1446-1473; bvh.py:66-74).

An env renders its soft mesh, its static rigid meshes and the instrument's visual mesh.
CPU: the layout of the concatenated arrays, the refit's face-shift table against a known
answer and the oracle's restatement of the reference arithmetic, the instrument's visual
points against hand-computed transforms, and the golden scene fixture (BVH topology
against the numpy build, boxes and images from the oracle).  GPU: the library's
instrument visual update, refit and render against the fixture bit for bit, and the
visual points after actions and steps against the oracle.
"""

import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden as mk  # noqa: E402
import oracle  # noqa: E402
from bvh_oracle import build_bvh  # noqa: E402
from ffsrl import SimBVH, SimModelDO, meshgen as mg  # noqa: E402
from ffsrl.bvh import reference_refit_source  # noqa: E402

TOPO_KEYS = ("left_node", "first_tri_id", "tri_count", "level", "tri_id")


def _tiny_scene(n_env=3):
    """M = 2 soft-mesh faces, Rg = 1 rigid face, Lf = 2 instrument faces per env."""
    mesh = mg.tiny_mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], triangle=[[0, 1, 2], [1, 3, 2]])
    rigid = {"vertex": np.array([[0, -1, 0], [1, -1, 0], [0, -1, 1]], np.float32), "triangle": [[0, 1, 2]]}
    inst = {"points": np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32),
            "faces": [[0, 1, 2], [0, 2, 3]], "slot": [6, 6, 4, 5], "color": np.full((4, 3), 0.9, np.float32)}
    m = SimModelDO(mg.with_rigids(mesh, [rigid]), n_env, "cpu", instrumentMesh=inst)
    return m, mesh, rigid, inst


def test_layout_of_objects():
    m, mesh, rigid, inst = _tiny_scene()
    # per env: 4 mesh points, 3 rigid points, 4 instrument points; 2 + 1 + 2 faces
    assert m.envVisPointStart.tolist() == [0, 11, 22, 33]
    assert m.envVisFaceStart.tolist() == [0, 5, 10, 15]
    assert m.envMapStart.tolist() == [0, 4, 8, 12] and m.numVisPoints == 12 and m.numAllVisPoints == 33
    assert m.envInstrumentPointStart.tolist() == [7, 18, 29]
    f = m.host["allVisFace"].reshape(-1, 3)
    assert f[5:10].tolist() == [[11, 12, 13], [12, 14, 13], [15, 16, 17], [18, 19, 20], [18, 20, 21]]
    vp = m.allVisPoint.numpy()
    np.testing.assert_array_equal(vp[15:18], rigid["vertex"])  # rigid points, static
    assert m.host["pointToVertex"].reshape(-1, 2)[:, 0].max() < 33
    assert (m.numEnvMeshesVisFaces, m.numEnvRigidsVisFaces, m.numEnvLaparoscopeVisFaces) == (2, 1, 2)
    # objects of each env: soft mesh from face 0, rigid from face 2, instrument from face 3
    assert m.host["objectTexture"].reshape(-1, 5)[:, 0].tolist() == [0, 2, 3]
    assert m.host["envObjects"].reshape(-1, 2).tolist() == [[0, 3]] * 3


def test_refit_shift_known_answer(oracle_lib):
    m, *_ = _tiny_scene()
    # env e's local face M = 2 boxed from env e+1's face 0, M + Rg = 3 from env e+1's face 2;
    # the last env wraps to env 0's faces 2 and 3 (its own global faces 12, 13 are shifted)
    expect = [0, 1, 5, 7, 4, 5, 6, 10, 12, 9, 10, 11, 2, 3, 14]
    assert reference_refit_source(m).tolist() == expect
    assert oracle.reference_refit_source(3, 2, 1, 2, m.envVisFaceStart[:-1]).tolist() == expect
    # no shift for one env, and none without extra objects
    m1, *_ = _tiny_scene(1)
    assert reference_refit_source(m1) is None
    plain = SimModelDO(mg.tiny_mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0]], triangle=[[0, 1, 2]]), 2, "cpu")
    assert reference_refit_source(plain) is None


@pytest.mark.parametrize("counts", [(5, 0, 3), (4, 2, 0), (3, 2, 2), (1, 1, 1)])
def test_refit_shift_matches_reference_arithmetic(oracle_lib, counts):
    M, Rg, Lf = counts
    N = 4
    mesh = mg.tiny_mesh(np.random.default_rng(0).uniform(size=(M + 2, 3)), triangle=[[k, k + 1, k + 2]
                                                                                      for k in range(M)])
    rig = [{"vertex": np.zeros((3, 3), np.float32), "triangle": [[0, 1, 2]] * Rg}] if Rg else []
    inst = None if Lf == 0 else {"points": np.zeros((3, 3), np.float32), "faces": [[0, 1, 2]] * Lf,
                                 "slot": [6, 6, 6], "color": np.zeros((3, 3), np.float32)}
    m = SimModelDO(mg.with_rigids(mesh, rig), N, "cpu", instrumentMesh=inst)
    got = reference_refit_source(m)
    ref = oracle.reference_refit_source(N, M, Rg, Lf, m.envVisFaceStart[:-1])
    assert got is not None and np.array_equal(got, ref)


def test_instrument_visual_known_answer(oracle_lib):
    # slot 6 = translation (10, 0, 0); slot 4 = rotation of 90 degrees about z then
    # translation (0, 5, 0); slot 5 = identity -- stored as transposes
    X = np.zeros((2, 7, 4, 4), np.float32)
    X[:] = np.eye(4, dtype=np.float32)
    T6 = np.eye(4); T6[:3, 3] = (10, 0, 0)
    T4 = np.array([[0, -1, 0, 0], [1, 0, 0, 5], [0, 0, 1, 0], [0, 0, 0, 1]], np.float64)
    X[1, 6], X[1, 4] = T6.T, T4.T
    o = oracle.OracleInstrument(X.reshape(2, 112), np.zeros(8), np.zeros((8, 3)), np.zeros((8, 3)))
    local = np.array([[1, 2, 3], [1, 2, 3], [1, 2, 3]], np.float32)
    vis = np.zeros((10, 3), np.float32)
    o.visual(local, [6, 4, 5], vis, [1, 5])
    np.testing.assert_array_equal(vis[1:4], local)  # env 0: identities
    np.testing.assert_array_equal(vis[5:8], [[11, 2, 3], [-2, 6, 3], [1, 2, 3]])
    assert not vis[[0, 4, 8, 9]].any()


def test_meshgen_instrument_and_box():
    im = mg.instrument_mesh(rod=10.0, clamp=1.0, radii=(0.2, 0.05, 0.05))
    z = im["points"][:, 2]
    rod, clamps = im["slot"] == 6, im["slot"] != 6
    np.testing.assert_allclose([z[rod].min(), z[rod].max()], [-5.2, 5.2], atol=1e-6)  # centred rod
    np.testing.assert_allclose([z[clamps].min(), z[clamps].max()], [-0.05, 1.05], atol=1e-6)  # from the pivot
    for p, f in ((im["points"], im["faces"]), (mg.rigid_box([0, 0, 0], [1, 2, 3])["vertex"],
                                                mg.rigid_box([0, 0, 0], [1, 2, 3])["triangle"])):
        P = np.asarray(p, np.float64)[np.asarray(f)]
        assert np.einsum("ij,ij->i", P[:, 0], np.cross(P[:, 1], P[:, 2])).sum() > 0  # closed, outward


def test_golden_scene_oracle(oracle_lib):
    import torch
    z = np.load(GOLDEN / "scene.npz")
    mesh, inst = mk.unpack_scene(z)
    m = mk.scene_model("cpu", mesh, inst)
    vis0 = oracle.OracleSim(m).vis_points(oracle.OracleInstrument.from_model(m))
    assert np.array_equal(vis0, z["vis_point_rest"])
    m.allVisPoint.copy_(torch.as_tensor(vis0))
    bvh = SimBVH("cpu", m)
    faces = m.host["allVisFace"].reshape(-1, 3)
    f0, f1, p0, p1 = int(m.envVisFaceStart[0]), int(m.envVisFaceStart[1]), 0, int(m.envVisPointStart[1])
    ref = build_bvh(vis0[p0:p1], faces[f0:f1] - p0)
    for key in TOPO_KEYS:
        assert np.array_equal(bvh.topologies[0][key], z[f"topo0_{key}"]), key
        assert np.array_equal(ref[key], z[f"topo0_{key}"]), key
    assert np.array_equal(bvh.refitSource.numpy(), z["refit_source"])
    oi = oracle.OracleInstrument(z["xform"], z["height"], z["tool_base"], z["tool_tip"])
    o = oracle.OracleSim(m, {"vertex": z["vertex"]})
    vis = o.vis_points(oi)
    assert np.array_equal(vis, z["vis_point"])
    lo, hi = oracle.refit(bvh, vis, m.host["allVisFace"])
    assert np.array_equal(lo, z["aabb_min"]) and np.array_equal(hi, z["aabb_max"])
    r = mk.renderer("cpu", m, [mesh] * mk.SCENE_ENVS)
    for mode in mk.SCENE_MODES:
        r.render_mode = mode
        col, dep, _ = oracle.render(r, bvh, vis, aabb=(lo, hi))
        assert np.array_equal(col, z[f"color_mode{mode}"]) and np.array_equal(dep, z["depth"])
    # the instrument and the rigid box are in view, the texture shows
    assert (z["depth"] > 0).mean() > 0.2
    assert np.abs(z["color_mode1"] - z["color_mode3"]).max() > 0.05


# ------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_golden_scene_gpu(gpu, fused):
    import torch
    z = np.load(GOLDEN / "scene.npz")
    mesh, inst = mk.unpack_scene(z)
    m = mk.scene_model("cuda:0", mesh, inst)
    # the instrument at its initial pose, placed by the library's own visual update
    assert np.array_equal(m.allVisPoint.cpu().numpy(), z["vis_point_rest"])
    bvh = SimBVH("cuda:0", m)
    for key in TOPO_KEYS:
        assert np.array_equal(bvh.topologies[0][key], z[f"topo0_{key}"]), key
    assert np.array_equal(bvh.refitSource.cpu().numpy(), z["refit_source"])
    m.setInstrument(z["xform"], z["height"])
    m.vertex.copy_(torch.as_tensor(z["vertex"], device="cuda:0"))
    m.transformSimMeshData()
    torch.cuda.synchronize()
    assert np.array_equal(m.allVisPoint.cpu().numpy(), z["vis_point"])
    bvh.refitBVH(fused=fused)
    torch.cuda.synchronize()
    assert np.array_equal(bvh.aabbMin.cpu().numpy(), z["aabb_min"])
    assert np.array_equal(bvh.aabbMax.cpu().numpy(), z["aabb_max"])
    r = mk.renderer("cuda:0", m, [mesh] * mk.SCENE_ENVS)
    r.fused = fused
    for mode in mk.SCENE_MODES:
        r.render_mode = mode
        img = r.renderNew(bvh, m)
        torch.cuda.synchronize()
        r.checkErrors()
        assert np.array_equal(r.depthImages().cpu().numpy(), z["depth"]), mode
        if fused:
            assert np.array_equal(img.cpu().numpy(), z[f"color_mode{mode}"]), mode
        else:  # its normal sums use float atomics
            assert np.abs(img.cpu().numpy() - z[f"color_mode{mode}"]).max() < 1e-5, mode


@pytest.mark.gpu
def test_instrument_visual_follows_actions_and_steps(gpu, oracle_lib):
    import torch
    from ffsrl import SimIntegratorDO, scenarios as sc
    meshes, _ = sc.mixed_meshes(5, pool_size=3, seed=4, t_lo=300, t_hi=700)
    m, _ = sc.liver_model("cuda:0", 5, meshes=meshes)
    o = oracle.OracleInstrument.from_model(m)
    rng = np.random.default_rng(11)
    integ = SimIntegratorDO("cuda:0")
    for _ in range(6):
        a = rng.uniform(-0.08, 0.08, size=(5, 5)).astype(np.float32)
        m.applyActions(torch.as_tensor(a, device="cuda:0"))
        o.apply_actions(a)
        integ.stepModel(m)  # ends with the visual update, as the reference's stepModel
    torch.cuda.synchronize()
    # the kinematics agree to rounding (their sines and cosines are not bit-exact)...
    X = m.laparoscopeXForm.cpu().numpy()
    assert np.abs(X - o.xform).max() / max(np.abs(o.xform).max(), 1.0) < 1e-5
    # ...and the visual points are exactly the oracle's transform of the library's transforms
    vis = m.allVisPoint.cpu().numpy()
    exp = vis.copy()
    o.xform[:] = X
    o.visual(m.instrumentMesh["points"], m.instrumentMesh["slot"], exp, m.envInstrumentPointStart)
    assert np.array_equal(vis, exp)
    # the env-list form updates only the listed envs
    ids = torch.tensor([1, 3], dtype=torch.int32, device="cuda:0")
    m.allVisPoint.zero_()
    m.transformSimLaparoscopeMeshData(env_ids=ids)
    torch.cuda.synchronize()
    got = m.allVisPoint.cpu().numpy()
    Lp = m.numEnvLaparoscopeVisPoints
    for e in range(5):
        s = slice(int(m.envInstrumentPointStart[e]), int(m.envInstrumentPointStart[e]) + Lp)
        if e in (1, 3):
            assert np.array_equal(got[s], exp[s])
        else:
            assert not got[s].any()
