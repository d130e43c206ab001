"""Array scene files carrying the reference's USD attribute schema (modelDO.py:545-700,
1646-1690): round trips, the schema's attribute names, the prim transform convention,
merged soft bodies, and models built from a file equal to models built from the arrays
(on CPU the host arrays, on the GPU a step and a render bit for bit)."""

import numpy as np
import pytest

from ffsrl import SimModelDO, meshgen as mg, scenarios as sc
from ffsrl import scene as scene_io

HOST_KEYS = ("vertex", "inverseMass", "tetrahedron", "tetrahedronRestVolume", "tetrahedronRestVolumeSigned",
             "tetrahedronDmInv", "edge", "edgeRestLength", "triangle", "allVisFace", "allVisPointColor",
             "pointToVertex", "texture", "texCoords", "texIndices", "objectTexture", "envObjects")


def _mesh():
    base = mg.ellipsoid_for_tets(400, seed=12)
    lo, hi = base["vertex"].min(axis=0), base["vertex"].max(axis=0)
    box = mg.rigid_box([lo[0] - 1, lo[1] - 1, lo[2] - 1], [hi[0] + 1, lo[1] - 0.5, hi[2] + 1])
    return mg.with_rigids(mg.add_texture(base, size=8, seed=1), [box])


def test_round_trip_and_schema_names(tmp_path):
    mesh = _mesh()
    p = tmp_path / "s.npz"
    sc.write_liver_scene(p, mesh, rigids=mesh["rigids"])
    z = np.load(p)
    for attr in ("extMesh:vertex", "extMesh:elem", "extMesh:edge", "extMesh:edgeRestLength", "extMesh:triangle",
                 "extMesh:inverseMass", "extMesh:tetrahedronRestVolume", "extMesh:inverseRestPosition", "points",
                 "faceVertexIndices", "primvars:displayColor", "mapping:pointToVertex", "simMesh",
                 "material:diffuse_texture", "primvars:st", "primvars:st:indices"):
        assert f"/World/Mesh0.{attr}" in z.files, attr
    assert "/World/Rigid0.simRigid" in z.files and "/World/Laparoscope.laparoscope:transforms" in z.files
    s = scene_io.read_scene(p)
    for key in ("vertex", "rest_vertex", "inverse_mass", "tetrahedron", "tetrahedron_rest_volume",
                "tetrahedron_rest_volume_signed", "edge", "edge_rest_length", "triangle", "vis_face",
                "point_to_vertex", "vis_point_color", "fixed", "texture", "tex_coords", "tex_indices"):
        assert np.array_equal(np.asarray(s.mesh[key]), np.asarray(mesh[key]).reshape(np.shape(s.mesh[key]))), key
    np.testing.assert_array_equal(s.mesh["tetrahedron_dm_inv"], np.asarray(mesh["tetrahedron_dm_inv"]).reshape(-1, 9))
    for key in ("vertex", "triangle", "color"):
        assert np.array_equal(s.mesh["rigids"][0][key], mesh["rigids"][0][key]), key
    im = mg.instrument_mesh()
    for key in ("points", "faces", "slot", "color"):
        assert np.array_equal(s.instrument["mesh"][key], im[key]), key


def test_model_from_file_equals_model_from_arrays(tmp_path):
    mesh = _mesh()
    p = tmp_path / "s.npz"
    sc.write_liver_scene(p, mesh, rigids=mesh["rigids"])
    a, _ = sc.liver_model("cpu", 3, meshes=[mesh] * 3)
    b, _ = sc.liver_model("cpu", 3, scene=p)
    for key in HOST_KEYS:
        assert np.array_equal(a.host[key], b.host[key]), key
    for key in ("base", "tip", "radius", "xform", "height"):
        assert np.array_equal(np.asarray(a.toolHost[key]), np.asarray(b.toolHost[key])), key
    assert np.array_equal(a.laparoscopeXForm.numpy(), b.laparoscopeXForm.numpy())
    assert len(b.meshes) == 1 and b.hasTextures and b.numEnvRigidsVisFaces == 12


def test_prim_transform_row_vector_convention(tmp_path):
    # USD applies a prim's local-to-world matrix to row vectors: p' = p M, translation in
    # the last row (utils.py:77-82, Gf.Matrix4d.Transform)
    mesh = mg.tiny_mesh([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], tetrahedron=[[3, 0, 1, 2]],
                        triangle=[[0, 1, 2]])
    p = tmp_path / "t.npz"
    scene_io.write_scene(p, mesh, params={"density": 1.06, "ksDistance": 0.5})
    z = dict(np.load(p))
    M = np.eye(4)
    M[:3, :3] = [[0, 1, 0], [-1, 0, 0], [0, 0, 1]]  # +90 degrees about z for row vectors
    M[3, :3] = [10, 20, 30]
    z["/World/Mesh0.xformOp:transform"] = M
    np.savez(p, **z)
    s = scene_io.read_scene(p)
    np.testing.assert_array_equal(s.mesh["vertex"], [[10, 21, 30], [9, 20, 30], [10, 20, 31], [10, 20, 30]])
    assert s.params["/World/Mesh0"] == {"density": 1.06, "ksDistance": 0.5}
    assert s.instrument is None


def test_several_soft_bodies_merge(tmp_path):
    a, b = mg.ellipsoid_for_tets(300, seed=1), mg.ellipsoid_for_tets(350, seed=2)
    p = tmp_path / "two.npz"
    scene_io.write_scene(p, [a, b])
    s = scene_io.read_scene(p)
    nv = len(a["vertex"])
    assert len(s.mesh["vertex"]) == nv + len(b["vertex"])
    assert np.array_equal(s.mesh["tetrahedron"][len(a["tetrahedron"]):], b["tetrahedron"] + nv)
    assert np.array_equal(s.mesh["point_to_vertex"][len(a["point_to_vertex"]):],
                          b["point_to_vertex"] + np.array([len(a["point_to_vertex"]), nv]))
    m = SimModelDO(str(p), 2, "cpu")
    assert m.numVertices == 2 * (nv + len(b["vertex"]))


def test_scene_without_soft_body_is_refused(tmp_path):
    p = tmp_path / "empty.npz"
    np.savez(p, **{"/World/Rigid0.simRigid": np.int32(1)})
    with pytest.raises(ValueError):
        scene_io.read_scene(p)


@pytest.mark.gpu
def test_model_from_file_steps_and_renders_like_arrays(gpu, tmp_path):
    import torch
    from ffsrl import SimBVH, SimIntegratorDO
    mesh = _mesh()
    p = tmp_path / "s.npz"
    sc.write_liver_scene(p, mesh, rigids=mesh["rigids"])
    out = []
    for kw in ({"meshes": [mesh] * 3}, {"scene": p}):
        m, meshes = sc.liver_model("cuda:0", 3, **kw)
        bvh = SimBVH("cuda:0", m)
        r = sc_renderer(m, meshes)
        m.graspNearest(torch.ones(3, dtype=torch.int32, device="cuda:0"))
        SimIntegratorDO("cuda:0").stepModel(m, 3)
        bvh.refitBVH()
        img = r.renderNew(bvh, m)
        torch.cuda.synchronize()
        out.append((m.vertex.cpu().numpy(), m.allVisPoint.cpu().numpy(), img.cpu().numpy()))
    for x, y in zip(*out):
        assert np.array_equal(x, y)
    assert (out[0][2] > 0).any()


def sc_renderer(m, meshes):
    from ffsrl import WarpRaycastRendererDO
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO("cuda:0", m, resolution=16, mode="headless", verticalAperture=ap, horizontalAperture=ap)
    r.setCameras(*sc.env_cameras(meshes, seed=2))
    return r
