"""Shading modes of the ray-cast renderer (render.py:17-25, 123-148, 350-409).

CPU: known answers of the oracle for each mode on a flat triangle facing the camera --
grayscale is the Lambert term, the normal map is n/2 + 1/2, the depth map repeats the
depth image, a linear texture is sampled back exactly, and envs without a texture fall
back to the vertex colour.  GPU: every mode, with textured and untextured meshes in one
batch, against the oracle (fused path bit-exact; reference-shaped path within 1e-5, its
normal sums use float atomics).
"""

import numpy as np
import pytest
import torch

import oracle
from ffsrl import RenderMode, SimBVH, SimIntegratorDO, SimModelDO, WarpRaycastRendererDO, meshgen as mg
from ffsrl import scenarios as sc

BIG = 100.0
R = 4


def _flat(texture=None, coords=None):
    mesh = mg.tiny_mesh([[-BIG, -BIG, 0], [BIG, -BIG, 0], [0, BIG, 0]], triangle=[[0, 1, 2]],
                        inverse_mass=[1.0, 1.0, 1.0])
    if texture is not None:
        mesh["texture"], mesh["tex_coords"] = texture, coords
    return mesh


def _render(meshes, mode):
    m = SimModelDO(meshes, len(meshes), "cpu", environmentGravity=(0.0, 0.0, 0.0), environmentGroundLevel=-100.0)
    bvh = SimBVH("cpu", m)
    r = WarpRaycastRendererDO("cpu", m, cameraPos=(0.0, 0.0, 1.0), resolution=R, mode="headless",
                              lightPos=(0.0, 0.0, 2.0), lightIntensity=0.25, render_mode=mode)
    vp = np.concatenate([mm["vertex"][mm["point_to_vertex"][:, 1]] for mm in meshes])
    return oracle.render(r, bvh, vp), r


def _ray_points(r):
    """Hit point (a, b) of each of a pixel's 4 rays on z = 0 (camera at z = 1, no rotation)."""
    W, tan = 2 * R, r.camera_tan
    pts = np.zeros((R, R, 4, 2))
    for py in range(R):
        for px in range(R):
            for q in range(4):
                et = (2 * py + q // 2) * W + 2 * px + q % 2
                x, y = et % W, W - et // W
                pts[py, px, q] = ((2 * x / W - 1) * tan, (2 * y / W - 1) * tan)
    return pts


def test_grayscale_normal_and_depth_maps(oracle_lib):
    (col, dep, _), _ = _render([_flat()], RenderMode.grayscale)
    np.testing.assert_allclose(col[0], 0.5, rtol=1e-6)  # lambert 0.25 * dot((0,0,1), (0,0,2))
    (col, _, _), _ = _render([_flat()], RenderMode.normal_map)
    np.testing.assert_allclose(col[0], np.broadcast_to([0.5, 0.5, 1.0], col[0].shape), rtol=1e-6)
    (col, dep, _), _ = _render([_flat()], RenderMode.depth_map)
    for c in range(3):
        np.testing.assert_array_equal(col[0, ..., c], dep[0])
    (col3, _, _), _ = _render([_flat()], RenderMode.vertex_color)
    (col1, _, _), _ = _render([_flat()], RenderMode.texture)  # no texture: the vertex colour
    np.testing.assert_array_equal(col1, col3)
    np.testing.assert_allclose(col3[0], 0.25, rtol=1e-6)


def test_linear_texture_is_sampled_back(oracle_lib):
    # texel (i, j) sits at first + j + i*S (render.py:139-142) and holds (i, j)/(S-1);
    # bilinear interpolation of a linear field is exact, so channel 0 reads the tex u and
    # channel 1 reads 1 - v at the hit point
    S = 9
    g = np.arange(S, dtype=np.float32) / (S - 1)
    tex = np.zeros((S, S, 3), np.float32)
    tex[..., 0] = g[:, None]
    tex[..., 1] = g[None, :]
    tex[..., 2] = 0.5
    vtx = np.array([[-BIG, -BIG], [BIG, -BIG], [0, BIG]])
    coords = ((vtx + BIG) / (2 * BIG)).astype(np.float32)
    (col, dep, _), r = _render([_flat(tex, coords)], RenderMode.texture)
    assert (dep[0] > 0).all()
    uv = (_ray_points(r) + BIG) / (2 * BIG)
    lam = 0.5
    np.testing.assert_allclose(col[0, ..., 0], (lam * uv[..., 0]).mean(axis=2), atol=2e-6)
    np.testing.assert_allclose(col[0, ..., 1], (lam * (1.0 - uv[..., 1])).mean(axis=2), atol=2e-6)
    np.testing.assert_allclose(col[0, ..., 2], lam * 0.5, atol=2e-6)


def test_constant_texture_and_per_env_fallback(oracle_lib):
    S = 4
    tex = np.full((S, S, 3), 0.8, np.float32)
    coords = np.array([[0.0, 0.0], [1.0, 0.0], [0.5, 1.0]], np.float32)
    plain = _flat()
    (col, _, _), _ = _render([_flat(tex, coords), plain, plain], RenderMode.texture)
    np.testing.assert_allclose(col[0], 0.4, rtol=1e-5)  # lambert 0.5 * texel 0.8
    np.testing.assert_allclose(col[1:], 0.25, rtol=1e-6)  # untextured envs: vertex colour 0.5


def test_texture_tables_per_distinct_mesh():
    S = 4
    tex = np.full((S, S, 3), 0.8, np.float32)
    a = _flat(tex, np.zeros((3, 2), np.float32))
    b = _flat()
    m = SimModelDO([a, b, a, b], 4, "cpu", environmentGravity=(0.0, 0.0, 0.0))
    assert m.hasTextures
    assert m.host["texture"].size == 3 * S * S  # stored once for the two envs that share it
    # one object per env (the soft mesh): (first face, first texel, S, first coord, first index)
    assert m.host["objectTexture"].reshape(-1, 5).tolist() == [[0, 0, S, 0, 0], [0, 0, 0, 0, 0]]
    assert m.host["envObjects"].reshape(4, 2).tolist() == [[0, 1], [1, 1]] * 2
    bad = _flat(tex, np.zeros((2, 2), np.float32))  # vis_face refers to tex coord 2
    with pytest.raises(ValueError):
        SimModelDO(bad, 1, "cpu")


def test_meshgen_texture_coordinates():
    mesh = mg.ellipsoid_for_tets(400, seed=1)
    t = mg.add_texture(mesh, size=16, seed=2)
    assert t["texture"].shape == (16, 16, 3) and t["texture"].min() >= 0 and t["texture"].max() <= 1
    assert t["tex_coords"].min() >= 0 and t["tex_coords"].max() <= 1
    assert np.array_equal(t["tex_indices"], mesh["vis_face"].reshape(-1))
    c = mg.add_texture(mesh, size=16, seed=2, per_corner=True)
    np.testing.assert_array_equal(c["tex_coords"][c["tex_indices"]], t["tex_coords"][t["tex_indices"]])
    assert "texture" not in mesh


def test_invalid_render_mode_is_rejected():
    with pytest.raises(ValueError):
        WarpRaycastRendererDO("cpu", SimModelDO(_flat(), 1, "cpu"), mode="headless", render_mode=7)


# ------------------------------------------------------------------------- GPU
def _textured_setup(n_env=4, res=24):
    base = [mg.ellipsoid_for_tets(1500, seed=7), mg.ellipsoid_for_tets(900, seed=8)]
    pool = [mg.add_texture(base[0], size=32, seed=1), base[1],
            mg.add_texture(base[1], size=17, seed=2, per_corner=True)]
    meshes = [pool[e % 3] for e in range(n_env)]
    m, meshes = sc.liver_model("cuda:0", n_env, meshes=meshes)
    assert m.hasTextures
    bvh = SimBVH("cuda:0", m)
    r = WarpRaycastRendererDO("cuda:0", m, resolution=res, mode="headless", verticalAperture=sc.fov_aperture(60.0),
                              horizontalAperture=sc.fov_aperture(60.0), lightPos=(0.3, 1.0, 0.5),
                              lightIntensity=0.8)
    pos, rot = sc.env_cameras(meshes, seed=3)
    r.setCameras(pos, rot)
    return m, bvh, r


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_render_modes_gpu_match_oracle(gpu, oracle_lib, fused):
    m, bvh, r = _textured_setup()
    r.fused = fused
    SimIntegratorDO("cuda:0").stepModel(m, 2)
    bvh.refitBVH()
    aabb = (bvh.aabbMin.cpu().numpy(), bvh.aabbMax.cpu().numpy())
    vp = m.allVisPoint.cpu().numpy()
    seen = {}
    for mode in range(5):
        r.render_mode = mode
        img = r.renderNew(bvh, m)
        torch.cuda.synchronize()
        r.checkErrors()
        col, dep, _ = oracle.render(r, bvh, vp, aabb=aabb)
        g_col, g_dep = img.cpu().numpy(), r.depthImages().cpu().numpy()
        assert (dep > 0).mean() > 0.05
        assert np.array_equal(g_dep, dep)
        if fused:
            assert np.array_equal(g_col, col), f"mode {mode}"
        else:
            assert np.abs(g_col - col).max() < 1e-5, f"mode {mode}"
        seen[mode] = g_col
    # the texture changes the textured envs only
    ot, eo = m.host["objectTexture"].reshape(-1, 5), m.host["envObjects"].reshape(-1, 2)
    tex_env = ot[eo[:, 0], 2] > 0  # the env's soft mesh has a texture
    assert not np.allclose(seen[1][tex_env], seen[3][tex_env], atol=1e-3)
    if fused:
        assert np.array_equal(seen[1][~tex_env], seen[3][~tex_env])
    else:  # each render sums the normals again with float atomics
        assert np.abs(seen[1][~tex_env] - seen[3][~tex_env]).max() < 1e-5
    print(f"[render modes] fused={fused}: modes 0-4 match the oracle, textured envs {int(tex_env.sum())}")


@pytest.mark.gpu
def test_render_mode_bad_value_is_rejected(gpu):
    m, bvh, r = _textured_setup(n_env=2, res=8)
    r.render_mode = 9
    from ffsrl._lib import FFSRLError
    with pytest.raises(FFSRLError):
        r.renderNew(bvh, m)
