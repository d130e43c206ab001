"""Known-answer tests of the CPU oracle (the reference ships no golden vectors).

Each case has an answer derived by hand from the reference kernel it exercises; they pin
the oracle that every GPU parity test is checked against.
"""

import math

import numpy as np
import pytest

import oracle
from bvh_oracle import build_bvh
from ffsrl import SimModelDO, SimBVH, WarpRaycastRendererDO, _lib as L, meshgen as mg


def model(mesh, flags, n_env=1, **kw):
    kw.setdefault("environmentGravity", (0.0, 0.0, 0.0))
    kw.setdefault("environmentGroundLevel", -100.0)
    kw.setdefault("simSubsteps", 1)
    kw.setdefault("simConstraintsSteps", 1)
    return SimModelDO(mesh, n_env, "cpu", constraints=flags, **kw)


def test_distance_single_edge_known_answer(oracle_lib):
    # integrator.py:65-109: A (w=1) and B (w=3), rest 1, stretched to 1.5 along x:
    # delta = -C n kS / (wA+wB) = (-0.125,0,0); A += 0.125, B -= 0.375
    mesh = mg.tiny_mesh([[0, 1, 0], [1, 1, 0]], edge=[[0, 1]], inverse_mass=[1.0, 3.0])
    m = model(mesh, L.DISTANCE)
    o = oracle.OracleSim(m, {"vertex": [[0, 1, 0], [1.5, 1, 0]]})
    o.step(1)
    np.testing.assert_allclose(o.a["vertex"], [[0.125, 1, 0], [1.125, 1, 0]], atol=1e-7)
    dt = np.float32(m.simDt)
    np.testing.assert_allclose(o.a["velocity"][1], [-0.375 / dt, 0, 0], rtol=1e-6)


def test_distance_fixed_pair_is_skipped(oracle_lib):
    mesh = mg.tiny_mesh([[0, 1, 0], [1, 1, 0]], edge=[[0, 1]], inverse_mass=[0.0, 0.0])
    o = oracle.OracleSim(model(mesh, L.DISTANCE), {"vertex": [[0, 1, 0], [2, 1, 0]]})
    o.step(1)
    np.testing.assert_array_equal(o.a["vertex"], [[0, 1, 0], [2, 1, 0]])


def _tet(neg=True):
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    t = [[0, 2, 1, 3]] if neg else [[0, 1, 2, 3]]
    return x, t


def test_volume_restores_one_sixth_of_deficit(oracle_lib):
    # integrator.py:444-504 with equal masses: the correction q_i*dlambda*m_i has no 1/6
    # on the gradient, so to first order it restores C/6 of the volume deficit C.
    x, t = _tet(neg=True)
    mesh = mg.tiny_mesh(x, tetrahedron=t)
    s = 0.99
    o = oracle.OracleSim(model(mesh, L.VOLUME), {"vertex": x * s})
    o.step(1)
    v0 = 1.0 / 6.0
    vol_before = v0 * s ** 3
    a, b, c, d = o.a["vertex"][[0, 2, 1, 3]].astype(np.float64)
    vol_after = abs(np.dot(np.cross(b - a, c - a), d - a)) / 6.0
    C = v0 - vol_before
    assert vol_after > vol_before
    assert (vol_after - vol_before) / C == pytest.approx(1.0 / 6.0, rel=2e-2)


def test_neohookean_rest_state_is_balanced(oracle_lib):
    # integrator.py:578-698: at F = I the hydrostatic term (C = -mu/lambda) and the
    # deviatoric term (C = sqrt(3), gradient Dm^-T / sqrt(3)) cancel to first order when
    # the compliance dominates w.
    x, t = _tet(neg=True)
    x = x * 0.01
    mesh = mg.tiny_mesh(x, tetrahedron=t, inverse_mass=[1.0, 1.0, 1.0, 1.0])
    m = model(mesh, L.NEOHOOKEAN, globalVolumeCompliance=1e-2, globalDeviatoricCompliance=2e-2)
    o = oracle.OracleSim(m, {"vertex": x})
    o.step(1)
    disp = np.abs(o.a["vertex"] - x).max()
    # the individual hydrostatic displacement would be ~ mu dt^2 V0 |grad| ~ 1e-9 here
    dt = m.simDt
    single = (1 / 2e-2) * dt * dt * (0.01 ** 3 / 6) * (1 / 0.01)
    assert disp < 1e-3 * single + 1e-12


def test_neohookean_stretched_tet_contracts(oracle_lib):
    x, t = _tet(neg=True)
    x = x * 0.01
    mesh = mg.tiny_mesh(x, tetrahedron=t)
    m = model(mesh, L.NEOHOOKEAN, globalVolumeCompliance=1e-9, globalDeviatoricCompliance=1e-3)
    xs = x * np.array([1.2, 1.0, 1.0])
    o = oracle.OracleSim(m, {"vertex": xs})
    o.step(1)
    ext = o.a["vertex"][:, 0].max() - o.a["vertex"][:, 0].min()
    assert ext < 0.012 - 1e-6


def test_gravity_quirk_free_fall(oracle_lib):
    # integrator.py:40-63: v += g * invMass * dt * (1 - damping); x' = x + v dt
    mesh = mg.tiny_mesh([[0, 5, 0], [1, 5, 0]], inverse_mass=[2.0, 0.0])
    m = model(mesh, 0, environmentGravity=(0.0, -9.8, 0.0), environmentVelocityDampening=0.1)
    o = oracle.OracleSim(m)
    o.step(1)
    dt = np.float32(m.simDt)
    v = np.float32(-9.8) * np.float32(2.0) * dt * (np.float32(1.0) - np.float32(0.1))
    assert o.a["vertex"][0, 1] == pytest.approx(5.0 + v * dt, abs=1e-6)
    assert o.a["vertex"][1, 1] == 5.0  # invMass 0: velocity forced to 0


def test_ground_clamp(oracle_lib):
    mesh = mg.tiny_mesh([[0, 0.001, 0], [1, 5, 0]], inverse_mass=[1.0, 0.0])
    m = model(mesh, 0, environmentGravity=(0.0, -100.0, 0.0), environmentGroundLevel=0.0)
    o = oracle.OracleSim(m)
    o.step(1)
    assert o.a["vertex"][0, 1] == 0.0
    assert o.a["velocity"][0, 1] == pytest.approx(-0.001 / m.simDt, rel=1e-5)


def test_drag_pulls_half_way_to_right_clamp_tip(oracle_lib):
    # integrator.py:412-442: x -= |d| normalize(d) drag ks / 2 toward laparoscopeTip[4e+2]
    mesh = mg.tiny_mesh([[0.01, 0, 0], [1, 5, 0]], inverse_mass=[1.0, 0.0])
    m = model(mesh, L.DRAG)
    tip = m.toolHost["tip"].copy()
    tip[2] = [0, 0, 0]
    o = oracle.OracleSim(m, {"laparoscope_tip": tip, "active_drag_constraint": [1.0, 0.0]})
    o.step(1)
    np.testing.assert_allclose(o.a["vertex"][0], [0.005, 0, 0], atol=1e-9)


def _np_closest_bary(a, b, c, p):
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = ab @ ap, ac @ ap
    if d1 <= 0 and d2 <= 0:
        return np.array([1.0, 0, 0])
    bp = p - b
    d3, d4 = ab @ bp, ac @ bp
    if d3 >= 0 and d4 <= d3:
        return np.array([0, 1.0, 0])
    vc = d1 * d4 - d3 * d2
    if vc <= 0 and d1 >= 0 and d3 <= 0:
        v = d1 / (d1 - d3)
        return np.array([1 - v, v, 0])
    cp = p - c
    d5, d6 = ab @ cp, ac @ cp
    if d6 >= 0 and d5 <= d6:
        return np.array([0, 0, 1.0])
    vb = d5 * d2 - d1 * d6
    if vb <= 0 and d2 >= 0 and d6 <= 0:
        w = d2 / (d2 - d6)
        return np.array([1 - w, 0, w])
    va = d3 * d6 - d5 * d4
    if va <= 0 and (d4 - d3) >= 0 and (d5 - d6) >= 0:
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6))
        return np.array([0, w, 1 - w])
    den = 1 / (va + vb + vc)
    return np.array([1 - vb * den - vc * den, vb * den, vc * den])


def test_capsule_contact_response(oracle_lib):
    # integrator.py:981-1050, 1302-1355 with the triangle near the origin, where the
    # reference's barycentric triple (passed as a point to closestPointOnEdge) lies on
    # the capsule's side; expected value from a float64 evaluation of the same steps.
    A, B, Cc = np.array([0.6, 0.0, -0.2]), np.array([-0.2, 0.0, 0.6]), np.array([-0.2, 0.0, -0.2])
    mesh = mg.tiny_mesh([A, B, Cc], triangle=[[0, 1, 2]], inverse_mass=[1.0, 1.0, 1.0])
    m = model(mesh, L.COLLIDE)
    base, tip, rad = m.toolHost["base"].copy(), m.toolHost["tip"].copy(), m.toolHost["radius"].copy()
    base[0], tip[0], rad[0] = [0.1, -0.3, 0.1], [0.1, 0.9, 0.1], 0.4
    o = oracle.OracleSim(m, {"laparoscope_base": base, "laparoscope_tip": tip, "laparoscope_radius": rad})
    o.step(1)
    n = np.cross(B - A, Cc - A)
    n /= np.linalg.norm(n)
    centre = (A + B + Cc) * 0.3333
    cn = (tip[0] - base[0]) / np.linalg.norm(tip[0] - base[0])
    posA, posB = base[0] + cn * rad[0], tip[0] - cn * rad[0]
    t = n @ (centre - base[0]) / (n @ cn)
    ref = _np_closest_bary(A, B, Cc, base[0] + cn * t)
    d = posB - posA
    tt = np.clip(d @ (ref - posA) / (d @ d), 0, 1)
    sc = posA + d * tt
    bary = _np_closest_bary(A, B, Cc, sc)
    contact = A * bary[0] + B * bary[1] + Cc * bary[2]
    sv = sc - contact
    dist = np.linalg.norm(sv)
    assert dist <= rad[0]
    pv = (rad[0] / dist - 1) * sv
    resp = pv / np.linalg.norm(pv) * (np.linalg.norm(pv) / (bary @ bary))
    expect = np.stack([A, B, Cc]) - np.outer(bary, resp)
    np.testing.assert_allclose(o.a["vertex"], expect, atol=2e-6)
    assert o.a["laparoscope_in_collision"][0] == 1


def test_ray_depth_and_shading_known_answer(oracle_lib):
    # render.py:276-409, 661-724: camera at z=1 looking down -z at a large triangle in
    # z=0; each ray's t = sqrt(1 + a^2 + b^2), a = sx*tan*aspect, b = sy*tan.
    big = 100.0
    mesh = mg.tiny_mesh([[-big, -big, 0], [big, -big, 0], [0, big, 0]], triangle=[[0, 1, 2]],
                        inverse_mass=[1.0, 1.0, 1.0])
    m = model(mesh, 0)
    bvh = SimBVH("cpu", m)
    R = 4
    r = WarpRaycastRendererDO("cpu", m, cameraPos=(0.0, 0.0, 1.0), resolution=R, mode="headless",
                              lightPos=(0.0, 0.0, 2.0), lightIntensity=0.25)
    col, dep, nrm = oracle.render(r, bvh, m.host["vertex"][[0, 1, 2]])
    W = 2 * R
    tan = r.camera_tan
    expect = np.zeros((R, R))
    for py in range(R):
        for px in range(R):
            acc = 0.0
            for i in range(2):
                for j in range(2):
                    et = (2 * py + i) * W + 2 * px + j
                    x, y = et % W, W - et // W
                    a, b = (2 * x / W - 1) * tan, (2 * y / W - 1) * tan
                    acc += math.sqrt(1 + a * a + b * b) / 50.0
            expect[py, px] = acc / 4
    np.testing.assert_allclose(dep[0], expect, rtol=1e-6)
    # flat triangle: normal (0,0,1); lambert = 0.25 * 2 = 0.5; colour 0.5 -> 0.25
    np.testing.assert_allclose(nrm, [[0, 0, 1]] * 3, atol=1e-7)
    np.testing.assert_allclose(col[0], 0.25, rtol=1e-6)


def test_bvh_four_triangles_known_topology():
    # bvh.py:281-518 by hand: centroids at x = 1/3 + 10k; the root splits {0,1}|{2,3},
    # each child splits into single-triangle leaves.
    pts, faces = [], []
    for k in range(4):
        pts += [[10 * k, 0, 0], [10 * k + 1, 0, 0], [10 * k, 1, 0]]
        faces.append([3 * k, 3 * k + 1, 3 * k + 2])
    t = build_bvh(np.array(pts, dtype=np.float32), np.array(faces))
    assert t["left_node"].tolist() == [1, 3, 5, -1, -1, -1, -1]
    assert t["first_tri_id"].tolist() == [0, 0, 2, 0, 1, 2, 3]
    assert t["tri_count"].tolist() == [0, 0, 0, 1, 1, 1, 1]
    assert t["level"].tolist() == [0, 1, 1, 2, 2, 2, 2]
    assert t["tri_id"].tolist() == [0, 1, 2, 3]


def test_refit_known_boxes(oracle_lib):
    pts, faces = [], []
    for k in range(4):
        pts += [[10 * k, 0, 0], [10 * k + 1, 0, 0], [10 * k, 1, 0]]
        faces.append([3 * k, 3 * k + 1, 3 * k + 2])
    mesh = mg.tiny_mesh(pts, triangle=faces)
    m = model(mesh, 0)
    bvh = SimBVH("cpu", m)
    moved = np.array(pts, dtype=np.float32) + np.array([0, 0, 2], dtype=np.float32)
    lo, hi = oracle.refit(bvh, moved, m.host["allVisFace"])
    np.testing.assert_array_equal(lo[0], [0, 0, 2])
    np.testing.assert_array_equal(hi[0], [31, 1, 2])
    np.testing.assert_array_equal(lo[6], [30, 0, 2])
    np.testing.assert_array_equal(hi[2], [31, 1, 2])


def test_threaded_scene_matches_serial(oracle_lib):
    # the CPU baseline's threaded step (solve, remap, refit, render spread over envs)
    # must give the serial oracle's boxes and images bit for bit
    from ffsrl import scenarios as sc
    meshes, _ = sc.mixed_meshes(3, pool_size=3, seed=5, t_lo=150, t_hi=400)
    m, _ = sc.liver_model("cpu", 3, meshes=meshes)
    bvh = SimBVH("cpu", m)
    r = WarpRaycastRendererDO("cpu", m, resolution=8, mode="headless", verticalAperture=sc.fov_aperture(60.0),
                              horizontalAperture=sc.fov_aperture(60.0))
    pos, rot = sc.env_cameras(meshes, seed=1)
    r.setCameras(pos, rot)
    scene = oracle.OracleScene(m, bvh, r)
    scene.step(threads=3)
    o = oracle.OracleSim(m)
    o.step(1)
    vp = o.vis_points(oracle.OracleInstrument.from_model(m))
    lo, hi = oracle.refit(bvh, vp, m.host["allVisFace"])
    col, dep, _ = oracle.render(r, bvh, vp, aabb=(lo, hi))
    np.testing.assert_array_equal(scene.sim.a["vertex"], o.a["vertex"])
    np.testing.assert_array_equal(scene.bvh_arrays["aabb_min"], lo)
    np.testing.assert_array_equal(scene.bvh_arrays["aabb_max"], hi)
    np.testing.assert_array_equal(scene.a["color"].reshape(col.shape), col)
    np.testing.assert_array_equal(scene.a["depth"].reshape(dep.shape), dep)
    assert (dep > 0).any()
