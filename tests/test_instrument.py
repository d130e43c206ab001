"""Instrument kinematics (modelDO.py:26-416, 1331-1419, 1570-1587).

CPU: known answers of the oracle's restatement -- the host builder's capsule ends,
insertion along the axis, Cartesian moves of the effector about the rotation centre, the
workspace clip, the clamp's angle limits and grasp flags, and moving the rotation centre.
GPU: the CUDA kernels against the oracle over seeded action sequences.
"""

import numpy as np
import pytest

import oracle
from ffsrl import scenarios as sc

PTS = np.array([[0.0, 5.0, 0.0], [1.0, 6.0, 2.0], [-2.0, 4.0, 1.5]])


def make(points=PTS, **kw):
    xf, h, b, t, r = sc.instrument_xforms(points, **kw)
    return oracle.OracleInstrument(xf, h, b, t), (xf, h, b, t, r)


def ends(o):
    return o.base.reshape(-1, 4, 3), o.tip.reshape(-1, 4, 3)


def clamp_angle(o, e):
    """Right-clamp pivot angle about the rod's x axis, degrees (rotateClampsFunc)."""
    X = o.xform.reshape(-1, 7, 4, 4)[e]
    rod, right = X[0].T.astype(np.float64), X[5].T.astype(np.float64)
    return np.degrees(np.arcsin((np.linalg.inv(rod) @ right)[2, 1]))


def test_builder_matches_update(oracle_lib):
    o, (_, _, b, t, _) = make()
    o.update()
    np.testing.assert_allclose(o.base, b.reshape(-1), atol=1e-5)
    np.testing.assert_allclose(o.tip, t.reshape(-1), atol=1e-5)
    np.testing.assert_allclose(ends(o)[1][:, 3], PTS, atol=1e-5)  # drag point at the effector


def test_rod_insertion_moves_every_capsule_along_the_axis(oracle_lib):
    o, _ = make()
    b0, t0 = (a.copy() for a in ends(o))
    a = np.zeros((3, 5), np.float32)
    a[:, 0] = 0.5  # forward along local z, here -y
    o.apply_actions(a)
    b1, t1 = ends(o)
    np.testing.assert_allclose(b1 - b0, np.broadcast_to([0.0, -0.5, 0.0], b0.shape), atol=2e-5)
    np.testing.assert_allclose(t1 - t0, np.broadcast_to([0.0, -0.5, 0.0], t0.shape), atol=2e-5)


def test_cartesian_action_moves_the_effector(oracle_lib):
    o, _ = make()
    rng = np.random.default_rng(0)
    target = PTS.copy()
    for _ in range(20):
        a = rng.uniform(-0.1, 0.1, size=(3, 3)).astype(np.float32)
        o.cartesian(a)
        target += a
    np.testing.assert_allclose(ends(o)[1][:, 3], target, atol=1e-3)
    # the rod still passes through the rotation centre (a rigid pivot about it)
    X = o.xform.reshape(-1, 7, 4, 4)
    for e in range(3):
        c = X[e, 3].T[:3, 3].astype(np.float64)
        b, t = ends(o)[0][e, 3].astype(np.float64), ends(o)[1][e, 3].astype(np.float64)
        d = np.cross(t - b, c - b)
        assert np.linalg.norm(d) / np.linalg.norm(t - b) < 1e-3


def test_workspace_drops_components_and_flags(oracle_lib):
    o, _ = make()
    before = ends(o)[1][:, 3].copy()
    ws = [-100.0, 4.95, -100.0, 100.0, 100.0, 100.0]  # y may not go below 4.95
    o.cartesian(np.array([[0.1, -0.1, 0.0]] * 3, np.float32), workspace=ws)
    after = ends(o)[1][:, 3]
    assert o.violation.tolist() == [1, 0, 1]  # env 2 starts below the bound
    np.testing.assert_allclose(after[0] - before[0], [0.1, 0.0, 0.0], atol=2e-4)  # y component dropped
    np.testing.assert_allclose(after[1] - before[1], [0.1, -0.1, 0.0], atol=2e-4)
    np.testing.assert_allclose(after[2] - before[2], [0.1, 0.0, 0.0], atol=2e-4)


def test_clamp_limits_and_grasp_flags(oracle_lib):
    o, _ = make(clamp_angle=60.0)
    close = np.zeros((3, 5), np.float32)
    close[:, 4] = -0.2  # about -11.5 degrees per action
    assert abs(clamp_angle(o, 0) - 60.0) < 1e-3
    o.apply_actions(close)
    assert abs(clamp_angle(o, 0) - (60.0 - np.degrees(0.2))) < 1e-3 and o.dch[0] == 0
    for _ in range(4):
        o.apply_actions(close)
    assert abs(clamp_angle(o, 0) - 40.0) < 1e-3  # stops at the minimum
    assert o.dch.reshape(-1, 3)[:, 0].tolist() == [1, 1, 1]  # grasping below 43 degrees
    opened = close.copy()
    opened[:, 4] = 0.5
    for _ in range(3):
        o.apply_actions(opened)
    assert abs(clamp_angle(o, 0) - 85.0) < 1e-3 and o.dch[0] == 0  # released, opened to the maximum


def test_set_rotation_center_carries_the_instrument(oracle_lib):
    o, _ = make()
    X0 = o.xform.reshape(-1, 7, 4, 4).copy()
    rel0 = [np.linalg.inv(X0[e, 3].T.astype(np.float64)) @ np.append(ends(o)[1][e, 3], 1.0) for e in range(3)]
    t = np.array([[0.0, 20.0, 0.0], [1.0, 19.0, 1.0], [0.0, 18.0, -1.0]], np.float32)
    r = np.array([[0.0, 0.0, 0.0], [0.1, 0.0, 0.0], [0.0, 0.2, 0.1]], np.float32)
    o.set_rotation_center(t, r)
    X = o.xform.reshape(-1, 7, 4, 4)
    for e in range(3):
        np.testing.assert_allclose(X[e, 3].T[:3, 3], t[e], atol=1e-5)
        rel = np.linalg.inv(X[e, 3].T.astype(np.float64)) @ np.append(ends(o)[1][e, 3], 1.0)
        np.testing.assert_allclose(rel, rel0[e], atol=1e-4)


# ------------------------------------------------------------------------- GPU
def _gpu_model(n=6):
    meshes, _ = sc.mixed_meshes(n, pool_size=3, seed=9, t_lo=300, t_hi=700)
    m, _ = sc.liver_model("cuda:0", n, meshes=meshes)
    return m


def _oracle_of(m):
    return oracle.OracleInstrument(m.laparoscopeXForm.cpu().numpy(), m.laparoscopeHeight.cpu().numpy(),
                                   m.laparoscopeBase.cpu().numpy(), m.laparoscopeTip.cpu().numpy(),
                                   m.laparoscopeDragCutHeat.cpu().numpy(), m.laparoscopeDragCutHeatUpdate.cpu().numpy())


@pytest.mark.gpu
def test_kinematics_gpu_matches_oracle(gpu, oracle_lib):
    import torch
    m = _gpu_model()
    o = _oracle_of(m)
    rng = np.random.default_rng(3)
    n = m.numEnvs
    m.workspaceLow, m.workspaceHigh = (-100.0, 3.0, -100.0), (100.0, 100.0, 100.0)
    ws = list(m.workspaceLow) + list(m.workspaceHigh)
    centre = np.asarray(m.toolHost["xform"]).reshape(n, 7, 4, 4)[:, 3, 3, :3]
    t = (rng.uniform(-1, 1, size=(n, 3)) + centre).astype(np.float32)
    r = rng.uniform(-0.1, 0.1, size=(n, 3)).astype(np.float32)
    m.setRotationCenter(torch.as_tensor(t, device="cuda:0"), torch.as_tensor(r, device="cuda:0"))
    o.set_rotation_center(t, r)
    for k in range(40):
        a = rng.uniform(-0.1, 0.1, size=(n, 5)).astype(np.float32)
        a[:, 4] = rng.choice([-0.1, 0.0, 0.1], size=n)
        m.applyActions(torch.as_tensor(a, device="cuda:0"))
        o.apply_actions(a)
        c = rng.uniform(-0.08, 0.08, size=(n, 3)).astype(np.float32)
        if k % 2:
            m.applyCartesianActionsInWorkspace(torch.as_tensor(c, device="cuda:0"))
            o.cartesian(c, workspace=ws)
        else:
            m.applyCartesianActions(torch.as_tensor(c, device="cuda:0"))
            o.cartesian(c)
    torch.cuda.synchronize()
    scale = np.abs(o.tip).max()
    e_tip = np.abs(m.laparoscopeTip.cpu().numpy().reshape(-1) - o.tip).max() / scale
    e_base = np.abs(m.laparoscopeBase.cpu().numpy().reshape(-1) - o.base).max() / scale
    e_x = np.abs(m.laparoscopeXForm.cpu().numpy() - o.xform).max() / max(np.abs(o.xform).max(), 1.0)
    print(f"[instrument] 40 action rounds: tips {e_tip:.2e}, bases {e_base:.2e}, transforms {e_x:.2e}")
    assert e_tip < 1e-5 and e_base < 1e-5 and e_x < 1e-5
    assert np.array_equal(m.laparoscopeDragCutHeat.cpu().numpy(), o.dch)
    assert np.array_equal(m.laparoscopeDragCutHeatUpdate.cpu().numpy(), o.dchu)
    assert np.array_equal(m.laparoscopeWorkspaceViolation.cpu().numpy(), o.violation)


@pytest.mark.gpu
def test_forced_clamp_grasps_near_the_drag_point(gpu):
    import torch
    m = _gpu_model(3)
    m.globalLaparoscopeDragLookupRadius = 0.5
    for _ in range(4):  # closing below 43 degrees grasps (updateClampsDragKernel)
        m.forceLaparoscopeClamp(torch.ones(3, device="cuda:0"))
    torch.cuda.synchronize()
    assert m.laparoscopeDragCutHeat.cpu().numpy().reshape(-1, 3)[:, 0].tolist() == [1, 1, 1]
    drag = m.activeDragConstraint.cpu().numpy()
    pred = m.predictedVertex.cpu().numpy()
    tips = m.getLaparoscopePositionsTensor().cpu().numpy()
    env = m.vertexToEnv.cpu().numpy()
    near = np.linalg.norm(pred - tips[env], axis=1) < 0.5
    assert np.array_equal(drag == 1.0, near)
