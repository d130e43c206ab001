"""lookAt (FF_SRL/FF_SRL/render.py:1186-1196): known answers on the CPU.

The reference points its camera with ``pitch = asin(dir.y)``, ``yaw = atan2(dir.x, dir.z)
- pi`` and ``q = quat_rpy(pitch, yaw, 0)``, dir the unit vector from the camera to the
target.  The camera looks down its local -z (the ray direction of the pixel centre,
render.py:836-878), so the rotated -z axis must be dir.
"""

import math

import numpy as np
import pytest

from ffsrl import WarpRaycastRendererDO, meshgen as mg, scenarios as sc
from ffsrl.render import look_at_rotation, quat_rpy


def rotate(q, v):
    """quat_rotate: v (2w^2 - 1) + 2 u (u.v) + 2 w (u x v), u = q.xyz."""
    q = np.asarray(q, dtype=np.float64)
    u, w = q[:3], q[3]
    v = np.asarray(v, dtype=np.float64)
    return v * (2 * w * w - 1) + 2 * u * np.dot(u, v) + 2 * w * np.cross(u, v)


def test_formula():
    rng = np.random.default_rng(3)
    for _ in range(20):
        pos, at = rng.normal(size=3) * 10, rng.normal(size=3) * 10
        d = (at - pos) / np.linalg.norm(at - pos)
        want = quat_rpy(math.asin(d[1]), math.atan2(d[0], d[2]) - math.pi, 0.0)
        assert np.array_equal(look_at_rotation(pos, at), want)


@pytest.mark.parametrize("d, q", [
    ((0.0, 0.0, -1.0), (0.0, 0.0, 0.0, 1.0)),                                   # already looking down -z
    ((1.0, 0.0, 0.0), (0.0, -math.sqrt(0.5), 0.0, math.sqrt(0.5))),            # yaw -pi/2 about y
    ((0.0, 0.0, 1.0), (0.0, -1.0, 0.0, 0.0)),                                   # yaw -pi (or pi) about y
    ((0.0, math.sqrt(0.5), -math.sqrt(0.5)), (math.sin(math.pi / 8), 0.0, 0.0, math.cos(math.pi / 8))),  # pitch 45
])
def test_known_answers(d, q):
    got = look_at_rotation((0.0, 0.0, 0.0), d)
    # q and -q are the same rotation
    assert min(np.abs(got - np.asarray(q)).max(), np.abs(got + np.asarray(q)).max()) < 1e-6


def test_the_camera_looks_at_the_target():
    rng = np.random.default_rng(7)
    for _ in range(50):
        pos = rng.normal(size=3) * 20
        at = pos + rng.normal(size=3)
        d = (at - pos) / np.linalg.norm(at - pos)
        if abs(d[1]) > 0.999:
            continue
        fwd = rotate(look_at_rotation(pos, at), (0.0, 0.0, -1.0))
        assert np.abs(fwd - d).max() < 2e-6


def test_renderer_lookat_sets_the_shared_camera():
    m, _ = sc.beam_model("cpu")
    r = WarpRaycastRendererDO("cpu", m, cameraPos=(5.0, 30.0, 40.0), resolution=8, mode="headless")
    r.lookAt((5.0, 12.0, 2.0))
    q = r.cameraRotT.numpy().reshape(4)
    assert np.array_equal(q, look_at_rotation((5.0, 30.0, 40.0), (5.0, 12.0, 2.0)))
    d = np.array([0.0, -18.0, -38.0]) / np.linalg.norm([0.0, -18.0, -38.0])
    assert np.abs(rotate(q, (0.0, 0.0, -1.0)) - d).max() < 2e-6
