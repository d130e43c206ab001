"""The ray-cast's traversal-stack check, through the Python renderer and the C handle.

A BVH deeper than the traversal stack (64 entries) cannot come from an ordinary surface
mesh.  This one is built on purpose: three families of flat triangles, each family
perpendicular to one axis, shrinking geometrically (ratio 0.3) towards the origin.  The
binned SAH build peels off the largest triangle level after level, so the tree is
about 110 levels deep, and every box along that chain contains the origin.  A camera at
the origin starts every ray inside all those boxes; the nearer-child-first traversal
keeps each level's farther child pending while it descends, so its stack overflows.
The kernels detect that (a bounds check, no out-of-range access) and set the error flag
that ``WarpRaycastRendererDO.checkErrors`` and ``ffsrl_render_handle_check`` report.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from ffsrl import SimBVH, SimModelDO, WarpRaycastRendererDO, _lib as L, meshgen as mg
from ffsrl.bvh import build_topology
from ffsrl.render import look_at_rotation


def deep_slab_mesh(ratio=0.3, smallest=1e-35, largest=1e4):
    n = int(np.log(smallest / largest) / np.log(ratio))
    pts, faces = [], []
    for axis in range(3):
        other = [a for a in range(3) if a != axis]
        for k in range(n):
            x = largest * ratio ** k
            base = len(pts)
            for u, v in ((-x, -x), (2 * x, -x), (-x, 2 * x)):
                p = [0.0, 0.0, 0.0]
                p[axis], p[other[0]], p[other[1]] = x, u, v
                pts.append(p)
            faces.append([base, base + 1, base + 2])
    pts = np.asarray(pts, dtype=np.float32)
    return mg.tiny_mesh(pts, triangle=np.asarray(faces), inverse_mass=np.zeros(len(pts)))


def test_deep_mesh_builds_a_tree_deeper_than_the_stack(built_lib):
    mesh = deep_slab_mesh()
    t = build_topology(mesh["vertex"], mesh["triangle"])
    assert t["max_level"] > 80, t["max_level"]


def _model(device):
    return SimModelDO(deep_slab_mesh(), 1, device, simSubsteps=1, simFrameRate=60, simConstraintsSteps=1,
                      environmentGroundLevel=-1e9, constraints=0, environmentGravity=(0.0, 0.0, 0.0))


def _camera():
    pos = np.zeros((1, 3), dtype=np.float32)
    rot = np.asarray(look_at_rotation((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), dtype=np.float32).reshape(1, 4)
    return pos, rot


@pytest.mark.gpu
def test_python_renderer_reports_the_overflow(gpu):
    m = _model("cuda:0")
    bvh = SimBVH("cuda:0", m)
    r = WarpRaycastRendererDO("cuda:0", m, resolution=8, mode="headless", render_mode=4)
    r.setCameras(*_camera())
    bvh.refitBVH()
    r.renderNew(bvh, m)
    torch.cuda.synchronize()
    with pytest.raises(L.FFSRLError) as e:
        r.checkErrors()
    assert e.value.code == L.ERR_STACK_OVERFLOW
    r.checkErrors()  # cleared by the report


@pytest.mark.gpu
def test_handle_render_check_reports_and_clears_the_overflow(gpu):
    m = _model("cuda:0")
    hm, keep = m.host_model()
    lib = L.lib()
    h = C.c_void_p()
    L.check(lib.ffsrl_create(C.byref(hm), C.byref(m.params()), 0, C.byref(h)))
    try:
        pts = np.ascontiguousarray(m.allVisPoint.cpu().numpy(), dtype=np.float32)
        faces = np.ascontiguousarray(m.host["allVisFace"], dtype=np.int32)
        cols = np.ascontiguousarray(m.allVisPointColor.cpu().numpy(), dtype=np.float32)
        ps = np.ascontiguousarray(m.envVisPointStart, dtype=np.int32)
        fs = np.ascontiguousarray(m.envVisFaceStart, dtype=np.int32)
        ld = np.array([[0.3, 1.0, 0.5]], dtype=np.float32)
        li = np.array([0.8], dtype=np.float32)
        c = L.RenderConfig(num_points=len(pts), num_faces=faces.size // 3, points=pts.ctypes.data,
                           faces=faces.ctypes.data, colors=cols.ctypes.data, num_map=0, point_to_vertex=None,
                           env_point_start=ps.ctypes.data, env_face_start=fs.ctypes.data, env_topology=None,
                           resolution=8, camera_tan=0.5, camera_aspect=1.0, num_lights=1, light_dir=ld.ctypes.data,
                           light_intensity=li.ctypes.data, render_mode=4)
        L.check(lib.ffsrl_attach_render(h, C.byref(c)))
        pos, rot = (torch.as_tensor(a, device="cuda:0") for a in _camera())
        color = torch.zeros((1, 8, 8, 3), dtype=torch.float32, device="cuda:0")
        depth = torch.zeros((1, 8, 8), dtype=torch.float32, device="cuda:0")
        L.check(lib.ffsrl_render_handle_check(h, None))  # nothing rendered yet
        L.check(lib.ffsrl_render_handle(h, pos.data_ptr(), rot.data_ptr(), 1, color.data_ptr(), depth.data_ptr(),
                                        None))
        assert lib.ffsrl_render_handle_check(h, None) == L.ERR_STACK_OVERFLOW
        assert b"stack" in L.lib().ffsrl_last_error()
        assert lib.ffsrl_render_handle_check(h, None) == L.OK  # the report cleared it
    finally:
        lib.ffsrl_destroy(h)
