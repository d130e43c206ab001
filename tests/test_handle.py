"""The owning C-ABI handle (ffsrl_create / ffsrl_step / ffsrl_get_device_model /
ffsrl_set_tool / ffsrl_set_drag): a model uploaded from host arrays steps to the same bits
as the Python layer's batched step over the same model."""

import ctypes as C

import numpy as np
import pytest
import torch

from ffsrl import SimIntegratorDO, _lib as L, scenarios as sc


def _vec3(ptr_value, n):
    """n vec3 of a device array the handle owns, copied into a torch tensor by the
    library's own remap (identity pairs)."""
    ident = torch.arange(n, dtype=torch.int32, device="cuda:0").repeat_interleave(2)
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda:0")
    L.check(L.lib().ffsrl_remap(out.data_ptr(), ptr_value, ident.data_ptr(), n, None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.gpu
def test_handle_steps_like_the_python_layer(gpu):
    meshes, _ = sc.mixed_meshes(5, pool_size=3, seed=13, t_lo=300, t_hi=1200)
    m, _ = sc.liver_model("cuda:0", 5, meshes=meshes)
    m.graspNearest(torch.ones(5, dtype=torch.int32, device="cuda:0"))
    torch.cuda.synchronize()
    hm, keep = m.host_model()
    params = m.params()
    lib = L.lib()
    h = C.c_void_p()
    L.check(lib.ffsrl_create(C.byref(hm), C.byref(params), 0, C.byref(h)))
    try:
        # the tool and the grasp set again through the setters, from host memory
        tip = m.laparoscopeTip.cpu().numpy().copy()
        drag = m.activeDragConstraint.cpu().numpy().copy()
        L.check(lib.ffsrl_set_tool(h, None, tip.ctypes.data, None, 1, None))
        L.check(lib.ffsrl_set_drag(h, drag.ctypes.data, 1, None))
        L.check(lib.ffsrl_step(h, 3, None))
        dm = L.Model()
        plan = C.c_void_p()
        L.check(lib.ffsrl_get_device_model(h, C.byref(dm), C.byref(plan)))
        assert plan.value and dm.num_vertices == m.numVertices
        got = _vec3(dm.vertex, m.numVertices)
        vel = _vec3(dm.velocity, m.numVertices)
    finally:
        lib.ffsrl_destroy(h)
    SimIntegratorDO("cuda:0").stepModel(m, 3)
    torch.cuda.synchronize()
    print(f"[handle] {m.numEnvs} envs, {m.numVertices} vertices, 3 steps: "
          f"max |x_handle - x_python| = {np.abs(got - m.vertex.cpu().numpy()).max():.1e}")
    assert np.array_equal(got, m.vertex.cpu().numpy())
    assert np.array_equal(vel, m.velocity.cpu().numpy())


@pytest.mark.gpu
def test_handle_render_matches_the_python_renderer(gpu):
    # ffsrl_attach_render / ffsrl_render_handle against SimBVH + WarpRaycastRendererDO on
    # the same model state: same BVHs (built on the same rest points), same images
    from ffsrl import SimBVH, WarpRaycastRendererDO
    meshes, _ = sc.mixed_meshes(4, pool_size=2, seed=17, t_lo=300, t_hi=900)
    m, meshes = sc.liver_model("cuda:0", 4, meshes=meshes, instrument_visual=False)
    m.graspNearest(torch.ones(4, dtype=torch.int32, device="cuda:0"))
    bvh = SimBVH("cuda:0", m)
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO("cuda:0", m, resolution=16, mode="headless", verticalAperture=ap,
                              horizontalAperture=ap, render_mode=3)
    r.setCameras(*sc.env_cameras(meshes, seed=4))
    torch.cuda.synchronize()
    hm, keep = m.host_model()
    lib = L.lib()
    h = C.c_void_p()
    L.check(lib.ffsrl_create(C.byref(hm), C.byref(m.params()), 0, C.byref(h)))
    try:
        pts = np.ascontiguousarray(m.allVisPoint.cpu().numpy(), dtype=np.float32)
        faces = np.ascontiguousarray(m.host["allVisFace"], dtype=np.int32)
        cols = np.ascontiguousarray(m.allVisPointColor.cpu().numpy(), dtype=np.float32)
        ptv = np.ascontiguousarray(m.host["pointToVertex"], dtype=np.int32)
        ps = np.ascontiguousarray(m.envVisPointStart, dtype=np.int32)
        fs = np.ascontiguousarray(m.envVisFaceStart, dtype=np.int32)
        topo = np.ascontiguousarray(m.envMesh, dtype=np.int32)
        ld = np.ascontiguousarray(r.lightDir.cpu().numpy(), dtype=np.float32)
        li = np.ascontiguousarray(r.lightIntensity.cpu().numpy(), dtype=np.float32)
        c = L.RenderConfig(num_points=len(pts), num_faces=len(faces) // 3 if faces.ndim == 1 else len(faces),
                           points=pts.ctypes.data, faces=faces.ctypes.data, colors=cols.ctypes.data,
                           num_map=len(ptv.reshape(-1)) // 2, point_to_vertex=ptv.ctypes.data,
                           env_point_start=ps.ctypes.data, env_face_start=fs.ctypes.data,
                           env_topology=topo.ctypes.data, resolution=16, camera_tan=r.camera_tan,
                           camera_aspect=r.camera_aspect, num_lights=len(li), light_dir=ld.ctypes.data,
                           light_intensity=li.ctypes.data, render_mode=3)
        L.check(lib.ffsrl_attach_render(h, C.byref(c)))
        L.check(lib.ffsrl_step(h, 2, None))
        color = torch.zeros((4, 16, 16, 3), dtype=torch.float32, device="cuda:0")
        depth = torch.zeros((4, 16, 16), dtype=torch.float32, device="cuda:0")
        L.check(lib.ffsrl_render_handle(h, r.cameraPosT.data_ptr(), r.cameraRotT.data_ptr(), int(r.cameraPosT.shape[0]),
                                        color.data_ptr(), depth.data_ptr(), None))
        torch.cuda.synchronize()
    finally:
        lib.ffsrl_destroy(h)
    SimIntegratorDO("cuda:0").stepModel(m, 2)
    bvh.refitBVH()
    r.renderNew(bvh, m)
    torch.cuda.synchronize()
    hit = float((depth > 0).float().mean())
    print(f"[handle] render: {hit:.2f} of the pixels hit; max |color diff| "
          f"{float((color - r.pixels.reshape(color.shape)).abs().max()):.1e}")
    assert hit > 0.05
    assert torch.equal(color, r.pixels.reshape(color.shape))
    assert torch.equal(depth, r.depth.reshape(depth.shape))
