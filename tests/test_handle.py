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
