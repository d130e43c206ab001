"""The step entry point that allocates nothing (ffsrl_step_model_noalloc).

It serves callers that cannot call cudaMalloc -- for example a host application that has
reserved the device's memory for its own pool, or a control loop that must never wait on
the driver's allocator.  Its accumulators live in an array compiled into the library, so
this test checks, through the C-ABI, that two calls in a row give the same positions as
the allocating entry point (ffsrl_step_model) within the parity tolerance of the other
GPU tests -- on a beam and on meshes pressed by the instrument, whose contact phase uses
the array's contact slice -- and that a model above its vertex limit is rejected.  Kept
in a file that pytest collects last.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from ffsrl import _lib as L, meshgen as mg, scenarios as sc

pytestmark = pytest.mark.gpu
POS_TOL = 1e-4


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def _contact_model():
    # two small ellipsoids with the instrument's closed clamps on their surfaces: the step
    # runs the contact phase, whose sums use the array's third slice
    mesh = mg.ellipsoid_for_tets(1500, seed=2)
    m, _ = sc.liver_model("cuda:0", 2, meshes=[mesh, mesh])
    return m


@pytest.mark.parametrize("scene", ["beam", "contact"])
def test_noalloc_step_matches_allocating_step(gpu, scene):
    build = (lambda: sc.beam_model("cuda:0")[0]) if scene == "beam" else _contact_model
    ref, new = build(), build()
    lib = L.lib()
    p = ref.params()
    s = L.stream_handle()
    for call in range(2):
        m_ref = ref.device_model()
        L.check(lib.ffsrl_step_model(C.byref(m_ref), C.byref(p), s))
        m_new = new.device_model()
        # the no-allocation entry ignores the model's accumulator pointers
        m_new.dp = None
        m_new.constraints_number = None
        m_new.collision_dp = None
        L.check(lib.ffsrl_step_model_noalloc(C.byref(m_new), C.byref(p), s))
        torch.cuda.synchronize()
        err = _rel(new.vertex, ref.vertex)
        print(f"[noalloc] call {call + 1}: max|dx|/max|x| = {err:.3e}")
        assert err < POS_TOL
        assert _rel(new.velocity, ref.velocity) < 1e-2 or float(ref.velocity.abs().max()) == 0.0
    assert float((new.vertex - new.initialVertex).abs().max()) > 1e-3  # the mesh moved
    if scene == "contact":
        assert int(new.laparoscopeInCollision.min()) > 0  # every env was in contact
        assert torch.equal(new.laparoscopeInCollision, ref.laparoscopeInCollision)


def test_noalloc_rejects_models_above_the_limit(gpu):
    m, _ = sc.beam_model("cuda:0")
    d = m.device_model()
    d.num_vertices = 65537
    p = m.params()
    rc = L.lib().ffsrl_step_model_noalloc(C.byref(d), C.byref(p), L.stream_handle())
    assert rc == L.ERR_INVALID_ARGUMENT
    assert b"65536" in L.lib().ffsrl_last_error()
