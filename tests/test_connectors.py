"""Connectors (triToPointDistanceConstraintsDO, integrator.py:300-353; SimConnectorDO,
modelDO.py:723-770, 977-1015): a known answer of the oracle, the model's global ids, the
scene-file prims, and the reference-shaped and batched GPU steps against the oracle."""

import numpy as np
import pytest

import oracle
from ffsrl import SimIntegratorDO, SimModelDO, _lib as L, meshgen as mg
from ffsrl import scene as scene_io


def _one_connector():
    # triangle a, b, c in z = 0 and point d above its centroid (tiny_mesh vertex order)
    mesh = mg.tiny_mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1 / 3, 1 / 3, 2]], triangle=[[0, 1, 2]])
    mesh["connector_vertex_id"] = [3]
    mesh["connector_triangle_id"] = [[0, 1, 2]]
    mesh["connector_tri_bar"] = [[1 / 3, 1 / 3, 1 / 3]]
    mesh["connector_rest_dist"] = [1.0]
    return mesh


def test_connector_known_answer(oracle_lib):
    # integrator.py:300-353 with massWeightRatio 0.75, kS 0.125, restLengthMul 0.5: the
    # point is 2 above the centroid, C = 2 - 0.5 = 1.5, s = 0.75 + 0.25 * 3/9,
    # delta = C / s * kS along +z.  Its dP is added after applyConstraints, so the first
    # iteration's corrections move the vertices at the second iteration's apply.
    m = SimModelDO(_one_connector(), 1, "cpu", constraints=L.CONNECTORS, simSubsteps=1, simConstraintsSteps=2,
                   environmentGravity=(0.0, 0.0, 0.0), environmentGroundLevel=-100.0,
                   globalConnectorMassWeightRatio=0.75, globalConnectorKs=0.125, globalConnectorRestLengthMul=0.5)
    assert m.simConnectors == 1
    o = oracle.OracleSim(m)
    o.step(1)
    delta = 1.5 / (0.75 + 0.25 / 3.0) * 0.125
    x = o.a["vertex"]
    np.testing.assert_allclose(x[3], [1 / 3, 1 / 3, 2 - 0.75 * delta], rtol=1e-6)
    np.testing.assert_allclose(x[:3, 2], [0.25 * delta / 3.0] * 3, rtol=1e-5)
    # the second iteration's corrections wait in dP for the next step, one count each
    assert o.a["constraints_number"].tolist() == [1, 1, 1, 1]
    assert o.a["dp"][3, 2] < 0


def _connected():
    a = mg.beam(4, 2, 2)
    b = dict(mg.beam(4, 2, 2))
    for k in ("vertex", "rest_vertex"):
        b[k] = b[k] + np.array([0.0, 1.05, 0.0], np.float32)
    return mg.connect_meshes(a, b, 0.8)


def test_model_connector_ids_are_global():
    body = _connected()
    m = SimModelDO(body, 2, "cpu")
    nv = len(body["vertex"])
    c = len(body["connector_vertex_id"])
    assert m.simConnectors == 2 * c
    ids = m.host["connectorVertexId"]
    assert np.array_equal(ids[:c], body["connector_vertex_id"]) and np.array_equal(ids[c:], body["connector_vertex_id"] + nv)
    tri = m.host["connectorTriangleId"].reshape(-1, 3)
    assert np.array_equal(tri[c:], body["connector_triangle_id"] + nv)
    bad = dict(body)
    bad["connector_vertex_id"] = np.array(body["connector_vertex_id"]) + nv
    with pytest.raises(ValueError):
        SimModelDO(bad, 1, "cpu")


def test_scene_file_connectors(tmp_path):
    body = _connected()
    p = tmp_path / "c.npz"
    scene_io.write_scene(p, body)
    z = np.load(p)
    assert "/World/Mesh0Connector.simConnector" in z.files and str(z["/World/Mesh0Connector.pointBody"]) == "/World/Mesh0"
    s = scene_io.read_scene(p)
    for key in ("connector_vertex_id", "connector_triangle_id", "connector_tri_bar", "connector_rest_dist"):
        assert np.array_equal(np.asarray(s.mesh[key]).reshape(np.shape(body[key])), body[key]), key


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_connectors_step_matches_oracle(gpu, oracle_lib, batched):
    import torch
    body = _connected()
    kw = dict(constraints=L.REFERENCE_STEP, simSubsteps=4, simConstraintsSteps=5, environmentGroundLevel=-100.0,
              environmentGravity=mg.gravity_force(body))
    m = SimModelDO([body, mg.beam(4, 2, 2), body], 3, "cuda:0", **kw)
    o = oracle.OracleSim(m)
    integ = SimIntegratorDO("cuda:0", batched=batched)
    for _ in range(3):  # separate calls: the pending corrections carry over between steps
        integ.stepModel(m, 1)
        o.step(1)
    torch.cuda.synchronize()
    x = m.vertex.cpu().numpy()
    e = np.abs(x - o.a["vertex"]).max() / np.abs(o.a["vertex"]).max()
    print(f"[connectors] batched={batched} step vs oracle, 3 steps: {e:.2e}")
    assert e < 1e-4
    if not batched:  # the reference-shaped step keeps them in the model's dP and counts
        assert np.array_equal(m.constraintsNumber.cpu().numpy(), o.a["constraints_number"])
    # without the connectors the bodies move differently: the test sees them
    free = SimModelDO([body, mg.beam(4, 2, 2), body], 3, "cuda:0", **(kw | {"constraints": L.REFERENCE_STEP & ~L.CONNECTORS}))
    SimIntegratorDO("cuda:0", batched=batched).stepModel(free, 3)
    torch.cuda.synchronize()
    assert np.abs(free.vertex.cpu().numpy() - x).max() > 100 * np.abs(x - o.a["vertex"]).max()
