"""Edge cases of the step on the GPU against the oracle: an env without tets (a cloth of
distance constraints) batched with tet envs, an env too large for the batched step's
16-bit env-local ids (refused there, stepped by the reference-shaped step), a zero-step
call, and a grasp with no vertex in reach."""

import numpy as np
import pytest
import torch

import oracle
from ffsrl import SimIntegratorDO, SimModelDO, _lib as L, meshgen as mg

pytestmark = pytest.mark.gpu


def _cloth(n=12, h=0.5):
    """An n x n grid of vertices in y = 5 joined by structural and shear edges, its first
    row fixed; the surface triangles are the grid's."""
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 2)
    x = np.zeros((n * n, 3))
    x[:, 0], x[:, 1], x[:, 2] = g[:, 0] * h, 5.0, g[:, 1] * h
    idx = lambda i, j: i * n + j
    edges, tris = [], []
    for i in range(n):
        for j in range(n):
            if i + 1 < n: edges.append((idx(i, j), idx(i + 1, j)))
            if j + 1 < n: edges.append((idx(i, j), idx(i, j + 1)))
            if i + 1 < n and j + 1 < n:
                edges.append((idx(i, j), idx(i + 1, j + 1)))
                tris += [(idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)), (idx(i, j), idx(i + 1, j + 1), idx(i, j + 1))]
    inv = np.ones(n * n)
    inv[:n] = 0.0
    return mg.tiny_mesh(x, edge=edges, triangle=tris, inverse_mass=inv)


def test_env_without_tets_in_a_batch(gpu, oracle_lib):
    meshes = [mg.beam(6, 3, 3), _cloth(), mg.beam(4, 2, 2)]
    kw = dict(constraints=L.REFERENCE_STEP, simSubsteps=4, simConstraintsSteps=5, environmentGroundLevel=-100.0,
              environmentGravity=(0.0, -98.0, 0.0))
    m = SimModelDO(meshes, 3, "cuda:0", **kw)
    assert int(m.envTetStart[2] - m.envTetStart[1]) == 0
    o = oracle.OracleSim(m)
    SimIntegratorDO("cuda:0").stepModel(m, 10)
    o.step(10)
    torch.cuda.synchronize()
    x = m.vertex.cpu().numpy()
    e = np.abs(x - o.a["vertex"]).max() / np.abs(o.a["vertex"]).max()
    print(f"[edge cases] beam + cloth + beam, 10 batched steps vs oracle: {e:.2e}")
    assert e < 1e-4
    cloth = m.envSlice(1)
    assert np.abs(x[cloth] - m.initialVertex.cpu().numpy()[cloth]).max() > 1e-2  # the cloth sags


def test_env_too_large_for_the_batched_step(gpu, oracle_lib):
    big = mg.beam(40, 40, 40)  # 41^3 = 68,921 vertices: more than 16-bit env-local ids hold
    assert len(big["vertex"]) > 65535
    m = SimModelDO(big, 1, "cuda:0", simSubsteps=1, simConstraintsSteps=1, environmentGroundLevel=-100.0)
    from ffsrl.integrator import BatchPlan
    with pytest.raises(L.FFSRLError) as err:
        BatchPlan(m)  # the batched tables cannot hold it
    assert err.value.code == L.ERR_UNSUPPORTED
    # the integrator routes the model to the reference-shaped step instead
    integ = SimIntegratorDO("cuda:0")
    assert integ.routesToPlain(m)
    o = oracle.OracleSim(m)
    with pytest.warns(UserWarning, match="65,535"):
        integ.stepModel(m)
    o.step(1)
    torch.cuda.synchronize()
    x = m.vertex.cpu().numpy()
    assert np.abs(x - o.a["vertex"]).max() / np.abs(o.a["vertex"]).max() < 1e-5
    assert integ.envStatus(m).tolist() == [0]


def test_check_status_raises_on_a_non_finite_env(gpu):
    mesh = mg.ellipsoid_for_tets(600, seed=1)
    from ffsrl import scenarios as sc
    m, _ = sc.liver_model("cuda:0", 3, meshes=[mesh] * 3)
    integ = SimIntegratorDO("cuda:0")
    integ.stepModel(m, 1, checkStatus=True)  # finite: no error
    m.vertex[m.envSlice(2).start + 3, 1] = float("inf")
    with pytest.raises(L.FFSRLError) as err:
        integ.stepModel(m, 1, checkStatus=True)
    assert err.value.code == L.ERR_NONFINITE and "[2]" in str(err.value)


def test_zero_steps_and_unreachable_grasp(gpu):
    m = SimModelDO(mg.beam(4, 2, 2), 2, "cuda:0", environmentGroundLevel=-100.0)
    x0 = m.vertex.clone()
    SimIntegratorDO("cuda:0").stepModel(m, 0)
    torch.cuda.synchronize()
    assert torch.equal(m.vertex, x0)
    # the instrument lifted 50 cm clear of the beam: nothing within 0.5 cm of the drag point
    lift = torch.zeros((2, 3), device="cuda:0")
    lift[:, 1] = 50.0
    m.moveTool(lift)
    m.graspNearest(torch.ones(2, dtype=torch.int32, device="cuda:0"), radius=0.5)
    torch.cuda.synchronize()
    assert not m.activeDragConstraint.any()
