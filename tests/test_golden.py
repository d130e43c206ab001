"""Golden fixtures (tests/golden/, written by tests/golden/make_golden.py from the oracle).

On CPU, the oracle and the host BVH builder must reproduce the fixtures bit for bit: this
pins the checker itself across machines and changes. On the GPU, the CUDA paths are
compared with the same fixtures: positions within 1e-4 of the position scale, contact
counts equal, BVH boxes and fused-render images bit-exact.
"""

import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden as mk  # noqa: E402
import oracle  # noqa: E402
from bvh_oracle import build_bvh  # noqa: E402
from ffsrl import SimBVH, SimIntegratorDO  # noqa: E402
from ffsrl import scenarios as sc  # noqa: E402
from ffsrl.bvh import build_topology  # noqa: E402

POS_TOL = 1e-4


def load(name):
    return np.load(GOLDEN / name)


def liver_inputs(device):
    z = load("liver3.npz")
    meshes = mk.unpack_meshes(z)
    m = mk.liver_model(device, meshes)
    # the instrument placement is part of the fixture's input
    np.testing.assert_array_equal(np.asarray(m.toolHost["base"], np.float32), z["tool_base"])
    np.testing.assert_array_equal(np.asarray(m.toolHost["tip"], np.float32), z["tool_tip"])
    np.testing.assert_array_equal(np.asarray(m.toolHost["radius"], np.float32), z["tool_radius"])
    return z, meshes, m


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


# ---------------------------------------------------------------- CPU: pin the oracle
def test_golden_beam_oracle(oracle_lib):
    z = load("beam.npz")
    m, _ = sc.beam_model("cpu", mesh=mk.unpack_meshes(z)[0])
    o = oracle.OracleSim(m)
    o.step(int(z["steps"]))
    assert np.array_equal(o.a["vertex"], z["vertex"])
    assert np.array_equal(o.a["velocity"], z["velocity"])
    V = m.numVertices
    x64 = np.asarray(m.host["vertex"], dtype=np.float64).reshape(-1, 3).copy()
    oracle.OracleSim(m).step_f64(int(z["steps"]), x64, np.zeros((V, 3)), np.zeros((V, 3)))
    assert np.array_equal(x64, z["vertex_f64"])


def test_golden_liver_oracle(oracle_lib):
    z, _, m = liver_inputs("cpu")
    o = oracle.OracleSim(m, {"active_drag_constraint": z["drag"]})
    o.step(int(z["steps"]))
    assert np.array_equal(o.a["vertex"], z["vertex"])
    assert np.array_equal(o.a["laparoscope_in_collision"], z["in_collision"])
    assert z["in_collision"].min() > 0 and z["drag"].sum() == 3  # contact and grasp happen


def test_golden_bvh_topology_and_render_oracle(oracle_lib):
    z, meshes, m = liver_inputs("cpu")
    r = load("render.npz")
    bvh = SimBVH("cpu", m)
    for k, t in enumerate(bvh.topologies):
        e = m.envMesh.index(k)
        p0, p1 = int(m.envVisPointStart[e]), int(m.envVisPointStart[e + 1])
        f0, f1 = int(m.envVisFaceStart[e]), int(m.envVisFaceStart[e + 1])
        pts = m.allVisPoint.numpy()[p0:p1]
        faces = m.host["allVisFace"].reshape(-1, 3)[f0:f1] - p0
        ref = build_bvh(pts, faces)
        host = build_topology(pts, faces)
        for key in ("left_node", "first_tri_id", "tri_count", "level", "tri_id"):
            assert np.array_equal(t[key], r[f"topo{k}_{key}"]), key
            assert np.array_equal(host[key], r[f"topo{k}_{key}"]), key
            assert np.array_equal(np.asarray(ref[key]), r[f"topo{k}_{key}"]), key
    lo, hi = oracle.refit(bvh, r["vis_point"], m.host["allVisFace"])
    assert np.array_equal(lo, r["aabb_min"]) and np.array_equal(hi, r["aabb_max"])
    rr = mk.renderer("cpu", m, meshes)
    col, dep, _ = oracle.render(rr, bvh, r["vis_point"], aabb=(lo, hi))
    assert np.array_equal(col, r["color"]) and np.array_equal(dep, r["depth"])
    assert (dep > 0).mean() > 0.1


# ---------------------------------------------------------------- GPU: CUDA vs fixtures
@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_golden_beam_gpu(gpu, batched):
    z = load("beam.npz")
    m, _ = sc.beam_model("cuda:0", mesh=mk.unpack_meshes(z)[0])
    SimIntegratorDO("cuda:0", batched=batched).stepModel(m, int(z["steps"]))
    x = m.vertex.cpu().numpy()
    e32, e64 = rel(x, z["vertex"]), rel(x, z["vertex_f64"])
    print(f"[golden] beam {int(z['steps'])} steps batched={batched}: vs oracle f32 {e32:.2e}, vs oracle f64 {e64:.2e}")
    assert e32 < POS_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_golden_liver_gpu(gpu, batched):
    import torch
    z, _, m = liver_inputs("cuda:0")
    m.activeDragConstraint.copy_(torch.as_tensor(z["drag"], device="cuda:0"))
    SimIntegratorDO("cuda:0", batched=batched).stepModel(m, int(z["steps"]))
    e = rel(m.vertex.cpu().numpy(), z["vertex"])
    print(f"[golden] liver3 batched={batched}: {e:.2e}")
    assert e < POS_TOL
    assert np.array_equal(m.laparoscopeInCollision.cpu().numpy(), z["in_collision"])


@pytest.mark.gpu
def test_golden_render_gpu(gpu):
    import torch
    z, meshes, m = liver_inputs("cuda:0")
    r = load("render.npz")
    bvh = SimBVH("cuda:0", m)  # built from the rest state, like the fixture
    for k, t in enumerate(bvh.topologies):
        assert np.array_equal(t["left_node"], r[f"topo{k}_left_node"])
    # the fixture's end state, then the library's own remap, refit and render
    m.vertex.copy_(torch.as_tensor(z["vertex"], device="cuda:0"))
    m.transformSimMeshData()
    assert np.array_equal(m.allVisPoint.cpu().numpy(), r["vis_point"])
    bvh.refitBVH()
    rr = mk.renderer("cuda:0", m, meshes)
    img = rr.renderNew(bvh, m)
    torch.cuda.synchronize()
    rr.checkErrors()
    assert np.array_equal(bvh.aabbMin.cpu().numpy(), r["aabb_min"])
    assert np.array_equal(bvh.aabbMax.cpu().numpy(), r["aabb_max"])
    assert np.array_equal(rr.depthImages().cpu().numpy(), r["depth"])
    assert np.array_equal(img.cpu().numpy(), r["color"])
