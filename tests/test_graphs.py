"""CUDA graphs of the step, the refit, the render and a whole RL step (the reference's
``wp.capture_begin`` / ``wp.capture_launch``: bvh.py:442-451, render.py:1108-1112,
tests/testLiverRetraction.py:77-85): replays give the eager results bit for bit (the
batched step; the reference-shaped step's float atomics differ run to run)."""

import numpy as np
import pytest

from ffsrl import SimBVH, SimIntegratorDO, WarpRaycastRendererDO, scenarios as sc
from ffsrl.graphs import Graph


def _setup(n=4):
    import torch
    meshes, _ = sc.mixed_meshes(n, pool_size=3, seed=21, t_lo=300, t_hi=900)
    m, meshes = sc.liver_model("cuda:0", n, meshes=meshes)
    m.graspNearest(torch.ones(n, dtype=torch.int32, device="cuda:0"))
    bvh = SimBVH("cuda:0", m)
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO("cuda:0", m, resolution=16, mode="headless", verticalAperture=ap, horizontalAperture=ap)
    r.setCameras(*sc.env_cameras(meshes, seed=4))
    return m, bvh, r


def _state(m, bvh, r):
    return [t.cpu().numpy() for t in (m.vertex, m.velocity, m.allVisPoint, bvh.aabbMin, bvh.aabbMax, r.pixels,
                                      r.depth, m.laparoscopeXForm)]


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [True, False])
def test_graphs_replay_the_eager_calls(gpu, batched):
    import torch
    out = []
    for use in (False, True):
        m, bvh, r = _setup()
        integ = SimIntegratorDO("cuda:0", batched=batched)
        for _ in range(3):
            integ.stepModel(m, 2, useGraph=use)
            bvh.refitBVH(useGraph=use)
            r.renderNew(bvh, m, useGraph=use)
        torch.cuda.synchronize()
        out.append(_state(m, bvh, r))
    for a, b in zip(*out):
        if batched:  # exact fixed-point sums: the same bits
            assert np.array_equal(a, b)
        else:  # the reference-shaped step sums with float atomics, in a different order each run
            assert np.abs(a - b).max() <= 1e-3 * max(np.abs(a).max(), 1.0)


@pytest.mark.gpu
def test_rl_step_graph_with_changing_actions(gpu):
    import torch
    rng = np.random.default_rng(2)
    acts = rng.uniform(-0.05, 0.05, size=(5, 4, 3)).astype(np.float32)
    out = []
    for use in (False, True):
        m, bvh, r = _setup()
        integ = SimIntegratorDO("cuda:0")
        static = torch.zeros((4, 3), device="cuda:0")

        def rl_step():
            m.resetCollisionInfo()
            m.applyCartesianActionsInWorkspace(static)
            integ.stepModel(m)
            bvh.refitBVH()
            r.renderNew(bvh, m)

        g = Graph(rl_step, prepare=lambda: integ.plan(m))
        for k in range(5):
            static.copy_(torch.as_tensor(acts[k], device="cuda:0"))
            g() if use else rl_step()
        torch.cuda.synchronize()
        out.append(_state(m, bvh, r) + [m.laparoscopeInCollision.cpu().numpy()])
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_native_graph_calls_replay_the_step_and_refit(gpu):
    # ffsrl_graph_begin / end / launch (the C caller's capture) around library calls only
    import torch
    from ffsrl.graphs import NativeGraph
    out = []
    for use in (False, True):
        m, bvh, r = _setup()
        integ = SimIntegratorDO("cuda:0")

        def step():
            integ.stepModel(m, 2)
            bvh.refitBVH()

        g = NativeGraph(step, prepare=lambda: integ.plan(m)) if use else step
        for _ in range(3):
            g()
        torch.cuda.synchronize()
        out.append([t.cpu().numpy() for t in (m.vertex, m.velocity, m.allVisPoint, bvh.aabbMin, bvh.aabbMax)])
        if use:
            g.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
