"""Cutting and heating on the GPU against the oracle: every kernel of ffsrl.cutting on a
three-env model of beams of two sizes, compared bit for bit (integer flags, holes, and
float values computed in the same order without contraction), then the batched and the
reference-shaped step over the cut topology against the oracle step."""

import numpy as np
import pytest
import torch

import oracle
from ffsrl import SimIntegratorDO, SimModelDO, _lib as L, meshgen as mg
from ffsrl.cutting import SimCutting

pytestmark = pytest.mark.gpu

MESHES = (mg.beam(6, 3, 3), mg.beam(4, 2, 2))
FLOATS = ("edgeBreaker", "tetrahedronBreaker", "tetrahedronHeat", "tetrahedronNewHeat", "vertexHeat")
INTS = ("flipEdge", "flipTetrahedron")
MODEL = {"activeEdge": "activeEdge", "activeTetrahedron": "activeTetrahedron", "hole": "hole"}


def _model():
    meshes = [MESHES[0], MESHES[1], MESHES[0]]
    return SimModelDO(meshes, 3, "cuda:0", constraints=L.REFERENCE_STEP, simSubsteps=4, simConstraintsSteps=5,
                      environmentGroundLevel=-100.0, environmentGravity=(0.0, -98.0, 0.0))


def _same(c, o, where):
    torch.cuda.synchronize()
    for k in FLOATS + INTS:
        g = getattr(c, k).cpu().numpy().reshape(-1)
        assert np.array_equal(g, o.a[k]), f"{where}: {k} differs at {np.nonzero(g != o.a[k])[0][:8]}"
    for k in MODEL:
        g = getattr(c.model, k).cpu().numpy().reshape(-1)
        assert np.array_equal(g, o.a[k]), f"{where}: model {k} differs at {np.nonzero(g != o.a[k])[0][:8]}"


def _stretch(m, seed=0, scale=0.25):
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = (torch.rand(m.predictedVertex.shape, generator=g) - 0.5) * 2 * scale
    m.predictedVertex.copy_(m.vertex + noise.to(m.vertex.device))


def test_breaking_and_fading_match_the_oracle(gpu, oracle_lib):
    m = _model()
    _stretch(m)
    c = SimCutting(m)
    o = oracle.OracleCutting.from_cutting(c)
    for _ in range(3):
        c.checkEdgeBreaking(breakFactor=2.0, breakThreshold=0.05)
        o.checkEdgeBreaking(breakFactor=2.0, breakThreshold=0.05)
        c.checkTetrahedronBreaking(breakFactor=3.0)
        o.checkTetrahedronBreaking(breakFactor=3.0)
    _same(c, o, "breakers")
    v = m.topologyVersion
    c.checkEdgeBreaking(breakFactor=2.0, breakThreshold=1e9, breakLimit=1e9)  # nothing new breaks
    assert m.topologyVersion == v
    o.checkEdgeBreaking(breakFactor=2.0, breakThreshold=1e9, breakLimit=1e9)
    flipped = int((c.flipEdge == -1).sum())
    print(f"[cutting] {flipped} of {m.numEdges} edges broke, {int((c.flipTetrahedron == -1).sum())} tets, "
          f"{int(m.hole.sum())} holes")
    assert 0 < flipped < m.numEdges
    for i in range(6):
        c.updateActiveValues()
        o.updateActiveValues()
        _same(c, o, f"fade {i}")
    assert int((m.activeEdge == 0).sum()) == flipped


def test_heat_matches_the_oracle(gpu, oracle_lib):
    m = _model()
    c = SimCutting(m)
    rng = np.random.default_rng(3)
    c.tetrahedronHeat.copy_(torch.as_tensor(rng.uniform(0, 4, m.numTetrahedrons).astype(np.float32)))
    act = np.ones(m.numTetrahedrons, np.float32)
    act[rng.choice(m.numTetrahedrons, 20, replace=False)] = 0.0
    m.activeTetrahedron.copy_(torch.as_tensor(act))
    o = oracle.OracleCutting.from_cutting(c)
    for i in range(4):
        c.propagateHeat(heatConduction=0.3, heatTransfer=0.5, heatLoss=0.02)
        o.propagateHeat(heatConduction=0.3, heatTransfer=0.5, heatLoss=0.02)
        _same(c, o, f"propagate {i}")
    c.checkHeat(heatLimit=2.5)
    o.checkHeat(heatLimit=2.5)
    _same(c, o, "check heat")
    c.checkHeat(heatLimit=3.0, volumeProportional=True)
    o.checkHeat(heatLimit=3.0, volumeProportional=True)
    _same(c, o, "check heat, volume-proportional")
    assert 0 < int((c.flipTetrahedron == -1).sum()) < m.numTetrahedrons


def test_instrument_heat_and_cut_match_the_oracle(gpu, oracle_lib):
    m = _model()
    c = SimCutting(m)
    tips = m.laparoscopeTip.cpu().numpy().reshape(-1, 4, 3).copy()
    tri = m.triangle.cpu().numpy().reshape(-1, 3)
    x = m.vertex.cpu().numpy()
    f0 = m.envTriStart
    for e in range(m.numEnvs):
        p = x[tri[f0[e] + 5][0]]                        # clamp midpoint on a surface vertex
        tips[e, 1], tips[e, 2] = p + [0.1, 0.0, 0.0], p - [0.1, 0.0, 0.0]
    m.laparoscopeTip.copy_(torch.as_tensor(tips.reshape(-1, 3)))
    o = oracle.OracleCutting.from_cutting(c)
    for _ in range(3):
        c.heatLaparoscope(heatSphereRadius=0.9, heatQuantum=0.75)
        o.heatLaparoscope(heatSphereRadius=0.9, heatQuantum=0.75)
    _same(c, o, "heat laparoscope")
    assert int((c.tetrahedronHeat > 0).sum()) > 0
    # clamp triangle in the plane x = 3.5 (2.5 for the small beam) across the whole section
    for e, nx in enumerate((6, 4, 6)):
        x0 = nx / 2 + 0.5
        tips[e, 0], tips[e, 1], tips[e, 2] = [x0, 9.0, -1.0], [x0, 33.0, -1.0], [x0, 9.0, 23.0]
    m.laparoscopeTip.copy_(torch.as_tensor(tips.reshape(-1, 3)))
    o.a["laparoscopeTip"] = tips.reshape(-1).astype(np.float32).copy()
    c.cutLaparoscope()
    o.cutLaparoscope()
    _same(c, o, "cut")
    per_env = [int((c.flipEdge[m.envEdgeStart[e]:m.envEdgeStart[e + 1]] == -1).sum()) for e in range(3)]
    print(f"[cutting] edges cut per env: {per_env}")
    assert all(n > 0 for n in per_env) and per_env[0] == per_env[2]


@pytest.mark.parametrize("fades", [2, 6])
def test_steps_over_the_cut_topology_match_the_oracle(gpu, oracle_lib, fades):
    """After a cut and `fades` fade calls (active values part-way down, or at 0), the
    batched step rebuilds its plan and both step forms follow the oracle."""
    outs = {}
    for batched in (True, False):
        m = _model()
        integ = SimIntegratorDO("cuda:0", batched=batched)
        integ.stepModel(m, 2)
        c = SimCutting(m)
        tips0 = m.laparoscopeTip.clone()
        tips = tips0.cpu().numpy().reshape(-1, 4, 3).copy()
        for e, nx in enumerate((6, 4, 6)):
            x0 = nx / 2 + 0.5
            tips[e, 0], tips[e, 1], tips[e, 2] = [x0, 9.0, -1.0], [x0, 33.0, -1.0], [x0, 9.0, 23.0]
        m.laparoscopeTip.copy_(torch.as_tensor(tips.reshape(-1, 3)))
        c.cutLaparoscope()
        m.laparoscopeTip.copy_(tips0)                    # the instrument back where it was
        for _ in range(fades):
            c.updateActiveValues()
        torch.cuda.synchronize()
        st = lambda t: t.cpu().numpy()
        o = oracle.OracleSim(m, state={"vertex": st(m.vertex), "velocity": st(m.velocity),
                                       "predicted_vertex": st(m.predictedVertex),
                                       "active_tetrahedron": st(m.activeTetrahedron),
                                       "active_edge": st(m.activeEdge), "hole": st(m.hole),
                                       "laparoscope_tip": st(m.laparoscopeTip),
                                       "laparoscope_base": st(m.laparoscopeBase)})
        v0 = m.topologyVersion
        integ.stepModel(m, 6)
        o.step(6)
        torch.cuda.synchronize()
        if batched:
            assert integ.plan(m).version == m.topologyVersion == v0
        got = m.vertex.cpu().numpy()
        err = np.abs(got - o.a["vertex"]).max() / np.abs(o.a["vertex"]).max()
        outs[batched] = err
        part = np.unique(m.activeEdge.cpu().numpy())
        print(f"[cutting] {'batched' if batched else 'reference-shaped'} step after {fades} fades "
              f"(active values {np.round(part, 3).tolist()}): {err:.2e}")
        assert err < (1e-4 if batched else 1e-5)
