"""Serving loop: slot budget (CPU), alone-vs-mix equality, eviction/restore, closed loop (GPU)."""

import numpy as np
import pytest

from ffsrl import meshgen as mg
from ffsrl.serve import plan_slots, slot_bytes


def _pool():
    return [mg.ellipsoid_for_tets(t, seed=i) for i, t in enumerate([300, 900, 2000])]


def test_slot_budget_planning():
    pool = _pool()
    actors = np.array([0, 0, 1, 1, 1, 2, 2, 2, 2])
    big = plan_slots(pool, actors, 60e9, 128)
    assert big.tolist() == [2, 3, 4]
    per = np.array([slot_bytes(m, 128) for m in pool])
    budget = float(per.sum()) * 1.5
    k = plan_slots(pool, actors, budget, 128)
    assert (k >= 1).all() and float((k * per).sum()) <= budget and k.sum() < len(actors)
    with pytest.raises(Exception):
        plan_slots(pool, actors, float(per.sum()) * 0.5, 128)


def _serve(actors, budget=60e9, resolution=16):
    from ffsrl.serve import EnvServer
    return EnvServer(_pool(), actors, "cuda:0", hbm_budget_bytes=budget, resolution=resolution)


def _tick(srv, reqs):
    from ffsrl.serve import Request
    for a, d, c in reqs:
        srv.submit(Request(a, np.asarray(d, dtype=np.float32), c, 0.0))
    while srv.pending:
        srv.launch()
        srv.poll()
    return {r.actor: r.result for r in srv.drain()} | {}


def _run(srv, plan):
    out = {}
    for reqs in plan:
        from ffsrl.serve import Request
        for a, d, c in reqs:
            srv.submit(Request(a, np.asarray(d, dtype=np.float32), c, 0.0))
        done = []
        while srv.pending or any(ln.batch for ln in srv.lanes):
            srv.launch()
            done += srv.poll()
        for r in done:
            out.setdefault(r.actor, []).append(r.result.copy())
    return out


def _state(srv, a):
    s = int(srv.actor_slot[a])
    if s < 0:
        return srv.snapshots[a]["vertex"].numpy()
    v0, v1 = int(srv.model.envVertexStart[s]), int(srv.model.envVertexStart[s + 1])
    return srv.model.vertex[v0:v1].cpu().numpy()


@pytest.mark.gpu
def test_alone_equals_mix(gpu):
    actors = [0, 1, 2, 0, 1, 2]
    d = [[0.05, 0.02, -0.01], [-0.03, 0.04, 0.0], [0.0, -0.05, 0.02]]
    alone = _serve(actors)
    mix = _serve(actors)
    plan_alone = [[(4, d[k], 1)] for k in range(3)]
    plan_mix = [[(a, d[(k + a) % 3] if a != 4 else d[k], 1) for a in range(6)] for k in range(3)]
    ra = _run(alone, plan_alone)
    rm = _run(mix, plan_mix)
    for k in range(3):
        assert np.array_equal(ra[4][k], rm[4][k])
    assert np.array_equal(_state(alone, 4), _state(mix, 4))
    assert np.isfinite(_state(mix, 4)).all()


@pytest.mark.gpu
def test_alone_equals_mix_across_server_models(gpu):
    # an actor served by a model of its own mesh alone gives the same bits as in a model
    # built from a whole pool and stepped with other actors: each env's fixed-point scale
    # comes from its own coordinates.  Both models get the same gravity force (the
    # reference's gravity is one vector per model, applied times each vertex's inverse
    # mass; by default a server takes it from the mean vertex mass of its own pool)
    from ffsrl.serve import EnvServer
    pool = _pool()
    g = mg.gravity_force(pool)
    alone = EnvServer([pool[1]], [0], "cuda:0", resolution=16, environmentGravity=g)
    mix = EnvServer(pool, [0, 1, 2, 0, 1, 2], "cuda:0", resolution=16, environmentGravity=g)
    d = [[0.05, 0.02, -0.01], [-0.03, 0.04, 0.0], [0.0, -0.05, 0.02]]
    ra = _run(alone, [[(0, d[k], 1)] for k in range(3)])
    rm = _run(mix, [[(a, d[k] if a == 4 else d[(k + a) % 3], 1) for a in range(6)] for k in range(3)])
    for k in range(3):
        assert np.array_equal(ra[0][k], rm[4][k])
    assert np.array_equal(_state(alone, 0), _state(mix, 4))


@pytest.mark.gpu
def test_eviction_restores_state(gpu):
    actors = [0, 0, 1, 1, 2, 2]
    pool = _pool()
    per = np.array([slot_bytes(m, 16) for m in pool])
    small = _serve(actors, budget=float(per.sum()) * 1.2)
    assert small.num_slots == 3
    roomy = _serve(actors)
    d = [0.04, 0.01, -0.02]
    plan = [[(0, d, 1)], [(1, d, 1)], [(0, d, 1)], [(1, d, 1)], [(0, d, 1)]]
    rs, rr = _run(small, plan), _run(roomy, plan)
    assert small.evictions >= 3
    for a in (0, 1):
        for x, y in zip(rs[a], rr[a]):
            assert np.array_equal(x, y)
        assert np.array_equal(_state(small, a), _state(roomy, a))


@pytest.mark.gpu
def test_closed_loop_reports_latency(gpu):
    srv = _serve([0, 1, 2, 0, 1, 2, 0, 1])
    st = srv.run_closed_loop(0.5, think_hz=60.0, warmup_s=0.2)
    print("[serve]", st)
    assert st["requests"] > 8
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    assert st["served_env_steps_per_s"] > 0


@pytest.mark.gpu
def test_episode_reset_restarts_from_rest(gpu):
    # actor 3 steps three times, then starts a new episode with displacement d; actor 0
    # (same mesh) takes d as its first request: both end in the same state
    from ffsrl.serve import Request
    actors = [0, 1, 2, 0]
    srv = _serve(actors)
    d = [0.04, -0.02, 0.01]
    _run(srv, [[(3, [0.05, 0.0, 0.0], 1)], [(3, [0.0, 0.05, 0.0], 1)], [(3, [0.0, 0.0, 0.05], 1)]])
    srv.submit(Request(3, np.asarray(d, dtype=np.float32), 1, 0.0, reset=True))
    srv.submit(Request(0, np.asarray(d, dtype=np.float32), 1, 0.0))
    done = []
    while srv.pending or any(ln.batch for ln in srv.lanes):
        srv.launch()
        done += srv.poll()
    res = {r.actor: r.result for r in done}
    assert np.array_equal(res[3], res[0])
    assert np.array_equal(_state(srv, 3), _state(srv, 0))


def _run_native(srv, plan):
    from ffsrl.serve import Request
    out = {}
    for reqs in plan:
        for a, d, c, *rst in reqs:
            srv.submit(Request(a, np.asarray(d, dtype=np.float32), c, 0.0, reset=bool(rst and rst[0])))
        done = []
        while srv._stats()[2] or srv._stats()[3]:
            srv.launch()
            done += srv.poll()
        for r in done:
            out.setdefault(r.actor, []).append(r.result.copy())
    return out


@pytest.mark.gpu
def test_native_server_matches_the_python_server(gpu):
    # the C server (ffsrl_server_*) against EnvServer on the same requests: a slot budget
    # that forces evictions, episode resets and clamp changes; results and states bit-equal
    from ffsrl.serve import EnvServer, NativeEnvServer
    actors = [0, 0, 1, 1, 2, 2]
    pool = _pool()
    per = np.array([slot_bytes(m, 16) for m in pool])
    kw = dict(hbm_budget_bytes=float(per.sum()) * 1.2, resolution=16)
    py = EnvServer(pool, actors, "cuda:0", **kw)
    nat = NativeEnvServer(pool, actors, "cuda:0", **kw)
    assert nat.num_slots == py.num_slots == 3
    rng = np.random.default_rng(5)
    plan = []
    for k in range(8):
        acts = rng.permutation(6)[:3]
        plan.append([(int(a), rng.uniform(-0.05, 0.05, 3).tolist(), int(k % 4 != 3), int(k == 5 and a % 2 == 0))
                     for a in acts])
    from ffsrl.serve import Request
    rp = {}
    for reqs in plan:
        for a, d, c, rst in reqs:
            py.submit(Request(a, np.asarray(d, dtype=np.float32), c, 0.0, reset=bool(rst)))
        done = []
        while py.pending or any(ln.batch for ln in py.lanes):
            py.launch()
            done += py.poll()
        for r in done:
            rp.setdefault(r.actor, []).append(r.result.copy())
    rn = _run_native(nat, plan)
    print(f"[serve] native: {nat.admissions} admissions, {nat.evictions} evictions; python: {py.admissions}, "
          f"{py.evictions}")
    assert nat.evictions == py.evictions >= 3 and nat.admissions == py.admissions
    assert sorted(rp) == sorted(rn)
    for a in rp:
        assert len(rp[a]) == len(rn[a])
        for x, y in zip(rp[a], rn[a]):
            assert np.array_equal(x, y)
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    assert np.array_equal(py.model.vertex.cpu().numpy(), nat.model.vertex.cpu().numpy())
    assert np.array_equal(py.renderer.pixels.cpu().numpy(), nat.renderer.pixels.cpu().numpy())
    nat.close()
