"""Env sharding across ranks, on CPU with gloo (world size 2).

Envs are independent, so stepping each rank's shard must give, env by env, exactly the
positions that stepping the whole list gives. The oracle steps both here: the property
under test is the sharding and the host-side reductions, not the kernels.
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from ffsrl import shard as sh

WORLD = 2
NUM_ENVS = 5


def _pool():
    from ffsrl import scenarios as sc
    return sc.mixed_meshes(NUM_ENVS, pool_size=3, seed=4, t_lo=150, t_hi=400)[0]


def _step(meshes, gravity):
    import oracle
    from ffsrl import scenarios as sc
    m, _ = sc.liver_model("cpu", len(meshes), meshes=meshes, environmentGravity=gravity)
    o = oracle.OracleSim(m)
    o.step(2)
    x = o.a["vertex"]
    per_env = [x[int(m.envVertexStart[e]):int(m.envVertexStart[e + 1])].copy() for e in range(len(meshes))]
    return per_env, o.a["laparoscope_in_collision"].copy()


def _rank_main(rank, port, out_dir):
    import torch.distributed as dist
    from ffsrl import meshgen as mg
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        meshes = _pool()
        gravity = mg.gravity_force(meshes[0])
        lo, hi = sh.env_range(NUM_ENVS, rank, WORLD)
        mine = sh.shard(meshes, rank, WORLD)
        assert len(mine) == hi - lo
        x, coll = _step(mine, gravity)
        rows = torch.tensor([[len(xe), float(np.abs(xe).sum()), float(c)] for xe, c in zip(x, coll)],
                            dtype=torch.float64)
        allrows = sh.gather_env_results(rows, NUM_ENVS)
        slowest = sh.max_over_ranks(10.0 + rank)
        total = sh.sum_over_ranks(hi - lo)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), lo=lo, hi=hi, coll=coll, rows=allrows.numpy(),
                 slowest=slowest, total=total, *x)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_env_range_partitions():
    for n in (0, 1, 5, 4096, 4097):
        for w in (1, 2, 3, 8):
            ranges = [sh.env_range(n, r, w) for r in range(w)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        sh.env_range(4, 2, 2)
    assert sh.max_over_ranks(3.5) == 3.5  # no process group: the value itself


def test_sharded_step_matches_unsharded(oracle_lib, tmp_path):
    from ffsrl import meshgen as mg
    mp.start_processes(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=WORLD, join=True,
                       start_method="spawn")
    meshes = _pool()
    full_x, full_coll = _step(meshes, mg.gravity_force(meshes[0]))
    seen = []
    for r in range(WORLD):
        d = np.load(tmp_path / f"rank{r}.npz")
        lo, hi = int(d["lo"]), int(d["hi"])
        seen.extend(range(lo, hi))
        for k, e in enumerate(range(lo, hi)):
            assert np.array_equal(d[f"arr_{k}"], full_x[e]), f"env {e} differs on rank {r}"
        assert np.array_equal(d["coll"], full_coll[lo:hi])
        # gathered rows agree on every rank and follow env order
        rows = d["rows"]
        assert rows.shape == (NUM_ENVS, 3)
        assert np.array_equal(rows[:, 0], [len(x) for x in full_x])
        assert np.array_equal(rows[:, 2], full_coll.astype(np.float64))
        assert float(d["slowest"]) == 10.0 + WORLD - 1
        assert float(d["total"]) == NUM_ENVS
    assert seen == list(range(NUM_ENVS))
