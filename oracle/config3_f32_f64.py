"""Config 3 in the oracle: the reference algorithm in float32 against float64.

Test infrastructure, like the rest of this directory.  The oracle (the serial
restatement of the reference kernels, in the reference's launch and thread order) steps
config 3 -- the 12/8/6 cm ellipsoid at Poisson ratio 0.49, 16 substeps x 50 iterations,
the liver constraint set without contact, one env -- once in float32 and once in
float64.  Every 25 steps it prints the float32 run's position error against the float64
run (max and RMS, relative to the largest coordinate) and both runs' volume error
|det F - 1| per tet.  This is the float32 error of the reference algorithm itself, to set
beside the batched kernel's (``python -m ffsrl.precision 3``, on a GPU).

    python oracle/config3_f32_f64.py [steps] [every]      # 300 and 25 by default

The two runs go to two processes; on one host core each, 300 steps take about 20 and
26 minutes.
"""

from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, os.path.join(ROOT, "ff-srl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def _model():
    from ffsrl import meshgen as mg, scenarios as sc
    return sc.liver_model("cpu", 1, meshes=[mg.ellipsoid()], nu=0.49, substeps=16, iterations=50, collide=False)[0]


def _run(prec: int, steps: int, every: int, q) -> None:
    import oracle
    m = _model()
    o = oracle.OracleSim(m)
    if prec == 64:
        x64 = o.a["vertex"].astype(np.float64).copy()
        xp64, v64 = np.zeros_like(x64), np.zeros_like(x64)
    done = 0
    while done < steps:
        k = min(every, steps - done)
        if prec == 64:
            o.step_f64(k, x64, xp64, v64)
            x = x64.copy()
        else:
            o.step(k)
            x = o.a["vertex"].astype(np.float64)
        done += k
        q.put((prec, done, x))


def _det_f(x, tets, rest_signed):
    t = tets.reshape(-1, 4)
    a = x[t[:, 0]]
    s6 = np.einsum("ij,ij->i", np.cross(x[t[:, 1]] - a, x[t[:, 2]] - a), x[t[:, 3]] - a)
    return (s6 / 6.0) / rest_signed.astype(np.float64)


def main(steps: int = 300, every: int = 25) -> None:
    m = _model()
    tets, rest = m.host["tetrahedron"], m.host["tetrahedronRestVolumeSigned"]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_run, args=(p, steps, every, q)) for p in (32, 64)]
    for p in procs:
        p.start()
    got: dict[int, dict[int, np.ndarray]] = {32: {}, 64: {}}
    for _ in range(2 * ((steps + every - 1) // every)):
        prec, k, x = q.get()
        got[prec][k] = x
        if k in got[32] and k in got[64]:
            x32, x64 = got[32].pop(k), got[64].pop(k)
            d = np.linalg.norm(x32 - x64, axis=1)
            scale = np.abs(x64).max()
            j32, j64 = _det_f(x32, tets, rest), _det_f(x64, tets, rest)
            print(json.dumps({"config": "3 ellipsoid, nu 0.49, 16 x 50, oracle", "steps": k,
                              "vertices": int(m.numVertices), "tets": int(m.numTetrahedrons),
                              "max_pos_err_rel": float(d.max() / scale),
                              "rms_pos_err_rel": float(np.sqrt((d ** 2).mean()) / scale),
                              "volume_err_f32": {"max": float(np.abs(j32 - 1).max()), "mean": float(np.abs(j32 - 1).mean())},
                              "volume_err_f64": {"max": float(np.abs(j64 - 1).max()), "mean": float(np.abs(j64 - 1).mean())},
                              "finite": bool(np.isfinite(x32).all() and np.isfinite(x64).all())}), flush=True)
    for p in procs:
        p.join()


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 300, int(sys.argv[2]) if len(sys.argv) > 2 else 25)
