"""Precision report: the batched step in float32 against the same kernel in float64.

Every run starts from the same state and uses the same constraint tables (rest volumes
and inverse rest-shape matrices computed in float64 by the mesh generator, stored in
float32), with the reference arithmetic (the reference kernels' expressions, IEEE
division and square root).  The float32 runs differ only in how each vertex's
corrections are summed:

* ``fixed``: every term rounded once to 32-bit fixed point (a quarter float ulp of the
  env's largest coordinate) and summed exactly, then rounded once to float;
* ``kahan``: float32 compensated summation, (sum, compensation) pairs per vertex;
* ``atomic``: plain float32 atomics, as the reference sums them.

The float64 run sums in double.  The report gives each float32 run's position error
against the float64 run, max and RMS, relative to the largest coordinate, and the
volume-conservation error of each tet as |det F - 1|, with F = Ds Dm^-1 = signed volume /
signed rest volume.
"""

from __future__ import annotations

import numpy as np

from . import scenarios as sc
from .integrator import BatchPlan

ACCUMULATIONS = ("fixed", "kahan", "atomic")


def det_f(x: np.ndarray, tets: np.ndarray, rest_signed: np.ndarray) -> np.ndarray:
    """det F per tet: current signed volume over the signed rest volume."""
    t = tets.reshape(-1, 4)
    a = x[t[:, 0]]
    s6 = np.einsum("ij,ij->i", np.cross(x[t[:, 1]] - a, x[t[:, 2]] - a), x[t[:, 3]] - a)
    return (s6 / 6.0) / rest_signed.astype(np.float64)


def compare(make, steps: int, accumulations=ACCUMULATIONS, every: int = 0, on_row=None) -> dict:
    """Steps identical models ``make()`` in each float32 accumulation and in the float64
    build, and reports every float32 run against the float64 run.  With ``every`` > 0 the
    runs advance in lock step and ``on_row`` receives the report at every ``every``-th
    step (the last one is returned)."""
    import torch
    m64 = make()
    p64 = BatchPlan(m64, precision=64)
    runs = {}
    for acc in accumulations:
        m = make()
        runs[acc] = (m, BatchPlan(m, accumulation=acc))
    tets = m64.host["tetrahedron"]
    rest = m64.host["tetrahedronRestVolumeSigned"]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms = {"f64": 0.0} | {acc: 0.0 for acc in accumulations}
    done = 0
    out = None
    chunk = every if every > 0 else steps
    while done < steps:
        k = min(chunk, steps - done)
        ev[0].record()
        p64.step(k)
        ev[1].record()
        torch.cuda.synchronize()
        ms["f64"] += ev[0].elapsed_time(ev[1])
        for acc, (m, p) in runs.items():
            ev[0].record()
            p.step(k)
            ev[1].record()
            torch.cuda.synchronize()
            ms[acc] += ev[0].elapsed_time(ev[1])
        done += k
        x64 = p64.state_f64()["vertex"]
        scale = np.abs(x64).max()
        j64 = det_f(x64, tets, rest)
        out = {"envs": int(m64.numEnvs), "steps": done, "substeps": m64.simSubsteps, "iterations": m64.simConstraints,
               "vertices": int(m64.numVertices), "tets": int(m64.numTetrahedrons), "ms_f64": ms["f64"],
               "volume_err_f64": {"max": float(np.abs(j64 - 1).max()), "mean": float(np.abs(j64 - 1).mean())},
               "finite": bool(np.isfinite(x64).all())}
        for acc, (m, p) in runs.items():
            x = m.vertex.cpu().numpy().astype(np.float64)
            d = np.linalg.norm(x - x64, axis=1)
            j = det_f(x, tets, rest)
            out[acc] = {"max_pos_err_rel": float(d.max() / scale), "rms_pos_err_rel": float(np.sqrt((d ** 2).mean()) / scale),
                        "volume_err": {"max": float(np.abs(j - 1).max()), "mean": float(np.abs(j - 1).mean())},
                        "ms": ms[acc], "status_nonzero": int((p.env_status() != 0).sum())}
            out["finite"] = out["finite"] and bool(np.isfinite(x).all())
        if on_row is not None:
            on_row(dict(out))
    return out


def config3(envs: int = 4, steps: int = 300, device: str = "cuda:0", accumulations=ACCUMULATIONS, every: int = 0,
            on_row=None) -> dict:
    """Config 3: the 12/8/6 cm ellipsoid at Poisson ratio 0.49, 16 substeps x 50 iterations,
    the liver constraint set without contact, ``envs`` identical envs."""
    from . import meshgen as mg
    mesh = mg.ellipsoid()
    make = lambda: sc.liver_model(device, envs, meshes=[mesh] * envs, nu=0.49, substeps=16, iterations=50,
                                  collide=False)[0]
    tag = {"config": "3 ellipsoid, nu 0.49, 16 x 50"}
    row = None if on_row is None else (lambda r: on_row(tag | r | {"nu": 0.49}))
    return tag | compare(make, steps, accumulations, every=every, on_row=row) | {"nu": 0.49}


def all_configs(device: str = "cuda:0", steps: int = 100, steps3: int = 300, envs3: int = 4, which=(0, 1, 2, 3)):
    """The float32-vs-float64 report for each workload, one row per workload as it
    finishes: the beam (config 0, reference step), the 12/8/6 cm ellipsoid (config 1,
    Neo-Hookean, grasp, contact), 16 envs with one mesh each from the generator shared by
    the throughput and serving workloads (configs 2 and 4), all ``steps`` steps, and the
    nearly incompressible ellipsoid (config 3, ``steps3`` steps)."""
    import torch
    from . import meshgen as mg

    def liver(meshes):
        m, _ = sc.liver_model(device, len(meshes), meshes=meshes)
        m.graspNearest(torch.ones(len(meshes), dtype=torch.int32, device=device), radius=0.5)
        return m

    if 0 in which:
        yield {"config": "0 beam, reference step"} | compare(lambda: sc.beam_model(device, 1)[0], steps)
    if 1 in which:
        ell = [mg.ellipsoid()]
        yield {"config": "1 ellipsoid, Neo-Hookean + grasp + contact"} | compare(lambda: liver(ell), steps)
    if 2 in which:
        pool, _ = sc.mixed_meshes(16, pool_size=0, seed=0)
        yield {"config": "2/4 one mesh per env, 16 envs"} | compare(lambda: liver(pool), steps)
    if 3 in which:
        yield config3(envs3, steps3, device)


if __name__ == "__main__":
    # python -m ffsrl.precision [configs, e.g. 012 or 3] [steps for config 3]
    import json
    import sys
    which = tuple(int(c) for c in sys.argv[1]) if len(sys.argv) > 1 else (0, 1, 2, 3)
    steps3 = int(sys.argv[2]) if len(sys.argv) > 2 else 300
    if which == (3,):
        # config 3 alone: one env, every 25 steps a row, so a long run reports as it goes
        config3(1, steps3, every=25, on_row=lambda r: print(json.dumps(r), flush=True))
    else:
        for row in all_configs(which=which, steps3=steps3):
            print(json.dumps(row), flush=True)
