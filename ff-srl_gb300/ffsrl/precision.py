"""Precision report: the batched step in float32 against the same kernel in float64.

Both runs start from the same state and use the same constraint tables (rest volumes
and inverse rest-shape matrices computed in float64 by the mesh generator, stored in
float32). The float32 run sums corrections exactly in fixed point and rounds once. The
float64 run sums in double. The report gives the position error of the float32 run
against the float64 run, max and RMS, relative to the largest coordinate. It also gives
the volume-conservation error of each tet as |det F - 1|, with
F = Ds Dm^-1 = signed volume / signed rest volume.
"""

from __future__ import annotations

import numpy as np

from . import scenarios as sc
from .integrator import BatchPlan


def det_f(x: np.ndarray, tets: np.ndarray, rest_signed: np.ndarray) -> np.ndarray:
    """det F per tet: current signed volume over the signed rest volume."""
    t = tets.reshape(-1, 4)
    a = x[t[:, 0]]
    s6 = np.einsum("ij,ij->i", np.cross(x[t[:, 1]] - a, x[t[:, 2]] - a), x[t[:, 3]] - a)
    return (s6 / 6.0) / rest_signed.astype(np.float64)


def precision_report(meshes, steps: int, substeps: int = 16, iterations: int = 50, nu: float = 0.49,
                     device: str = "cuda:0") -> dict:
    """Config-3 form: the liver constraint set (no contact) at Poisson ratio ``nu``."""
    make = lambda: sc.liver_model(device, len(meshes), meshes=meshes, nu=nu, substeps=substeps,
                                  iterations=iterations, collide=False)[0]
    return compare(make(), make(), steps) | {"substeps": substeps, "iterations": iterations, "nu": nu}


def compare(m32, m64, steps: int) -> dict:
    """Steps two identical models, one in the float32 batched kernel and one in its float64
    build, and reports the float32 run's errors against the float64 run."""
    import torch
    p32 = BatchPlan(m32)
    p64 = BatchPlan(m64, precision=64)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record()
    p32.step(steps)
    ev[1].record()
    p64.step(steps)
    ev[2].record()
    torch.cuda.synchronize()
    x32 = m32.vertex.cpu().numpy().astype(np.float64)
    x64 = p64.state_f64()["vertex"]
    scale = np.abs(x64).max()
    d = np.linalg.norm(x32 - x64, axis=1)
    tets = m32.host["tetrahedron"]
    rest = m32.host["tetrahedronRestVolumeSigned"]
    j32, j64 = det_f(x32, tets, rest), det_f(x64, tets, rest)
    return {
        "envs": int(m32.numEnvs), "steps": steps, "substeps": m32.simSubsteps, "iterations": m32.simConstraints,
        "vertices": int(m32.numVertices), "tets": int(m32.numTetrahedrons),
        "max_pos_err": float(d.max()), "rms_pos_err": float(np.sqrt((d ** 2).mean())),
        "max_pos_err_rel": float(d.max() / scale), "rms_pos_err_rel": float(np.sqrt((d ** 2).mean()) / scale),
        "volume_err_f32": {"max": float(np.abs(j32 - 1).max()), "mean": float(np.abs(j32 - 1).mean())},
        "volume_err_f64": {"max": float(np.abs(j64 - 1).max()), "mean": float(np.abs(j64 - 1).mean())},
        "ms_f32": ev[0].elapsed_time(ev[1]), "ms_f64": ev[1].elapsed_time(ev[2]),
        "finite": bool(np.isfinite(x32).all() and np.isfinite(x64).all()),
    }


def all_configs(device: str = "cuda:0") -> list[dict]:
    """The float32-vs-float64 report for each workload: the beam (config 0, reference
    step, 25 steps), the 12/8/6 cm ellipsoid (config 1, Neo-Hookean, grasp, 5 steps),
    envs of the mixed-size pool shared by the throughput and serving workloads (configs 2
    and 4, 16 envs, 5 steps) and the nearly incompressible ellipsoid (config 3, nu 0.49,
    16 substeps x 50 iterations, 3 steps).  The float64 build is slow, so the env counts
    and step counts are samples of each workload."""
    import torch
    from . import meshgen as mg
    out = []
    beam = lambda: sc.beam_model(device, 1)[0]
    out.append({"config": "0 beam, reference step"} | compare(beam(), beam(), 25))

    def liver(meshes, **kw):
        m, _ = sc.liver_model(device, len(meshes), meshes=meshes, **kw)
        m.graspNearest(torch.ones(len(meshes), dtype=torch.int32, device=device), radius=0.5)
        return m

    ell = [mg.ellipsoid()]
    out.append({"config": "1 ellipsoid, Neo-Hookean + grasp + contact"} | compare(liver(ell), liver(ell), 5))
    pool, _ = sc.mixed_meshes(16, pool_size=64, seed=0)
    out.append({"config": "2/4 mixed-size pool, 16 envs"} | compare(liver(pool), liver(pool), 5))
    out.append({"config": "3 ellipsoid, nu 0.49, 16 x 50"} | precision_report(ell, steps=3, device=device))
    return out


if __name__ == "__main__":
    import json
    for row in all_configs():
        print(json.dumps(row))
