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
    import torch
    m32, _ = sc.liver_model(device, len(meshes), meshes=meshes, nu=nu, substeps=substeps, iterations=iterations,
                            collide=False)
    m64, _ = sc.liver_model(device, len(meshes), meshes=meshes, nu=nu, substeps=substeps, iterations=iterations,
                            collide=False)
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
        "envs": len(meshes), "steps": steps, "substeps": substeps, "iterations": iterations, "nu": nu,
        "vertices": int(m32.numVertices), "tets": int(m32.numTetrahedrons),
        "max_pos_err": float(d.max()), "rms_pos_err": float(np.sqrt((d ** 2).mean())),
        "max_pos_err_rel": float(d.max() / scale), "rms_pos_err_rel": float(np.sqrt((d ** 2).mean()) / scale),
        "volume_err_f32": {"max": float(np.abs(j32 - 1).max()), "mean": float(np.abs(j32 - 1).mean())},
        "volume_err_f64": {"max": float(np.abs(j64 - 1).max()), "mean": float(np.abs(j64 - 1).mean())},
        "ms_f32": ev[0].elapsed_time(ev[1]), "ms_f64": ev[1].elapsed_time(ev[2]),
        "finite": bool(np.isfinite(x32).all() and np.isfinite(x64).all()),
    }
