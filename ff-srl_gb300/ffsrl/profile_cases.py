"""Small, self-ending workloads for profiling one kernel under ncu.

Each case builds its inputs, runs the kernel of interest once (plus whatever set-up
launches it needs) and exits. The inputs are larger than L2 but hold at most a few GB on
the device, so a capture of one to six launches ends within a minute or two.

    python -m ffsrl.profile_cases step_mixed [envs] [arithmetic] [pool]
                                       # every size-class launch of one batched step (default
                                       # 512 envs, fast arithmetic, one mesh per env)
    python -m ffsrl.profile_cases step_big            # one size class of large envs (12k-20k tets)
    python -m ffsrl.profile_cases step_uniform [constraints] [block]
                                       # 152 copies of one 16k-tet mesh, one step with the named
                                       # constraints (e.g. VOLUME+DISTANCE; default: all)
    python -m ffsrl.profile_cases render [envs]       # refit + vertex normals + ray-cast at 128x128
    python -m ffsrl.profile_cases plain [envs]        # one reference-shaped step (one launch per kernel)

The mixed cases draw per-env meshes from the same seeded generator as the 4096-env
throughput workload (tet counts log-uniform in [500, 20000]), so per-env-step figures
scale to it.
"""

from __future__ import annotations

import ctypes as C
import sys

import torch

from . import SimBVH, SimIntegratorDO, WarpRaycastRendererDO
from . import scenarios as sc


def step_mixed(envs: int = 512, arithmetic: str = "fast", pool: int = 0, device: str = "cuda:0") -> None:
    """The autotuned batched step; the step after tuning runs inside the NVTX range
    ``profiled_step`` (capture it with ``ncu --nvtx --nvtx-include profiled_step/``)."""
    meshes, _ = sc.mixed_meshes(envs, pool_size=pool, seed=0)
    m, _ = sc.liver_model(device, envs, meshes=meshes)
    m.graspNearest(torch.ones(envs, dtype=torch.int32, device=device), radius=0.5)
    integ = SimIntegratorDO(device, autotune=True, arithmetic=arithmetic)
    p = integ.plan(m)
    print(p.info(), integ.tuning)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profiled_step")
    p.step(1)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()


def step_big(device: str = "cuda:0") -> None:
    meshes, _ = sc.mixed_meshes(304, pool_size=8, seed=3, t_lo=12000, t_hi=20000)
    m, _ = sc.liver_model(device, 304, meshes=meshes)
    m.graspNearest(torch.ones(304, dtype=torch.int32, device=device), radius=0.5)
    p = SimIntegratorDO(device).plan(m)
    print(p.info())
    p.step(1)
    torch.cuda.synchronize()


def step_uniform(constraints: str = "", block: int = 1024, envs: int = 152, device: str = "cuda:0") -> None:
    from . import _lib as L
    from . import meshgen as mg
    mesh = mg.ellipsoid_for_tets(16000, seed=7)
    m, _ = sc.liver_model(device, envs, meshes=[mesh] * envs)
    if constraints:
        m.constraintFlags = 0
        for name in constraints.split("+"):
            m.constraintFlags |= getattr(L, name)
    p = SimIntegratorDO(device, blockThreads=block, arithmetic="fast").plan(m)
    print(p.info(), hex(m.constraintFlags))
    p.step(1)
    torch.cuda.synchronize()


def render(envs: int = 256, device: str = "cuda:0") -> None:
    meshes, _ = sc.mixed_meshes(envs, pool_size=0, seed=0)
    m, _ = sc.liver_model(device, envs, meshes=meshes)
    bvh = SimBVH(device, m)
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO(device, m, resolution=128, mode="headless", verticalAperture=ap,
                              horizontalAperture=ap)
    pos, rot = sc.env_cameras(meshes, seed=1)
    r.setCameras(pos, rot)
    bvh.refitBVH()
    r.renderNew(bvh, m)
    torch.cuda.synchronize()


def plain(envs: int = 512, device: str = "cuda:0") -> None:
    from . import _lib as L
    meshes, _ = sc.mixed_meshes(envs, pool_size=0, seed=0)
    m, _ = sc.liver_model(device, envs, meshes=meshes)
    m.graspNearest(torch.ones(envs, dtype=torch.int32, device=device), radius=0.5)
    dm, prm = m.device_model(), m.params()
    L.check(L.lib().ffsrl_step_model(C.byref(dm), C.byref(prm), None))
    torch.cuda.synchronize()


def main(argv: list[str]) -> None:
    case = argv[0] if argv else "step_mixed"
    if case == "step_mixed":
        step_mixed(int(argv[1]) if len(argv) > 1 else 512, argv[2] if len(argv) > 2 else "fast",
                   int(argv[3]) if len(argv) > 3 else 0)
    elif case == "step_big":
        step_big()
    elif case == "step_uniform":
        step_uniform(argv[1] if len(argv) > 1 else "", int(argv[2]) if len(argv) > 2 else 1024)
    elif case == "render":
        render(int(argv[1]) if len(argv) > 1 else 256)
    elif case == "plain":
        plain(int(argv[1]) if len(argv) > 1 else 512)
    else:
        raise SystemExit(f"unknown case {case!r}: step_mixed, step_big, step_uniform, render or plain")
    print("ok")


if __name__ == "__main__":
    main(sys.argv[1:])
