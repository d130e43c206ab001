"""Small, self-ending workloads for profiling one kernel under ncu.

Each case builds its inputs, runs the kernel of interest once (plus whatever set-up
launches it needs) and exits. The inputs are larger than L2 but hold at most a few GB on
the device, so a capture of one to six launches ends within a minute or two.

    python -m ffsrl.profile_cases step_mixed [envs]   # every size-class launch of one batched step
    python -m ffsrl.profile_cases step_big            # one size class of large envs (12k-20k tets)
    python -m ffsrl.profile_cases render              # refit + ray-cast of 256 envs at 128x128
    python -m ffsrl.profile_cases step_uniform [constraints] [block]
                                                      # 152 copies of one 16k-tet mesh, one step with the
                                                      # named constraints (e.g. VOLUME+DISTANCE; default: all)
    python -m ffsrl.profile_cases constraint_costs    # timed batched step per constraint subset (4096 envs)
    python -m ffsrl.profile_cases contact_costs       # timed batched step, contact on/off, tools pressed/lifted

The step cases draw their meshes from the same seeded 64-mesh pool as the 4096-env
throughput workload, so per-env-step figures scale to it.
"""

from __future__ import annotations

import sys

import torch

from . import SimBVH, SimIntegratorDO, WarpRaycastRendererDO
from . import scenarios as sc


def step_mixed(envs: int = 512, device: str = "cuda:0") -> None:
    meshes, _ = sc.mixed_meshes(envs, pool_size=64, seed=0)
    m, _ = sc.liver_model(device, envs, meshes=meshes)
    m.graspNearest(torch.ones(envs, dtype=torch.int32, device=device), radius=0.5)
    integ = SimIntegratorDO(device, autotune=True)
    p = integ.plan(m)
    print(p.info(), integ.tuning)
    p.step(1)
    torch.cuda.synchronize()


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
    p = SimIntegratorDO(device, blockThreads=block).plan(m)
    print(p.info(), hex(m.constraintFlags))
    p.step(1)
    torch.cuda.synchronize()


def render(envs: int = 256, device: str = "cuda:0") -> None:
    meshes, _ = sc.mixed_meshes(envs, pool_size=16, seed=0)
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


def _time_step(m, device, reps: int = 3) -> float:
    integ = SimIntegratorDO(device, autotune=True)
    p = integ.plan(m)
    p.step(1)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(reps):
        p.step(1)
    ev[1].record()
    torch.cuda.synchronize()
    return ev[0].elapsed_time(ev[1]) / reps


def constraint_costs(envs: int = 4096, device: str = "cuda:0") -> None:
    """Batched-step time of the 4096-env mixed pool with subsets of the constraint kernels
    (CUDA events, mean of 3 steps after one untimed), one JSON line per subset."""
    import json
    from . import _lib as L
    meshes, _ = sc.mixed_meshes(envs, pool_size=64, seed=0)
    V, D, N, DR, C = L.VOLUME, L.DISTANCE, L.NEOHOOKEAN, L.DRAG, L.COLLIDE
    subsets = {"all": V | D | N | DR | C, "all but contact": V | D | N | DR, "all but grasp": V | D | N | C,
               "Neo-Hookean": N, "volume": V, "distance": D, "volume + distance": V | D,
               "Neo-Hookean + volume": N | V, "none (gravity, apply, PBD step)": 0}
    for name, fl in subsets.items():
        m, _ = sc.liver_model(device, envs, meshes=meshes, instrument_visual=False)
        m.constraintFlags = fl
        m.graspNearest(torch.ones(envs, dtype=torch.int32, device=device), radius=0.5)
        print(json.dumps({"constraints": name, "ms": _time_step(m, device)}), flush=True)
        del m
        torch.cuda.empty_cache()


def contact_costs(envs: int = 4096, device: str = "cuda:0") -> None:
    """Batched-step time with and without the contact kernel, with the instruments pressed
    into the surface and lifted 50 cm away from it."""
    import json
    meshes, _ = sc.mixed_meshes(envs, pool_size=64, seed=0)
    for tools, lift in (("pressed", 0.0), ("lifted", 50.0)):
        for collide in (True, False):
            m, _ = sc.liver_model(device, envs, meshes=meshes, instrument_visual=False, collide=collide)
            if lift:
                d = torch.zeros((envs, 3), device=device)
                d[:, 1] = lift
                m.moveTool(d)
            m.graspNearest(torch.ones(envs, dtype=torch.int32, device=device), radius=0.5)
            ms = _time_step(m, device)
            print(json.dumps({"tools": tools, "contact": collide, "ms": ms,
                              "envs_in_contact": int((m.laparoscopeInCollision > 0).sum())}), flush=True)
            del m
            torch.cuda.empty_cache()


def main(argv: list[str]) -> None:
    case = argv[0] if argv else "step_mixed"
    if case == "step_mixed":
        step_mixed(int(argv[1]) if len(argv) > 1 else 512)
    elif case == "step_big":
        step_big()
    elif case == "step_uniform":
        step_uniform(argv[1] if len(argv) > 1 else "", int(argv[2]) if len(argv) > 2 else 1024)
    elif case == "render":
        render()
    elif case == "constraint_costs":
        constraint_costs()
    elif case == "contact_costs":
        contact_costs()
    else:
        raise SystemExit(f"unknown case {case!r}: step_mixed, step_big, step_uniform, render, constraint_costs "
                         "or contact_costs")
    print("ok")


if __name__ == "__main__":
    main(sys.argv[1:])
