"""Benchmark: env-steps/s of the multi-environment soft-tissue step at 4096 environments.

Workload (one "step"): every environment of a 4096-env batch drawn from a pool of
mixed-size ellipsoids (tet counts log-uniform in [500, 20000]) takes one RL step --
an effector displacement through the instrument's kinematic chain (0.5 mm random walk,
applyCartesianActionsInWorkspace), 8 substeps x 10 Jacobi iterations of
Neo-Hookean + volume + distance constraints with grasp and instrument contact, BVH refit,
and a 128x128 (2x2 supersampled) depth + colour ray-cast per environment.

  value  -- env-steps/s with inputs resident in HBM (CUDA events on the stream)
  e2e    -- the same through the public API with host buffers: each step copies the
            actions (N x 4 float32 from pinned memory) to the device and reads back the
            per-env result (effector position + contact count, N x 4 float32)
  plain  -- the reference-shaped drop-in (one launch per reference kernel) on the same GPU

Every env has a mesh of its own by default (config 2 draws a tet count per env);
``--pool K`` draws the 4096 envs from K shared meshes instead.  ``--arithmetic`` picks the
batched step's arithmetic for the headline (``fast``: hardware reciprocals; ``reference``:
the reference kernels' own expressions, IEEE division and square root); the step kernel
of the other form is timed beside it.

`--impl reference` times the reference algorithm's CPU implementation (the C++
restatement, all host threads) on a bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "ff-srl_gb300"))

METRIC = "env-steps/s at 4096 envs"
NUM_ENVS = 4096
RES = 128
POOL = 0  # 0: one mesh per env
GRASP_RADIUS = 0.5  # cm: grasp the nearest surface vertex within this distance of the drag point
EPISODE = 16  # RL episode length: every env returns to its rest state after this many steps


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ffsrl", choices=["ffsrl", "reference"])
    ap.add_argument("--envs", type=int, default=NUM_ENVS)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--serve-impl", choices=("native", "python"), default="native",
                    help="serving loop: the library's C server (ffsrl_server_*) or the Python EnvServer")
    ap.add_argument("--no-graph", action="store_true", help="launch the env-step eagerly instead of a CUDA graph")
    ap.add_argument("--pool", type=int, default=POOL, help="distinct meshes the envs draw from (0: one per env)")
    ap.add_argument("--arithmetic", choices=("fast", "reference"), default="fast",
                    help="batched-step arithmetic of the headline")
    ap.add_argument("--plain-steps", type=int, default=5)
    ap.add_argument("--pressure-seconds", type=float, default=5.0,
                    help="serving with a binding HBM budget (a quarter of one slot per actor), 64-mesh pool")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def config(envs, n, pool=POOL, arithmetic="fast"):
    return {"workload": f"{envs} mixed-size ellipsoid envs (tets log-uniform 500-20000), 8 substeps x 10 iterations, "
                        f"Neo-Hookean+volume+distance+grasp+contact, kinematic instrument (rendered), BVH refit, "
                        f"{RES}x{RES} depth+colour ray-cast",
            "envs_per_gpu": envs, "pool_meshes": pool if pool > 0 else envs, "substeps": 8, "iterations": 10,
            "resolution": RES, "arithmetic": arithmetic,
            "parallelism": f"env-shard x{n}", "l2": "working set (GBs) exceeds the 129 MB L2; no flush needed",
            "episode_steps": EPISODE, "episode_reset": "all envs to rest state + grasp, inside the timed region"}


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while active."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up briefly holds the GPU: the timed region starts after
            # its first reading
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 7 for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            for k in ("hbm_gbs", "hbm_GBs", "hbm"):
                if k in d:
                    return float(d[k]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def algorithmic_bytes(model, substeps=8, iterations=10, nh=True):
    """Per-step compulsory bytes of the constraint solve, summed over envs:
    B_iter = V*32 + E*12 + T*(20 [+36 NH]) + F*12; B_sub = I*B_iter + V*48; B = S*B_sub."""
    V, E, T, F = model.numVertices, model.numEdges, model.numTetrahedrons, model.numTriangles
    b_iter = V * 32 + E * 12 + T * (20 + (36 if nh else 0)) + F * 12
    return substeps * (iterations * b_iter + V * 48)


def build_workload(device, envs, seed, pool_size=POOL):
    import torch
    from ffsrl import SimBVH, SimIntegratorDO, WarpRaycastRendererDO, scenarios as sc
    meshes, pool = sc.mixed_meshes(envs, pool_size=pool_size, seed=seed)
    m, _ = sc.liver_model(device, envs, meshes=meshes)
    bvh = SimBVH(device, m)
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO(device, m, resolution=RES, mode="headless", verticalAperture=ap,
                              horizontalAperture=ap, lightPos=(0.3, 1.0, 0.5), lightIntensity=0.8)
    pos, rot = sc.env_cameras(meshes, seed=seed + 1)
    r.setCameras(pos, rot)
    m.graspNearest(torch.ones(envs, dtype=torch.int32, device=device), radius=GRASP_RADIUS)
    return m, meshes, pool, bvh, r


def cpu_sample(meshes, threads, n_env=16):
    """Oracle (C++ restatement) env-steps/s on a bounded sample of the workload: the full
    env-step of ``n_env`` envs -- solve, remap, BVH refit and the RES x RES ray-cast --
    with envs spread over ``threads`` host threads. Set-up is outside the timed call."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from ffsrl import SimBVH, WarpRaycastRendererDO, scenarios as sc
    m, _ = sc.liver_model("cpu", n_env, meshes=meshes[:n_env])
    bvh = SimBVH("cpu", m)
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO("cpu", m, resolution=RES, mode="headless", verticalAperture=ap,
                              horizontalAperture=ap, lightPos=(0.3, 1.0, 0.5), lightIntensity=0.8)
    pos, rot = sc.env_cameras(meshes[:n_env], seed=1)
    r.setCameras(pos, rot)
    scene = oracle.OracleScene(m, bvh, r)
    t0 = time.perf_counter()
    scene.step(threads=threads)
    dt = time.perf_counter() - t0
    return n_env / dt, dt


def warp_probe() -> str:
    """Whether the reference's own kernels could run here: they need warp-lang 0.10.1
    (FF_SRL/setup.py:24) for SimIntegratorDO.stepModel on device="cpu"."""
    try:
        import warp  # noqa: F401
    except Exception as e:  # not installed on this image
        return f"import warp failed: {type(e).__name__}: {e}"
    return f"warp {getattr(warp, '__version__', '?')} imports"


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    probe = warp_probe()
    from ffsrl import scenarios as sc
    threads = os.cpu_count() or 1
    meshes, _ = sc.mixed_meshes(args.envs, pool_size=args.pool, seed=0)
    sample = 32
    for _ in range(args.warmup):
        cpu_sample(meshes, threads, n_env=sample)
    vals = []
    for k in range(args.steps):
        v, dt = cpu_sample(meshes[k * sample % (len(meshes) - sample):], threads, n_env=sample)
        vals.append(v)
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": "env-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * sample / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": config(args.envs, world, args.pool, args.arithmetic) | {"sample": f"{sample} envs x 1 step per timed step"},
            "cpu_baseline": {"value": v, "unit": "env-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} envs of the same pool, 1 full env-step each (8x10 solve, refit, "
                                       f"{RES}x{RES} ray-cast), OpenMP over envs"},
            "e2e": {"value": v, "unit": "env-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "warp_probe": probe,
            "reference_kind_reason": "the reference's Warp kernels need warp-lang 0.10.1, which this image lacks "
                                     "(warp_probe); the arm times the C++ restatement of those kernels instead"}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    envs = args.envs
    setup = {}
    t_setup = time.perf_counter()
    m, meshes, pool, bvh, r = build_workload(device, envs, seed=rank, pool_size=args.pool)
    setup["workload_s"] = time.perf_counter() - t_setup
    from ffsrl import SimIntegratorDO, scenarios as sc, _lib as L
    from ffsrl.shard import max_over_ranks
    t_setup = time.perf_counter()
    integ = SimIntegratorDO(device, autotune=True, arithmetic=args.arithmetic)
    plan = integ.plan(m)
    torch.cuda.synchronize()
    setup["plan_and_autotune_s"] = time.perf_counter() - t_setup
    n_cls = plan.info()["num_classes"]
    K, W = args.steps, max(args.warmup, 3)
    walk = torch.as_tensor(sc.random_walk_steps(envs, K + W, seed=rank + 100), device=device)
    stream = torch.cuda.current_stream()

    grasp_all = torch.ones(envs, dtype=torch.int32, device=device)
    all_envs = range(envs)
    episode = {"steps": 0, "resets": 0}

    def episode_tick():
        # the soft meshes sag under gravity at 8 substeps x 10 iterations; RL episodes
        # restart from the rest state (reset + grasp), inside the timed region
        if episode["steps"] and episode["steps"] % EPISODE == 0:
            m.resetFixedModel(all_envs)
            m.graspNearest(grasp_all, radius=GRASP_RADIUS)
            episode["resets"] += 1
        episode["steps"] += 1

    def new_episode():
        m.resetFixedModel(all_envs)
        m.graspNearest(grasp_all, radius=GRASP_RADIUS)
        episode["steps"] = 1

    # one env-step (instrument move, batched step, visual points, refit, ray-cast) as a
    # CUDA graph replayed every step; the action is copied into the buffer it reads
    act_s = torch.zeros((envs, 3), dtype=torch.float32, device=device)

    def core():
        m.applyCartesianActionsInWorkspace(act_s)
        integ.stepModel(m, 1)
        bvh.refitBVH()
        r.renderNew(bvh, m)

    from ffsrl.graphs import Graph
    core_step = Graph(core, prepare=lambda: integ.plan(m)) if not args.no_graph else core

    def step(k):
        episode_tick()
        act_s.copy_(walk[k])
        core_step()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for k in range(W):
        step(k)
    barrier()
    resets0 = episode["resets"]
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(K + 1)]
    with Clocks(local) as clk:
        torch.cuda.nvtx.range_push("timed_steps")  # lets a profiler select the timed launches
        evs[0].record(stream)
        for k in range(K):
            step(W + k)
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    barrier()
    resets_timed = episode["resets"] - resets0
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(K)]
    total_ms = evs[0].elapsed_time(evs[K])
    total_ms = max_over_ranks(total_ms, device=device)
    r.checkErrors()
    status = integ.envStatus(m)
    value = envs * world * K / (total_ms / 1000.0)

    # dominant kernel: the batched step alone
    ks = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    kreps = min(max(3, K // 2), EPISODE - 1)
    new_episode()
    integ.plan(m).step(1)
    torch.cuda.synchronize()
    ks[0].record(stream)
    for _ in range(kreps):
        plan.step(1)
    ks[1].record(stream)
    torch.cuda.synchronize()
    step_kernel_ms = ks[0].elapsed_time(ks[1]) / kreps
    # the observation alone: fused refit, vertex normals and the ray-cast
    ks[0].record(stream)
    for _ in range(kreps):
        bvh.refitBVH()
        r.renderNew(bvh, m)
    ks[1].record(stream)
    torch.cuda.synchronize()
    observe_ms = ks[0].elapsed_time(ks[1]) / kreps
    # the step kernel in the other arithmetic form, same workload and episode phase
    other = "reference" if args.arithmetic == "fast" else "fast"
    t_other = time.perf_counter()
    integ_o = SimIntegratorDO(device, autotune=True, arithmetic=other)
    plan_o = integ_o.plan(m)
    new_episode()
    plan_o.step(1)
    torch.cuda.synchronize()
    ks[0].record(stream)
    for _ in range(kreps):
        plan_o.step(1)
    ks[1].record(stream)
    torch.cuda.synchronize()
    other_kernel_ms = ks[0].elapsed_time(ks[1]) / kreps
    setup["other_arithmetic_s"] = time.perf_counter() - t_other
    del plan_o, integ_o
    alg = algorithmic_bytes(m)
    peak, peak_kind = peaks()
    achieved = alg / (step_kernel_ms / 1000.0) / 1e9
    prof = ROOT / "profiles" / "batched_step_traffic.json"
    traffic = None
    if prof.exists():
        try:
            d = json.loads(prof.read_text())
            rec = d.get(f"{args.arithmetic}|{'distinct' if args.pool <= 0 else 'pool' + str(args.pool)}")
            if rec:
                traffic = rec["dram_bytes_per_env_step"] * envs
        except Exception:
            traffic = None

    # end to end through the public API with host buffers
    act_h = torch.empty((envs, 4), dtype=torch.float32, pin_memory=True)
    res_h = torch.empty((envs, 4), dtype=torch.float32, pin_memory=True)
    act_d = torch.empty((envs, 4), dtype=torch.float32, device=device)
    res_d = torch.empty((envs, 4), dtype=torch.float32, device=device)
    walk_h = walk.cpu()

    def e2e_step(k):
        episode_tick()
        act_h[:, :3] = walk_h[k % len(walk_h)]
        act_h[:, 3] = 1.0
        act_d.copy_(act_h, non_blocking=True)
        act_s.copy_(act_d[:, :3])
        core_step()
        res_d[:, :3] = m.laparoscopeTip[3::4]
        res_d[:, 3] = m.laparoscopeInCollision.float()
        res_h.copy_(res_d, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    # the same episode phase and walk steps as the device-timed region
    new_episode()
    for k in range(W):
        e2e_step(k)
    barrier()
    t0 = time.perf_counter()
    for k in range(K):
        e2e_step(W + k)
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e = envs * world * K / e2e_s

    plain = None
    if not args.no_plain:
        pint = SimIntegratorDO(device, batched=False)
        pint.stepModel(m, 1)
        torch.cuda.synchronize()
        pe = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        pk = max(1, args.plain_steps)
        pe[0].record(stream)
        for k in range(pk):
            m.applyCartesianActionsInWorkspace(walk[k])
            pint.stepModel(m, 1)
            bvh.refitBVH(fused=False)
            r.fused = False
            r.renderNew(bvh, m)
            r.fused = True
        pe[1].record(stream)
        torch.cuda.synchronize()
        plain_ms = pe[0].elapsed_time(pe[1]) / pk
        plain = {"value": envs / (plain_ms / 1000.0), "unit": "env-steps/s", "ms_per_step": plain_ms,
                 "speedup_batched_vs_plain": value / world / (envs / (plain_ms / 1000.0))}

    serving = None
    if args.serve_seconds > 0:
        # continuous-batching serving of the same pool: one closed-loop actor per env
        from ffsrl import scenarios as sc2
        from ffsrl.serve import EnvServer, NativeEnvServer
        meshes_s, pool_s = meshes, pool
        ids = {id(mm): k for k, mm in enumerate(pool_s)}
        Server = NativeEnvServer if args.serve_impl == "native" else EnvServer
        srv = Server(pool_s, [ids[id(mm)] for mm in meshes_s], device, hbm_budget_bytes=60e9, resolution=RES,
                     autotune=True, arithmetic=args.arithmetic)
        serving = srv.run_closed_loop(args.serve_seconds, think_hz=60.0, seed=rank, warmup_s=1.0)
        serving["server"] = args.serve_impl
        serving["what"] = ("closed-loop actors, Poisson think time at 60 Hz, each request = effector move + 8x10 step "
                           "+ refit + 128x128 ray-cast of its env; latency from arrival to result on the host")
        del srv
    serving_pressure = None
    if args.pressure_seconds > 0:
        # the same actor count on a 64-mesh pool, with the HBM budget at a quarter of what one
        # slot per actor needs: actors queue for slots, idle ones are evicted to host memory
        from ffsrl import scenarios as sc3
        from ffsrl.serve import NativeEnvServer, EnvServer, slot_bytes
        meshes_p, pool_p = sc3.mixed_meshes(envs, pool_size=64, seed=rank + 7)
        idp = {id(mm): k for k, mm in enumerate(pool_p)}
        need = float(sum(slot_bytes(mm, RES) for mm in meshes_p))
        Server = NativeEnvServer if args.serve_impl == "native" else EnvServer
        srv = Server(pool_p, [idp[id(mm)] for mm in meshes_p], device, hbm_budget_bytes=0.25 * need, resolution=RES,
                     autotune=True, arithmetic=args.arithmetic)
        serving_pressure = srv.run_closed_loop(args.pressure_seconds, think_hz=60.0, seed=rank, warmup_s=1.0)
        serving_pressure["server"] = args.serve_impl
        serving_pressure["budget_bytes"] = 0.25 * need
        serving_pressure["what"] = ("as serving, 64-mesh pool, HBM budget = 25% of one slot per actor: admission waits "
                                    "for a free slot or evicts the least recently used idle actor of the mesh type")
        del srv
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            threads = os.cpu_count() or 1
            cpu_sample(meshes[32:], threads, n_env=8)  # warm-up: page-in, thread pool, caches
            v, dt = cpu_sample(meshes, threads, n_env=32)
            cpu = {"value": v, "unit": "env-steps/s", "cores": threads, "kind": "port",
                   "sample": f"32 envs of the same pool, 1 full env-step (8x10 solve, refit, {RES}x{RES} ray-cast), "
                             "oracle restatement, OpenMP over envs"}
        # per step: instrument kinematics, one launch per size class, remap, instrument visual points,
        # fused refit, normal gather, rays; per episode reset: instrument visual points, remap and grasp
        launches = K * (n_cls + 6) + 3 * resets_timed
        line = {"metric": METRIC, "value": value, "unit": "env-steps/s", "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes and random-walk actions)",
                "config": config(envs, world, args.pool, args.arithmetic), "cuda_graph": not args.no_graph,
                "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                               "what": "full-batch step latency (all envs), per timed step"},
                "e2e": {"value": e2e, "unit": "env-steps/s", "h2d_bytes_per_step": envs * 16,
                        "d2h_bytes_per_step": envs * 16},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                             "kernel": "k_batched (batched step, all size classes)", "kernel_ms": step_kernel_ms,
                             "achieved_is": "algorithmic bytes of the step (every table and state byte of every "
                                            "iteration) per second; the kernel keeps each env in shared memory "
                                            "and L2, so DRAM moves a small fraction of them",
                             "dram_gbs": (traffic / (step_kernel_ms / 1000.0) / 1e9) if traffic else None,
                             "limiter": "instruction issue and the shared-memory pipe (profiles/k_batched_*.md)"},
                "other_arithmetic": {"arithmetic": other, "kernel_ms": other_kernel_ms,
                                     "what": "the batched step kernel of the other arithmetic form on the same "
                                             "workload (autotuned), CUDA events"},
                "setup_s": setup,
                "observe_ms": {"value": observe_ms, "what": f"fused BVH refit + vertex normals + {RES}x{RES} "
                                                          "ray-cast of all envs, per step"},
                "cpu_baseline": cpu, "plain": plain, "serving": serving, "serving_pressure": serving_pressure,
                "gpu_launches": launches,
                "autotune": integ.tuning,
                "clocks": clk.summary(), "env_status_nonzero": int((status != 0).sum())}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
