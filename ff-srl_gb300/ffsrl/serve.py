"""Continuous-batching server of RL step requests over device-resident environments.

Each actor owns one environment (a mesh from a mixed-size pool) and sends step
requests: a tool displacement and a clamp flag.  Environments live in slots of one
batched model, grouped by mesh type; a device-memory budget bounds the number of slots.
An actor without a slot is admitted into a free slot of its mesh type. If there is none,
the least recently used idle actor of that type is evicted: its state is copied to
host memory and restored when it returns.

Requests are served in ticks.  A tick takes every ready request (arrived, its actor not
already on the GPU, admitted) and runs, for exactly those environments: the tool move,
grasp changes, one batched step (substeps x iterations), the visual-point remap, the
BVH refit and the ray-cast observation; then the per-env result (effector position and
contact count) is copied back.  Two lanes -- each with its own stream, work lists and
staging -- let the next tick start while the previous one is still on the GPU, so
requests that arrive mid-tick are served by the next tick on the other lane.  Each
environment's result depends only on its own inputs (the batched step sums corrections
in fixed point, the renderer gathers normals in face order), so it is the same whether
the environment is stepped alone or in any mix.
"""

from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L
from . import meshgen as mg
from . import scenarios as sc
from ._lib import check, lib, ptr
from .bvh import SimBVH
from .integrator import SimIntegratorDO
from .render import WarpRaycastRendererDO


def slot_bytes(mesh: dict, resolution: int) -> int:
    """Device bytes one slot of ``mesh`` holds: model arrays, batch tables, BVH, images."""
    V, T, E = len(mesh["vertex"]), len(mesh["tetrahedron"]), len(mesh["edge"])
    F, P = len(mesh["triangle"]), len(mesh["point_to_vertex"])
    model = V * (12 * 6 + 4 * 4) + T * (16 + 4 * 5 + 36) + E * (8 + 4 * 3) + F * (12 + 8) + P * (12 * 3 + 8)
    plan = T * (8 + 8 + 36 + 4) + E * (4 + 8 + 4) + F * 8 + V * 4
    bvh = 2 * F * (24 + 16) + F * 4
    image = resolution * resolution * 16
    instrument = 112 * 4 + 16 * 4 * 3  # transforms, heights, capsule ends
    return int(model + plan + bvh + image + instrument)


def plan_slots(pool: list, actor_mesh, hbm_budget_bytes: float, resolution: int) -> np.ndarray:
    """Slots per mesh type: one per actor when they fit in the budget, otherwise scaled
    down (at least one per mesh type in use) until the total fits."""
    actor_mesh = np.asarray(actor_mesh, dtype=np.int64)
    want = np.bincount(actor_mesh, minlength=len(pool))
    per = np.array([slot_bytes(m, resolution) for m in pool], dtype=np.float64)
    if float((want * per).sum()) <= hbm_budget_bytes:
        return want
    k = np.floor(want * hbm_budget_bytes / float((want * per).sum())).astype(np.int64)
    k = np.where(want > 0, np.maximum(k, 1), 0)
    while float((k * per).sum()) > hbm_budget_bytes and k.max() > 1:
        k[np.argmax(k * per)] -= 1
    if float((k * per).sum()) > hbm_budget_bytes:
        raise L.FFSRLError(L.ERR_BUDGET, "HBM budget too small for one slot per mesh type in use")
    return k


@dataclass
class Request:
    actor: int
    disp: np.ndarray
    clamp: int
    t_arrival: float
    reset: bool = False  # start a new episode: the env returns to its rest state first
    t_done: float = 0.0
    result: np.ndarray | None = None


@dataclass
class _Lane:
    stream: torch.cuda.Stream
    ids_h: torch.Tensor
    act_h: torch.Tensor
    res_h: torch.Tensor
    ids_d: torch.Tensor
    act_d: torch.Tensor
    res_d: torch.Tensor
    gids_d: torch.Tensor
    gclamp_d: torch.Tensor
    rst_h: torch.Tensor
    rst_d: torch.Tensor
    gids_h: torch.Tensor
    gclamp_h: torch.Tensor
    event: torch.cuda.Event
    batch: list = field(default_factory=list)


class EnvServer:
    def __init__(self, pool: list, actor_mesh, device="cuda:0", hbm_budget_bytes: float = 60e9, resolution: int = 128,
                 lanes: int = 2, seed: int = 0, autotune: bool = False, block_threads: int = 0,
                 arithmetic: str = "reference", **model_kw):
        self.device = torch.device(device)
        self.pool = pool
        self.actor_mesh = np.asarray(actor_mesh, dtype=np.int64)
        self.num_actors = len(self.actor_mesh)
        self.resolution = resolution
        per = np.array([slot_bytes(m, resolution) for m in pool], dtype=np.float64)
        self.slot_bytes = per
        k = plan_slots(pool, self.actor_mesh, hbm_budget_bytes, resolution)
        self.slots_per_mesh = k
        self.slot_mesh = np.repeat(np.arange(len(pool)), k)
        self.num_slots = int(len(self.slot_mesh))
        self.budget_used = float((k * per).sum())
        meshes = [pool[m] for m in self.slot_mesh]
        # one gravity force for the model (the reference's per-model vector), from the
        # whole pool, so that it does not depend on which mesh takes the first slot
        model_kw.setdefault("environmentGravity", mg.gravity_force(pool))
        self.model, _ = sc.liver_model(device, self.num_slots, meshes=meshes, **model_kw)
        self.integ = SimIntegratorDO(device, blockThreads=block_threads, autotune=autotune, arithmetic=arithmetic)
        self.plan = self.integ.plan(self.model)
        self.bvh = SimBVH(device, self.model)
        ap = sc.fov_aperture(60.0)
        self.renderer = WarpRaycastRendererDO(device, self.model, resolution=resolution, mode="headless",
                                              verticalAperture=ap, horizontalAperture=ap, lightPos=(0.3, 1.0, 0.5),
                                              lightIntensity=0.8)
        pos, rot = sc.env_cameras(meshes, seed=seed + 1)
        self.renderer.setCameras(pos, rot)
        self.free = {m: list(np.nonzero(self.slot_mesh == m)[0][::-1]) for m in range(len(pool))}
        self.slot_actor = np.full(self.num_slots, -1, dtype=np.int64)
        self.actor_slot = np.full(self.num_actors, -1, dtype=np.int64)
        self.actor_clamp = np.zeros(self.num_actors, dtype=np.int32)
        self.last_used = np.zeros(self.num_actors)
        self.in_flight = np.zeros(self.num_actors, dtype=bool)
        self.snapshots: dict[int, dict] = {}
        self.evictions = 0
        self.admissions = 0
        n = self.num_slots
        pin = dict(pin_memory=True)
        self.lanes = [_Lane(stream=torch.cuda.Stream(device=self.device),
                            ids_h=torch.empty(n, dtype=torch.int32, **pin),
                            act_h=torch.empty((n, 4), dtype=torch.float32, **pin),
                            res_h=torch.empty((n, 4), dtype=torch.float32, **pin),
                            ids_d=torch.empty(n, dtype=torch.int32, device=self.device),
                            act_d=torch.empty((n, 4), dtype=torch.float32, device=self.device),
                            res_d=torch.empty((n, 4), dtype=torch.float32, device=self.device),
                            gids_d=torch.empty(n, dtype=torch.int32, device=self.device),
                            gclamp_d=torch.empty(n, dtype=torch.int32, device=self.device),
                            rst_h=torch.empty(n, dtype=torch.int32, **pin),
                            rst_d=torch.empty(n, dtype=torch.int32, device=self.device),
                            gids_h=torch.empty(n, dtype=torch.int32, **pin),
                            gclamp_h=torch.empty(n, dtype=torch.int32, **pin),
                            event=torch.cuda.Event())
                      for _ in range(lanes)]
        self.pending: list[Request] = []
        # per-tick device timing (start/end events on the lane stream), kept when enabled
        self.profile_ticks = False
        self.tick_log: list[tuple] = []
        torch.cuda.synchronize()

    # ------------------------------------------------------------ admission
    def _slot_views(self, s: int):
        m = self.model
        v0, v1 = int(m.envVertexStart[s]), int(m.envVertexStart[s + 1])
        return {"vertex": m.vertex[v0:v1], "velocity": m.velocity[v0:v1], "drag": m.activeDragConstraint[v0:v1],
                "base": m.laparoscopeBase[4 * s:4 * s + 4], "tip": m.laparoscopeTip[4 * s:4 * s + 4],
                "xform": m.laparoscopeXForm[112 * s:112 * s + 112], "incol": m.laparoscopeInCollision[s:s + 1]}

    def _evict(self, a: int, stream) -> None:
        s = int(self.actor_slot[a])
        with torch.cuda.stream(stream):
            snap = {k: v.to("cpu", non_blocking=True) for k, v in self._slot_views(s).items()}
        stream.synchronize()
        self.snapshots[a] = snap
        self.actor_slot[a] = -1
        self.slot_actor[s] = -1
        self.free[int(self.slot_mesh[s])].append(s)
        self.evictions += 1

    def _admit(self, a: int, stream, busy=()) -> bool:
        """Give actor a a slot; ``busy`` holds the actors of the tick being formed, which
        may not be evicted for it."""
        m = int(self.actor_mesh[a])
        if not self.free[m]:
            idle = [int(x) for x in self.slot_actor[self.slot_mesh == m]
                    if x >= 0 and not self.in_flight[x] and int(x) not in busy]
            if not idle:
                return False
            self._evict(min(idle, key=lambda x: self.last_used[x]), stream)
        s = self.free[m].pop()
        views = self._slot_views(s)
        mm = self.model
        with torch.cuda.stream(stream):
            if a in self.snapshots:
                snap = self.snapshots.pop(a)
                for k, v in views.items():
                    v.copy_(snap[k], non_blocking=True)
            else:
                self._rest_state(s, a)
        self.actor_slot[a] = s
        self.slot_actor[s] = a
        self.admissions += 1
        return True

    def _rest_state(self, s: int, a: int) -> None:
        """Slot s holds actor a's env at rest, instrument at its initial pose, no grasp
        (on the current stream)."""
        mm = self.model
        views = self._slot_views(s)
        v0, v1 = int(mm.envVertexStart[s]), int(mm.envVertexStart[s + 1])
        views["vertex"].copy_(mm.initialVertex[v0:v1])
        views["velocity"].zero_()
        views["drag"].zero_()
        views["base"].copy_(mm.laparoscopeInitialBase[4 * s:4 * s + 4])
        views["tip"].copy_(mm.laparoscopeInitialTip[4 * s:4 * s + 4])
        views["xform"].copy_(mm.laparoscopeInitialXForm[112 * s:112 * s + 112])
        views["incol"].zero_()
        self.actor_clamp[a] = 0

    # ------------------------------------------------------------ ticks
    def submit(self, req: Request) -> None:
        self.pending.append(req)

    def free_lane(self):
        for ln in self.lanes:
            if not ln.batch or ln.event.query():
                return ln
        return None

    def poll(self) -> list[Request]:
        done = []
        now = time.perf_counter()
        for ln in self.lanes:
            if ln.batch and ln.event.query():
                res = ln.res_h[:len(ln.batch)].numpy().copy()
                for i, r in enumerate(ln.batch):
                    r.t_done = now
                    r.result = res[i]
                    self.in_flight[r.actor] = False
                done += ln.batch
                ln.batch = []
        return done

    def launch(self, max_batch: int | None = None) -> int:
        """Start a tick on a free lane with every ready request; returns its size."""
        ln = self.free_lane()
        if ln is None or not self.pending:
            return 0
        if ln.batch:  # finished but not yet collected
            return 0
        batch, rest = [], []
        seen = set()
        for r in self.pending:
            if self.in_flight[r.actor] or r.actor in seen or (max_batch and len(batch) >= max_batch):
                rest.append(r)
                continue
            if self.actor_slot[r.actor] < 0 and not self._admit(r.actor, ln.stream, seen):
                rest.append(r)
                continue
            seen.add(r.actor)
            batch.append(r)
        self.pending = rest
        if not batch:
            return 0
        n = len(batch)
        ids = np.array([self.actor_slot[r.actor] for r in batch], dtype=np.int32)
        resets = [int(self.actor_slot[r.actor]) for r in batch if r.reset]
        for r in batch:
            if r.reset:
                self.actor_clamp[r.actor] = 0  # the grasp closes again below
        acts = np.array([[*r.disp, r.clamp] for r in batch], dtype=np.float32)
        trans = [i for i, r in enumerate(batch) if r.clamp != self.actor_clamp[r.actor]]
        m = self.model
        s = L.stream_handle(ln.stream)
        t_host = time.perf_counter()
        with torch.cuda.stream(ln.stream):
            if self.profile_ticks:
                ev0 = torch.cuda.Event(enable_timing=True)
                ev0.record(ln.stream)
            ln.ids_h[:n].copy_(torch.from_numpy(ids))
            ln.act_h[:n].copy_(torch.from_numpy(acts))
            ln.ids_d[:n].copy_(ln.ids_h[:n], non_blocking=True)
            ln.act_d[:n].copy_(ln.act_h[:n], non_blocking=True)
            if resets:
                nr = len(resets)
                ln.rst_h[:nr].copy_(torch.as_tensor(resets, dtype=torch.int32))
                ln.rst_d[:nr].copy_(ln.rst_h[:nr], non_blocking=True)
                check(lib().ffsrl_reset_envs(ptr(m.vertex), ptr(m.velocity), ptr(m.activeDragConstraint),
                                             ptr(m.initialVertex), ptr(m.laparoscopeBase), ptr(m.laparoscopeTip),
                                             ptr(m.laparoscopeInitialBase), ptr(m.laparoscopeInitialTip),
                                             ptr(m.laparoscopeInCollision), ptr(m.laparoscopeXForm),
                                             ptr(m.laparoscopeInitialXForm), ptr(m.envVertexStartT), ptr(ln.rst_d), nr,
                                             m.numEnvs, s))
            disp = ln.act_d[:n, :3].contiguous()
            if m.hasInstrumentKinematics:  # the effector moves through the instrument's kinematic chain
                check(lib().ffsrl_instrument_cartesian_envs(ptr(m.laparoscopeXForm), ptr(disp), None, None,
                                                            ptr(m.laparoscopeBase), ptr(m.laparoscopeTip),
                                                            ptr(m.laparoscopeHeight), ptr(ln.ids_d), n, m.numEnvs, s))
            else:
                check(lib().ffsrl_move_tool_envs(ptr(m.laparoscopeBase), ptr(m.laparoscopeTip), ptr(disp),
                                                 ptr(ln.ids_d), n, m.numEnvs, s))
            if trans:
                # pinned staging: a copy from pageable memory would wait for the stream
                nt = len(trans)
                ln.gids_h[:nt].copy_(torch.from_numpy(ids[np.asarray(trans)]))
                ln.gclamp_h[:nt].copy_(torch.tensor([batch[i].clamp for i in trans], dtype=torch.int32))
                ln.gids_d[:nt].copy_(ln.gids_h[:nt], non_blocking=True)
                ln.gclamp_d[:nt].copy_(ln.gclamp_h[:nt], non_blocking=True)
                check(lib().ffsrl_grasp_nearest_envs(ptr(m.vertex), ptr(m.graspCandStartT), ptr(m.graspCand),
                                                     ptr(m.laparoscopeTip), ptr(ln.gclamp_d), m.globalLaparoscopeDragLookupRadius,
                                                     ptr(m.activeDragConstraint), ptr(ln.gids_d), len(trans), m.numEnvs, s))
                for i in trans:
                    self.actor_clamp[batch[i].actor] = batch[i].clamp
            check(lib().ffsrl_batch_step_envs_lane(self.plan.handle, self.lanes.index(ln), ids.ctypes.data, n, 1, s))
            check(lib().ffsrl_remap_envs(ptr(m.allVisPoint), ptr(m.vertex), ptr(m.pointToVertex),
                                         ptr(m.envMapStartT), ptr(ln.ids_d), n, m.numEnvs, s))
            m.transformSimLaparoscopeMeshData(ln.stream, env_ids=ln.ids_d[:n])
            check(lib().ffsrl_bvh_refit_fused_envs(C.byref(self.bvh.desc), ptr(m.allVisPoint), ptr(m.allVisFace),
                                                   ptr(ln.ids_d), n, s))
            rd = self.renderer._desc(m)
            check(lib().ffsrl_render_fused_envs(C.byref(rd), C.byref(self.bvh.desc), ptr(ln.ids_d), n, s))
            idl = ln.ids_d[:n].long()
            ln.res_d[:n, :3] = m.laparoscopeTip[4 * idl + 3]
            ln.res_d[:n, 3] = m.laparoscopeInCollision[idl].float()
            ln.res_h[:n].copy_(ln.res_d[:n], non_blocking=True)
            ln.event.record(ln.stream)
            if self.profile_ticks:
                ev1 = torch.cuda.Event(enable_timing=True)
                ev1.record(ln.stream)
        now = time.perf_counter()
        if self.profile_ticks:
            self.tick_log.append((self.lanes.index(ln), n, ev0, ev1, (now - t_host) * 1e3))
        for r in batch:
            self.in_flight[r.actor] = True
            self.last_used[r.actor] = now
        ln.batch = batch
        return n

    def drain(self) -> list[Request]:
        done = []
        while any(ln.batch for ln in self.lanes):
            done += self.poll()
            time.sleep(0.0002)
        return done

    # ------------------------------------------------------------ load generator
    def run_closed_loop(self, duration_s: float, think_hz: float = 60.0, seed: int = 0, warmup_s: float = 0.5,
                        max_batch: int | None = None, episode: int = 16) -> dict:
        """Every actor sends its next request an exponential think time (mean 1/think_hz)
        after its previous result arrives; requests carry U[-0.1, 0.1] cm displacements
        and a clamp flag that closes on the first request of each episode; every
        ``episode`` requests an actor starts a new episode from the rest state.  Returns
        latency percentiles (arrival to result on the host) and served env-steps/s over
        ``duration_s``."""
        rng = np.random.Generator(np.random.PCG64(seed))
        A = self.num_actors
        t0 = time.perf_counter()
        nxt = t0 + rng.exponential(1.0 / think_hz, size=A)
        waiting = np.zeros(A, dtype=bool)  # request outstanding
        lat, served, t_meas = [], 0, t0 + warmup_s
        t_end = t_meas + duration_s
        ticks, batch_sizes = 0, []
        sent = np.zeros(A, dtype=np.int64)
        ev_meas = None  # evictions when the measured window opens
        while True:
            now = time.perf_counter()
            if ev_meas is None and now >= t_meas:
                ev_meas = self.evictions
            if now >= t_end:
                break
            due = np.nonzero((~waiting) & (nxt <= now))[0]
            for a in due:
                reset = bool(sent[a]) and episode > 0 and sent[a] % episode == 0
                self.submit(Request(int(a), rng.uniform(-0.1, 0.1, size=3).astype(np.float32), 1, float(nxt[a]),
                                    reset=reset))
                sent[a] += 1
            waiting[due] = True
            for r in self.poll():
                waiting[r.actor] = False
                nxt[r.actor] = r.t_done + rng.exponential(1.0 / think_hz)
                if r.t_arrival >= t_meas:
                    lat.append(r.t_done - r.t_arrival)
                    served += 1
            b = self.launch(max_batch)
            if b:
                ticks += 1
                batch_sizes.append(b)
            else:
                time.sleep(0.0001)
        self.drain()
        torch.cuda.synchronize()
        lat_ms = np.array(lat) * 1e3
        prof = None
        if self.profile_ticks and self.tick_log:
            first = self.tick_log[0][2]
            spans = [(ln, n, first.elapsed_time(a), first.elapsed_time(b), h) for ln, n, a, b, h in self.tick_log]
            dev = np.array([b - a for _, _, a, b, _ in spans])
            ends = max(b for _, _, _, b, _ in spans)
            busy = np.zeros(int(ends) + 1)
            for _, _, a, b, _ in spans:
                busy[int(a):int(b) + 1] += 1
            prof = {"tick_device_ms_p50": float(np.median(dev)), "tick_device_ms_mean": float(dev.mean()),
                    "host_launch_ms_mean": float(np.mean([h for *_, h in spans])),
                    "frac_time_two_lanes_busy": float((busy >= 2).mean()), "frac_time_idle": float((busy == 0).mean()),
                    "ticks": [(ln, n, round(a, 2), round(b, 2), round(h, 2)) for ln, n, a, b, h in spans[-40:]]}
            self.tick_log = []
        return {"p50_ms": float(np.percentile(lat_ms, 50)) if len(lat_ms) else None,
                "p99_ms": float(np.percentile(lat_ms, 99)) if len(lat_ms) else None,
                "served_env_steps_per_s": served / duration_s, "requests": served, "ticks": ticks,
                "mean_batch": float(np.mean(batch_sizes)) if batch_sizes else 0.0, "actors": A,
                "slots": self.num_slots, "evictions": self.evictions,
                "evictions_measured": self.evictions - (ev_meas if ev_meas is not None else self.evictions),
                "budget_bytes_used": self.budget_used,
                "episode_requests": episode, "env_status_nonzero": int((self.plan.env_status() != 0).sum()),
                **({"tick_profile": prof} if prof else {})}


class NativeEnvServer(EnvServer):
    """``EnvServer`` with its ticks run by the library's C server (``ffsrl_server_*``): the
    same slots, model, plan, BVH and renderer, with admission, eviction, the lanes and each
    tick's launch sequence in native code.  Results equal ``EnvServer``'s for the same
    requests (each env's result depends only on its own inputs)."""

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        m = self.model
        self._dm = m.device_model()
        self._rd = self.renderer._desc(m)
        self._slot_mesh = np.ascontiguousarray(self.slot_mesh, dtype=np.int32)
        self._actor_mesh = np.ascontiguousarray(self.actor_mesh, dtype=np.int32)
        c = L.ServerConfig()
        c.num_slots, c.slot_mesh = self.num_slots, self._slot_mesh.ctypes.data
        c.num_actors, c.actor_mesh = self.num_actors, self._actor_mesh.ctypes.data
        c.lanes = len(self.lanes)
        c.plan = self.plan.handle
        c.model = C.pointer(self._dm)
        c.initial_vertex = ptr(m.initialVertex)
        c.initial_base, c.initial_tip = ptr(m.laparoscopeInitialBase), ptr(m.laparoscopeInitialTip)
        if m.hasInstrumentKinematics:
            c.xform, c.initial_xform = ptr(m.laparoscopeXForm), ptr(m.laparoscopeInitialXForm)
            c.height = ptr(m.laparoscopeHeight)
            if m.instrumentMesh is not None:
                c.inst_local_point, c.inst_point_slot = ptr(m.laparoscopeVertex), ptr(m.laparoscopeVertexToXForm)
                c.inst_num_points = int(m.laparoscopeVertexToXForm.numel())
                c.env_inst_first_point = ptr(m.envInstrumentPointStartT)
        c.grasp_cand_start, c.grasp_cand = ptr(m.graspCandStartT), ptr(m.graspCand)
        c.grasp_radius = m.globalLaparoscopeDragLookupRadius
        c.vis_point, c.point_to_vertex, c.env_map_start = ptr(m.allVisPoint), ptr(m.pointToVertex), ptr(m.envMapStartT)
        c.bvh, c.vis_face, c.render = C.pointer(self.bvh.desc), ptr(m.allVisFace), C.pointer(self._rd)
        self._cfg = c
        h = C.c_void_p()
        check(lib().ffsrl_server_create(C.byref(c), C.byref(h)))
        self.handle = h
        self._reqs: dict[int, Request] = {}
        self._tag = 0
        cap = self.num_slots * len(self.lanes)
        self._tags = np.zeros(cap, dtype=np.int64)
        self._actors = np.zeros(cap, dtype=np.int32)
        self._res = np.zeros((cap, 4), dtype=np.float32)

    def _stats(self):
        a, e = C.c_int64(), C.c_int64()
        p, f = C.c_int32(), C.c_int32()
        check(lib().ffsrl_server_stats(self.handle, C.byref(a), C.byref(e), C.byref(p), C.byref(f)))
        return int(a.value), int(e.value), int(p.value), int(f.value)

    @property
    def evictions(self) -> int:
        return self._stats()[1] if getattr(self, "handle", None) is not None else 0

    @evictions.setter
    def evictions(self, _):  # EnvServer's own counter; the C server keeps the count here
        pass

    @property
    def admissions(self) -> int:
        return self._stats()[0] if getattr(self, "handle", None) is not None else 0

    @admissions.setter
    def admissions(self, _):
        pass

    def submit(self, req: Request) -> None:
        d = np.ascontiguousarray(np.asarray(req.disp, dtype=np.float32).reshape(3))
        self._tag += 1
        self._reqs[self._tag] = req
        check(lib().ffsrl_server_submit(self.handle, int(req.actor), d.ctypes.data, int(req.clamp), int(req.reset),
                                        self._tag))

    def launch(self, max_batch: int | None = None) -> int:
        n = C.c_int32()
        check(lib().ffsrl_server_launch(self.handle, int(max_batch or 0), C.byref(n)))
        return int(n.value)

    def poll(self) -> list[Request]:
        n = C.c_int32()
        check(lib().ffsrl_server_poll(self.handle, len(self._tags), self._tags.ctypes.data, self._actors.ctypes.data,
                                      self._res.ctypes.data, C.byref(n)))
        now = time.perf_counter()
        done = []
        for i in range(n.value):
            r = self._reqs.pop(int(self._tags[i]))
            r.t_done = now
            r.result = self._res[i].copy()
            done.append(r)
        return done

    def drain(self) -> list[Request]:
        done = []
        while self._stats()[3] > 0:
            done += self.poll()
            time.sleep(0.0002)
        return done

    def close(self) -> None:
        if getattr(self, "handle", None) is not None and self.handle.value:
            torch.cuda.synchronize()
            lib().ffsrl_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
