"""Block-size autotuner for the batched step.

The batched step runs one launch per size class (environments grouped by vertex count).
For each class this times the class's environments for one step at every block size
that has a kernel instantiation and fits on an SM, with and without the L1 prefetch of
the tet records, keeps the fastest, and records the
choice in a JSON cache keyed by the device and the class's shape, so later plans with
the same classes skip the timing.  The model's state is saved before and restored after
the timing runs.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
from pathlib import Path

import numpy as np
import torch

from ._lib import FFSRLError, check, lib

CANDIDATES = (128, 256, 512, 640, 768, 1024)
PREFETCH = (0, 1, 2)  # next tet record: not fetched ahead, into L1, into registers


def cache_path() -> Path:
    p = os.environ.get("FFSRL_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "ffsrl" / "autotune.json"


def _classes(plan):
    n = plan.info()["num_classes"]
    out = []
    for c in range(n):
        mx, mode, blk, ne = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().ffsrl_batch_class_info(plan.handle, c, C.byref(mx), C.byref(mode), C.byref(blk), C.byref(ne)))
        ids = np.zeros(max(ne.value, 1), dtype=np.int32)
        check(lib().ffsrl_batch_class_envs(plan.handle, c, ids.ctypes.data))
        out.append({"max_nv": mx.value, "mode": mode.value, "block": blk.value, "envs": ids[:ne.value]})
    return out


def _key(plan, cls) -> str:
    m = plan.model
    props = torch.cuda.get_device_properties(m.device)
    tets = int(sum(int(m.envTetStart[e + 1] - m.envTetStart[e]) for e in cls["envs"]))
    sig = f"v4|{props.name}|{props.multi_processor_count}|{m.constraintFlags}|{m.simSubsteps}|{m.simConstraints}|" \
          f"{cls['mode']}|{cls['max_nv']}|{len(cls['envs'])}|{tets}|{plan.precision}|" \
          f"{getattr(plan, 'arithmetic', '')}|{getattr(plan, 'accumulation', '')}"
    return hashlib.sha1(sig.encode()).hexdigest()[:16]


def _time(plan, envs, reps: int) -> float:
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    plan.step_envs(envs, 1)
    ev[0].record()
    for _ in range(reps):
        plan.step_envs(envs, 1)
    ev[1].record()
    torch.cuda.synchronize()
    return ev[0].elapsed_time(ev[1]) / reps


def autotune(plan, reps: int = 2, use_cache: bool = True, verbose: bool = False) -> list[dict]:
    """Pick each class's block size; returns [{class, block, ms}]."""
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except Exception:
            cache = {}
    m = plan.model
    saved = [t.clone() for t in (m.vertex, m.velocity, m.predictedVertex, m.laparoscopeInCollision,
                                 m.tetrahedronLambda, m.edgeLambda)]
    result = []
    try:
        for ci, cls in enumerate(_classes(plan)):
            key = _key(plan, cls)
            if key in cache:
                c = cache[key]
                check(lib().ffsrl_batch_set_class_prefetch(plan.handle, ci, 0))
                check(lib().ffsrl_batch_set_class_block(plan.handle, ci, int(c["block"])))
                check(lib().ffsrl_batch_set_class_prefetch(plan.handle, ci, int(c.get("prefetch", 0))))
                result.append({"class": ci, "block": c["block"], "prefetch": c.get("prefetch", 0), "ms": c["ms"],
                               "cached": True})
                continue
            best = None
            for b in CANDIDATES:
                check(lib().ffsrl_batch_set_class_prefetch(plan.handle, ci, 0))
                if lib().ffsrl_batch_set_class_block(plan.handle, ci, b) != 0:
                    continue
                for pf in PREFETCH:
                    if lib().ffsrl_batch_set_class_prefetch(plan.handle, ci, pf) != 0:
                        continue
                    ms = _time(plan, cls["envs"], reps)
                    if verbose:
                        print(f"autotune class {ci} (max_nv {cls['max_nv']}, {len(cls['envs'])} envs): "
                              f"block {b} prefetch {pf} {ms:.3f} ms")
                    if best is None or ms < best[2]:
                        best = (b, pf, ms)
            if best is None:
                raise FFSRLError(6, f"autotune: no block size fits class {ci}")
            check(lib().ffsrl_batch_set_class_prefetch(plan.handle, ci, 0))
            check(lib().ffsrl_batch_set_class_block(plan.handle, ci, best[0]))
            check(lib().ffsrl_batch_set_class_prefetch(plan.handle, ci, best[1]))
            cache[key] = {"block": best[0], "prefetch": best[1], "ms": best[2]}
            result.append({"class": ci, "block": best[0], "prefetch": best[1], "ms": best[2], "cached": False})
    finally:
        for t, s in zip((m.vertex, m.velocity, m.predictedVertex, m.laparoscopeInCollision, m.tetrahedronLambda,
                         m.edgeLambda), saved):
            t.copy_(s)
        torch.cuda.synchronize()
    if use_cache:
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return result
