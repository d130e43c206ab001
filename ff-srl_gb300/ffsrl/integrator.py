"""SimIntegratorDO: the multi-environment step (reference ``FF_SRL/FF_SRL/integrator.py:1634-1744``).

``stepModel(simModel)`` advances every environment by one step of ``simSubsteps``
substeps x ``simConstraints`` Jacobi iterations and then maps the simulated vertices
onto the visual points (``transformSimMeshData``), as the reference does.

Two GPU forms with the same semantics:

* ``batched=True`` (default): the env-resident batched kernel -- one persistent launch per
  mesh-size class, every substep and iteration of an environment on one SM, shared-memory
  positions and deterministic fixed-point correction sums.  ``arithmetic="reference"``
  (default) evaluates every constraint with the reference kernel's expressions (IEEE
  division and square root, no fused multiply-add); ``"fast"`` uses hardware
  reciprocals and a reformulated Neo-Hookean constraint.  ``accumulation`` selects
  ``"fixed"`` (default), ``"kahan"`` (compensated float32) or ``"atomic"`` (float32
  atomics, as the reference);
* ``batched=False``: the reference-shaped form -- one kernel launch per reference kernel
  in the reference's launch order, float atomics.
"""

from __future__ import annotations

import contextlib
import ctypes as C

import numpy as np
import torch

from . import _lib, graphs
from ._lib import check, lib, ptr


ARITHMETIC = {"reference": _lib.ARITH_REFERENCE, "fast": _lib.ARITH_FAST}
ACCUMULATION = {"fixed": _lib.ACC_FIXED, "kahan": _lib.ACC_KAHAN, "atomic": _lib.ACC_ATOMIC}


class BatchPlan:
    """Owner of an ffsrl_batch handle (packed constraint tables, work lists, streams)."""

    def __init__(self, model, block_threads: int = 0, precision: int = 32, arithmetic: str = "reference",
                 accumulation: str = "fixed"):
        model.require_cuda()
        if arithmetic not in ARITHMETIC or accumulation not in ACCUMULATION:
            raise ValueError(f"arithmetic in {list(ARITHMETIC)}, accumulation in {list(ACCUMULATION)}")
        hm, self._host_arrays = model.host_model()
        self._dm = model.device_model()
        self._params = model.params()
        opts = _lib.BatchOptions()
        opts.block_threads = int(block_threads)
        opts.arithmetic = ARITHMETIC[arithmetic]
        opts.accumulation = ACCUMULATION[accumulation]
        opts.precision = int(precision)
        self.arithmetic, self.accumulation = arithmetic, accumulation
        h = C.c_void_p()
        check(lib().ffsrl_batch_create(C.byref(hm), C.byref(self._dm), C.byref(self._params), C.byref(opts),
                                       C.byref(h)))
        self.handle = h
        self.model = model
        self.precision = precision
        self.version = getattr(model, "topologyVersion", 0)
        self._host_arrays = None  # the plan has copied what it needs

    def step(self, n_steps: int = 1, stream=None) -> None:
        graphs.keep(self)
        check(lib().ffsrl_batch_step(self.handle, int(n_steps), _lib.stream_handle(stream)))

    def step_envs(self, env_ids, n_steps: int = 1, stream=None) -> None:
        graphs.keep(self)
        ids = np.ascontiguousarray(np.asarray(env_ids, dtype=np.int32))
        check(lib().ffsrl_batch_step_envs(self.handle, ids.ctypes.data, int(ids.size), int(n_steps),
                                          _lib.stream_handle(stream)))

    def info(self) -> dict:
        nbytes = C.c_int64()
        ncls = C.c_int32()
        check(lib().ffsrl_batch_info(self.handle, C.byref(nbytes), C.byref(ncls), None))
        blocks = np.zeros(max(ncls.value, 1), dtype=np.int32)
        check(lib().ffsrl_batch_info(self.handle, None, None, blocks.ctypes.data))
        return {"device_bytes": int(nbytes.value), "num_classes": int(ncls.value),
                "block_threads": blocks[:ncls.value].tolist()}

    def env_status(self) -> np.ndarray:
        out = np.zeros(self.model.numEnvs, dtype=np.int32)
        check(lib().ffsrl_batch_env_status(self.handle, out.ctypes.data, self.model.numEnvs))
        return out

    def state_f64(self) -> dict:
        V = self.model.numVertices
        out = np.zeros(9 * V, dtype=np.float64)
        check(lib().ffsrl_batch_state_f64(self.handle, out.ctypes.data))
        return {"vertex": out[:3 * V].reshape(-1, 3), "velocity": out[3 * V:6 * V].reshape(-1, 3),
                "predicted_vertex": out[6 * V:].reshape(-1, 3)}

    def close(self) -> None:
        if getattr(self, "handle", None) is not None and self.handle.value:
            lib().ffsrl_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SimIntegratorDO:
    """Reference-compatible integrator: ``SimIntegratorDO(device).stepModel(simModel)``."""

    def __init__(self, device="cuda:0", batched: bool = True, blockThreads: int = 0, autotune: bool = False,
                 arithmetic: str = "reference", accumulation: str = "fixed") -> None:
        self.device = device
        self.batched = bool(batched)
        self.arithmetic = arithmetic
        self.accumulation = accumulation
        self.blockThreads = int(blockThreads)
        self.autotune = bool(autotune)
        self.tuning = None
        self._plans = {}
        self._graphs = {}

    def plan(self, simModel) -> BatchPlan:
        """The model's batched plan, built on first use and rebuilt when the model's active
        values or holes have changed since (``simModel.topologyVersion``, bumped by the
        cutting and heating calls).  A rebuild starts with empty connector accumulators."""
        key = id(simModel)
        p = self._plans.get(key)
        if p is None or p.model is not simModel or p.version != simModel.topologyVersion:
            p = BatchPlan(simModel, self.blockThreads, arithmetic=self.arithmetic, accumulation=self.accumulation)
            self._plans[key] = p
            if self.autotune and self.blockThreads == 0:
                from .autotune import autotune
                self.tuning = autotune(p)
        return p

    def stepModel(self, simModel, steps: int = 1, stream=None, useGraph: bool = False,
                  checkStatus: bool = False) -> None:
        """integrator.py:1640-1744: ``steps`` env-steps, then the visual points.  With
        ``useGraph`` the launches are captured into a CUDA graph on the first call and the
        graph is replayed afterwards (the reference RL loop's ``wp.capture_launch``,
        ``tests/testLiverRetraction.py:77-85``); one graph per model and step count.
        ``checkStatus`` waits for the step and raises if an env's state became non-finite
        (the reference has no such check; without it, poll ``envStatus``)."""
        if checkStatus:
            self.stepModel(simModel, steps, stream, useGraph)
            if stream is not None:
                stream.synchronize()
            self.checkStatus(simModel)
            return
        simModel.require_cuda()
        if useGraph:
            from .graphs import Graph
            key = (id(simModel), int(steps))
            g = self._graphs.get(key)
            if g is None or g[0] is not simModel or g[2] != simModel.topologyVersion:
                # a changed topology rebuilds the plan, so the graph holding the old one goes
                prep = (lambda: self.plan(simModel)) if self.batched else None
                g = (simModel, Graph(lambda: self._step(simModel, steps, None), prep), simModel.topologyVersion)
                self._graphs[key] = g
            with torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext():
                g[1]()
            return
        self._step(simModel, steps, stream)

    MAX_BATCHED_ENV_VERTICES = 65535  # env-local vertex ids of the batched tables are 16-bit

    def routesToPlain(self, simModel) -> bool:
        """True when the batched step cannot hold the model (an env with more than 65,535
        vertices): stepModel then runs the reference-shaped step, which has no such limit."""
        sizes = np.diff(np.asarray(simModel.envVertexStart, dtype=np.int64))
        return bool(self.batched and len(sizes) and sizes.max() > self.MAX_BATCHED_ENV_VERTICES)

    def _step(self, simModel, steps, stream) -> None:
        if self.batched and self.routesToPlain(simModel):
            if not getattr(self, "_warned_plain", False):
                import warnings
                warnings.warn("an env has more than 65,535 vertices: stepping this model with the reference-shaped "
                              "step instead of the batched one")
                self._warned_plain = True
            m = simModel.device_model()
            prm = simModel.params()
            s = _lib.stream_handle(stream)
            for _ in range(int(steps)):
                check(lib().ffsrl_step_model(C.byref(m), C.byref(prm), s))
        elif self.batched:
            self.plan(simModel).step(steps, stream)
        else:
            m = simModel.device_model()
            prm = simModel.params()
            s = _lib.stream_handle(stream)
            for _ in range(int(steps)):
                check(lib().ffsrl_step_model(C.byref(m), C.byref(prm), s))
        simModel.transformSimMeshData(stream)
        simModel.transformSimLaparoscopeMeshData(stream)

    def envStatus(self, simModel) -> np.ndarray:
        """Per-env status of the last batched step (0 ok, 7 non-finite state); zeros for a
        model the batched step routes to the reference-shaped step."""
        if self.routesToPlain(simModel):
            return np.zeros(simModel.numEnvs, dtype=np.int32)
        return self.plan(simModel).env_status()

    def checkStatus(self, simModel) -> None:
        """Raises FFSRLError (ERR_NONFINITE) naming the envs whose state the last batched
        step left non-finite.  It reads the per-env status back from the device, so it
        waits for the step; stepModel(checkStatus=True) calls it after every step."""
        st = self.envStatus(simModel)
        bad = np.nonzero(st)[0]
        if len(bad):
            raise _lib.FFSRLError(int(st[bad[0]]), f"non-finite state in envs {bad[:16].tolist()}"
                                                   f"{' ...' if len(bad) > 16 else ''}")
