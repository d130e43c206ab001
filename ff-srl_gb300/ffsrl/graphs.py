"""CUDA graphs of the library's calls (the reference's ``wp.capture_begin`` /
``wp.capture_launch``: ``bvh.py:442-451``, ``render.py:1108-1112``,
``tests/testLiverRetraction.py:77-85``).

``Graph(fn)`` records every launch ``fn`` makes on the current stream into one CUDA graph
on its first call and replays that graph on every later call, as the reference does.
The captured launches keep the device pointers and the scalar arguments they were
recorded with, so the arrays ``fn`` uses must stay the same tensors (the model's arrays
do) and host-side choices inside ``fn`` (a render mode, a step count) are fixed at
capture; make a new ``Graph`` after changing them.  Everything the library launches goes
to the current stream, which is the capture stream during the capture, so its calls
record with no change; anything that must run before the first capture (plan building,
autotuning, kernel attributes) is done by ``prepare``.

A graph holds a reference to every batched-step plan its capture launched, so a plan
the integrator replaces (after cutting changes the model's active values or holes) stays
allocated while an older graph can still replay it; such a graph steps the topology it
was captured with until it is made again.
"""

from __future__ import annotations

from typing import Callable

import torch

_capturing: list[list] = []


def keep(obj) -> None:
    """Tie ``obj`` (a plan a launch reads) to the graph being captured, if any."""
    if _capturing:
        _capturing[-1].append(obj)


class Graph:
    def __init__(self, fn: Callable[[], None], prepare: Callable[[], None] | None = None):
        self.fn = fn
        self.prepare = prepare
        self.graph = None
        self._kept: list = []

    def capture(self) -> None:
        if self.prepare is not None:
            self.prepare()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        kept: list = []
        _capturing.append(kept)
        try:
            with torch.cuda.stream(side), torch.cuda.graph(g, stream=side):
                self.fn()
        finally:
            _capturing.pop()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = g
        self._kept = kept

    def __call__(self) -> None:
        """Capture on the first call (which then replays once, so the call has its effect),
        replay afterwards; the replay is ordered on the current stream."""
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def reset(self) -> None:
        self.graph = None
        self._kept = []


class NativeGraph:
    """The same capture through the C-ABI's graph calls (``ffsrl_graph_begin`` /
    ``ffsrl_graph_end`` / ``ffsrl_graph_launch``), as a C caller would use them.  ``fn`` must
    make library calls only: torch operations that allocate are not recorded by torch's
    allocator here (use ``Graph`` for those)."""

    def __init__(self, fn: Callable[[], None], prepare: Callable[[], None] | None = None):
        self.fn = fn
        self.prepare = prepare
        self.handle = None
        self._kept: list = []

    def capture(self) -> None:
        import ctypes as C
        from ._lib import check, lib
        if self.prepare is not None:
            self.prepare()
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        h = C.c_void_p()
        kept: list = []
        _capturing.append(kept)
        try:
            with torch.cuda.stream(side):
                check(lib().ffsrl_graph_begin(side.cuda_stream))
                try:
                    self.fn()
                finally:
                    check(lib().ffsrl_graph_end(side.cuda_stream, C.byref(h)))
        finally:
            _capturing.pop()
        torch.cuda.current_stream().wait_stream(side)
        self.handle = h
        self._kept = kept

    def __call__(self) -> None:
        from ._lib import check, lib
        if self.handle is None:
            self.capture()
        check(lib().ffsrl_graph_launch(self.handle, torch.cuda.current_stream().cuda_stream or None))

    def close(self) -> None:
        from ._lib import lib
        if self.handle is not None and self.handle.value:
            lib().ffsrl_graph_destroy(self.handle)
        self.handle = None
        self._kept = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
