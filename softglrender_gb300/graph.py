"""CUDA graphs of renderer calls (sglc_graph_*): capture a frame once, replay it with one launch.

Draws inside a capture must be synchronisation-free (Renderer.setCapacity) and the captured
sequence must have run once uncaptured, so that every working array already has its size.
"""
from __future__ import annotations

import ctypes as C

from . import api as A

_P = C.c_void_p
GRAPH_SIGS = {
    "graph_begin": [_P],
    "graph_end": [_P, C.POINTER(_P)],
    "graph_launch": [_P],
    "graph_destroy": [_P],
}
GRAPH_FUNCTIONS = tuple(GRAPH_SIGS)


class Graph:
    """A captured sequence of calls on one renderer; `launch()` enqueues one replay."""

    def __init__(self, renderer: A.Renderer):
        self.r = renderer
        self.fn = {}
        for name, args in GRAPH_SIGS.items():
            f = getattr(renderer.lib.cdll, "sglc_" + name)
            f.argtypes = args
            f.restype = C.c_int32
            self.fn[name] = f
        self.h = None

    def _check(self, st: int, name: str) -> None:
        if st != 0:
            msg = self.r.lib.fn["last_error"](self.r.ctx)
            raise A.SoftGLError(st, "sglc_" + name, msg.decode() if msg else "")

    def capture(self, frame) -> "Graph":
        """Capture the calls `frame()` enqueues."""
        self._check(self.fn["graph_begin"](self.r.ctx), "graph_begin")
        try:
            frame()
        finally:
            h = _P()
            st = self.fn["graph_end"](self.r.ctx, C.byref(h))
        self._check(st, "graph_end")
        self.h = h
        return self

    def launch(self) -> None:
        self._check(self.fn["graph_launch"](self.h), "graph_launch")

    def destroy(self) -> None:
        if self.h:
            self.fn["graph_destroy"](self.h)
            self.h = None
