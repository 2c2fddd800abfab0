"""Autotuner for synchronisation-free frames: picks working-array capacities, the raster tile shape,
the raster tile order and eager-versus-graph submission for a given frame by measuring them.

1. Calibration: the frame runs once with exact sizing (one count read-back per draw); the peak
   counts over its draws (clip vertices and polygons, appended primitives, bin entries) times a
   headroom give the capacities, doubled until the frame runs without overflow (sglc_get_overflow);
   all candidates then share them.
2. Candidates: the deferred raster's tile shape (16x16 pixels with 256 threads, or 16x8 with 128;
   capacities calibrated for each, the reference's counterpart is its raster block size,
   RendererSoft.h:128), raster tiles longest-list-first or in index order, and the frame enqueued
   call by call or captured once in a CUDA graph and replayed. Each runs `reps` times after
   warm-up, timed with CUDA events on the renderer's stream; the fastest wins.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional

import numpy as np

from . import api as A
from .graph import Graph


@dataclass
class TuneResult:
    capacity: A.Capacity
    heavy_first: int
    graph: bool
    ms: float
    table: List[Dict[str, object]] = field(default_factory=list)
    tile: int = 16
    threads_per_tile: int = 256

    def describe(self) -> Dict[str, object]:
        c = self.capacity
        return {"tile": self.tile, "threads_per_tile": self.threads_per_tile, "heavy_first": self.heavy_first,
                "graph": self.graph, "ms": round(self.ms, 4),
                "capacity": {"clip_vertices": c.clip_vertices, "clip_polygons": c.clip_polygons,
                             "appended_primitives": c.appended_primitives, "bin_entries": c.bin_entries,
                             "fragments": c.fragments},
                "candidates": self.table}


class Tuned:
    """A frame with its tuned submission: `run()` enqueues one frame."""

    def __init__(self, r: A.Renderer, frame: Callable[[], None], result: TuneResult, graph: Optional[Graph]):
        self.r, self.frame, self.result, self.graph = r, frame, result, graph

    def run(self) -> None:
        if self.graph is not None:
            self.graph.launch()
        else:
            self.r.setTileSize(self.result.tile)
            self.frame()

    def destroy(self) -> None:
        if self.graph is not None:
            self.graph.destroy()
            self.graph = None


def _timer(r: A.Renderer):
    import torch
    stream = torch.cuda.ExternalStream(r.stream())

    def time_ms(fn: Callable[[], None], reps: int) -> float:
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for s, e in ev:
            with torch.cuda.stream(stream):
                s.record(stream)
            fn()
            with torch.cuda.stream(stream):
                e.record(stream)
        r.waitIdle()
        torch.cuda.synchronize()
        return float(np.median([s.elapsed_time(e) for s, e in ev]))
    return time_ms


def _calibrate(r: A.Renderer, frame: Callable[[], None], headroom: float) -> A.Capacity:
    """Capacities from the peak counts of an exactly sized run, times a headroom, doubled until the
    frame runs without overflow."""
    r.setCapacity(None)
    r.getPeakCounts()   # reset
    frame()
    r.waitIdle()
    pk = r.getPeakCounts()
    cap = A.Capacity(max(1024, int(pk.clip_vertices * headroom) + 1024),
                     max(1024, int(pk.clip_polygons * headroom) + 1024),
                     max(1024, int(pk.appended_primitives * headroom) + 1024),
                     max(4096, int(pk.bin_entries * headroom) + 4096), 1,
                     int(pk.fragments * headroom) + 4096 if pk.fragments else 0)
    for _ in range(8):
        r.setCapacity(cap)
        frame()
        if r.getOverflow() == 0:
            return cap
        cap = A.Capacity(cap.clip_vertices * 2, cap.clip_polygons * 2, cap.appended_primitives * 2,
                         cap.bin_entries * 2, 1, cap.fragments * 2)
    r.setCapacity(None)
    raise RuntimeError("autotune: the frame does not fit its capacities")


def autotune(r: A.Renderer, frame: Callable[[], None], headroom: float = 1.25, reps: int = 5,
             heavy_first=(1, 0), graph=(False, True), tiles=(16, 8)) -> Tuned:
    """Search tile height (16x16 or 16x8 raster tiles of the deferred kernels, sglc_set_tile_size)
    x tile order x eager-or-graph submission; capacities are calibrated per tile height. The winner's
    settings stay on the renderer (and its graph, when it won, is captured afresh under them)."""
    time_ms = _timer(r)
    table, best, best_cap = [], None, None
    for tile in tiles:
        r.setTileSize(tile)
        cap = _calibrate(r, frame, headroom)
        for hf in heavy_first:
            for use_graph in graph:
                cap.heavy_first = hf
                r.setCapacity(cap)
                g = None
                if use_graph:
                    frame()   # the uncaptured run that sizes every working array
                    r.waitIdle()
                    g = Graph(r).capture(frame)
                    run = g.launch
                else:
                    run = frame
                for _ in range(2):
                    run()
                ms = time_ms(run, reps)
                ok = r.getOverflow() == 0
                table.append({"tile": tile, "threads_per_tile": 16 * tile, "heavy_first": hf, "graph": use_graph,
                              "ms": round(ms, 4), "fits": ok})
                if g is not None:
                    g.destroy()
                if ok and (best is None or ms < best.ms):
                    best = TuneResult(A.Capacity(cap.clip_vertices, cap.clip_polygons, cap.appended_primitives,
                                                 cap.bin_entries, hf, cap.fragments), hf, use_graph, ms,
                                      tile=tile, threads_per_tile=16 * tile)
    if best is None:
        r.setCapacity(None)
        raise RuntimeError("autotune: no candidate fitted its capacities")
    best.table = table
    r.setTileSize(best.tile)
    r.setCapacity(best.capacity)
    g = None
    if best.graph:
        frame()   # sizes the arrays for the winner's settings, then the graph is captured under them
        r.waitIdle()
        g = Graph(r).capture(frame)
    return Tuned(r, frame, best, g)
