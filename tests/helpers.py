"""Shared comparison helpers for the parity tests."""
from __future__ import annotations

import numpy as np

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S


def render(lib, scene, layout=A.Layout_Linear, early_z=True, threads=None):
    r = A.Renderer(lib, 0)
    if threads is not None:
        lib.cdll.sglo_set_threads(r.ctx, threads)
    r.setEnableEarlyZ(early_z)
    inst = S.SceneInstance(r, scene, layout=layout)
    inst.render()
    r.waitIdle()
    outs = [inst.outputs(i) for i in range(len(scene.passes))]
    stats = r.drawStats()
    r.destroy()
    return outs, stats


def assert_depth_exact(a, b, what=""):
    da, db = a.view(np.uint32), b.view(np.uint32)
    bad = np.argwhere(da != db)
    assert bad.size == 0, f"{what}: {len(bad)} depth values differ, first at {bad[:5].tolist()}"


def color_stats(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return d.max(), float((d <= 1).mean()), int((d > 1).sum())


# the colour bar: within 1 LSB per channel on at least 99.9% of channels
COLOR_MIN_FRACTION = 0.999


def assert_outputs_match(gpu, cpu, what="", exact_color=False):
    for p, (g, c) in enumerate(zip(gpu, cpu)):
        if "depth" in c:
            assert_depth_exact(g["depth"], c["depth"], f"{what} pass {p}")
        for key in ("color", "resolved"):
            if key not in c:
                continue
            mx, frac, nbad = color_stats(g[key], c[key])
            if exact_color:
                assert mx == 0, f"{what} pass {p} {key}: max diff {mx}"
            else:
                assert frac >= COLOR_MIN_FRACTION, f"{what} pass {p} {key}: {nbad} channels > 1 LSB ({frac:.6f})"
