"""Shared comparison helpers for the parity tests.

The colour bar is per PIXEL: a pixel passes when every channel (of every sample, for a multi-sample
attachment) is within 1 LSB of the checker's, and at least 99.9% of pixels must pass. Depth is
compared bit for bit. Every comparison's pixel fraction and max-abs difference is appended to the
JSON-lines file named by SGLC_PARITY_LOG when that variable is set."""
from __future__ import annotations

import json
import os

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
    """(max abs difference, fraction of pixels with every channel within 1 LSB, pixels failing).
    Axes 0 and 1 are the pixel grid; the remaining axes (channels, samples) belong to the pixel."""
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    if d.ndim > 2:
        per_pixel = d.reshape(d.shape[0], d.shape[1], -1).max(axis=2)
    else:
        per_pixel = d
    return int(d.max(initial=0)), float((per_pixel <= 1).mean()) if per_pixel.size else 1.0, \
        int((per_pixel > 1).sum())


# the colour bar: every channel within 1 LSB on at least 99.9% of pixels
COLOR_MIN_FRACTION = 0.999


def log_parity(what, key, mx, frac, nbad, npix):
    path = os.environ.get("SGLC_PARITY_LOG")
    if not path:
        return
    with open(path, "a") as f:
        f.write(json.dumps({"case": what, "image": key, "pixel_fraction": frac, "max_abs": mx,
                            "pixels_over_1lsb": nbad, "pixels": npix}) + "\n")


def assert_color_bar(g, c, what="", key="color", max_abs=None):
    """Per-pixel colour bar; `max_abs` optionally bounds the largest channel difference too."""
    mx, frac, nbad = color_stats(g, c)
    log_parity(what, key, mx, frac, nbad, int(g.shape[0] * g.shape[1]) if g.ndim >= 2 else g.size)
    assert frac >= COLOR_MIN_FRACTION, \
        f"{what} {key}: {nbad} pixels > 1 LSB ({frac:.6f} of pixels pass, max abs {mx})"
    if max_abs is not None:
        assert mx <= max_abs, f"{what} {key}: max abs {mx} > {max_abs}"
    return mx, frac


def assert_outputs_match(gpu, cpu, what="", exact_color=False):
    for p, (g, c) in enumerate(zip(gpu, cpu)):
        if "depth" in c:
            assert_depth_exact(g["depth"], c["depth"], f"{what} pass {p}")
        for key in ("color", "resolved"):
            if key not in c:
                continue
            if exact_color:
                mx, frac, nbad = color_stats(g[key], c[key])
                log_parity(f"{what} pass {p}", key, mx, frac, nbad, int(g[key].shape[0] * g[key].shape[1]))
                assert mx == 0, f"{what} pass {p} {key}: max diff {mx}"
            else:
                assert_color_bar(g[key], c[key], f"{what} pass {p}", key)
