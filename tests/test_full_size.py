"""Parity at the full sizes of the measured workloads, against the CPU oracle run on all host cores
(its band-parallel mode gives the single-threaded result, test_oracle_vs_reference.py):

- the 1M-triangle vertex-colour soup at 1920x1080, 4x MSAA, opaque then blended pass, reversed Z;
- the 200k-triangle PBR+IBL sphere at 1920x1080, 4x MSAA (the frames/s workload), drawn eagerly and
  replayed from the autotuned CUDA graph with set capacities (the submission the throughput is
  measured on);
- 256 batched views at 256x256 after a 2048x2048 shadow pass (one batched draw against the
  reference viewer's one pass per view);
- the extremes of the 64-scene uneven batch: 1.9M triangles at 1024x1024 PBR MSAA 4x, 830k at
  2048x2048 PBR, 889k at 128x128 PBR, 1.7M at 512x512 Blinn-Phong, 960 at 2048x2048 PBR; and all 64
  scenes as multi-scene draws against their own render passes.

Depth bit for bit; colour within the colour bar (exactly, for vertex colours)."""
import os

import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S
from softglrender_gb300.autotune import autotune
from softglrender_gb300.batch import BatchConfig, BatchedViews
from softglrender_gb300.uneven import UnevenBatch, UnevenConfig

from helpers import assert_outputs_match, render

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_geometry_stress_full(cuda_lib, oracle_lib):
    scene = S.config_geometry_stress()
    gpu, gs = render(cuda_lib, scene)
    cpu, cs = render(oracle_lib, scene, threads=THREADS)
    assert_outputs_match(gpu, cpu, "soup 1M", exact_color=True)
    assert gs["primitives"] == cs["primitives"] and gs["clip_vertices"] == cs["clip_vertices"]


def test_pbr_ibl_full_eager_and_tuned_graph(cuda_lib, oracle_lib):
    scene = S.config_pbr()
    cpu, _ = render(oracle_lib, scene, threads=THREADS)
    r = A.Renderer(cuda_lib, 0)
    inst = S.SceneInstance(r, scene)
    inst.render()
    r.waitIdle()
    eager = inst.outputs()
    assert_outputs_match([eager], cpu, "pbr 1080p eager")
    tuned = autotune(r, inst.render, reps=2)
    tuned.run()
    r.waitIdle()
    assert r.getOverflow() == 0
    replay = inst.outputs()
    for k in eager:
        assert np.array_equal(replay[k].view(np.uint8), eager[k].view(np.uint8)), k
    tuned.destroy()
    r.destroy()


def _views(lib, cfg, batched, threads=None):
    r = A.Renderer(lib, 0)
    if threads:
        lib.cdll.sglo_set_threads(r.ctx, threads)
    b = BatchedViews(r, cfg)
    b.render() if batched else b.render_looped()
    r.waitIdle()
    outs = [b.view_outputs(v) for v in range(cfg.views)]
    shadow = b.shadow_tex.readImage()
    r.destroy()
    return outs, shadow


def test_batched_views_full(cuda_lib, oracle_lib):
    cfg = BatchConfig()
    g, gs = _views(cuda_lib, cfg, True)
    c, cs = _views(oracle_lib, cfg, False, THREADS)
    assert np.array_equal(gs.view(np.uint32), cs.view(np.uint32))
    for v in range(cfg.views):
        assert_outputs_match([g[v]], [c[v]], f"view {v}")


UNEVEN_EXTREMES = [63, 19, 57, 40, 43]


def _uneven(lib, threads=None):
    r = A.Renderer(lib, 0)
    if threads:
        lib.cdll.sglo_set_threads(r.ctx, threads)
    u = UnevenBatch(r, UnevenConfig(), only=UNEVEN_EXTREMES)
    u.render(UNEVEN_EXTREMES)
    r.waitIdle()
    outs = {s: u.outputs(s) for s in UNEVEN_EXTREMES}
    tris = {s: u.triangles[s] for s in UNEVEN_EXTREMES}
    r.destroy()
    return outs, tris


def test_uneven_extremes_full(cuda_lib, oracle_lib):
    g, tris = _uneven(cuda_lib)
    c, _ = _uneven(oracle_lib, THREADS)
    assert max(tris.values()) > 1_800_000 and min(tris.values()) < 1000
    for s in UNEVEN_EXTREMES:
        assert_outputs_match([g[s]], [c[s]], f"scene {s}")


def test_uneven_full_multi_scene_equals_per_scene(cuda_lib):
    """All 64 scenes of the uneven batch (1k-2M triangles, 128^2-2048^2, Blinn-Phong and PBR MSAA 4x)
    drawn as one multi-scene draw per class equal their own render passes bit for bit (the per-scene
    passes are checked against the oracle above), eagerly and replayed from the tuned graph."""
    r = A.Renderer(cuda_lib, 0)
    u = UnevenBatch(r, UnevenConfig())
    u.render()
    r.waitIdle()
    single = {s: u.outputs(s) for s in range(u.cfg.scenes)}
    u.render_batched()
    r.waitIdle()
    for s in range(u.cfg.scenes):
        o = u.outputs(s)
        for k in single[s]:
            assert np.array_equal(o[k].view(np.uint8), single[s][k].view(np.uint8)), ("eager", s, k)
    t = autotune(r, u.render_batched, reps=1, heavy_first=(1,), graph=(True,))
    t.run()
    r.waitIdle()
    assert r.getOverflow() == 0
    for s in range(u.cfg.scenes):
        o = u.outputs(s)
        for k in single[s]:
            assert np.array_equal(o[k].view(np.uint8), single[s][k].view(np.uint8)), ("graph", s, k)
    t.destroy()
    r.destroy()
