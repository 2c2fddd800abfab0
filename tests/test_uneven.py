"""Uneven batch (scenes of different size, resolution, shading and sample count in one
submission): every scene matches the CPU oracle, the CUDA-graph replay of the whole batch
matches its eager submission, and the batch split over concurrent renderers (lanes) gives the
same images."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300.autotune import autotune
from softglrender_gb300.uneven import UnevenBatch, UnevenConfig, UnevenLanes, assign_lanes, scene_plan

from helpers import assert_outputs_match

SMALL = UnevenConfig(scenes=6, tri_min=200, tri_max=20000, resolutions=(48, 96, 128), seed=5100, pbr_tex=64,
                     prefilter=32, irradiance=8, blinn_tex=64)


def test_plan_is_seeded_and_mixed():
    a, b = scene_plan(SMALL), scene_plan(SMALL)
    assert a == b
    assert {p["pbr"] for p in a} == {0, 1}
    full = scene_plan(UnevenConfig())
    tris = [2 * p["lon"] * (p["lat"] - 1) for p in full]
    assert len(full) == 64 and min(tris) < 5000 and max(tris) > 500000
    assert {p["res"] for p in full} == {128, 512, 1024, 2048}


def _render(lib, cfg):
    r = A.Renderer(lib, 0)
    u = UnevenBatch(r, cfg)
    u.render()
    r.waitIdle()
    outs = [u.outputs(s) for s in range(cfg.scenes)]
    r.destroy()
    return outs


@pytest.mark.gpu
def test_uneven_batch_matches_oracle(cuda_lib, oracle_lib):
    g = _render(cuda_lib, SMALL)
    c = _render(oracle_lib, SMALL)
    for s in range(SMALL.scenes):
        assert_outputs_match([g[s]], [c[s]], f"scene {s}")


def _render_both(lib, cfg):
    """Per-scene render passes and the multi-scene draws of the same batch on one renderer."""
    r = A.Renderer(lib, 0)
    u = UnevenBatch(r, cfg)
    u.render()
    r.waitIdle()
    single = [u.outputs(s) for s in range(cfg.scenes)]
    u.render_batched()
    r.waitIdle()
    batched = [u.outputs(s) for s in range(cfg.scenes)]
    r.destroy()
    return single, batched


def _assert_same(a, b, what):
    for s in range(len(a)):
        for k in a[s]:
            assert np.array_equal(a[s][k].view(np.uint8), b[s][k].view(np.uint8)), (what, s, k)


def test_multi_scene_draw_is_per_scene_passes_on_oracle(oracle_lib):
    single, batched = _render_both(oracle_lib, SMALL)
    _assert_same(single, batched, "oracle")


@pytest.mark.gpu
def test_multi_scene_draw_matches_per_scene_passes(cuda_lib, oracle_lib):
    """One pipeline pass per class of scenes gives every scene's images bit for bit as its own
    render pass does, and within the parity bar of the oracle; also with capacities set (no
    read-back) and replayed from a CUDA graph, twice."""
    single, batched = _render_both(cuda_lib, SMALL)
    _assert_same(single, batched, "cuda")
    c = _render(oracle_lib, SMALL)
    for s in range(SMALL.scenes):
        assert_outputs_match([batched[s]], [c[s]], f"multi-scene draw, scene {s}")
    r = A.Renderer(cuda_lib, 0)
    u = UnevenBatch(r, SMALL)
    t = autotune(r, u.render_batched, reps=2, heavy_first=(1,), graph=(True,))
    for _ in range(2):
        t.run()
        r.waitIdle()
        _assert_same(single, [u.outputs(s) for s in range(SMALL.scenes)], "graph")
    assert r.getOverflow() == 0
    t.destroy()
    r.destroy()


@pytest.mark.gpu
def test_uneven_graph_replay_matches_eager(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    u = UnevenBatch(r, SMALL)
    u.render()
    r.waitIdle()
    eager = [u.outputs(s) for s in range(SMALL.scenes)]
    t = autotune(r, u.render, reps=2, heavy_first=(1,), graph=(True,))
    assert t.result.graph
    t.run()
    r.waitIdle()
    for s in range(SMALL.scenes):
        o = u.outputs(s)
        for k in eager[s]:
            assert np.array_equal(o[k].view(np.uint8), eager[s][k].view(np.uint8)), (s, k)
    t.destroy()
    r.destroy()


def test_assign_lanes_covers_and_balances():
    cost = [float(c) for c in (50, 1, 1, 1, 20, 20, 5, 3, 2, 30)]
    groups = assign_lanes(cost, 3)
    assert sorted(sum(groups, [])) == list(range(len(cost)))
    loads = [sum(cost[s] for s in g) for g in groups]
    assert max(loads) == 50.0 and min(loads) >= 30.0   # the longest scene alone; the rest spread
    assert assign_lanes(cost, 3) == groups               # deterministic
    assert assign_lanes(cost, 1) == [list(range(len(cost)))]


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_uneven_lanes_match_single_renderer(cuda_lib, batched):
    r = A.Renderer(cuda_lib, 0)
    u = UnevenBatch(r, SMALL)
    u.render()
    r.waitIdle()
    single = [u.outputs(s) for s in range(SMALL.scenes)]
    rs = [A.Renderer(cuda_lib, 0) for _ in range(3)]
    ul = UnevenLanes(rs, SMALL, [float(t) for t in u.triangles], batched=batched)
    assert sorted(sum(ul.groups, [])) == list(range(SMALL.scenes))
    ul.tune(reps=2)
    for _ in range(2):   # two submissions in a row
        ul.launch()
        ul.wait()
        for s in range(SMALL.scenes):
            o = ul.outputs(s)
            for k in single[s]:
                assert np.array_equal(o[k].view(np.uint8), single[s][k].view(np.uint8)), (s, k)
    ul.release()
    for x in rs:
        x.destroy()
    r.destroy()
