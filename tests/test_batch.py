"""Batched views (sglc_draw_views): one pipeline pass over many views must give, view for view,
exactly the images of drawing the views one render pass at a time (the reference viewer's
sequence), after a depth-only shadow pass whose PCF lookup feeds the Blinn-Phong shader."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300.batch import BatchConfig, BatchedViews

from helpers import assert_outputs_match

SMALL = BatchConfig(views=6, size=96, shadow=256, lon=48, lat=24, tex=64)


def _render(lib, cfg, batched, layout=A.Layout_Linear):
    r = A.Renderer(lib, 0)
    b = BatchedViews(r, cfg, layout=layout)
    if batched:
        b.render()
    else:
        b.render_looped()
    r.waitIdle()
    outs = [b.view_outputs(v) for v in range(cfg.views)]
    shadow = b.shadow_tex.readImage()
    r.destroy()
    return outs, shadow


def test_oracle_batched_equals_looped(oracle_lib):
    a, sa = _render(oracle_lib, SMALL, True)
    b, sb = _render(oracle_lib, SMALL, False)
    for v in range(SMALL.views):
        assert np.array_equal(a[v]["color"], b[v]["color"]) and np.array_equal(a[v]["depth"], b[v]["depth"])
    # the views differ from one another and the shadow map is non-trivial
    assert not np.array_equal(a[0]["color"], a[1]["color"])
    assert 0.05 < (sa < 1).mean() < 0.95


@pytest.mark.gpu
def test_gpu_batched_equals_gpu_looped(cuda_lib):
    a, sa = _render(cuda_lib, SMALL, True)
    b, sb = _render(cuda_lib, SMALL, False)
    assert np.array_equal(sa.view(np.uint32), sb.view(np.uint32))
    for v in range(SMALL.views):
        assert np.array_equal(a[v]["color"], b[v]["color"]), v
        assert np.array_equal(a[v]["depth"].view(np.uint32), b[v]["depth"].view(np.uint32)), v


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [SMALL, BatchConfig(views=1, size=64, shadow=128, lon=32, lat=16, tex=64),
                                 BatchConfig(views=17, size=57, shadow=200, lon=40, lat=20, tex=64, seed=4100)])
def test_gpu_batched_matches_oracle(cfg, cuda_lib, oracle_lib):
    g, gs = _render(cuda_lib, cfg, True)
    c, cs = _render(oracle_lib, cfg, False)
    assert np.array_equal(gs.view(np.uint32), cs.view(np.uint32))
    for v in range(cfg.views):
        assert_outputs_match([g[v]], [c[v]], f"view {v}")
