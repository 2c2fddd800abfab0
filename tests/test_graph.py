"""Synchronisation-free draws (capacities instead of count read-backs), CUDA-graph capture and
replay of a whole frame, overflow reporting, and the autotuner: each must reproduce, image for
image, the default (exactly sized) draws."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S
from softglrender_gb300.autotune import autotune
from softglrender_gb300.batch import BatchConfig, BatchedViews
from softglrender_gb300.graph import Graph

pytestmark = pytest.mark.gpu

CFG = BatchConfig(views=5, size=80, shadow=256, lon=48, lat=24, tex=64, seed=4200)


def _outs(b):
    b.r.waitIdle()
    return [b.view_outputs(v) for v in range(b.cfg.views)]


def _same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x["color"], y["color"])
        assert np.array_equal(x["depth"].view(np.uint32), y["depth"].view(np.uint32))


@pytest.fixture()
def batch(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    b = BatchedViews(r, CFG)
    yield b
    r.destroy()


def test_capacity_mode_matches_exact(batch):
    b = batch
    b.render()
    exact = _outs(b)
    b.r.setCapacity(A.Capacity(1 << 16, 1 << 14, 1 << 14, 1 << 20, 1))
    b.render()
    _same(_outs(b), exact)
    assert b.r.getOverflow() == 0
    b.r.setCapacity(A.Capacity(1 << 16, 1 << 14, 1 << 14, 1 << 20, 0))   # tiles in index order
    b.render()
    _same(_outs(b), exact)


def test_overflow_is_reported_not_faulted(batch):
    b = batch
    b.r.setCapacity(A.Capacity(1 << 16, 1 << 14, 1 << 14, 64, 1))
    b.render()
    assert b.r.getOverflow() & 8          # bin entries
    assert b.r.getOverflow() == 0         # reading clears
    b.r.setCapacity(None)
    b.render()                            # the context stays usable
    assert len(_outs(b)) == CFG.views


def test_graph_replay_matches_eager(batch):
    b = batch
    b.render()
    exact = _outs(b)
    b.r.setCapacity(A.Capacity(1 << 16, 1 << 14, 1 << 14, 1 << 20, 1))
    b.render()                            # sizes every working array before the capture
    g = Graph(b.r).capture(b.render)
    # change view 0's camera and render eagerly: the replay must restore the captured frame
    ub = [u for u in b.res[0].blocks.values() if u.name == "UniformsModel"][0]
    ub.setData(S.uniforms_model(np.eye(4), np.eye(4) * 0.5, None, False))
    b.render()
    assert not np.array_equal(_outs(b)[0]["color"], exact[0]["color"])
    g.launch()
    g.launch()
    _same(_outs(b), exact)
    assert b.r.getOverflow() == 0
    g.destroy()


def test_autotune_picks_a_fitting_configuration(batch):
    b = batch
    b.render()
    exact = _outs(b)
    t = autotune(b.r, b.render, reps=3)
    d = t.result.describe()
    # two tile shapes x two tile orders x eager / graph, all fitting their capacities
    assert d["tile"] in (16, 8) and d["threads_per_tile"] == 16 * d["tile"]
    assert len(d["candidates"]) == 8 and all(c["fits"] for c in d["candidates"])
    assert {c["tile"] for c in d["candidates"]} == {16, 8}
    t.run()
    _same(_outs(b), exact)
    t.destroy()


def test_graph_is_invalidated_by_its_own_renderer_only(batch, cuda_lib):
    """Frees in another renderer (working arrays grown, resources released) leave a graph
    replayable; releasing a resource of the graph's own renderer makes it refuse to replay."""
    b = batch
    b.render()
    exact = _outs(b)
    b.r.setCapacity(A.Capacity(1 << 16, 1 << 14, 1 << 14, 1 << 20, 1))
    b.render()
    g = Graph(b.r).capture(b.render)
    other = A.Renderer(cuda_lib, 0)
    ob = BatchedViews(other, BatchConfig(views=3, size=160, shadow=512, lon=64, lat=32, tex=64, seed=4300))
    ob.render()                                    # grows the other renderer's working arrays
    spare = other.createTexture(A.TextureDesc(64, 64, A.TextureType_2D, A.TextureFormat_RGBA8,
                                              A.TextureUsage_Sampler, False, False))
    spare.initImageData()
    other.release(spare)
    other.waitIdle()
    g.launch()
    _same(_outs(b), exact)
    own = b.r.createTexture(A.TextureDesc(64, 64, A.TextureType_2D, A.TextureFormat_RGBA8,
                                          A.TextureUsage_Sampler, False, False))
    own.initImageData()
    b.r.release(own)
    with pytest.raises(A.SoftGLError):
        g.launch()
    g.destroy()
    other.destroy()
