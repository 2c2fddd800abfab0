"""Deferred shading (coverage / depth kernel, fragment-shader kernel over the fragment records, ordered
colour operations) against the single fused raster kernel: the same images bit for bit, for every
shading model it serves, single and batched draws, exact sizing and set capacities; a fragment-record
capacity that is too small is reported, not faulted."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S
from softglrender_gb300.batch import BatchConfig, BatchedViews
from softglrender_gb300.ibl import IBLGenerator, equirect_sky

from helpers import render

pytestmark = pytest.mark.gpu

SCENES = {
    "blinn_dir_mips": lambda: S.config_plain_small(width=300, height=200, lon=48, lat=24, tex=64),
    "pbr_msaa4": lambda: S.config_pbr(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=8),
    "pbr_msaa1": lambda: S.config_pbr(width=256, height=144, samples=1, lon=64, lat=32, tex=64, prefilter=32,
                                      irradiance=8),
}


def _render_mode(lib, scene, deferred):
    r = A.Renderer(lib, 0)
    r.setDeferredShading(deferred)
    inst = S.SceneInstance(r, scene)
    inst.render()
    r.waitIdle()
    out = inst.outputs()
    r.destroy()
    return out


@pytest.mark.parametrize("name", sorted(SCENES))
def test_deferred_equals_fused(name, cuda_lib):
    scene = SCENES[name]()
    a = _render_mode(cuda_lib, scene, True)
    b = _render_mode(cuda_lib, scene, False)
    for k in a:
        x, y = a[k], b[k]
        if x.dtype == np.float32:
            x, y = x.view(np.uint32), y.view(np.uint32)
        assert np.array_equal(x, y), k


def test_deferred_equals_fused_ibl(cuda_lib):
    outs = []
    for deferred in (True, False):
        r = A.Renderer(cuda_lib, 0)
        r.setDeferredShading(deferred)
        g = IBLGenerator(r)
        eq = r.createTexture(A.TextureDesc(64, 32, A.TextureType_2D, A.TextureFormat_RGBA8,
                                           A.TextureUsage_Sampler | A.TextureUsage_UploadData, False, False))
        eq.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE,
                                        A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE))
        eq.setImageData([equirect_sky(64, 32, 7)])
        cube = g.convert_equirectangular(eq, 32)
        pf = g.prefilter(cube, 16, 3)
        r.waitIdle()
        outs.append([cube.readImage(f) for f in range(6)] + [pf.readImage(f, 1) for f in range(6)])
        r.destroy()
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


CFG = BatchConfig(views=6, size=96, shadow=256, lon=48, lat=24, tex=64, seed=4300)


def _batch_outputs(lib, deferred, capacity=None):
    r = A.Renderer(lib, 0)
    r.setDeferredShading(deferred)
    b = BatchedViews(r, CFG)
    if capacity is not None:
        r.setCapacity(capacity)
    b.render()
    r.waitIdle()
    out = [b.view_outputs(v) for v in range(CFG.views)]
    flags = r.getOverflow() if capacity is not None else 0
    r.destroy()
    return out, flags


def test_batched_deferred_equals_fused_and_capacity_mode(cuda_lib):
    fused, _ = _batch_outputs(cuda_lib, False)
    exact, _ = _batch_outputs(cuda_lib, True)
    capped, flags = _batch_outputs(cuda_lib, True, A.Capacity(1 << 16, 1 << 14, 1 << 14, 1 << 20, 1, 1 << 22))
    assert flags == 0
    for a, b, c in zip(fused, exact, capped):
        for k in ("color", "depth"):
            x, y, z = a[k], b[k], c[k]
            if x.dtype == np.float32:
                x, y, z = x.view(np.uint32), y.view(np.uint32), z.view(np.uint32)
            assert np.array_equal(x, y) and np.array_equal(x, z), k


def test_fragment_capacity_overflow_is_reported(cuda_lib):
    out, flags = _batch_outputs(cuda_lib, True, A.Capacity(1 << 16, 1 << 14, 1 << 14, 1 << 20, 1, 64))
    assert flags & 32                    # fragment records
    assert len(out) == CFG.views         # the context stayed usable and the draw completed
