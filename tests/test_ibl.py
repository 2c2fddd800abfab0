"""IBL precompute (IBLGenerator, Environment.cpp:25-195): equirectangular -> cube, irradiance and
prefiltered specular maps drawn through the renderer with the skybox / IBL shaders. The CPU
restatement must equal the unmodified reference (same host, same maths library), and the GPU must
match the restatement within the colour bar."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300.ibl import IBLGenerator, equirect_sky

from helpers import assert_color_bar


def _run(lib, env=32, irr=8, pre=16, levels=3):
    r = A.Renderer(lib, 0)
    g = IBLGenerator(r)
    eq = r.createTexture(A.TextureDesc(64, 32, A.TextureType_2D, A.TextureFormat_RGBA8,
                                       A.TextureUsage_Sampler | A.TextureUsage_UploadData, False, False))
    eq.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE,
                                    A.Wrap_CLAMP_TO_EDGE))
    eq.setImageData([equirect_sky(64, 32, 7)])
    cube = g.convert_equirectangular(eq, env)
    ir = g.irradiance(cube, irr)
    pf = g.prefilter(cube, pre, levels)
    r.waitIdle()
    out = {"cube": np.stack([cube.readImage(f) for f in range(6)]),
           "irradiance": np.stack([ir.readImage(f) for f in range(6)])}
    for lv in range(levels):
        out[f"prefilter{lv}"] = np.stack([pf.readImage(f, lv) for f in range(6)])
    r.destroy()
    return out


def test_restatement_equals_reference(oracle_lib, reference_lib):
    a = _run(oracle_lib)
    b = _run(reference_lib)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    # the maps are not trivial: the cube has the sky's range, irradiance is smooth
    assert a["cube"][..., :3].std() > 10 and a["irradiance"][..., :3].std() < a["cube"][..., :3].std()


@pytest.mark.gpu
def test_gpu_matches_restatement(cuda_lib, oracle_lib):
    g = _run(cuda_lib)
    c = _run(oracle_lib)
    for k in c:
        # the six faces stacked into one pixel grid (6*h rows)
        gk, ck = g[k].reshape(-1, *g[k].shape[2:]), c[k].reshape(-1, *c[k].shape[2:])
        assert_color_bar(gk, ck, "ibl", k, max_abs=2)
