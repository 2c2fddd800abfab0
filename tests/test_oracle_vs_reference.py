"""Pins the CPU oracle (oracle/softgl_oracle.cpp) to the UNMODIFIED reference RendererSoft built
from the reference sources (oracle/_ref): bit-identical colour, MSAA samples, resolved colour and
depth on every case. Skipped where the reference cannot be built (no reference tree / not x86)."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

from golden.cases import CASES, soup
from helpers import assert_outputs_match, render


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference(name, oracle_lib, reference_lib):
    scene = CASES[name]()
    ref, rs = render(reference_lib, scene)
    orc, os_ = render(oracle_lib, scene)
    assert_outputs_match(orc, ref, name, exact_color=True)


@pytest.mark.parametrize("func", range(8))
def test_depth_functions_vs_reference(func, oracle_lib, reference_lib):
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=func)
    scene = soup(1500, 64, 48, 4, [st, st], clear_depth=0.5)
    assert_outputs_match(render(oracle_lib, scene)[0], render(reference_lib, scene)[0], f"func {func}", True)


@pytest.mark.parametrize("src,dst,fn", [(3, 7, 0), (1, 1, 0), (4, 0, 2), (5, 9, 3), (8, 3, 4), (6, 2, 0)])
def test_blending_vs_reference(src, dst, fn, oracle_lib, reference_lib):
    bp = A.BlendParameters()
    bp.SetBlendFactor(src, dst)
    bp.SetBlendFunc(fn)
    scene = soup(2000, 96, 64, 4, [A.RenderStates(depthTest=True),
                                   A.RenderStates(blend=True, blendParams=bp, depthTest=True, depthMask=False)])
    assert_outputs_match(render(oracle_lib, scene)[0], render(reference_lib, scene)[0], "blend", True)


@pytest.mark.parametrize("filt", range(6))
@pytest.mark.parametrize("wrap", range(4))
def test_sampling_vs_reference(filt, wrap, oracle_lib, reference_lib):
    scene = S.config_plain_small(width=160, height=120, lon=32, lat=16, tex=64, filter_min=filt)
    ts = scene.passes[0].draws[0].textures[0]
    ts.sampler = A.SamplerDesc(filt, A.Filter_LINEAR, wrap, wrap, wrap, A.Border_WHITE)
    scene.passes[0].draws[0].vertexes[:, 4:6] = scene.passes[0].draws[0].vertexes[:, 4:6] * 2.5 - 0.7
    assert_outputs_match(render(oracle_lib, scene)[0], render(reference_lib, scene)[0], "sampling", True)


def test_early_z_off_vs_reference(oracle_lib, reference_lib):
    scene = S.config_geometry_stress(n_tris=4000, width=128, height=96)
    assert_outputs_match(render(oracle_lib, scene, early_z=False)[0], render(reference_lib, scene, early_z=False)[0],
                         "early z off", True)


@pytest.mark.parametrize("variant", ["tiled", "morton"])
def test_reference_buffer_layouts(variant, oracle_lib):
    """The reference's compile-time Tiled/Morton layouts (Buffer.h:140-213) change addressing only:
    at sizes that are multiples of the layout tile the result equals the linear-layout oracle."""
    import oracle
    lib = oracle.reference(variant)
    if lib is None:
        pytest.skip("reference checker not buildable here")
    scene = S.config_pbr(width=256, height=128, lon=64, lat=32, tex=128, prefilter=64, irradiance=16)
    assert_outputs_match(render(oracle_lib, scene)[0], render(lib, scene)[0], variant, True)


def test_parallel_oracle_equals_serial(oracle_lib):
    """Row-band parallel mode (the CPU baseline) gives the serial result."""
    scene = S.config_geometry_stress(n_tris=8000, width=200, height=150)
    a, _ = render(oracle_lib, scene, threads=1)
    b, _ = render(oracle_lib, scene, threads=7)
    assert_outputs_match(a, b, "threads", True)
