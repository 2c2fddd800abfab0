"""Parity of the CUDA renderer with the CPU oracle (a restatement of RendererSoft pinned to the
reference itself by test_oracle_vs_reference.py), on identical seeded inputs, through the C ABI.

The bar: depth (hence coverage, culling and depth-test outcomes) bit-identical; RGBA8 colour with
every channel within 1 LSB on at least 99.9% of pixels (tests/helpers.py COLOR_MIN_FRACTION). Shading
models whose arithmetic has no transcendental functions (vertex colour, base colour) must match
bit for bit."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

from golden.cases import soup
from helpers import assert_outputs_match, render

pytestmark = pytest.mark.gpu

CASES = {
    "plain_small_320": lambda: S.config_plain_small(width=320, height=240),
    "plain_small_full": lambda: S.config_plain_small(),
    "plain_small_close": lambda: S.config_plain_small(width=400, height=300, distance=1.6),
    "geometry_stress_20k": lambda: S.config_geometry_stress(n_tris=20000, width=320, height=180),
    "geometry_stress_100k_1x": lambda: S.config_geometry_stress(n_tris=100000, width=640, height=360, samples=1),
    "pbr_small": lambda: S.config_pbr(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=16),
    "pbr_view3": lambda: S.config_pbr(width=480, height=270, lon=128, lat=64, tex=256, prefilter=128, irradiance=16,
                                      view=3),
    # sub-pixel triangles (most cover no sample point and are not binned) and a dense sphere at a
    # low resolution, opaque (LESS) and with reversed Z
    "tiny_soup_msaa4": lambda: soup(40000, 160, 120, 4, [A.RenderStates(depthTest=True, depthMask=True,
                                                                        depthFunc=A.DepthFunc_LESS)],
                                    seed=31, median_px=0.15),
    "tiny_soup_1x_reversed": lambda: soup(40000, 160, 120, 1, [A.RenderStates(depthTest=True, depthMask=True,
                                                                              depthFunc=A.DepthFunc_GREATER)],
                                          seed=32, clear_depth=0.0, reverse=True, median_px=0.3),
    "dense_sphere_96px": lambda: S.config_plain_small(width=96, height=72, lon=512, lat=256, tex=64),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_parity_configs(name, cuda_lib, oracle_lib):
    scene = CASES[name]()
    gpu, gstats = render(cuda_lib, scene)
    cpu, cstats = render(oracle_lib, scene)
    exact = all(d.shading in (A.Shading_VertexColor, A.Shading_BaseColor) for p in scene.passes for d in p.draws)
    assert_outputs_match(gpu, cpu, name, exact_color=exact)
    assert gstats["primitives"] == cstats["primitives"]
    assert gstats["clip_vertices"] == cstats["clip_vertices"]


@pytest.mark.parametrize("layout", [A.Layout_Tiled, A.Layout_Morton])
def test_texture_layouts(layout, cuda_lib, oracle_lib):
    """Linear / Tiled 4x4 / Morton 32x32 storage changes addressing only (Buffer.h:140-213)."""
    scene = S.config_pbr(width=256, height=144, lon=64, lat=32, tex=128, prefilter=64, irradiance=16)
    gpu, _ = render(cuda_lib, scene, layout=layout)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, f"layout {layout}")


@pytest.mark.parametrize("filt", range(6))
@pytest.mark.parametrize("wrap", range(4))
def test_sampler_filters_wraps(filt, wrap, cuda_lib, oracle_lib):
    scene = S.config_plain_small(width=200, height=150, lon=32, lat=16, tex=64, filter_min=filt)
    ts = scene.passes[0].draws[0].textures[0]
    ts.sampler = A.SamplerDesc(filt, A.Filter_LINEAR, wrap, wrap, wrap, A.Border_WHITE)
    # stretch the texture coordinates outside [0, 1] so the wrap mode matters
    scene.passes[0].draws[0].vertexes[:, 4:6] = scene.passes[0].draws[0].vertexes[:, 4:6] * 2.5 - 0.7
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, f"filter {filt} wrap {wrap}")


def test_early_z_off(cuda_lib, oracle_lib):
    scene = S.config_geometry_stress(n_tris=5000, width=160, height=120)
    gpu, _ = render(cuda_lib, scene, early_z=False)
    cpu, _ = render(oracle_lib, scene, early_z=False)
    assert_outputs_match(gpu, cpu, "early z off", exact_color=True)


def _soup_scene(n, w, h, samples, states_list, seed=7, clear_depth=1.0, reverse=False):
    eye = np.array([0.2, 0.1, 1.8])
    P = S.perspective(np.deg2rad(70.0), w / h, 0.3, reverse, far=3.0)
    V = S.look_at(eye, [0, 0, 0], [0, 1, 0])
    VP = S.mm4(P, V)
    rows, idx, _ = S.triangle_soup(n, seed, VP, w, h, median_px=60.0)
    blocks = {"UniformsModel": S.uniforms_model(np.eye(4), VP, None, reverse),
              "UniformsMaterial": S.uniforms_material(False, False, False, 1.0, 0.0, [1, 1, 1, 1])}
    draws = []
    k = len(states_list)
    per = n // k
    for i, st in enumerate(states_list):
        r = rows[3 * per * i:3 * per * (i + 1)]
        draws.append(S.DrawSpec(r, 32, np.arange(len(r), dtype=np.int32), A.Shading_VertexColor, (), st, blocks))
    clear = A.ClearStates(True, True, (0.1, 0.2, 0.3, 0.4), clear_depth)
    return S.Scene("soup", [S.PassSpec(w, h, samples, clear, draws)])


@pytest.mark.parametrize("func", range(8))
def test_depth_functions(func, cuda_lib, oracle_lib):
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=func)
    scene = _soup_scene(3000, 96, 64, 4, [st, st], clear_depth=0.5)
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, f"depth func {func}", exact_color=True)


@pytest.mark.parametrize("src,dst,fn", [(3, 7, 0), (1, 1, 0), (2, 6, 1), (4, 0, 2), (5, 9, 3), (8, 3, 4), (0, 1, 0)])
def test_blending(src, dst, fn, cuda_lib, oracle_lib):
    bp = A.BlendParameters()
    bp.SetBlendFactor(src, dst)
    bp.SetBlendFunc(fn)
    opaque = A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS)
    blend = A.RenderStates(blend=True, blendParams=bp, depthTest=True, depthMask=False, depthFunc=A.DepthFunc_LESS)
    scene = _soup_scene(4000, 128, 96, 4, [opaque, blend])
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, f"blend {src},{dst},{fn}", exact_color=True)


@pytest.mark.parametrize("w,h,samples", [(1, 1, 1), (17, 13, 4), (31, 33, 1), (300, 7, 4)])
def test_odd_framebuffer_sizes(w, h, samples, cuda_lib, oracle_lib):
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS, cullFace=False)
    scene = _soup_scene(2000, w, h, samples, [st])
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, f"fbo {w}x{h}x{samples}", exact_color=True)


def test_empty_and_degenerate_draws(cuda_lib, oracle_lib):
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS)
    scene = _soup_scene(600, 64, 48, 1, [st])
    d = scene.passes[0].draws[0]
    empty = S.DrawSpec(d.vertexes[:0], 32, np.zeros(0, np.int32), d.shading, (), st, d.blocks)
    degen_rows = d.vertexes[:30].copy()
    degen_rows[1::3, :3] = degen_rows[0::3, :3]          # two identical vertices per triangle
    degen = S.DrawSpec(degen_rows, 32, np.arange(30, dtype=np.int32), d.shading, (), st, d.blocks)
    scene.passes[0].draws = [empty, degen, d]
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, "empty/degenerate", exact_color=True)


def test_clear_only_pass(cuda_lib, oracle_lib):
    st = A.RenderStates(depthTest=True)
    scene = _soup_scene(60, 40, 30, 4, [st])
    scene.passes[0].draws = []
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_depth_equal = gpu[0]["depth"].view(np.uint32) == cpu[0]["depth"].view(np.uint32)
    assert assert_depth_equal.all()
    assert np.array_equal(gpu[0]["color"], cpu[0]["color"])


def test_all_geometry_clipped(cuda_lib, oracle_lib):
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS)
    scene = _soup_scene(500, 64, 48, 1, [st])
    d = scene.passes[0].draws[0]
    d.vertexes[:, 2] += 50.0      # everything behind the camera / beyond the far plane
    gpu, gs = render(cuda_lib, scene)
    cpu, cs = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, "all clipped", exact_color=True)
    assert gs["primitives"] == cs["primitives"]
