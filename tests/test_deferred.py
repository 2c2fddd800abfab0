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

from helpers import assert_outputs_match, render

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


def _spheres_scene(samples, func, mask, clear_depth, w=160, h=120):
    """Three overlapping spheres drawn without culling (two to four fragments per pixel), directional
    Blinn-Phong (a deferred shading model), one depth function and depth-write setting for all."""
    vert, idx = S.uv_sphere(40, 20)
    eye = np.array([0.0, 0.0, 3.2])
    Pm = S.perspective(np.pi / 3.0, w / h, 0.05, False)
    VP = S.mm4(Pm, S.look_at(eye, [0, 0, 0], [0, 1, 0]))
    scene_block = S.uniforms_scene([0.15, 0.15, 0.15], eye, S.normalize(np.array([0.4, 0.7, 0.6])), [1, 1, 1])
    material = S.uniforms_material(True, False, False, 1.0, 0.6, [1, 1, 1, 1])
    tex = S.TextureSpec("u_albedoMap", A.TextureDesc(64, 64, A.TextureType_2D, A.TextureFormat_RGBA8,
                                                     A.TextureUsage_Sampler | A.TextureUsage_UploadData, True, False),
                        A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR, A.Filter_LINEAR, A.Wrap_REPEAT, A.Wrap_REPEAT,
                                      A.Wrap_REPEAT), layers=[S.checkerboard(64, 8, 11)])
    st = A.RenderStates(blend=False, depthTest=True, depthMask=mask, depthFunc=func, cullFace=False)
    draws = []
    for t in ([-0.45, 0.0, 0.0], [0.4, 0.15, -0.35], [0.0, -0.25, 0.45]):
        M = np.eye(4)
        M[:3, 3] = t
        blocks = {"UniformsModel": S.uniforms_model(M, S.mm4(VP, M), None, False), "UniformsScene": scene_block,
                  "UniformsMaterial": material}
        draws.append(S.DrawSpec(vert, 64, idx, A.Shading_BlinnPhongDir, ("ALBEDO_MAP",), st, blocks, [tex]))
    clear = A.ClearStates(True, True, (0.05, 0.05, 0.08, 1.0), clear_depth)
    return S.Scene("spheres", [S.PassSpec(w, h, samples, clear, draws)])


@pytest.mark.parametrize("samples", [1, 4])
@pytest.mark.parametrize("mask", [True, False])
@pytest.mark.parametrize("func", range(8))
def test_deferred_depth_functions_equal_fused(func, mask, samples, cuda_lib):
    """The coverage kernel evaluates a pixel's fragments as a scan for LESS / LEQUAL / GREATER /
    GEQUAL with depth writes (and for any function without them) and in order on the pixel's lane
    for the rest; both give the fused kernel's images bit for bit."""
    far = func in (A.DepthFunc_LESS, A.DepthFunc_LEQUAL, A.DepthFunc_EQUAL)
    scene = _spheres_scene(samples, func, mask, 1.0 if far else 0.0 if func != A.DepthFunc_NOTEQUAL else 0.5)
    a = _render_mode(cuda_lib, scene, True)
    b = _render_mode(cuda_lib, scene, False)
    for k in a:
        x, y = a[k], b[k]
        if x.dtype == np.float32:
            x, y = x.view(np.uint32), y.view(np.uint32)
        assert np.array_equal(x, y), k


@pytest.mark.parametrize("func", [A.DepthFunc_LESS, A.DepthFunc_LEQUAL, A.DepthFunc_GREATER, A.DepthFunc_GEQUAL])
def test_deferred_depth_functions_match_oracle(func, cuda_lib, oracle_lib):
    scene = _spheres_scene(4, func, True, 1.0 if func in (A.DepthFunc_LESS, A.DepthFunc_LEQUAL) else 0.0)
    gpu, _ = render(cuda_lib, scene)
    cpu, _ = render(oracle_lib, scene)
    assert_outputs_match(gpu, cpu, f"spheres depth func {func}")


def test_deferred_early_z_off_equals_fused(cuda_lib):
    scene = _spheres_scene(4, A.DepthFunc_LEQUAL, True, 1.0)
    outs = []
    for deferred in (True, False):
        r = A.Renderer(cuda_lib, 0)
        r.setDeferredShading(deferred)
        r.setEnableEarlyZ(False)
        inst = S.SceneInstance(r, scene)
        inst.render()
        r.waitIdle()
        outs.append(inst.outputs())
        r.destroy()
    for k in outs[0]:
        assert np.array_equal(outs[0][k].view(np.uint8), outs[1][k].view(np.uint8)), k


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


def _render_tma(lib, scene, tma):
    r = A.Renderer(lib, 0)
    r.setTmaStore(tma)
    inst = S.SceneInstance(r, scene)
    inst.render()
    r.waitIdle()
    out = [inst.outputs(i) for i in range(len(scene.passes))]
    r.destroy()
    return out


TMA_SCENES = {
    "pbr_msaa4_320x180": lambda: S.config_pbr(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64,
                                              irradiance=8),
    "blinn_1x_300x200": lambda: S.config_plain_small(width=300, height=200, lon=48, lat=24, tex=64),
    # rows of 257 pixels are not a multiple of 16 bytes: per-thread stores stay in use
    "soup_1x_257x131": lambda: S.config_geometry_stress(n_tris=4000, width=257, height=131, samples=1),
    "soup_msaa4_250x150": lambda: S.config_geometry_stress(n_tris=6000, width=250, height=150, samples=4),
}


@pytest.mark.parametrize("name", sorted(TMA_SCENES))
def test_tma_tile_write_back_equals_per_thread_stores(name, cuda_lib, oracle_lib):
    """Whole tiles written back from shared memory by TMA bulk tensor stores (colour, resolved and
    depth; edge tiles clipped by the copy) give the images of per-thread stores, and the oracle's."""
    scene = TMA_SCENES[name]()
    a = _render_tma(cuda_lib, scene, True)
    b = _render_tma(cuda_lib, scene, False)
    for pa, pb in zip(a, b):
        for k in pb:
            assert np.array_equal(pa[k].view(np.uint8), pb[k].view(np.uint8)), k
    assert_outputs_match(a, render(oracle_lib, scene)[0], name, exact_color=name.startswith("soup"))


def _render_tile(lib, scene, tile):
    r = A.Renderer(lib, 0)
    r.setTileSize(tile)
    inst = S.SceneInstance(r, scene)
    inst.render()
    r.waitIdle()
    out = [inst.outputs(i) for i in range(len(scene.passes))]
    r.destroy()
    return out


TILE_SCENES = {
    "pbr_msaa4": lambda: S.config_pbr(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=8),
    "blinn_1x_odd": lambda: S.config_plain_small(width=301, height=203, lon=48, lat=24, tex=64),
    # dense enough that the heaviest tiles are split over four CTAs
    "dense_pbr_msaa4": lambda: S.config_pbr(width=160, height=96, lon=512, lat=256, tex=64, prefilter=32,
                                            irradiance=8),
    "soup_msaa4_two_passes": lambda: S.config_geometry_stress(n_tris=20000, width=250, height=150, samples=4),
}


@pytest.mark.parametrize("name", sorted(TILE_SCENES))
def test_16x8_tiles_equal_16x16_tiles(name, cuda_lib, oracle_lib):
    """The deferred raster on 16x8 tiles (4 warps per CTA) gives the images of 16x16 tiles (8 warps)
    and the oracle's: a pixel still belongs to one warp, whose list keeps the primitive order."""
    scene = TILE_SCENES[name]()
    a = _render_tile(cuda_lib, scene, 8)
    b = _render_tile(cuda_lib, scene, 16)
    for pa, pb in zip(a, b):
        for k in pb:
            assert np.array_equal(pa[k].view(np.uint8), pb[k].view(np.uint8)), k
    assert_outputs_match(a, render(oracle_lib, scene)[0], name, exact_color=name.startswith("soup"))


def test_tile_size_rejects_other_shapes(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    with pytest.raises(A.SoftGLError):
        r.setTileSize(32)
    r.destroy()
