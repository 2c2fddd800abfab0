"""Multi-scene draws (sglc_draw_scenes) on edge cases: frames of sizes that are not tile multiples,
4x MSAA, clipped triangles, a scene without triangles, one scene alone, and the errors the call
returns. Each scene's images must equal its own render pass (bit for bit, GPU and oracle alike) and,
on the GPU, the oracle's (vertex colour: exact colour)."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

# (triangles, width, height) of each scene: the vertex-colour soup with clipping, opaque draw
SIZES = [(400, 37, 23), (1500, 96, 64), (0, 20, 12), (60, 16, 16), (800, 130, 70)]


def _scenes():
    out = []
    for k, (n, w, h) in enumerate(SIZES):
        sc = S.config_geometry_stress(seed=2100 + k, n_tris=max(n, 1), width=w, height=h, samples=4)
        d = sc.passes[0].draws[0]
        if n == 0:   # a scene without triangles: an empty vertex array
            d = S.DrawSpec(np.zeros((0, 8), np.float32), d.stride, np.zeros(0, np.int32), d.shading, d.defines,
                           d.states, d.blocks)
        out.append((sc.passes[0], d))
    return out


def _setup(r, scenes):
    prog = r.createShaderProgram()
    prog.SetShaders(A.Shading_VertexColor)
    states = r.createPipelineStates(scenes[0][1].states)
    items = []
    for ps, d in scenes:
        ct = r.createTexture(A.TextureDesc(ps.width, ps.height, A.TextureType_2D, A.TextureFormat_RGBA8,
                                           A.TextureUsage_AttachmentColor, False, True))
        ct.initImageData()
        dt = r.createTexture(A.TextureDesc(ps.width, ps.height, A.TextureType_2D, A.TextureFormat_FLOAT32,
                                           A.TextureUsage_AttachmentDepth, False, True))
        dt.initImageData()
        fb = r.createFrameBuffer(True)
        fb.setColorAttachment(ct, 0)
        fb.setDepthAttachment(dt)
        vao = r.createVertexArrayObject(d.vertexes, d.stride, d.indices)
        res = r.createShaderResources()
        for name, data in d.blocks.items():
            ub = r.createUniformBlock(name, len(data))
            ub.setData(data)
            res.setBlock(S._BLOCK_KEYS[name], ub)
        items.append({"w": ps.width, "h": ps.height, "fb": fb, "vao": vao, "res": res, "ct": ct, "dt": dt,
                      "clear": ps.clear})
    return prog, states, items


def _read(items):
    return [{"color": it["ct"].readImage(), "resolved": it["ct"].readImage(resolved=True),
             "depth": it["dt"].readImage()} for it in items]


def _per_scene(r, prog, states, items):
    for it in items:
        r.beginRenderPass(it["fb"], it["clear"])
        r.setViewPort(0, 0, it["w"], it["h"])
        r.setVertexArrayObject(it["vao"])
        r.setShaderProgram(prog)
        r.setShaderResources(it["res"])
        r.setPipelineStates(states)
        r.draw()
        r.endRenderPass()
    r.waitIdle()
    return _read(items)


def _multi(r, prog, states, items, subset=None):
    its = items if subset is None else [items[k] for k in subset]
    r.setShaderProgram(prog)
    r.setPipelineStates(states)
    r.drawScenes([it["vao"] for it in its], [it["fb"] for it in its], [it["res"] for it in its], its[0]["clear"])
    r.waitIdle()
    return _read(items)


def _both(lib):
    r = A.Renderer(lib, 0)
    prog, states, items = _setup(r, _scenes())
    single = _per_scene(r, prog, states, items)
    multi = _multi(r, prog, states, items)
    r.destroy()
    return single, multi


def _same(a, b, what):
    for s in range(len(a)):
        for k in a[s]:
            assert np.array_equal(a[s][k].view(np.uint8), b[s][k].view(np.uint8)), (what, s, k)


def test_multi_scene_edge_cases_on_oracle(oracle_lib):
    single, multi = _both(oracle_lib)
    _same(single, multi, "oracle")
    assert any(np.any(o["depth"] != 0.0) for o in multi)   # something was drawn (reversed Z clears to 0)


@pytest.mark.gpu
def test_multi_scene_edge_cases_on_gpu(cuda_lib, oracle_lib):
    single, multi = _both(cuda_lib)
    _same(single, multi, "cuda")
    _, ref = _both(oracle_lib)
    _same(multi, ref, "cuda vs oracle")   # vertex colour: colour and depth exact


@pytest.mark.gpu
def test_multi_scene_one_scene_equals_draw(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    prog, states, items = _setup(r, _scenes())
    single = _per_scene(r, prog, states, items)
    for k in range(len(items)):
        got = _multi(r, prog, states, items, subset=[k])
        _same([single[k]], [got[k]], f"scene {k} alone")
    r.destroy()


@pytest.mark.gpu
def test_multi_scene_errors(cuda_lib):
    r = A.Renderer(cuda_lib, 0)
    prog, states, items = _setup(r, _scenes())
    r.setShaderProgram(prog)
    r.setPipelineStates(states)
    # a vertex array of another stride
    other = r.createVertexArrayObject(np.zeros((3, 16), np.float32), 64, np.arange(3, dtype=np.int32))
    with pytest.raises(A.SoftGLError) as e:
        r.drawScenes([items[0]["vao"], other], [items[0]["fb"], items[1]["fb"]], [items[0]["res"], items[1]["res"]])
    assert e.value.status == A.SGLC_ERR_INVALID_VALUE and "stride" in str(e.value)
    # a scene that binds another texture than scene 0 for the same sampler
    tdesc = A.TextureDesc(8, 8, A.TextureType_2D, A.TextureFormat_RGBA8, A.TextureUsage_Sampler, False, False)
    t0, t1 = r.createTexture(tdesc), r.createTexture(tdesc)
    for t in (t0, t1):
        t.setImageData([np.zeros((8, 8, 4), np.uint8)])
    prog2 = r.createShaderProgram()   # a shader that samples u_albedoMap
    prog2.addDefines(("ALBEDO_MAP",))
    prog2.SetShaders(A.Shading_BlinnPhongDir)
    res = []
    for t in (t0, t1):
        us = r.createUniformSampler("u_albedoMap", tdesc)
        us.setTexture(t)
        rr = r.createShaderResources()
        rr.setSampler(0, us)
        res.append(rr)
    r.setShaderProgram(prog2)
    with pytest.raises(A.SoftGLError) as e:
        r.drawScenes([items[0]["vao"], items[1]["vao"]], [items[0]["fb"], items[1]["fb"]], res)
    assert e.value.status == A.SGLC_ERR_INVALID_VALUE and "scene 0" in str(e.value)
    # an invalid vertex array handle is an error (not the silent no-op of a draw without one)
    with pytest.raises(A.SoftGLError) as e:
        r.drawScenes([items[0]["vao"], A.VertexArrayObject(r, 99999)], [items[0]["fb"], items[1]["fb"]],
                     [items[0]["res"], items[1]["res"]])
    assert e.value.status == A.SGLC_ERR_INVALID_HANDLE
    # the context still draws correctly afterwards
    r.setShaderProgram(prog)
    single = _per_scene(r, prog, states, items)
    multi = _multi(r, prog, states, items)
    _same(single, multi, "after errors")
    r.destroy()
