"""Texture files and the IBL cache (TextureSoft::storeToFile / loadFromFile, TextureSoft.h:166-215;
IBLGenerator::loadFromCache / storeToCache, Environment.cpp:197-239): every layer, every level, the
raw texels in buffer-layout order. The restatement writes the bytes the unmodified reference writes
(Linear build; the Tiled / Morton builds at every texel that is not layout padding), reads files the
reference wrote, and the GPU reads and writes the same files."""
import hashlib
import os

import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S
from softglrender_gb300.ibl import IBLGenerator, cache_key, equirect_sky

from golden.cases import soup
from helpers import render


# ---- a Python restatement of the layouts (Buffer::convertIndex, Buffer.h:31-33, 151-157, 193-202)
def _spread5(v):
    r = np.zeros_like(v)
    for b in range(5):
        r |= ((v >> b) & 1) << (2 * b)
    return r


def _storage(layout, w, h):
    """(storage texel count, storage index of every (y, x))."""
    y, x = np.mgrid[0:h, 0:w]
    if layout == A.Layout_Tiled:
        tw = (w + 3) // 4
        return tw * 4 * ((h + 3) // 4) * 4, (((y >> 2) * tw + (x >> 2)) << 4) + ((y & 3) << 2) + (x & 3)
    if layout == A.Layout_Morton:
        tw = (w + 31) // 32
        return tw * 32 * ((h + 31) // 32) * 32, (((y >> 5) * tw + (x >> 5)) << 10) + (_spread5(x & 31) | (_spread5(y & 31) << 1))
    return w * h, y * w + x


def _levels(w, h, mips):
    n = int(np.floor(np.log2(max(w, h)))) + 1 if mips else 1
    return [(max(1, w >> l), max(1, h >> l)) for l in range(n)]


def parse(raw: bytes, w, h, layers, mips, layout, samples=1):
    """The file as [layer][level] linear arrays of uint32 (x samples); asserts the exact size."""
    words = np.frombuffer(raw, np.uint32)
    out, o = [], 0
    for _ in range(layers):
        lv = []
        for (lw, lh) in _levels(w, h, mips):
            n, idx = _storage(layout, lw, lh)
            block = words[o:o + n * samples].reshape(n, samples)
            lv.append(block[idx])
            o += n * samples
        out.append(lv)
    assert o == len(words), (o, len(words))
    return out


def _rng_image(w, h, seed):
    return np.random.default_rng(seed).integers(0, 256, (h, w, 4), dtype=np.uint8)


def _textures(r, layout):
    """(name, texture, mips, layers) for a mip-mapped odd-sized 2D RGBA8, a float cube, an MSAA colour
    attachment after a draw and its MSAA depth attachment."""
    out = []
    d = A.TextureDesc(37, 23, A.TextureType_2D, A.TextureFormat_RGBA8, A.TextureUsage_Sampler | A.TextureUsage_UploadData,
                      True, False)
    d.layout = layout
    t = r.createTexture(d)
    t.setImageData([_rng_image(37, 23, 1)])
    out.append(("rgba_mips", t, True, 1))
    d = A.TextureDesc(12, 12, A.TextureType_CUBE, A.TextureFormat_FLOAT32, A.TextureUsage_Sampler, False, False)
    d.layout = layout
    t = r.createTexture(d)
    t.setImageData([np.random.default_rng(2 + f).random((12, 12), dtype=np.float32) for f in range(6)])
    out.append(("float_cube", t, False, 6))
    return out


@pytest.mark.parametrize("variant,layout", [("", A.Layout_Linear), ("tiled", A.Layout_Tiled),
                                            ("morton", A.Layout_Morton)])
def test_store_equals_reference(variant, layout, tmp_path, oracle_lib):
    import oracle
    ref = oracle.reference(variant)
    if ref is None:
        pytest.skip("reference checker not buildable here")
    files = {}
    for tag, lib in (("oracle", oracle_lib), ("ref", ref)):
        r = A.Renderer(lib, 0)
        for name, t, mips, layers in _textures(r, layout):
            p = str(tmp_path / f"{tag}_{name}.tex")
            t.storeToFile(p)
            files.setdefault(name, {})[tag] = (open(p, "rb").read(), t, mips, layers)
        r.destroy()
    for name, v in files.items():
        (a, ta, mips, layers), (b, _, _, _) = v["oracle"], v["ref"]
        assert len(a) == len(b), name
        if layout == A.Layout_Linear:
            assert a == b, name
        else:   # the reference leaves layout padding uninitialised: compare the texels
            pa = parse(a, ta.width, ta.height, layers, mips, layout)
            pb = parse(b, ta.width, ta.height, layers, mips, layout)
            for la, lb in zip(pa, pb):
                for x, y in zip(la, lb):
                    assert np.array_equal(x, y), name


def test_rendered_attachments_equal_reference(tmp_path, oracle_lib, reference_lib):
    """MSAA colour and depth attachments after a draw (4 samples per texel)."""
    scene = soup(300, 40, 24, 4, [A.RenderStates(depthTest=True, depthMask=True)])
    data = {}
    for tag, lib in (("oracle", oracle_lib), ("ref", reference_lib)):
        r = A.Renderer(lib, 0)
        inst = S.SceneInstance(r, scene)
        inst.render()
        r.waitIdle()
        for k, t in (("color", inst.color_tex[0]), ("depth", inst.depth_tex[0])):
            p = str(tmp_path / f"{tag}_{k}.tex")
            t.storeToFile(p)
            data[(tag, k)] = open(p, "rb").read()
        r.destroy()
    for k in ("color", "depth"):
        assert data[("oracle", k)] == data[("ref", k)], k
        assert len(data[("oracle", k)]) == 40 * 24 * 4 * 4


def test_load_reference_file(tmp_path, oracle_lib, reference_lib):
    """A file the reference wrote loads into the restatement; a short file or a missing one fails and
    leaves the texture as it was."""
    r_ref, r_or = A.Renderer(reference_lib, 0), A.Renderer(oracle_lib, 0)
    (_, src, _, _) = _textures(r_ref, A.Layout_Linear)[0]
    p = str(tmp_path / "ref.tex")
    src.storeToFile(p)
    d = A.TextureDesc(37, 23, A.TextureType_2D, A.TextureFormat_RGBA8, A.TextureUsage_Sampler, True, False)
    dst = r_or.createTexture(d)
    dst.initImageData()
    assert dst.loadFromFile(p)
    for lv in range(len(_levels(37, 23, True))):
        assert np.array_equal(dst.readImage(0, lv), src.readImage(0, lv)), lv
    before = dst.readImage(0, 0)
    short = str(tmp_path / "short.tex")
    open(short, "wb").write(open(p, "rb").read()[:100])
    assert not dst.loadFromFile(short)
    assert not dst.loadFromFile(str(tmp_path / "missing.tex"))
    assert np.array_equal(dst.readImage(0, 0), before)
    r_ref.destroy()
    r_or.destroy()


def _ibl(lib, cache_dir, env=32, irr=8, pre=16):
    r = A.Renderer(lib, 0)
    g = IBLGenerator(r, cache_dir)
    eq = r.createTexture(A.TextureDesc(64, 32, A.TextureType_2D, A.TextureFormat_RGBA8,
                                       A.TextureUsage_Sampler | A.TextureUsage_UploadData, False, False))
    eq.tag = "sky.hdr"
    eq.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE,
                                    A.Wrap_CLAMP_TO_EDGE))
    eq.setImageData([equirect_sky(64, 32, 7)])
    cube = g.convert_equirectangular(eq, env)
    ir = g.irradiance(cube, irr)
    pf = g.prefilter(cube, pre, 3)
    r.waitIdle()
    out = {"cube": np.stack([cube.readImage(f) for f in range(6)]),
           "irradiance": np.stack([ir.readImage(f) for f in range(6)]),
           "prefilter": [np.stack([pf.readImage(f, lv) for f in range(6)]) for lv in range(5)],
           "hits": g.cache_hits, "tags": (cube.tag, ir.tag, pf.tag)}
    r.destroy()
    return out


def test_ibl_cache(tmp_path, oracle_lib, reference_lib):
    """The first run draws and stores the three maps under md5(tag + width + height).tex; a second
    run loads all three and draws nothing; the cache the reference wrote serves the restatement."""
    cache = str(tmp_path / "IBL")
    first = _ibl(reference_lib, cache)
    assert first["hits"] == 0
    assert first["tags"] == ("sky.hdr.cubeMap", "sky.hdr.cubeMap.irradianceMap", "sky.hdr.cubeMap.prefilterMap")
    names = sorted(os.listdir(cache))
    want = sorted(hashlib.md5((t + str(s) + str(s)).encode()).hexdigest() + ".tex"
                  for t, s in zip(first["tags"], (32, 8, 16)))
    assert names == want
    again = _ibl(oracle_lib, cache)
    assert again["hits"] == 3
    for k in ("cube", "irradiance"):
        assert np.array_equal(again[k], first[k]), k
    for lv in range(5):
        assert np.array_equal(again["prefilter"][lv], first["prefilter"][lv]), lv


# ---- GPU -----------------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("layout", [A.Layout_Linear, A.Layout_Tiled, A.Layout_Morton])
def test_gpu_store_load(layout, tmp_path, cuda_lib, oracle_lib):
    """The GPU's file of an uploaded texture equals the restatement's (layout padding is zero in
    both), and the GPU loads the restatement's file back to the same texels."""
    rg, ro = A.Renderer(cuda_lib, 0), A.Renderer(oracle_lib, 0)
    tg, to = _textures(rg, layout), _textures(ro, layout)
    for (name, a, mips, layers), (_, b, _, _) in zip(tg, to):
        pa, pb = str(tmp_path / f"g_{name}.tex"), str(tmp_path / f"o_{name}.tex")
        a.storeToFile(pa)
        b.storeToFile(pb)
        ga, ob = open(pa, "rb").read(), open(pb, "rb").read()
        assert ga == ob, name
        d = A.TextureDesc(a.width, a.height, a.type, a.format, A.TextureUsage_Sampler, a.useMipmaps, False)
        d.layout = layout
        c = rg.createTexture(d)
        c.initImageData()
        assert c.loadFromFile(pb)
        for layer in range(layers):
            for lv in range(len(_levels(a.width, a.height, mips))):
                assert np.array_equal(c.readImage(layer, lv), b.readImage(layer, lv)), (name, layer, lv)
    rg.destroy()
    ro.destroy()


@pytest.mark.gpu
def test_gpu_ibl_cache(tmp_path, cuda_lib, oracle_lib):
    """Maps the GPU generated and cached load back bit for bit; the restatement's cache serves the
    GPU too."""
    cache_g, cache_o = str(tmp_path / "g"), str(tmp_path / "o")
    first = _ibl(cuda_lib, cache_g)
    again = _ibl(cuda_lib, cache_g)
    assert first["hits"] == 0 and again["hits"] == 3
    assert np.array_equal(again["cube"], first["cube"]) and np.array_equal(again["irradiance"], first["irradiance"])
    ref = _ibl(oracle_lib, cache_o)
    served = _ibl(cuda_lib, cache_o)
    assert served["hits"] == 3
    assert np.array_equal(served["cube"], ref["cube"]) and np.array_equal(served["irradiance"], ref["irradiance"])
    for lv in range(5):
        assert np.array_equal(served["prefilter"][lv], ref["prefilter"][lv]), lv
