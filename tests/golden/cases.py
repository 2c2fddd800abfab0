"""Scenes pinned by golden fixtures: each builder is deterministic (see softglrender_gb300.scenes)."""
import numpy as np

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S


def soup(n, w, h, samples, states_list, seed=7, clear_depth=1.0, reverse=False, median_px=60.0):
    eye = np.array([0.2, 0.1, 1.8])
    P = S.perspective(np.deg2rad(70.0), w / h, 0.3, reverse, far=3.0)
    V = S.look_at(eye, [0, 0, 0], [0, 1, 0])
    VP = S.mm4(P, V)
    rows, idx, _ = S.triangle_soup(n, seed, VP, w, h, median_px=median_px)
    blocks = {"UniformsModel": S.uniforms_model(np.eye(4), VP, None, reverse),
              "UniformsMaterial": S.uniforms_material(False, False, False, 1.0, 0.0, [1, 1, 1, 1])}
    draws = []
    per = n // len(states_list)
    for i, st in enumerate(states_list):
        r = rows[3 * per * i:3 * per * (i + 1)]
        draws.append(S.DrawSpec(r, 32, np.arange(len(r), dtype=np.int32), A.Shading_VertexColor, (), st, blocks))
    clear = A.ClearStates(True, True, (0.1, 0.2, 0.3, 0.4), clear_depth)
    return S.Scene("soup", [S.PassSpec(w, h, samples, clear, draws)])


def _blend(src, dst, fn):
    bp = A.BlendParameters()
    bp.SetBlendFactor(src, dst)
    bp.SetBlendFunc(fn)
    return A.RenderStates(blend=True, blendParams=bp, depthTest=True, depthMask=False)


def _filters(filt, wrap):
    sc = S.config_plain_small(width=200, height=150, lon=32, lat=16, tex=64, filter_min=filt)
    ts = sc.passes[0].draws[0].textures[0]
    ts.sampler = A.SamplerDesc(filt, A.Filter_LINEAR, wrap, wrap, wrap, A.Border_WHITE)
    sc.passes[0].draws[0].vertexes[:, 4:6] = sc.passes[0].draws[0].vertexes[:, 4:6] * 2.5 - 0.7
    return sc


def _point_light_blinn():
    sc = S.config_plain_small(width=240, height=180)
    d = sc.passes[0].draws[0]
    d.shading = A.Shading_BlinnPhong
    d.blocks["UniformsScene"] = S.uniforms_scene([0.1, 0.1, 0.1], [0, 0, 3.0], [1.5, 1.5, 2.0], [1.0, 0.9, 0.8])
    return sc


def _base_color():
    sc = S.config_plain_small(width=160, height=120)
    d = sc.passes[0].draws[0]
    d.shading = A.Shading_BaseColor
    d.defines = ()
    d.textures = []
    d.blocks = {"UniformsModel": d.blocks["UniformsModel"],
                "UniformsMaterial": S.uniforms_material(False, False, False, 1.0, 0.0, [0.25, 0.5, 0.75, 1.0])}
    return sc


CASES = {
    "plain_small_320": lambda: S.config_plain_small(width=320, height=240),
    "plain_small_1024": lambda: S.config_plain_small(),
    "plain_point_light": _point_light_blinn,
    "base_color": _base_color,
    "geometry_stress_20k": lambda: S.config_geometry_stress(n_tris=20000, width=320, height=180),
    "pbr_small": lambda: S.config_pbr(width=320, height=180, lon=96, lat=48, tex=128, prefilter=64, irradiance=16),
    "soup_depth_equal": lambda: soup(3000, 96, 64, 4, [A.RenderStates(depthTest=True, depthFunc=A.DepthFunc_EQUAL)] * 2,
                                     clear_depth=0.5),
    "soup_blend_sub": lambda: soup(4000, 128, 96, 4, [A.RenderStates(depthTest=True), _blend(2, 6, 1)]),
    "soup_17x13": lambda: soup(2000, 17, 13, 4, [A.RenderStates(depthTest=True)]),
    "filter_nearest_mirror": lambda: _filters(A.Filter_NEAREST_MIPMAP_LINEAR, A.Wrap_MIRRORED_REPEAT),
    "filter_trilinear_border": lambda: _filters(A.Filter_LINEAR_MIPMAP_LINEAR, A.Wrap_CLAMP_TO_BORDER),
}
