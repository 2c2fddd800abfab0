"""Batched views with a shadow pass: one displaced sphere rendered from many seeded orbit cameras,
each view with its own RGBA8 colour and FP32 depth attachments, after a depth-only shadow-map pass
from a directional light whose 3x3 PCF lookup (BlinnPhongSoft.h:165-189) feeds the fragment shader.

`BatchedViews.render()` issues the shadow pass and then all views in one `drawViews` call (one
pipeline pass over every (view, triangle) and (view, tile) work item on the GPU);
`render_looped()` issues the same frame the way the reference viewer would, one render pass per
view (Viewer::drawShadowMap then one Viewer::drawFrame per camera, Viewer.cpp:100-168), which is
what the CPU oracle and the reference run. Both must give identical images.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import api as A
from . import scenes as S


@dataclass
class BatchConfig:
    views: int = 256
    size: int = 256
    shadow: int = 2048
    lon: int = 224                 # 2 * lon * (lat - 1) triangles: 49,728 at 224 x 112
    lat: int = 112
    tex: int = 512
    seed: int = 4000


def _bias() -> np.ndarray:
    """Viewer::updateUniformModel's bias matrix (Viewer.cpp:694-697), NDC xy -> [0, 1]."""
    B = np.eye(4)
    B[0, 0] = B[1, 1] = 0.5
    B[0, 3] = B[1, 3] = 0.5
    return B


def orbit_camera(seed: int, v: int):
    """Seeded orbit camera v: yaw uniform [0, 360), pitch uniform [-60, 60] degrees, distance [2, 5]."""
    yaw = 2.0 * np.pi * S.hash_u01(seed, 60, v)
    pitch = np.deg2rad(-60.0 + 120.0 * S.hash_u01(seed, 61, v))
    dist = 2.0 + 3.0 * S.hash_u01(seed, 62, v)
    eye = np.array([dist * S.det_cos(pitch) * S.det_sin(yaw), dist * S.det_sin(pitch),
                    dist * S.det_cos(pitch) * S.det_cos(yaw)])
    return eye


class BatchedViews:
    """Resources of the batched-views frame on one renderer (product, oracle or reference library)."""

    def __init__(self, r: A.Renderer, cfg: Optional[BatchConfig] = None, layout: int = A.Layout_Linear):
        self.r = r
        self.cfg = cfg = cfg or BatchConfig()
        vert, idx = S.uv_sphere(cfg.lon, cfg.lat, 1.0, displace_seed=cfg.seed, amplitude=0.1)
        self.triangles = len(idx) // 3
        self.vao = r.createVertexArrayObject(vert, 64, idx)
        # directional light, orthographic shadow camera covering the sphere
        ld = S.normalize(np.array([0.4, 0.8, 0.45]))
        self.light_dir = ld
        Vl = S.look_at(ld * 4.0, [0, 0, 0], [0, 1, 0])
        Pl = S.ortho(1.3, 1.3, 2.0, 6.0)
        light_vp = S.mm4(Pl, Vl)
        shadow_mvp = S.mm4(_bias(), light_vp)
        # shadow pass: depth-only framebuffer (the fragment shader does not run)
        sd = A.TextureDesc(cfg.shadow, cfg.shadow, A.TextureType_2D, A.TextureFormat_FLOAT32,
                           A.TextureUsage_Sampler | A.TextureUsage_AttachmentDepth, False, False)
        self.shadow_tex = r.createTexture(sd)
        self.shadow_tex.setSamplerDesc(A.SamplerDesc(A.Filter_NEAREST, A.Filter_NEAREST, A.Wrap_CLAMP_TO_BORDER,
                                                     A.Wrap_CLAMP_TO_BORDER, A.Wrap_CLAMP_TO_BORDER, A.Border_WHITE))
        self.shadow_tex.initImageData()
        self.shadow_fbo = r.createFrameBuffer(offscreen=True)
        self.shadow_fbo.setDepthAttachment(self.shadow_tex)
        self.shadow_prog = r.createShaderProgram()
        self.shadow_prog.SetShaders(A.Shading_BaseColor)
        self.shadow_res = r.createShaderResources()
        for name, data in {"UniformsModel": S.uniforms_model(np.eye(4), light_vp, None, False),
                           "UniformsMaterial": S.uniforms_material(False, False, False, 1.0, 0.0, [1, 1, 1, 1])}.items():
            ub = r.createUniformBlock(name, len(data))
            ub.setData(data)
            self.shadow_res.setBlock(S._BLOCK_KEYS[name], ub)
        self.states = r.createPipelineStates(A.RenderStates(depthTest=True, depthMask=True,
                                                            depthFunc=A.DepthFunc_LESS, cullFace=True))
        # view pass: Blinn-Phong (directional light, shininess 32) with the shadow map
        self.prog = r.createShaderProgram()
        self.prog.addDefines(("ALBEDO_MAP",))
        self.prog.SetShaders(A.Shading_BlinnPhongDir)
        td = A.TextureDesc(cfg.tex, cfg.tex, A.TextureType_2D, A.TextureFormat_RGBA8,
                           A.TextureUsage_Sampler | A.TextureUsage_UploadData, True, False)
        td.layout = layout
        self.albedo = r.createTexture(td)
        self.albedo.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR, A.Filter_LINEAR, A.Wrap_REPEAT,
                                                 A.Wrap_REPEAT, A.Wrap_REPEAT))
        self.albedo.setImageData([S.noise_texture(cfg.tex, cfg.seed + 10, "albedo")])
        us_alb = r.createUniformSampler("u_albedoMap", td)
        us_alb.setTexture(self.albedo)
        us_sh = r.createUniformSampler("u_shadowMap", sd)
        us_sh.setTexture(self.shadow_tex)
        P = S.perspective(np.pi / 3.0, 1.0, 0.05, False)
        material = S.uniforms_material(True, False, True, 1.0, 0.6, [1, 1, 1, 1])
        self.color, self.depth, self.fbos, self.res = [], [], [], []
        for v in range(cfg.views):
            eye = orbit_camera(cfg.seed, v)
            Vm = S.look_at(eye, [0, 0, 0], [0, 1, 0])
            blocks = {"UniformsModel": S.uniforms_model(np.eye(4), S.mm4(P, Vm), shadow_mvp, False),
                      "UniformsScene": S.uniforms_scene([0.15, 0.15, 0.15], eye, ld, [1.0, 1.0, 1.0]),
                      "UniformsMaterial": material}
            ct = r.createTexture(A.TextureDesc(cfg.size, cfg.size, A.TextureType_2D, A.TextureFormat_RGBA8,
                                               A.TextureUsage_AttachmentColor | A.TextureUsage_RendererOutput,
                                               False, False))
            ct.initImageData()
            dt = r.createTexture(A.TextureDesc(cfg.size, cfg.size, A.TextureType_2D, A.TextureFormat_FLOAT32,
                                               A.TextureUsage_AttachmentDepth, False, False))
            dt.initImageData()
            fbo = r.createFrameBuffer(offscreen=True)
            fbo.setColorAttachment(ct, 0)
            fbo.setDepthAttachment(dt)
            res = r.createShaderResources()
            for name, data in blocks.items():
                ub = r.createUniformBlock(name, len(data))
                ub.setData(data)
                res.setBlock(S._BLOCK_KEYS[name], ub)
            res.setSampler(0, us_alb)
            res.setSampler(1, us_sh)
            self.color.append(ct)
            self.depth.append(dt)
            self.fbos.append(fbo)
            self.res.append(res)
        self.clear = A.ClearStates(True, True, (0.05, 0.05, 0.08, 1.0), 1.0)

    def shadow_pass(self) -> None:
        r, cfg = self.r, self.cfg
        r.beginRenderPass(self.shadow_fbo, A.ClearStates(True, False, (0, 0, 0, 0), 1.0))
        r.setViewPort(0, 0, cfg.shadow, cfg.shadow)
        r.setVertexArrayObject(self.vao)
        r.setShaderProgram(self.shadow_prog)
        r.setShaderResources(self.shadow_res)
        r.setPipelineStates(self.states)
        r.draw()
        r.endRenderPass()

    def render(self) -> None:
        """Shadow pass, then every view in one batched draw."""
        r = self.r
        self.shadow_pass()
        r.setViewPort(0, 0, self.cfg.size, self.cfg.size)
        r.setVertexArrayObject(self.vao)
        r.setShaderProgram(self.prog)
        r.setPipelineStates(self.states)
        r.drawViews(self.fbos, self.res, self.clear)

    def render_looped(self, views: Optional[List[int]] = None) -> None:
        """Shadow pass, then one render pass per view (the reference viewer's sequence)."""
        r = self.r
        self.shadow_pass()
        for v in (range(self.cfg.views) if views is None else views):
            r.beginRenderPass(self.fbos[v], self.clear)
            r.setViewPort(0, 0, self.cfg.size, self.cfg.size)
            r.setVertexArrayObject(self.vao)
            r.setShaderProgram(self.prog)
            r.setShaderResources(self.res[v])
            r.setPipelineStates(self.states)
            r.draw()
            r.endRenderPass()

    def view_outputs(self, v: int):
        return {"color": self.color[v].readImage(), "depth": self.depth[v].readImage()}
