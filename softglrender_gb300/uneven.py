"""Uneven batch: many independent scenes of very different size rendered as one submission.

Each scene is a seeded displaced sphere whose triangle count is drawn log-uniformly from
[tri_min, tri_max] and whose square resolution is drawn from `resolutions`; even scenes use
directional Blinn-Phong without MSAA, odd scenes PBR+IBL with 4x MSAA: the material maps of the
1080p PBR scene under one of `pbr_materials` environments (material 0 is the 1080p scene's own IBL
maps, the others channel-rotated variants of them), optionally with the neural IBL shader bound per
material where it met its PSNR threshold (otherwise that material keeps the plain shader: the
fallback). `render()` issues the scenes one render pass each; `render_batched()` draws each class
of scenes (Blinn-Phong; PBR of one material) with one multi-scene draw, a single pipeline pass whose
raster stage takes the (scene, tile) work items of all its scenes from one heaviest-first queue. On
the GPU either sequence is captured once in a CUDA graph (softglrender_gb300/graph.py) and replayed
with one launch. `UnevenLanes` splits the scenes over several renderers
whose submissions run concurrently. Meshes with the same tessellation share their
displacement seed (the tessellation is rounded to a multiple of 16 longitude segments), which keeps
the set-up time of 64 scenes of up to 2M triangles within seconds.
"""
from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import api as A
from . import scenes as S


@dataclass
class UnevenConfig:
    scenes: int = 64
    tri_min: int = 1000
    tri_max: int = 2_000_000
    resolutions: Tuple[int, ...] = (128, 512, 1024, 2048)
    seed: int = 5000
    pbr_tex: int = 1024
    prefilter: int = 512
    irradiance: int = 32
    blinn_tex: int = 512
    pbr_materials: int = 2   # PBR materials (environments) the PBR scenes alternate between


# host-side scene assets, generated once per process and shared by every batch built from them
# (several renderers of one batch upload the same arrays; the arrays are never written)
@lru_cache(maxsize=None)
def _noise_texture(size: int, seed: int, kind: str) -> np.ndarray:
    return S.noise_texture(size, seed, kind)


@lru_cache(maxsize=None)
def _ibl_maps(seed: int, prefilter: int, irradiance: int, variant: int = 0):
    return S.ibl_maps(seed, prefilter, irradiance, variant=variant)


@lru_cache(maxsize=None)
def _checkerboard(size: int, seed: int) -> np.ndarray:
    return S.checkerboard(size, 8, seed)


@lru_cache(maxsize=None)
def _sphere(lon: int, lat: int, seed: int):
    return S.uv_sphere(lon, lat, 1.0, displace_seed=seed, amplitude=0.1)


def material_of(cfg: UnevenConfig, s: int) -> int:
    """PBR material of scene s (the odd scenes alternate between the materials)."""
    return (s // 2) % max(1, cfg.pbr_materials)


def scene_plan(cfg: UnevenConfig) -> List[Dict[str, int]]:
    """(kind, longitude segments, latitude segments, resolution, samples) of every scene."""
    plan = []
    for s in range(cfg.scenes):
        u = float(S.hash_u01(cfg.seed, 70, s))
        tris = float(np.exp(np.log(cfg.tri_min) + u * (np.log(cfg.tri_max) - np.log(cfg.tri_min))))
        lon = max(16, int(round(np.sqrt(tris) / 16.0)) * 16)   # 2 lon (lat - 1) ~ tris with lat = lon / 2
        lat = max(8, lon // 2)
        res = cfg.resolutions[int(S.hash_u01(cfg.seed, 71, s) * len(cfg.resolutions)) % len(cfg.resolutions)]
        pbr = s % 2 == 1
        plan.append({"pbr": int(pbr), "lon": lon, "lat": lat, "res": res, "samples": 4 if pbr else 1})
    return plan


class UnevenBatch:
    def __init__(self, r: A.Renderer, cfg: Optional[UnevenConfig] = None, only: Optional[List[int]] = None):
        """`only`: create just these scenes (the others are skipped by render())."""
        self.r = r
        self.cfg = cfg = cfg or UnevenConfig()
        self.plan = scene_plan(cfg)
        self.only = set(range(cfg.scenes)) if only is None else set(only)
        meshes: Dict[int, A.VertexArrayObject] = {}
        self.triangles = []
        # shared materials
        tdesc = A.TextureDesc(cfg.pbr_tex, cfg.pbr_tex, A.TextureType_2D, A.TextureFormat_RGBA8,
                              A.TextureUsage_Sampler | A.TextureUsage_UploadData, True, False)
        trilinear = A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR, A.Filter_LINEAR, A.Wrap_REPEAT, A.Wrap_REPEAT,
                                  A.Wrap_REPEAT)
        material_maps = []
        for k, (name, kind) in enumerate((("u_albedoMap", "albedo"), ("u_normalMap", "normal"),
                                          ("u_metalRoughnessMap", "metal_rough"))):
            t = r.createTexture(tdesc)
            t.setSamplerDesc(trilinear)
            t.setImageData([_noise_texture(cfg.pbr_tex, 3000 + 10 * (k + 1), kind)])
            us = r.createUniformSampler(name, tdesc)
            us.setTexture(t)
            material_maps.append(us)
        # PBR material m: the shared material maps under environment m (the 1080p PBR scene's IBL
        # maps, variant m: material 0 is that scene's own environment)
        self.pbr_samplers = []
        for m in range(max(1, cfg.pbr_materials)):
            pre, irr = _ibl_maps(3000, cfg.prefilter, cfg.irradiance, m)
            cdesc = A.TextureDesc(cfg.irradiance, cfg.irradiance, A.TextureType_CUBE, A.TextureFormat_RGBA8,
                                  A.TextureUsage_Sampler | A.TextureUsage_UploadData, False, False)
            t = r.createTexture(cdesc)
            t.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE,
                                           A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE))
            t.setImageData(irr)
            irr_us = r.createUniformSampler("u_irradianceMap", cdesc)
            irr_us.setTexture(t)
            pdesc = A.TextureDesc(cfg.prefilter, cfg.prefilter, A.TextureType_CUBE, A.TextureFormat_RGBA8,
                                  A.TextureUsage_Sampler, True, False)
            t = r.createTexture(pdesc)
            t.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE,
                                           A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE))
            t.initImageData()
            for lev, imgs in enumerate(pre):
                for layer, img in enumerate(imgs):
                    t.setLevelData(layer, lev, img)
            pre_us = r.createUniformSampler("u_prefilterMap", pdesc)
            pre_us.setTexture(t)
            self.pbr_samplers.append(material_maps + [irr_us, pre_us])
        bdesc = A.TextureDesc(cfg.blinn_tex, cfg.blinn_tex, A.TextureType_2D, A.TextureFormat_RGBA8,
                              A.TextureUsage_Sampler | A.TextureUsage_UploadData, True, False)
        bt = r.createTexture(bdesc)
        bt.setSamplerDesc(trilinear)
        bt.setImageData([_checkerboard(cfg.blinn_tex, cfg.seed)])
        blinn_sampler = r.createUniformSampler("u_albedoMap", bdesc)
        blinn_sampler.setTexture(bt)
        self.states = r.createPipelineStates(A.RenderStates(depthTest=True, depthMask=True,
                                                            depthFunc=A.DepthFunc_LESS, cullFace=True))
        self.items: Dict[int, dict] = {}
        for s, pl in enumerate(self.plan):
            if s not in self.only:
                self.triangles.append(2 * pl["lon"] * (pl["lat"] - 1))
                continue
            key = pl["lon"]
            if key not in meshes:
                vert, idx = _sphere(pl["lon"], pl["lat"], cfg.seed + key)
                meshes[key] = (r.createVertexArrayObject(vert, 64, idx), len(idx) // 3)
            vao, ntri = meshes[key]
            self.triangles.append(ntri)
            res = pl["res"]
            prog = r.createShaderProgram()
            resources = r.createShaderResources()
            if pl["pbr"]:
                prog.addDefines(("ALBEDO_MAP", "NORMAL_MAP", "METALROUGHNESS_MAP"))
                prog.SetShaders(A.Shading_PBR)
                blocks = S.pbr_view_blocks(cfg.seed + 1, s, res, res)
                for k, us in enumerate(self.pbr_samplers[material_of(cfg, s)]):
                    resources.setSampler(k, us)
            else:
                prog.addDefines(("ALBEDO_MAP",))
                prog.SetShaders(A.Shading_BlinnPhongDir)
                yaw = 2.0 * np.pi * S.hash_u01(cfg.seed, 72, s)
                eye = np.array([3.0 * S.det_sin(yaw), 0.8, 3.0 * S.det_cos(yaw)])
                Pm = S.perspective(np.pi / 3.0, 1.0, 0.05, False)
                Vm = S.look_at(eye, [0, 0, 0], [0, 1, 0])
                light = S.normalize(np.array([0.5, 0.7, 0.5]))
                blocks = {"UniformsModel": S.uniforms_model(np.eye(4), S.mm4(Pm, Vm), None, False),
                          "UniformsScene": S.uniforms_scene([0.15, 0.15, 0.15], eye, light, [1.0, 1.0, 1.0]),
                          "UniformsMaterial": S.uniforms_material(True, False, False, 1.0, 0.6, [1, 1, 1, 1])}
                resources.setSampler(0, blinn_sampler)
            for name, data in blocks.items():
                ub = r.createUniformBlock(name, len(data))
                ub.setData(data)
                resources.setBlock(S._BLOCK_KEYS[name], ub)
            ms = pl["samples"] > 1
            ct = r.createTexture(A.TextureDesc(res, res, A.TextureType_2D, A.TextureFormat_RGBA8,
                                               A.TextureUsage_AttachmentColor | A.TextureUsage_RendererOutput,
                                               False, ms))
            ct.initImageData()
            dt = r.createTexture(A.TextureDesc(res, res, A.TextureType_2D, A.TextureFormat_FLOAT32,
                                               A.TextureUsage_AttachmentDepth, False, ms))
            dt.initImageData()
            fbo = r.createFrameBuffer(offscreen=True)
            fbo.setColorAttachment(ct, 0)
            fbo.setDepthAttachment(dt)
            self.items[s] = {"vao": vao, "prog": prog, "res": resources, "fbo": fbo, "color": ct, "depth": dt,
                             "size": res, "pbr": bool(pl["pbr"]),
                             "material": material_of(cfg, s) if pl["pbr"] else -1}
        self.clear = A.ClearStates(True, True, (0.02, 0.02, 0.03, 1.0), 1.0)

    def pbr_programs(self, material: Optional[int] = None) -> List[A.ShaderProgram]:
        """Programs of the PBR scenes (of one material when given)."""
        return [it["prog"] for it in self.items.values() if it["pbr"] and material in (None, it["material"])]

    def render_scene(self, s: int) -> None:
        r, it = self.r, self.items[s]
        r.beginRenderPass(it["fbo"], self.clear)
        r.setViewPort(0, 0, it["size"], it["size"])
        r.setVertexArrayObject(it["vao"])
        r.setShaderProgram(it["prog"])
        r.setShaderResources(it["res"])
        r.setPipelineStates(self.states)
        r.draw()
        r.endRenderPass()

    def render(self, scenes: Optional[List[int]] = None) -> None:
        for s in (sorted(self.items) if scenes is None else scenes):
            self.render_scene(s)

    def classes(self) -> Dict[Tuple[int, int], List[int]]:
        """Scenes that share a program configuration, samplers and sample count: the Blinn-Phong
        scenes (key (0, -1)) and the PBR scenes of each material (key (1, m))."""
        out: Dict[Tuple[int, int], List[int]] = {}
        for s in sorted(self.items):
            it = self.items[s]
            out.setdefault((int(it["pbr"]), it["material"]), []).append(s)
        return out

    def render_batched(self) -> None:
        """The same frames as render(), each class of scenes in one multi-scene draw
        (Renderer.drawScenes): one pipeline pass, one launch per stage over all of its scenes'
        vertices, triangles and raster tiles. The class's first program stands for the class
        (its uniforms come from each scene's resources; a neural binding is per material)."""
        r = self.r
        for scenes in self.classes().values():
            its = [self.items[s] for s in scenes]
            r.setShaderProgram(its[0]["prog"])
            r.setPipelineStates(self.states)
            r.drawScenes([it["vao"] for it in its], [it["fbo"] for it in its], [it["res"] for it in its],
                         self.clear)

    def outputs(self, s: int):
        it = self.items[s]
        out = {"color": it["color"].readImage(), "depth": it["depth"].readImage()}
        if it["pbr"]:
            out["resolved"] = it["color"].readImage(resolved=True)
        return out


def assign_lanes(cost: Sequence[float], lanes: int) -> List[List[int]]:
    """Scenes to `lanes` groups: longest first, each to the group with the least cost so far."""
    groups: List[List[int]] = [[] for _ in range(lanes)]
    load = [0.0] * lanes
    for s in sorted(range(len(cost)), key=lambda i: (-cost[i], i)):
        k = min(range(lanes), key=lambda j: (load[j], j))
        groups[k].append(s)
        load[k] += cost[s]
    return [sorted(g) for g in groups]


class UnevenLanes:
    """The uneven batch over several renderers ("lanes"): each lane has its own stream, working
    memory and copy of the shared materials, and renders its share of the scenes as one
    submission (CUDA graph or eager, picked by the autotuner). The lanes' submissions are
    independent, so the GPU runs them concurrently: scenes too small to fill the GPU (a 128^2
    target has 64 raster tiles for 152 SMs) overlap instead of running one after another.
    Every scene's images equal the single-renderer batch's (a scene is drawn the same way on any
    renderer)."""

    def __init__(self, renderers: Sequence[A.Renderer], cfg: UnevenConfig, cost: Sequence[float],
                 batched: bool = False):
        """`batched`: each lane draws its scenes with one multi-scene draw per class
        (UnevenBatch.render_batched) instead of one render pass per scene."""
        self.renderers = list(renderers)
        self.cfg = cfg
        self.batched = batched
        self.groups = assign_lanes(cost, len(self.renderers))
        self.batches = [UnevenBatch(r, cfg, only=g) for r, g in zip(self.renderers, self.groups)]
        self.tuned = []

    def tune(self, reps: int = 3) -> None:
        """Capacities, tile order and graph-or-eager per lane (softglrender_gb300/autotune.py)."""
        from .autotune import autotune
        self.release()
        for r, b in zip(self.renderers, self.batches):
            r.setCapacity(None)
            self.tuned.append(autotune(r, b.render_batched if self.batched else b.render, reps=reps))

    def launch(self) -> None:
        """Enqueue every lane's submission (each on its own renderer's stream)."""
        for t in self.tuned:
            t.run()

    def wait(self) -> None:
        for r in self.renderers:
            r.waitIdle()

    def lane_of(self, s: int) -> int:
        return next(k for k, g in enumerate(self.groups) if s in g)

    def outputs(self, s: int):
        return self.batches[self.lane_of(s)].outputs(s)

    def release(self) -> None:
        for t in self.tuned:
            t.destroy()
        self.tuned = []
