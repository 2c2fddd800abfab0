"""Image-based-lighting precompute on the renderer: equirectangular map -> cube map, irradiance
convolution and the prefiltered specular chain, drawn exactly as IBLGenerator draws them
(Environment.cpp:25-195): a unit cube seen from its centre through six 90-degree cameras, one render
pass per cube face (and per mip level for the prefiltered map) into the face of the output cube
texture, with the skybox / IBL-irradiance / IBL-prefilter shaders. On the GPU these are ordinary
draws of the corresponding shading models (their fragment shaders run on the CUDA raster path).
"""
from __future__ import annotations

import hashlib
import os
from typing import Optional

import numpy as np

from . import api as A
from . import scenes as S

K_IRRADIANCE_SIZE = 32        # Environment.h:20
K_PREFILTER_LEVELS = 5        # Environment.h:21
K_PREFILTER_SIZE = 128        # Environment.h:22

# IBLGenerator::drawCubeFaces capture views (Environment.cpp:154-161): (center, up), eye at the origin
CAPTURE_VIEWS = (((1.0, 0.0, 0.0), (0.0, -1.0, 0.0)), ((-1.0, 0.0, 0.0), (0.0, -1.0, 0.0)),
                 ((0.0, 1.0, 0.0), (0.0, 0.0, 1.0)), ((0.0, -1.0, 0.0), (0.0, 0.0, -1.0)),
                 ((0.0, 0.0, 1.0), (0.0, -1.0, 0.0)), ((0.0, 0.0, -1.0), (0.0, -1.0, 0.0)))


def cube_mesh() -> (np.ndarray, np.ndarray):
    """A unit cube of 12 triangles as 64-byte View::Vertex rows (positions only), 36 vertices."""
    corners = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float32)
    faces = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
             (3, 6, 2), (3, 7, 6), (0, 4, 7), (0, 7, 3), (1, 2, 6), (1, 6, 5)]
    rows = np.zeros((36, 16), np.float32)
    for t, f in enumerate(faces):
        for k in range(3):
            rows[3 * t + k, 0:3] = corners[f[k]]
    return rows, np.arange(36, dtype=np.int32)


def _face_mvp(face: int) -> np.ndarray:
    """Projection (90 degrees, aspect 1, near 0.1) times the rotation part of the face's view."""
    center, up = CAPTURE_VIEWS[face]
    V = S.look_at([0.0, 0.0, 0.0], center, up)
    R = np.eye(4)
    R[:3, :3] = V[:3, :3]   # glm::mat4(glm::mat3(viewMatrix)): rotation only
    P = S.perspective(np.pi / 2.0, 1.0, 0.1, False)
    return S.mm4(P, R)


def cache_key(tex: A.Texture) -> str:
    """IBLGenerator::getTextureHashKey (Environment.cpp:197-199): MD5 of tag + width + height, as
    32 lower-case hex digits."""
    return hashlib.md5((tex.tag + str(tex.width) + str(tex.height)).encode()).hexdigest()


class IBLGenerator:
    """`cache_dir` (IBL_TEX_CACHE_DIR, Environment.cpp:17): when set, every generated map is looked
    up in the cache first (loadFromCache) and stored there after it is drawn (storeToCache),
    one <md5>.tex file per map in the TextureSoft::storeToFile format."""

    def __init__(self, r: A.Renderer, cache_dir: Optional[str] = None):
        self.r = r
        self.cache_dir = cache_dir
        self.cache_hits = 0
        rows, idx = cube_mesh()
        self.vao = r.createVertexArrayObject(rows, 64, idx)
        self.fbo = r.createFrameBuffer(offscreen=True)
        self.states = r.createPipelineStates(A.RenderStates())
        self.model_blocks = []
        for f in range(6):
            ub = r.createUniformBlock("UniformsModel", 256)
            ub.setData(S.uniforms_model(np.eye(4), _face_mvp(f), None, False))
            self.model_blocks.append(ub)

    def _draw_faces(self, shading: int, defines, sampler_name: str, tex_in: A.Texture, tex_out: A.Texture,
                    level: int = 0, prefilter: Optional[bytes] = None) -> None:
        r = self.r
        prog = r.createShaderProgram()
        prog.addDefines(defines)
        prog.SetShaders(shading)
        us = r.createUniformSampler(sampler_name, tex_in.desc)
        us.setTexture(tex_in)
        w, h = tex_out.getLevelWidth(level), tex_out.getLevelHeight(level)
        pre_ub = None
        if prefilter is not None:
            pre_ub = r.createUniformBlock("UniformsPrefilter", len(prefilter))
            pre_ub.setData(prefilter)
        for face in range(6):
            res = r.createShaderResources()
            res.setBlock(S._BLOCK_KEYS["UniformsModel"], self.model_blocks[face])
            if pre_ub is not None:
                res.setBlock(20, pre_ub)
            res.setSampler(0, us)
            self.fbo.setColorAttachment(tex_out, level, face)
            r.beginRenderPass(self.fbo, A.ClearStates(False, True, (0.0, 0.0, 0.0, 0.0), 1.0))
            r.setViewPort(0, 0, w, h)
            r.setVertexArrayObject(self.vao)
            r.setShaderProgram(prog)
            r.setShaderResources(res)
            r.setPipelineStates(self.states)
            r.draw()
            r.endRenderPass()

    def cache_path(self, tex: A.Texture) -> str:
        """IBLGenerator::getCacheFilePath (Environment.cpp:201-204)."""
        return os.path.join(self.cache_dir, cache_key(tex) + ".tex")

    def _load_from_cache(self, tex: A.Texture) -> bool:
        """IBLGenerator::loadFromCache (Environment.cpp:206-222)."""
        if self.cache_dir is None or not os.path.exists(self.cache_path(tex)):
            return False
        ok = tex.loadFromFile(self.cache_path(tex))
        self.cache_hits += int(ok)
        return ok

    def _store_to_cache(self, tex: A.Texture) -> None:
        """IBLGenerator::storeToCache (Environment.cpp:224-239)."""
        if self.cache_dir is None:
            return
        os.makedirs(self.cache_dir, exist_ok=True)
        tex.storeToFile(self.cache_path(tex))

    def _cube(self, size: int, mipmaps: bool) -> A.Texture:
        t = self.r.createTexture(A.TextureDesc(size, size, A.TextureType_CUBE, A.TextureFormat_RGBA8,
                                               A.TextureUsage_AttachmentColor | A.TextureUsage_Sampler,
                                               mipmaps, False))
        t.setSamplerDesc(A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR if mipmaps else A.Filter_LINEAR,
                                       A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE,
                                       A.Wrap_CLAMP_TO_EDGE))
        t.initImageData()
        return t

    def convert_equirectangular(self, equirect: A.Texture, size: int) -> A.Texture:
        """IBLGenerator::convertEquirectangular: the skybox shader with EQUIRECTANGULAR_MAP."""
        out = self._cube(size, False)
        out.tag = equirect.tag + ".cubeMap"
        if self._load_from_cache(out):
            return out
        self._draw_faces(A.Shading_Skybox, ("EQUIRECTANGULAR_MAP",), "u_equirectangularMap", equirect, out)
        self._store_to_cache(out)
        return out

    def irradiance(self, cube: A.Texture, size: int = K_IRRADIANCE_SIZE) -> A.Texture:
        """IBLGenerator::generateIrradianceMap."""
        out = self._cube(size, False)
        out.tag = cube.tag + ".irradianceMap"
        if self._load_from_cache(out):
            return out
        self._draw_faces(A.Shading_IBL_Irradiance, (), "u_cubeMap", cube, out)
        self._store_to_cache(out)
        return out

    def prefilter(self, cube: A.Texture, size: int = K_PREFILTER_SIZE, levels: int = K_PREFILTER_LEVELS) -> A.Texture:
        """IBLGenerator::generatePrefilterMap: roughness level / (levels - 1) for mip `level`."""
        out = self._cube(size, True)
        out.tag = cube.tag + ".prefilterMap"
        if self._load_from_cache(out):
            return out
        for level in range(levels):
            block = np.array([float(cube.width), level / float(levels - 1)], np.float32).tobytes()
            self._draw_faces(A.Shading_IBL_Prefilter, (), "u_cubeMap", cube, out, level, block)
        self._store_to_cache(out)
        return out


def equirect_sky(width: int, height: int, seed: int) -> np.ndarray:
    """A seeded equirectangular RGBA8 sky: vertical gradient with three sun lobes."""
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    lon = (x + 0.5) / width * 2.0 * np.pi - np.pi
    lat = np.pi / 2.0 - (y + 0.5) / height * np.pi
    d = np.stack([np.cos(lat) * np.cos(lon), np.sin(lat), np.cos(lat) * np.sin(lon)], axis=-1)
    base = np.stack([0.25 + 0.35 * (d[..., 1] * 0.5 + 0.5), 0.35 + 0.35 * (d[..., 1] * 0.5 + 0.5),
                     0.55 + 0.4 * (d[..., 1] * 0.5 + 0.5)], axis=-1)
    for k in range(3):
        s = S.normalize(S.hash_u01(seed, 400 + k, np.arange(3)) * 2.0 - 1.0 + np.array([0.0, 0.7, 0.0]))
        c = np.clip(d @ s, 0.0, 1.0)
        base += (c ** (40.0 * (k + 1)))[..., None] * np.array([1.0, 0.9, 0.7])
    img = np.zeros((height, width, 4), np.uint8)
    img[..., :3] = np.clip(base * 255.0, 0, 255).astype(np.uint8)
    img[..., 3] = 255
    return img
