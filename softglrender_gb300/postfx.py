"""Screen-space post passes on the renderer: QuadFilter (QuadFilter.cpp:12-112) drawing a
full-screen quad with a screen shader, here FXAA (FxaaSoft.h), from an input colour texture into an
output colour texture of the same size (Viewer::processFXAASetup / processFXAADraw,
Viewer.cpp:170-213). On the GPU the pass is an ordinary two-triangle draw of the FXAA shading model.
"""
from __future__ import annotations

import struct

import numpy as np

from . import api as A


class QuadFilter:
    def __init__(self, r: A.Renderer, width: int, height: int, shading: int = A.Shading_FXAA):
        self.r, self.width, self.height = r, width, height
        # the reference's quad: 4 vertices, indices {0, 1, 2, 1, 2, 3} (QuadFilter.cpp:22-28)
        rows = np.zeros((4, 16), np.float32)
        for k, (pos, uv) in enumerate((((1.0, -1.0), (1.0, 0.0)), ((-1.0, -1.0), (0.0, 0.0)),
                                       ((1.0, 1.0), (1.0, 1.0)), ((-1.0, 1.0), (0.0, 1.0)))):
            rows[k, 0:2] = pos
            rows[k, 4:6] = uv
        self.vao = r.createVertexArrayObject(rows, 64, np.array([0, 1, 2, 1, 2, 3], np.int32))
        self.fbo = r.createFrameBuffer(offscreen=False)
        self.prog = r.createShaderProgram()
        self.prog.SetShaders(shading)
        self.res = r.createShaderResources()
        desc = A.TextureDesc(width, height, A.TextureType_2D, A.TextureFormat_RGBA8, A.TextureUsage_AttachmentColor,
                             False, False)
        self.tex_in = r.createUniformSampler("u_screenTexture", desc)
        self.res.setSampler(0, self.tex_in)
        self.ub = r.createUniformBlock("UniformsQuadFilter", 8)
        self.ub.setData(struct.pack("<2f", float(width), float(height)))
        self.res.setBlock(30, self.ub)
        self.states = r.createPipelineStates(A.RenderStates())

    def set_textures(self, tex_in: A.Texture, tex_out: A.Texture) -> None:
        assert (tex_in.width, tex_in.height) == (self.width, self.height) == (tex_out.width, tex_out.height)
        self.tex_in.setTexture(tex_in)
        self.fbo.setColorAttachment(tex_out, 0)

    def draw(self) -> None:
        r = self.r
        r.beginRenderPass(self.fbo, A.ClearStates(False, True, (0.0, 0.0, 0.0, 0.0), 1.0))
        r.setViewPort(0, 0, self.width, self.height)
        r.setVertexArrayObject(self.vao)
        r.setShaderProgram(self.prog)
        r.setShaderResources(self.res)
        r.setPipelineStates(self.states)
        r.draw()
        r.endRenderPass()


def fxaa(r: A.Renderer, image: np.ndarray, filter_mode: int = A.Filter_LINEAR) -> np.ndarray:
    """FXAA of an (h, w, 4) RGBA8 image on renderer r; returns the filtered image."""
    h, w = image.shape[:2]
    tin = r.createTexture(A.TextureDesc(w, h, A.TextureType_2D, A.TextureFormat_RGBA8,
                                        A.TextureUsage_Sampler | A.TextureUsage_UploadData, False, False))
    tin.setSamplerDesc(A.SamplerDesc(filter_mode, filter_mode, A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE,
                                     A.Wrap_CLAMP_TO_EDGE))
    tin.setImageData([np.ascontiguousarray(image)])
    tout = r.createTexture(A.TextureDesc(w, h, A.TextureType_2D, A.TextureFormat_RGBA8,
                                         A.TextureUsage_AttachmentColor | A.TextureUsage_Sampler, False, False))
    tout.initImageData()
    q = QuadFilter(r, w, h)
    q.set_textures(tin, tout)
    q.draw()
    r.waitIdle()
    return tout.readImage()
