"""Test infrastructure: a Scene (softglrender_gb300/scenes.py) as a flat little-endian file that the C++
driver tests/integration/drive_renderer.cpp reads and renders through SoftGL::Renderer.

Layout (all integers int32 unless noted, floats IEEE float32):
  "SGLSCN01", pass count
  per pass: width, height, samples, color, depth, clear depthFlag, colorFlag, clearColor[4] (f32),
            clearDepth (f32), draw count
  per draw: stride, vertex bytes (int64) + bytes, index count (int64) + int32 indices, shading model,
            define count + strings, RenderStates (13 int32 + lineWidth f32), block count + blocks,
            texture count + textures
  block:    name, key (UniformBlockType), byte count + bytes
  texture:  id (textures shared by draws keep one id), sampler name, TextureDesc (width, height, type,
            format, usage, useMipmaps, multiSample), SamplerDesc (6 int32), source (0: level-0 image per
            layer for setImageData; 1: explicit [level][layer] images), then the images as
            (byte count (int64) + bytes) in that order
  string:   length + UTF-8 bytes
"""
from __future__ import annotations

import struct
from typing import Dict

import numpy as np

from softglrender_gb300 import scenes as S

MAGIC = b"SGLSCN01"
_BLOCK_KEYS = {"UniformsScene": 0, "UniformsModel": 1, "UniformsMaterial": 2}   # UniformBlockType


def _i(*v) -> bytes:
    return struct.pack(f"<{len(v)}i", *[int(x) for x in v])


def _f(*v) -> bytes:
    return struct.pack(f"<{len(v)}f", *[float(x) for x in v])


def _str(s: str) -> bytes:
    b = s.encode()
    return _i(len(b)) + b


def _blob(arr) -> bytes:
    b = arr if isinstance(arr, (bytes, bytearray)) else np.ascontiguousarray(arr).tobytes()
    return struct.pack("<q", len(b)) + b


def encode(scene: S.Scene) -> bytes:
    out = [MAGIC, _i(len(scene.passes))]
    tex_ids: Dict[int, int] = {}
    for p in scene.passes:
        c = p.clear
        out += [_i(p.width, p.height, p.samples, p.color, p.depth, c.depthFlag, c.colorFlag),
                _f(*c.clearColor, c.clearDepth), _i(len(p.draws))]
        for d in p.draws:
            rs = d.states
            bp = rs.blendParams
            out += [_i(d.stride), _blob(np.asarray(d.vertexes, np.float32)),
                    struct.pack("<q", len(d.indices)), np.ascontiguousarray(d.indices, np.int32).tobytes(),
                    _i(d.shading, len(d.defines))]
            out += [_str(x) for x in d.defines]
            out += [_i(rs.blend, bp.blendFuncRgb, bp.blendSrcRgb, bp.blendDstRgb, bp.blendFuncAlpha,
                       bp.blendSrcAlpha, bp.blendDstAlpha, rs.depthTest, rs.depthMask, rs.depthFunc,
                       rs.cullFace, rs.primitiveType, rs.polygonMode), _f(rs.lineWidth)]
            out.append(_i(len(d.blocks)))
            for k, (name, data) in enumerate(d.blocks.items()):
                out += [_str(name), _i(_BLOCK_KEYS.get(name, 10 + k)), _blob(data)]
            out.append(_i(len(d.textures)))
            for t in d.textures:
                tid = tex_ids.setdefault(id(t), len(tex_ids))
                td, sd = t.desc, t.sampler
                out += [_i(tid), _str(t.name),
                        _i(td.width, td.height, td.type, td.format, td.usage, td.useMipmaps, td.multiSample),
                        _i(sd.filterMin, sd.filterMag, sd.wrapS, sd.wrapT, sd.wrapR, sd.borderColor)]
                if t.levels is not None:
                    out += [_i(1, len(t.levels), len(t.levels[0]))]
                    out += [_blob(img) for lev in t.levels for img in lev]
                else:
                    out += [_i(0, len(t.layers))]
                    out += [_blob(img) for img in t.layers]
    return b"".join(out)


def write(scene: S.Scene, path: str) -> None:
    with open(path, "wb") as f:
        f.write(encode(scene))
