"""Host-side mirror of SoftGLRender's back-end abstraction over the C ABI of include/softgl_cuda.h.

`Renderer` exposes the reference's own method names and argument meaning
(src/Render/Renderer.h:24-59) and the resource objects expose theirs (FrameBuffer
src/Render/Framebuffer.h:20-91, Texture src/Render/Texture.h:87-105, VertexArrayObject
src/Render/Vertex.h:15-19, ShaderProgram src/Render/ShaderProgram.h:15-58, UniformBlock /
UniformSampler / ShaderResources src/Render/Uniform.h:20-64), so a script written against the
reference's call sequence (Viewer::pipelineDraw, src/Viewer/Viewer.cpp:388-396) reads the same here.

The class is generic over a loaded C-ABI library and its symbol prefix; the product package only
ever loads the CUDA library (see `softglrender_gb300.load_library`). Errors surface as
`SoftGLError` carrying the status code and the library's last-error text; the reference logs and
returns instead (RendererSoft.cpp:33,137-139), which a caller gets by catching the exception.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence

import numpy as np

# ---- enums (values equal to the reference's, see include/softgl_cuda.h) -------------------------
TextureType_2D, TextureType_CUBE = 0, 1
TextureFormat_RGBA8, TextureFormat_FLOAT32 = 0, 1
(Filter_NEAREST, Filter_LINEAR, Filter_NEAREST_MIPMAP_NEAREST, Filter_LINEAR_MIPMAP_NEAREST,
 Filter_NEAREST_MIPMAP_LINEAR, Filter_LINEAR_MIPMAP_LINEAR) = range(6)
Wrap_REPEAT, Wrap_MIRRORED_REPEAT, Wrap_CLAMP_TO_EDGE, Wrap_CLAMP_TO_BORDER = range(4)
Border_BLACK, Border_WHITE = 0, 1
Layout_Linear, Layout_Tiled, Layout_Morton = 0, 1, 2
(DepthFunc_NEVER, DepthFunc_LESS, DepthFunc_EQUAL, DepthFunc_LEQUAL, DepthFunc_GREATER,
 DepthFunc_NOTEQUAL, DepthFunc_GEQUAL, DepthFunc_ALWAYS) = range(8)
(BlendFactor_ZERO, BlendFactor_ONE, BlendFactor_SRC_COLOR, BlendFactor_SRC_ALPHA, BlendFactor_DST_COLOR,
 BlendFactor_DST_ALPHA, BlendFactor_ONE_MINUS_SRC_COLOR, BlendFactor_ONE_MINUS_SRC_ALPHA,
 BlendFactor_ONE_MINUS_DST_COLOR, BlendFactor_ONE_MINUS_DST_ALPHA) = range(10)
BlendFunc_ADD, BlendFunc_SUBTRACT, BlendFunc_REVERSE_SUBTRACT, BlendFunc_MIN, BlendFunc_MAX = range(5)
PolygonMode_POINT, PolygonMode_LINE, PolygonMode_FILL = range(3)
Primitive_POINT, Primitive_LINE, Primitive_TRIANGLE = range(3)
TextureUsage_Sampler, TextureUsage_UploadData = 1 << 0, 1 << 1
TextureUsage_AttachmentColor, TextureUsage_AttachmentDepth, TextureUsage_RendererOutput = 1 << 2, 1 << 3, 1 << 4

Shading_BaseColor = 1
Shading_BlinnPhong = 2
Shading_PBR = 3
Shading_Skybox = 4
Shading_IBL_Irradiance = 5
Shading_IBL_Prefilter = 6
Shading_FXAA = 7
Shading_BlinnPhongDir = 100
Shading_VertexColor = 101

# CubeMapFace (Texture.h:33-40)
TEXTURE_CUBE_MAP_POSITIVE_X, TEXTURE_CUBE_MAP_NEGATIVE_X = 0, 1
TEXTURE_CUBE_MAP_POSITIVE_Y, TEXTURE_CUBE_MAP_NEGATIVE_Y = 2, 3
TEXTURE_CUBE_MAP_POSITIVE_Z, TEXTURE_CUBE_MAP_NEGATIVE_Z = 4, 5


# sglc_status (softgl_cuda.h)
(SGLC_OK, SGLC_ERR_INVALID_HANDLE, SGLC_ERR_INVALID_VALUE, SGLC_ERR_OUT_OF_MEMORY, SGLC_ERR_DEVICE,
 SGLC_ERR_UNSUPPORTED, SGLC_ERR_OVERFLOW, SGLC_ERR_NO_DEVICE) = range(8)


class SoftGLError(RuntimeError):
    def __init__(self, status: int, call: str, message: str):
        super().__init__(f"{call} failed with status {status}: {message}")
        self.status = status


# ---- ABI structs -------------------------------------------------------------------------------
class _TextureDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("type", C.c_int32), ("format", C.c_int32),
                ("usage", C.c_uint32), ("use_mipmaps", C.c_int32), ("multi_sample", C.c_int32),
                ("layout", C.c_int32)]


class _SamplerDesc(C.Structure):
    _fields_ = [("filter_min", C.c_int32), ("filter_mag", C.c_int32), ("wrap_s", C.c_int32),
                ("wrap_t", C.c_int32), ("wrap_r", C.c_int32), ("border_color", C.c_int32)]


class _RenderStates(C.Structure):
    _fields_ = [("blend", C.c_int32), ("blend_func_rgb", C.c_int32), ("blend_src_rgb", C.c_int32),
                ("blend_dst_rgb", C.c_int32), ("blend_func_alpha", C.c_int32), ("blend_src_alpha", C.c_int32),
                ("blend_dst_alpha", C.c_int32), ("depth_test", C.c_int32), ("depth_mask", C.c_int32),
                ("depth_func", C.c_int32), ("cull_face", C.c_int32), ("primitive_type", C.c_int32),
                ("polygon_mode", C.c_int32), ("line_width", C.c_float)]


class _ClearStates(C.Structure):
    _fields_ = [("depth_flag", C.c_int32), ("color_flag", C.c_int32), ("clear_color", C.c_float * 4),
                ("clear_depth", C.c_float)]


class _DrawStats(C.Structure):
    _fields_ = [("vertices_in", C.c_int64), ("triangles_in", C.c_int64), ("clip_vertices", C.c_int64),
                ("primitives", C.c_int64), ("bin_entries", C.c_int64), ("fragments_shaded", C.c_int64),
                ("geometry_ms", C.c_float), ("binning_ms", C.c_float), ("raster_ms", C.c_float),
                ("kernel_launches", C.c_int32), ("coverage_ms", C.c_float), ("shading_ms", C.c_float),
                ("rop_ms", C.c_float)]


# ---- reference value types ---------------------------------------------------------------------
@dataclass
class TextureDesc:
    """TextureDesc (Texture.h:76-85) + the buffer layout (compile-time in the reference)."""
    width: int = 0
    height: int = 0
    type: int = TextureType_2D
    format: int = TextureFormat_RGBA8
    usage: int = TextureUsage_Sampler
    useMipmaps: bool = False
    multiSample: bool = False
    layout: int = Layout_Linear


@dataclass
class SamplerDesc:
    """SamplerDesc (Texture.h:47-56)."""
    filterMin: int = Filter_NEAREST
    filterMag: int = Filter_NEAREST
    wrapS: int = Wrap_CLAMP_TO_EDGE
    wrapT: int = Wrap_CLAMP_TO_EDGE
    wrapR: int = Wrap_CLAMP_TO_EDGE
    borderColor: int = Border_BLACK


@dataclass
class BlendParameters:
    """BlendParameters (RenderStates.h:53-73)."""
    blendFuncRgb: int = BlendFunc_ADD
    blendSrcRgb: int = BlendFactor_ONE
    blendDstRgb: int = BlendFactor_ZERO
    blendFuncAlpha: int = BlendFunc_ADD
    blendSrcAlpha: int = BlendFactor_ONE
    blendDstAlpha: int = BlendFactor_ZERO

    def SetBlendFactor(self, src: int, dst: int) -> None:
        self.blendSrcRgb = self.blendSrcAlpha = src
        self.blendDstRgb = self.blendDstAlpha = dst

    def SetBlendFunc(self, func: int) -> None:
        self.blendFuncRgb = self.blendFuncAlpha = func


@dataclass
class RenderStates:
    """RenderStates (RenderStates.h:79-92)."""
    blend: bool = False
    blendParams: BlendParameters = field(default_factory=BlendParameters)
    depthTest: bool = False
    depthMask: bool = True
    depthFunc: int = DepthFunc_LESS
    cullFace: bool = False
    primitiveType: int = Primitive_TRIANGLE
    polygonMode: int = PolygonMode_FILL
    lineWidth: float = 1.0


@dataclass
class ClearStates:
    """ClearStates (RenderStates.h:94-99)."""
    depthFlag: bool = False
    colorFlag: bool = False
    clearColor: Sequence[float] = (0.0, 0.0, 0.0, 0.0)
    clearDepth: float = 1.0


# ---- library binding ---------------------------------------------------------------------------
_SIGS = {
    "create": [C.POINTER(C.c_void_p), C.c_int32],
    "destroy": [C.c_void_p],
    "release": [C.c_void_p, C.c_int32],
    "create_framebuffer": [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)],
    "framebuffer_set_color_attachment": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32],
    "framebuffer_set_depth_attachment": [C.c_void_p, C.c_int32, C.c_int32],
    "framebuffer_is_valid": [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)],
    "create_texture": [C.c_void_p, C.POINTER(_TextureDesc), C.POINTER(C.c_int32)],
    "texture_set_sampler_desc": [C.c_void_p, C.c_int32, C.POINTER(_SamplerDesc)],
    "texture_init_image_data": [C.c_void_p, C.c_int32],
    "texture_set_image_data": [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p), C.c_size_t],
    "texture_set_level_data": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t],
    "texture_read_image": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t],
    "texture_store_to_file": [C.c_void_p, C.c_int32, C.c_char_p],
    "texture_load_from_file": [C.c_void_p, C.c_int32, C.c_char_p],
    "create_vertex_array": [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t,
                            C.POINTER(C.c_int32)],
    "vertex_array_update": [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t],
    "create_shader_program": [C.c_void_p, C.POINTER(C.c_int32)],
    "program_add_define": [C.c_void_p, C.c_int32, C.c_char_p],
    "program_set_shaders": [C.c_void_p, C.c_int32, C.c_int32],
    "create_pipeline_states": [C.c_void_p, C.POINTER(_RenderStates), C.POINTER(C.c_int32)],
    "create_uniform_block": [C.c_void_p, C.c_char_p, C.c_int32, C.POINTER(C.c_int32)],
    "uniform_block_set_sub_data": [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32],
    "uniform_block_set_data": [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32],
    "create_uniform_sampler": [C.c_void_p, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32)],
    "uniform_sampler_set_texture": [C.c_void_p, C.c_int32, C.c_int32],
    "create_shader_resources": [C.c_void_p, C.POINTER(C.c_int32)],
    "shader_resources_set_block": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32],
    "shader_resources_set_sampler": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32],
    "begin_render_pass": [C.c_void_p, C.c_int32, C.POINTER(_ClearStates)],
    "set_viewport": [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32],
    "set_vertex_array": [C.c_void_p, C.c_int32],
    "set_shader_program": [C.c_void_p, C.c_int32],
    "set_shader_resources": [C.c_void_p, C.c_int32],
    "set_pipeline_states": [C.c_void_p, C.c_int32],
    "draw": [C.c_void_p],
    "end_render_pass": [C.c_void_p],
    "wait_idle": [C.c_void_p],
    "set_enable_early_z": [C.c_void_p, C.c_int32],
    "get_draw_stats": [C.c_void_p, C.POINTER(_DrawStats)],
    "get_stream": [C.c_void_p, C.POINTER(C.c_void_p)],
    "set_stats_level": [C.c_void_p, C.c_int32],
    "draw_views": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32, C.c_void_p],
    "draw_scenes": [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32,
                    C.c_void_p],
    "set_capacity": [C.c_void_p, C.c_void_p],
    "get_overflow": [C.c_void_p, C.POINTER(C.c_int32)],
    "get_peak_counts": [C.c_void_p, C.c_void_p],
    "set_tile_size": [C.c_void_p, C.c_int32],
    "set_deferred_shading": [C.c_void_p, C.c_int32],
    "set_tma_store": [C.c_void_p, C.c_int32],
}

ABI_FUNCTIONS = tuple(_SIGS) + ("last_error",)


class Capacity(C.Structure):
    """sglc_capacity: working-array capacities of synchronisation-free draws."""
    _fields_ = [("clip_vertices", C.c_int64), ("clip_polygons", C.c_int64), ("appended_primitives", C.c_int64),
                ("bin_entries", C.c_int64), ("heavy_first", C.c_int32), ("fragments", C.c_int64)]


class Library:
    """A loaded C-ABI library (product, oracle or reference) with its symbol prefix."""

    def __init__(self, cdll: C.CDLL, prefix: str):
        self.cdll = cdll
        self.prefix = prefix
        self.fn = {}
        for name, args in _SIGS.items():
            f = getattr(cdll, prefix + name)
            f.argtypes = args
            f.restype = C.c_int32
            self.fn[name] = f
        le = getattr(cdll, prefix + "last_error")
        le.argtypes = [C.c_void_p]
        le.restype = C.c_char_p
        self.fn["last_error"] = le


def _as_bytes_ptr(arr: np.ndarray):
    arr = np.ascontiguousarray(arr)
    return arr, arr.ctypes.data_as(C.c_void_p)


# ---- resource objects (reference names) --------------------------------------------------------
class _Resource:
    def __init__(self, renderer: "Renderer", handle: int):
        self.renderer = renderer
        self.handle = handle

    def getId(self) -> int:
        return self.handle


class FrameBuffer(_Resource):
    def __init__(self, renderer, handle, offscreen):
        super().__init__(renderer, handle)
        self.offscreen = offscreen
        self.colorAttachment: Optional["Texture"] = None
        self.depthAttachment: Optional["Texture"] = None

    def setColorAttachment(self, tex: "Texture", level: int = 0, face: int = 0) -> None:
        self.renderer._call("framebuffer_set_color_attachment", self.handle, tex.handle, face, level)
        self.colorAttachment = tex

    def setDepthAttachment(self, tex: "Texture") -> None:
        self.renderer._call("framebuffer_set_depth_attachment", self.handle, tex.handle)
        self.depthAttachment = tex

    def isValid(self) -> bool:
        v = C.c_int32(0)
        self.renderer._call("framebuffer_is_valid", self.handle, C.byref(v))
        return bool(v.value)


class Texture(_Resource):
    def __init__(self, renderer, handle, desc: TextureDesc):
        super().__init__(renderer, handle)
        self.desc = desc
        self.width, self.height = desc.width, desc.height
        self.type, self.format = desc.type, desc.format
        self.useMipmaps, self.multiSample = desc.useMipmaps, desc.multiSample
        self.tag = ""   # Texture::tag (Texture.h:98): names the IBL cache entry

    @property
    def layerCount(self) -> int:
        return 6 if self.type == TextureType_CUBE else 1

    def getLevelWidth(self, level: int) -> int:
        return max(1, self.width >> level)

    def getLevelHeight(self, level: int) -> int:
        return max(1, self.height >> level)

    def setSamplerDesc(self, s: SamplerDesc) -> None:
        sd = _SamplerDesc(s.filterMin, s.filterMag, s.wrapS, s.wrapT, s.wrapR, s.borderColor)
        self.renderer._call("texture_set_sampler_desc", self.handle, C.byref(sd))

    def initImageData(self) -> None:
        self.renderer._call("texture_init_image_data", self.handle)

    def setImageData(self, layers: Sequence[np.ndarray]) -> None:
        """One (height, width[, 4]) array per layer: uint8 RGBA for RGBA8, float32 for FLOAT32."""
        keep = [np.ascontiguousarray(a) for a in layers]
        nbytes = keep[0].nbytes
        ptrs = (C.c_void_p * len(keep))(*[a.ctypes.data for a in keep])
        self.renderer._call("texture_set_image_data", self.handle, len(keep), ptrs, nbytes)

    def setLevelData(self, layer: int, level: int, data: np.ndarray) -> None:
        arr, p = _as_bytes_ptr(data)
        self.renderer._call("texture_set_level_data", self.handle, layer, level, p, arr.nbytes)

    def readImage(self, layer: int = 0, level: int = 0, resolved: bool = False) -> np.ndarray:
        """Texture::dumpImage analogue: the level as an array, linear row-major order."""
        w, h = self.getLevelWidth(level), self.getLevelHeight(level)
        if self.multiSample and not resolved:
            shape = (h, w, 4, 4) if self.format == TextureFormat_RGBA8 else (h, w, 4)
        else:
            shape = (h, w, 4) if self.format == TextureFormat_RGBA8 else (h, w)
        dtype = np.uint8 if self.format == TextureFormat_RGBA8 else np.float32
        if resolved and self.format != TextureFormat_RGBA8:
            raise ValueError("only RGBA8 attachments have a resolved image")
        out = np.empty(shape, dtype=dtype)
        self.renderer._call("texture_read_image", self.handle, layer, level, int(resolved),
                            out.ctypes.data_as(C.c_void_p), out.nbytes)
        return out


    def storeToFile(self, path: str) -> None:
        """TextureSoft::storeToFile: every layer and level, raw texels in storage layout order."""
        self.renderer._call("texture_store_to_file", self.handle, os.fsencode(path))

    def loadFromFile(self, path: str) -> bool:
        """TextureSoft::loadFromFile: False (texture unchanged) when the file is missing or short."""
        try:
            self.renderer._call("texture_load_from_file", self.handle, os.fsencode(path))
        except SoftGLError as e:
            if e.status != SGLC_ERR_INVALID_VALUE:
                raise
            return False
        return True


class VertexArrayObject(_Resource):
    def updateVertexData(self, data: np.ndarray) -> None:
        arr, p = _as_bytes_ptr(data)
        self.renderer._call("vertex_array_update", self.handle, p, arr.nbytes)


class ShaderProgram(_Resource):
    def addDefine(self, name: str) -> None:
        self.renderer._call("program_add_define", self.handle, name.encode())

    def addDefines(self, names) -> None:
        for n in sorted(names):
            self.addDefine(n)

    def SetShaders(self, shading_model: int) -> None:
        self.renderer._call("program_set_shaders", self.handle, shading_model)


class PipelineStates(_Resource):
    def __init__(self, renderer, handle, states: RenderStates):
        super().__init__(renderer, handle)
        self.renderStates = states


class UniformBlock(_Resource):
    def __init__(self, renderer, handle, name, size):
        super().__init__(renderer, handle)
        self.name, self.blockSize = name, size

    def setSubData(self, data: bytes, offset: int) -> None:
        buf = C.create_string_buffer(bytes(data), len(data))
        self.renderer._call("uniform_block_set_sub_data", self.handle, buf, len(data), offset)

    def setData(self, data: bytes) -> None:
        buf = C.create_string_buffer(bytes(data), len(data))
        self.renderer._call("uniform_block_set_data", self.handle, buf, len(data))


class UniformSampler(_Resource):
    def __init__(self, renderer, handle, name):
        super().__init__(renderer, handle)
        self.name = name

    def setTexture(self, tex: Texture) -> None:
        self.renderer._call("uniform_sampler_set_texture", self.handle, tex.handle)


class ShaderResources(_Resource):
    """ShaderResources (Uniform.h:60-64): integer-keyed blocks and samplers."""

    def __init__(self, renderer, handle):
        super().__init__(renderer, handle)
        self.blocks: Dict[int, UniformBlock] = {}
        self.samplers: Dict[int, UniformSampler] = {}

    def setBlock(self, key: int, ub: UniformBlock) -> None:
        self.renderer._call("shader_resources_set_block", self.handle, key, ub.handle)
        self.blocks[key] = ub

    def setSampler(self, key: int, us: UniformSampler) -> None:
        self.renderer._call("shader_resources_set_sampler", self.handle, key, us.handle)
        self.samplers[key] = us


class Renderer:
    """SoftGL::Renderer (Renderer.h:24-59) over one C-ABI library."""

    def __init__(self, library: Library, device: int = 0):
        self.lib = library
        ctx = C.c_void_p()
        st = library.fn["create"](C.byref(ctx), device)
        if st != 0:
            raise SoftGLError(st, "create", "context creation failed (no usable device?)")
        self.ctx = ctx

    # -- plumbing
    def _call(self, name: str, *args) -> None:
        st = self.lib.fn[name](self.ctx, *args)
        if st != 0:
            msg = self.lib.fn["last_error"](self.ctx)
            raise SoftGLError(st, self.lib.prefix + name, msg.decode() if msg else "")

    def _new(self, name: str, *args) -> int:
        h = C.c_int32(0)
        self._call(name, *args, C.byref(h))
        return h.value

    def destroy(self) -> None:
        if self.ctx:
            self.lib.fn["destroy"](self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def release(self, res: _Resource) -> None:
        self._call("release", res.handle)

    # -- factories
    def createFrameBuffer(self, offscreen: bool = False) -> FrameBuffer:
        return FrameBuffer(self, self._new("create_framebuffer", int(offscreen)), offscreen)

    def createTexture(self, desc: TextureDesc) -> Texture:
        d = _TextureDesc(desc.width, desc.height, desc.type, desc.format, desc.usage, int(desc.useMipmaps),
                         int(desc.multiSample), desc.layout)
        return Texture(self, self._new("create_texture", C.byref(d)), desc)

    def createVertexArrayObject(self, vertexes: np.ndarray, stride: int, indices: np.ndarray) -> VertexArrayObject:
        v = np.ascontiguousarray(vertexes)
        i = np.ascontiguousarray(indices, dtype=np.int32)
        h = self._new("create_vertex_array", v.ctypes.data_as(C.c_void_p), v.nbytes, stride,
                      i.ctypes.data_as(C.c_void_p), i.nbytes)
        return VertexArrayObject(self, h)

    def createShaderProgram(self) -> ShaderProgram:
        return ShaderProgram(self, self._new("create_shader_program"))

    def createPipelineStates(self, rs: RenderStates) -> PipelineStates:
        b = rs.blendParams
        s = _RenderStates(int(rs.blend), b.blendFuncRgb, b.blendSrcRgb, b.blendDstRgb, b.blendFuncAlpha,
                          b.blendSrcAlpha, b.blendDstAlpha, int(rs.depthTest), int(rs.depthMask), rs.depthFunc,
                          int(rs.cullFace), rs.primitiveType, rs.polygonMode, rs.lineWidth)
        return PipelineStates(self, self._new("create_pipeline_states", C.byref(s)), rs)

    def createUniformBlock(self, name: str, size: int) -> UniformBlock:
        return UniformBlock(self, self._new("create_uniform_block", name.encode(), size), name, size)

    def createUniformSampler(self, name: str, desc: TextureDesc) -> UniformSampler:
        return UniformSampler(self, self._new("create_uniform_sampler", name.encode(), desc.type, desc.format), name)

    def createShaderResources(self) -> ShaderResources:
        return ShaderResources(self, self._new("create_shader_resources"))

    # -- pipeline
    def beginRenderPass(self, fb: FrameBuffer, states: ClearStates) -> None:
        cs = _ClearStates(int(states.depthFlag), int(states.colorFlag), (C.c_float * 4)(*states.clearColor),
                          states.clearDepth)
        self._call("begin_render_pass", fb.handle, C.byref(cs))

    def setViewPort(self, x: int, y: int, width: int, height: int) -> None:
        self._call("set_viewport", x, y, width, height)

    def setVertexArrayObject(self, vao: VertexArrayObject) -> None:
        self._call("set_vertex_array", vao.handle)

    def setShaderProgram(self, program: ShaderProgram) -> None:
        self._call("set_shader_program", program.handle)

    def setShaderResources(self, resources: ShaderResources) -> None:
        self._call("set_shader_resources", resources.handle)

    def setPipelineStates(self, states: PipelineStates) -> None:
        self._call("set_pipeline_states", states.handle)

    def draw(self) -> None:
        self._call("draw")

    def endRenderPass(self) -> None:
        self._call("end_render_pass")

    def setCapacity(self, cap: Optional[Capacity]) -> None:
        """Synchronisation-free draws with these capacities (None: exact sizing, one read-back per draw)."""
        self._call("set_capacity", C.byref(cap) if cap is not None else None)

    def getPeakCounts(self) -> "Capacity":
        c = Capacity()
        self._call("get_peak_counts", C.byref(c))
        return c

    def getOverflow(self) -> int:
        f = C.c_int32(0)
        self._call("get_overflow", C.byref(f))
        return f.value

    def drawViews(self, framebuffers: Sequence[FrameBuffer], resources: Sequence[ShaderResources],
                  clear: Optional[ClearStates] = None) -> None:
        """Batched views (extension): the bound vertex array / program / states drawn into each
        framebuffer with the matching resources' uniform blocks; equal to one render pass per view."""
        n = len(framebuffers)
        assert len(resources) == n
        fbs = (C.c_int32 * n)(*[f.handle for f in framebuffers])
        res = (C.c_int32 * n)(*[r.handle for r in resources])
        cs = None
        if clear is not None:
            cs = _ClearStates(int(clear.depthFlag), int(clear.colorFlag), (C.c_float * 4)(*clear.clearColor),
                              clear.clearDepth)
        self._call("draw_views", fbs, res, n, C.byref(cs) if cs is not None else None)

    def drawScenes(self, vaos: Sequence["VertexArrayObject"], framebuffers: Sequence[FrameBuffer],
                   resources: Sequence[ShaderResources], clear: Optional[ClearStates] = None) -> None:
        """Multi-scene draw (extension): independent scenes (own vertex array, framebuffer of any
        size, uniform blocks) sharing the bound program, states and samplers, in one pipeline pass;
        equal to one render pass per scene with the viewport over the scene's whole frame."""
        n = len(framebuffers)
        assert len(resources) == n and len(vaos) == n
        vas = (C.c_int32 * n)(*[v.handle for v in vaos])
        fbs = (C.c_int32 * n)(*[f.handle for f in framebuffers])
        res = (C.c_int32 * n)(*[r.handle for r in resources])
        cs = None
        if clear is not None:
            cs = _ClearStates(int(clear.depthFlag), int(clear.colorFlag), (C.c_float * 4)(*clear.clearColor),
                              clear.clearDepth)
        self._call("draw_scenes", vas, fbs, res, n, C.byref(cs) if cs is not None else None)

    def waitIdle(self) -> None:
        self._call("wait_idle")

    def setEnableEarlyZ(self, enable: bool) -> None:
        self._call("set_enable_early_z", int(enable))

    # -- extensions
    def drawStats(self) -> dict:
        s = _DrawStats()
        self._call("get_draw_stats", C.byref(s))
        return {k: getattr(s, k) for k, _ in _DrawStats._fields_}

    def setStatsLevel(self, level: int) -> None:
        self._call("set_stats_level", level)

    def stream(self) -> int:
        p = C.c_void_p()
        self._call("get_stream", C.byref(p))
        return p.value or 0

    def setTileSize(self, tile: int) -> None:
        self._call("set_tile_size", tile)

    def setDeferredShading(self, enable: bool) -> None:
        """Extension: rasterise heavy shading models in coverage / shade / ROP kernels (default) or
        in one fused kernel; the images are the same."""
        self._call("set_deferred_shading", int(enable))

    def setTmaStore(self, enable: bool) -> None:
        """Extension: write whole raster tiles back with TMA bulk stores (default) or per-thread
        stores; the images are the same."""
        self._call("set_tma_store", int(enable))
