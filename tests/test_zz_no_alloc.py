"""The allocation-free draw (sglc_draw_vertex_color_noalloc) for callers that cannot call
cudaMalloc -- code whose device memory belongs to a host framework's pool, real-time render
threads that must not enter the CUDA allocator, library code that must not grow the process's
footprint. It renders one vertex-colour draw into caller-owned device buffers using only a fixed
device array inside the library.

Checked here against the regular entry point (a context, resources and sglc_draw) on the same
inputs, on two calls in a row with different scenes, bit for bit (vertex-colour shading has no
transcendental arithmetic, so the bar for this shading model is exact equality); that sizes
beyond the stated maximum are rejected with a message; that a draw whose triangles need more bin
entries than the fixed array holds reports SGLC_ERR_OVERFLOW and an out-of-range index
SGLC_ERR_INVALID_VALUE, both as status codes read back from the device (the kernels stop at the
capacity and skip the bad triangle, nothing is written out of bounds), and that a normal call
after each still matches the regular draw. This file is collected last so that a run
stopping at the first failure has run every other test first."""
import ctypes as C

import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

from golden.cases import soup
from helpers import render

pytestmark = pytest.mark.gpu


class NoAllocDraw(C.Structure):
    _fields_ = [("vertexes", C.c_void_p), ("vertex_count", C.c_int32), ("stride", C.c_int32),
                ("indices", C.c_void_p), ("triangle_count", C.c_int32), ("uniforms_model", C.c_void_p),
                ("uniforms_material", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32),
                ("samples", C.c_int32), ("color", C.c_void_p), ("resolved", C.c_void_p), ("depth", C.c_void_p),
                ("states", A._RenderStates), ("early_z", C.c_int32), ("error", C.c_char_p), ("error_len", C.c_size_t)]


def _states(rs):
    b = rs.blendParams
    return A._RenderStates(int(rs.blend), b.blendFuncRgb, b.blendSrcRgb, b.blendDstRgb, b.blendFuncAlpha,
                           b.blendSrcAlpha, b.blendDstAlpha, int(rs.depthTest), int(rs.depthMask), rs.depthFunc,
                           int(rs.cullFace), rs.primitiveType, rs.polygonMode, rs.lineWidth)


def _noalloc_render(cdll, scene, expect=0):
    import torch
    p = scene.passes[0]
    d = p.draws[0]
    w, h, s = p.width, p.height, p.samples
    dev = torch.device("cuda:0")
    verts = torch.from_numpy(np.ascontiguousarray(d.vertexes)).to(dev)
    idx = torch.from_numpy(np.ascontiguousarray(d.indices, dtype=np.int32)).to(dev)
    cc = p.clear.clearColor
    clear_rgba = sum((int(c * 255) & 255) << (8 * k) for k, c in enumerate(cc))
    clear_i32 = int(np.array([clear_rgba], dtype=np.uint32).view(np.int32)[0])
    color = torch.full((h * w * s,), clear_i32, dtype=torch.int32, device=dev)
    depth = torch.full((h * w * s,), p.clear.clearDepth, dtype=torch.float32, device=dev)
    resolved = torch.zeros((h * w,), dtype=torch.int32, device=dev)
    model = C.create_string_buffer(d.blocks["UniformsModel"], 256)
    material = C.create_string_buffer(d.blocks["UniformsMaterial"], 48)
    err = C.create_string_buffer(256)
    desc = NoAllocDraw(verts.data_ptr(), d.vertexes.shape[0], d.stride, idx.data_ptr(), len(d.indices) // 3,
                       C.addressof(model), C.addressof(material), w, h, s, color.data_ptr(),
                       resolved.data_ptr() if s == 4 else None, depth.data_ptr(), _states(d.states), 1,
                       C.cast(err, C.c_char_p), 256)
    stream = torch.cuda.current_stream(dev)
    st = cdll.sglc_draw_vertex_color_noalloc(C.byref(desc), C.c_void_p(stream.cuda_stream))
    assert st == expect, (st, err.value)
    torch.cuda.synchronize()
    if expect != 0:
        return err.value
    out = {"color": color.cpu().numpy().view(np.uint8).reshape(h, w, s, 4) if s == 4
           else color.cpu().numpy().view(np.uint8).reshape(h, w, 4),
           "depth": depth.cpu().numpy().reshape((h, w, 4) if s == 4 else (h, w))}
    if s == 4:
        out["resolved"] = resolved.cpu().numpy().view(np.uint8).reshape(h, w, 4)
    return out


def _bind(cuda_lib):
    f = cuda_lib.cdll.sglc_draw_vertex_color_noalloc
    f.argtypes = [C.POINTER(NoAllocDraw), C.c_void_p]
    f.restype = C.c_int32
    return cuda_lib.cdll


def test_noalloc_matches_regular_draw_twice(cuda_lib):
    cdll = _bind(cuda_lib)
    blend = A.BlendParameters()
    blend.SetBlendFactor(A.BlendFactor_SRC_ALPHA, A.BlendFactor_ONE_MINUS_SRC_ALPHA)
    scenes = [
        soup(6000, 320, 180, 4, [A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS)], seed=11),
        soup(4000, 257, 131, 1, [A.RenderStates(blend=True, blendParams=blend, depthTest=True, depthMask=False,
                                                depthFunc=A.DepthFunc_LEQUAL, cullFace=True)], seed=12),
    ]
    for k, scene in enumerate(scenes):       # two calls in a row: the array keeps the first call's data
        got = _noalloc_render(cdll, scene)
        want, _ = render(cuda_lib, scene)
        for key, arr in want[0].items():
            assert np.array_equal(got[key].view(np.uint8), arr.view(np.uint8)), f"call {k}: {key} differs"


def test_noalloc_rejects_sizes_beyond_the_maximum(cuda_lib):
    cdll = _bind(cuda_lib)
    err = C.create_string_buffer(256)
    desc = NoAllocDraw(None, 0, 32, None, 0, None, None, 2048, 16, 1, None, None, None, A._RenderStates(), 1,
                       C.cast(err, C.c_char_p), 256)
    assert cdll.sglc_draw_vertex_color_noalloc(C.byref(desc), None) == 2   # SGLC_ERR_INVALID_VALUE
    assert b"1024" in err.value


def _quads(n_quads, w, h, bad_index=False):
    """n_quads copies of a full-viewport quad (identity transform, z = 0.5): every triangle's
    bounding box covers every 16x16 tile."""
    corners = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=np.float32)
    rows = np.zeros((4 * n_quads, 8), dtype=np.float32)
    for q in range(n_quads):
        rows[4 * q:4 * q + 4, 0:2] = corners
        rows[4 * q:4 * q + 4, 2] = 0.5
        rows[4 * q:4 * q + 4, 4:8] = [(q % 7) / 7.0, (q % 5) / 5.0, (q % 3) / 3.0, 1.0]
    idx = np.concatenate([np.array([0, 1, 2, 0, 2, 3], dtype=np.int32) + 4 * q for q in range(n_quads)])
    if bad_index:
        idx[4] = 4 * n_quads + 100       # one vertex beyond the array
    blocks = {"UniformsModel": S.uniforms_model(np.eye(4), np.eye(4), None, False),
              "UniformsMaterial": S.uniforms_material(False, False, False, 1.0, 0.0, [1, 1, 1, 1])}
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LEQUAL)
    draw = S.DrawSpec(rows, 32, idx, A.Shading_VertexColor, (), st, blocks)
    clear = A.ClearStates(True, True, (0.1, 0.2, 0.3, 0.4), 1.0)
    return S.Scene("quads", [S.PassSpec(w, h, 1, clear, [draw])])


def _normal_call_matches(cuda_lib, cdll, seed):
    scene = soup(3000, 200, 120, 4, [A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS)],
                 seed=seed)
    got = _noalloc_render(cdll, scene)
    want, _ = render(cuda_lib, scene)
    for key, arr in want[0].items():
        assert np.array_equal(got[key].view(np.uint8), arr.view(np.uint8)), f"after the error: {key} differs"


def test_noalloc_reports_bin_overflow_then_recovers(cuda_lib):
    cdll = _bind(cuda_lib)
    # 140 triangles x 4096 tiles = 573,440 bin entries against a fixed 262,144
    msg = _noalloc_render(cdll, _quads(70, 1024, 1024), expect=6)    # SGLC_ERR_OVERFLOW
    assert b"capacity" in msg
    _normal_call_matches(cuda_lib, cdll, 21)


def test_noalloc_reports_bad_index_then_recovers(cuda_lib):
    cdll = _bind(cuda_lib)
    msg = _noalloc_render(cdll, _quads(4, 128, 96, bad_index=True), expect=2)   # SGLC_ERR_INVALID_VALUE
    assert b"index out of range" in msg
    _normal_call_matches(cuda_lib, cdll, 22)
