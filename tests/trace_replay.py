"""Test infrastructure: replays a trace of C-ABI calls (recorded by tests/integration/trace_abi.cpp
while the C++ binding RendererCUDA ran a scene) through any library that exports the ABI of
include/softgl_cuda.h: the CUDA renderer, the oracle restatement or the reference-backed checker.

A trace line is "<function> <argument>...", each argument tagged i:<int>, h:<handle made earlier>,
o:<handle this call makes>, s:<hex string>, b:<hex bytes>, H:<handles, comma-separated>. Handles are
renumbered through a map, so
the replay's handles need not equal the recorded ones. `replay` returns the images the trace read
back, in order, shaped like `Texture.readImage`."""
from __future__ import annotations

import ctypes as C
import gzip
from dataclasses import dataclass
from typing import List

import numpy as np

from softglrender_gb300 import api as A

# calls whose bytes argument is followed by its length in bytes (create_vertex_array: two such pairs)
_WITH_LENGTH = {"texture_set_level_data", "vertex_array_update", "uniform_block_set_sub_data",
                "uniform_block_set_data", "create_vertex_array"}


@dataclass
class ReadBack:
    width: int
    height: int
    format: int
    multi_sample: bool
    resolved: bool
    image: np.ndarray


def load(path: str) -> List[List[str]]:
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rt") as f:
        return [line.split() for line in f if line.strip()]


def _shape(desc: A._TextureDesc, level: int, resolved: bool):
    w, h = max(1, desc.width >> level), max(1, desc.height >> level)
    rgba = desc.format == A.TextureFormat_RGBA8
    if desc.multi_sample and not resolved:
        shape = (h, w, 4, 4) if rgba else (h, w, 4)
    else:
        shape = (h, w, 4) if rgba else (h, w)
    return shape, (np.uint8 if rgba else np.float32)


def replay(lib: A.Library, lines: List[List[str]], device: int = 0) -> List[ReadBack]:
    renderer = A.Renderer(lib, device)
    handles = {}
    descs = {}
    out: List[ReadBack] = []
    keep = []   # buffers alive for the duration of each call
    try:
        for toks in lines:
            name, args = toks[0], toks[1:]
            if name in ("create", "destroy"):
                continue   # the replay's own context stands in for the recorded one
            fn = lib.fn[name]
            types = fn.argtypes[1:]
            call = [renderer.ctx]
            outs = []
            keep.clear()
            if name == "texture_set_image_data":
                h, n, nbytes = handles[int(args[0][2:])], int(args[1][2:]), int(args[2][2:])
                bufs = [bytes.fromhex(a[2:]) for a in args[3:3 + n]]
                cbufs = [C.create_string_buffer(b, len(b)) for b in bufs]
                keep.extend(cbufs)
                ptrs = (C.c_void_p * n)(*[C.addressof(b) for b in cbufs])
                keep.append(ptrs)
                call += [h, n, ptrs, nbytes]
            elif name == "draw_scenes":
                arrs = [[handles[int(v)] for v in a[2:].split(",")] for a in args[:3]]
                n = int(args[3][2:])
                carr = [(C.c_int32 * n)(*x) for x in arrs]
                keep.extend(carr)
                cs = C.create_string_buffer(bytes.fromhex(args[4][2:]))
                keep.append(cs)
                call += [*carr, n, C.addressof(cs)]
            elif name == "texture_read_image":
                h = handles[int(args[0][2:])]
                layer, level, resolved, nbytes = (int(a[2:]) for a in args[1:5])
                shape, dtype = _shape(descs[h], level, bool(resolved))
                img = np.zeros(shape, dtype)
                assert img.nbytes == nbytes, (name, img.nbytes, nbytes)
                call += [h, layer, level, resolved, img.ctypes.data_as(C.c_void_p), nbytes]
                d = descs[h]
                out.append(ReadBack(d.width, d.height, d.format, bool(d.multi_sample), bool(resolved), img))
            else:
                k = 0
                for a in args:
                    tag, val = a[:1], a[2:]
                    if tag == "i":
                        call.append(int(val))
                        k += 1
                    elif tag == "h":
                        call.append(handles[int(val)])
                        k += 1
                    elif tag == "s":
                        call.append(bytes.fromhex(val))
                        k += 1
                    elif tag == "o":
                        o = C.c_int32(0)
                        outs.append((int(val), o))
                        call.append(C.byref(o))
                        k += 1
                    elif tag == "b":
                        raw = bytes.fromhex(val)
                        buf = C.create_string_buffer(raw, max(1, len(raw)))
                        keep.append(buf)
                        t = types[k]
                        if t is C.c_void_p:
                            call.append(C.addressof(buf))
                        else:
                            call.append(C.cast(buf, t))
                        k += 1
                        if name in _WITH_LENGTH:
                            call.append(len(raw))
                            k += 1
                    else:
                        raise ValueError(f"unknown argument tag in {a!r}")
            st = fn(*call)
            if st != 0:
                msg = lib.fn["last_error"](renderer.ctx)
                raise A.SoftGLError(st, lib.prefix + name, msg.decode() if msg else "")
            for recorded, o in outs:
                handles[recorded] = o.value
            if name == "create_texture":
                descs[handles[int(args[-1][2:])]] = A._TextureDesc.from_buffer_copy(bytes.fromhex(args[0][2:]))
        renderer.waitIdle()
    finally:
        renderer.destroy()
    return out


def as_pass_outputs(reads: List[ReadBack]) -> List[dict]:
    """Group read-backs into per-pass dicts (colour [+ resolved], depth), the order the driver reads
    them in, matching `SceneInstance.outputs`."""
    passes: List[dict] = []
    cur: dict = {}
    for r in reads:
        if r.format == A.TextureFormat_RGBA8:
            key = "resolved" if r.resolved else "color"
            if key == "color" and cur:
                passes.append(cur)
                cur = {}
            cur[key] = r.image
        else:
            cur["depth"] = r.image
            passes.append(cur)
            cur = {}
    if cur:
        passes.append(cur)
    return passes
