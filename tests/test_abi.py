"""The C-ABI boundary: every entry point include/softgl_cuda.h declares is exported by the CUDA
library, by the CPU oracle and by the reference-backed checker, with identical names modulo the
prefix; on a host without a GPU the CUDA library loads and refuses to create a context with
SGLC_ERR_NO_DEVICE (no compute is attempted)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "softgl_cuda.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"SGLC_API\s+[\w\s\*]+?\b(sglc_\w+)\s*\(", text)))


# product-only extensions (no Renderer counterpart): not exported by the checkers; the allocation-free
# draw is bound by its own test, the neural shader by softglrender_gb300/neural.py, CUDA graphs by
# softglrender_gb300/graph.py
PRODUCT_ONLY = {"sglc_draw_vertex_color_noalloc"}


def neural_abi():
    return [n for n in declared() if n.startswith("sglc_neural_") or n == "sglc_program_set_neural_shader"]


def graph_abi():
    return [n for n in declared() if n.startswith("sglc_graph_")]


def renderer_abi():
    return [n for n in declared() if n not in PRODUCT_ONLY and n not in neural_abi() and n not in graph_abi()]


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_header_declares_the_renderer_interface():
    names = declared()
    # Renderer (Renderer.h:26-58) + resource sub-interfaces
    for fn in ("create", "destroy", "create_framebuffer", "create_texture", "create_vertex_array",
               "create_shader_program", "create_pipeline_states", "create_uniform_block", "create_uniform_sampler",
               "begin_render_pass", "set_viewport", "set_vertex_array", "set_shader_program",
               "set_shader_resources", "set_pipeline_states", "draw", "end_render_pass", "wait_idle"):
        assert "sglc_" + fn in names
    assert len(names) >= 40


def test_cuda_library_exports_every_symbol():
    from softglrender_gb300 import build
    lib = build.build()
    missing = [n for n in declared() if n not in exported(lib)]
    assert not missing, missing


def test_python_binding_covers_every_symbol():
    from softglrender_gb300.api import ABI_FUNCTIONS
    from softglrender_gb300.neural import NEURAL_FUNCTIONS
    assert sorted("sglc_" + n for n in ABI_FUNCTIONS) == renderer_abi()
    assert sorted("sglc_" + n for n in NEURAL_FUNCTIONS) == sorted(neural_abi())
    from softglrender_gb300.graph import GRAPH_FUNCTIONS
    assert sorted("sglc_" + n for n in GRAPH_FUNCTIONS) == sorted(graph_abi())


def test_oracle_exports_same_abi(oracle_lib):
    ex = exported(oracle_lib.cdll._name)
    missing = [n for n in renderer_abi() if n.replace("sglc_", "sglo_") not in ex]
    assert not missing, missing


def test_reference_checker_exports_same_abi(reference_lib):
    ex = exported(reference_lib.cdll._name)
    missing = [n for n in renderer_abi() if n.replace("sglc_", "sglr_") not in ex]
    assert not missing, missing


def test_no_device_is_reported_not_faulted():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from softglrender_gb300 import build
    lib = ctypes.CDLL(build.build())
    ctx = ctypes.c_void_p()
    lib.sglc_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32]
    assert lib.sglc_create(ctypes.byref(ctx), 0) == 7   # SGLC_ERR_NO_DEVICE
    assert not ctx.value
