"""The reference-side binding (softglrender_gb300/host/RendererCUDA.{h,cpp}) compiles against the
reference's own headers, links against the CUDA library and drives it through SoftGL::Renderer only;
on a host without a GPU the renderer reports the missing device instead of faulting. Skipped where the
reference tree is absent (as on the GPU host)."""
import os
import subprocess

import pytest

import oracle
from softglrender_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    ref = oracle.reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    lib = B.build()
    exe = str(tmp_path / "drive_renderer")
    cmd = ["g++", "-std=gnu++11", "-O1", "-w", f"-I{ref}/src", f"-I{ref}/third_party/glm",
           f"-I{ref}/third_party/stb/include", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "softglrender_gb300", "host"),
           os.path.join(ROOT, "softglrender_gb300", "host", "RendererCUDA.cpp"),
           os.path.join(ROOT, "tests", "integration", "drive_renderer.cpp"),
           f"{ref}/src/Base/Logger.cpp", f"{ref}/src/Base/ImageUtils.cpp",
           lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_binding_builds_against_reference_headers_and_reports_no_device(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 3 and "no device" in r.stdout, (r.returncode, r.stdout, r.stderr)
