"""Regenerate tests/golden/renderer_cuda_<scene>.trace.gz: the C-ABI calls the C++ binding
RendererCUDA (softglrender_gb300/host/RendererCUDA.cpp) makes when the driver
tests/integration/drive_renderer.cpp renders a scene through SoftGL::Renderer (and, for "multi", the
multi-scene call it makes with the binding's handles).

The binding and the driver are compiled against the reference's own headers (src/Render/*.h,
src/Base/Buffer.h, GLM), which only the build host has, and linked against the call recorder
tests/integration/trace_abi.cpp instead of the CUDA library. The traces are committed so that a host
without the reference tree (the GPU host) can replay exactly those calls through the CUDA renderer
(tests/trace_replay.py, tests/test_renderer_cuda_trace.py).

    python tests/golden/make_renderer_traces.py
"""
import gzip
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from softglrender_gb300 import scenes as S  # noqa: E402

# small variants of the benchmark configurations: Blinn-Phong with a mip-mapped checkerboard;
# the vertex-colour soup (clipping, reversed Z, MSAA 4x, an alpha-blended second draw); PBR+IBL with
# material maps, an irradiance cube and a prefiltered cube chain (MSAA 4x)
def multi_scene():
    """Three independent vertex-colour soups of different frame sizes (4x MSAA, reversed Z, clipped
    triangles), one pass each: the driver draws them with one multi-scene call."""
    passes = []
    for k, (n, w, h) in enumerate([(300, 40, 24), (900, 96, 48), (150, 24, 40)]):
        ps = S.config_geometry_stress(seed=2200 + k, n_tris=n, width=w, height=h, samples=4).passes[0]
        passes.append(S.PassSpec(ps.width, ps.height, ps.samples, ps.clear, [ps.draws[0]]))
    return S.Scene("multi", passes)


SCENES = {
    "plain_small": lambda: S.config_plain_small(width=192, height=144, lon=32, lat=16, tex=64),
    "geometry_stress": lambda: S.config_geometry_stress(n_tris=1200, width=160, height=96, samples=4),
    "pbr": lambda: S.config_pbr(width=160, height=96, samples=4, lon=48, lat=24, tex=64, prefilter=32,
                                irradiance=8),
    "multi": multi_scene,
}
DRIVER_ARGS = {"multi": ["multi"]}   # recorded through the multi-scene extension


def trace_path(name: str) -> str:
    return os.path.join(HERE, f"renderer_cuda_{name}.trace.gz")


def build_driver(ref: str, exe: str) -> None:
    """The binding + driver against the reference headers, linked to the call recorder."""
    inc = os.path.join(ROOT, "include")
    host = os.path.join(ROOT, "softglrender_gb300", "host")
    integ = os.path.join(ROOT, "tests", "integration")
    cmd = ["g++", "-std=gnu++11", "-O1", "-w", f"-I{ref}/src", f"-I{ref}/third_party/glm",
           f"-I{ref}/third_party/stb/include", "-I", inc, "-I", host,
           os.path.join(host, "RendererCUDA.cpp"), os.path.join(integ, "drive_renderer.cpp"),
           os.path.join(integ, "trace_abi.cpp"), f"{ref}/src/Base/Logger.cpp", f"{ref}/src/Base/ImageUtils.cpp",
           "-o", exe]
    subprocess.run(cmd, check=True)


def record(exe: str, name: str, workdir: str) -> bytes:
    """Runs the driver on one scene; returns the recorded trace text."""
    from integration import scene_file
    scene_path = os.path.join(workdir, name + ".scene")
    trace = os.path.join(workdir, name + ".trace")
    scene_file.write(SCENES[name](), scene_path)
    env = dict(os.environ, SGLC_TRACE=trace)
    r = subprocess.run([exe, scene_path, os.path.join(workdir, name + ".out"), *DRIVER_ARGS.get(name, [])], env=env,
                       capture_output=True, text=True, timeout=120)
    if r.returncode != 0:
        raise RuntimeError(f"driver failed on {name}: {r.stdout} {r.stderr}")
    with open(trace, "rb") as f:
        return f.read()


def main():
    ref = oracle.reference_tree()
    if ref is None:
        raise SystemExit("the reference tree is not available on this host")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "drive_trace")
        build_driver(ref, exe)
        for name in SCENES:
            text = record(exe, name, tmp)
            with open(trace_path(name), "wb") as f:
                f.write(gzip.compress(text, compresslevel=9, mtime=0))
            print(name, len(text), "bytes of trace,", os.path.getsize(trace_path(name)), "compressed")


if __name__ == "__main__":
    main()
