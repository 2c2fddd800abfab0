"""The C++ binding RendererCUDA (softglrender_gb300/host/RendererCUDA.cpp) on real scenes.

The binding compiles only against the reference's headers, which the GPU host does not have, so the
committed traces in tests/golden/renderer_cuda_<scene>.trace.gz record the C-ABI calls it makes while
tests/integration/drive_renderer.cpp renders a scene through SoftGL::Renderer (the viewer's call
sequence, textures handed over in linear, tiled and Morton Buffer<T> layouts; "multi": three
independent scenes drawn by one multi-scene call with the binding's handles). Replaying a trace
through a library makes exactly those calls:

* on the CPU, the oracle's images from the trace equal its images from the Python harness
  (SceneInstance) and the reference-backed checker's images from the trace;
* where the reference tree is present, re-recording reproduces the committed traces;
* on the GPU, the CUDA renderer's images from the trace meet the parity bar against the oracle's."""
import gzip
import os
import sys
import tempfile

import numpy as np
import pytest

import oracle
from helpers import assert_outputs_match, render
import trace_replay as T

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_renderer_traces as M  # noqa: E402

NAMES = sorted(M.SCENES)


def _outputs(lib, name):
    return T.as_pass_outputs(T.replay(lib, T.load(M.trace_path(name))))


def _assert_identical(a, b, what):
    assert len(a) == len(b), what
    for p, (x, y) in enumerate(zip(a, b)):
        assert sorted(x) == sorted(y), (what, p, sorted(x), sorted(y))
        for k in x:
            assert x[k].dtype == y[k].dtype and x[k].shape == y[k].shape, (what, p, k)
            assert np.array_equal(x[k].view(np.uint8), y[k].view(np.uint8)), f"{what} pass {p} {k} differs"


@pytest.mark.parametrize("name", NAMES)
def test_trace_replay_equals_python_harness_on_oracle(name, oracle_lib):
    """The binding's calls render the same images as the harness's calls for the same scene."""
    from_trace = _outputs(oracle_lib, name)
    harness, _ = render(oracle_lib, M.SCENES[name]())
    assert any(np.any(o["depth"] != o["depth"].flat[0]) for o in from_trace), "nothing drawn"
    _assert_identical(from_trace, harness, name)


@pytest.mark.parametrize("name", NAMES)
def test_trace_replay_reference_equals_oracle(name, oracle_lib, reference_lib):
    _assert_identical(_outputs(reference_lib, name), _outputs(oracle_lib, name), name)


def test_traces_are_what_the_binding_records():
    ref = oracle.reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "drive_trace")
        M.build_driver(ref, exe)
        for name in NAMES:
            text = M.record(exe, name, tmp)
            with gzip.open(M.trace_path(name), "rb") as f:
                assert f.read() == text, f"{name}: committed trace differs from the binding's calls"


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_binding_trace_renders_on_gpu(name, cuda_lib, oracle_lib):
    """The calls RendererCUDA makes, run on the GB300, against the oracle: depth bit-exact, colour
    within the per-pixel bar (exact for the vertex-colour scene)."""
    gpu = _outputs(cuda_lib, name)
    cpu = _outputs(oracle_lib, name)
    assert_outputs_match(gpu, cpu, f"RendererCUDA trace {name}", exact_color=name in ("geometry_stress", "multi"))
