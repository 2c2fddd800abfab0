"""FXAA screen pass (QuadFilter + FxaaSoft.h): the CPU restatement equals the unmodified reference,
the GPU matches the restatement within the colour bar, and the pass does anti-alias (it changes
edge pixels and leaves flat regions alone)."""
import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S
from softglrender_gb300.postfx import fxaa

from helpers import assert_color_bar, render


@pytest.fixture(scope="module")
def aliased(oracle_lib):
    scene = S.config_geometry_stress(n_tris=3000, width=160, height=120, samples=1)
    outs, _ = render(oracle_lib, scene)
    return outs[-1]["color"]


@pytest.mark.parametrize("filt", [A.Filter_LINEAR, A.Filter_NEAREST])
def test_restatement_equals_reference(filt, aliased, oracle_lib, reference_lib):
    a = fxaa(A.Renderer(oracle_lib, 0), aliased, filt)
    b = fxaa(A.Renderer(reference_lib, 0), aliased, filt)
    assert np.array_equal(a, b)
    changed = np.any(a != aliased, axis=-1).mean()
    assert 0.01 < changed < 0.9


@pytest.mark.gpu
@pytest.mark.parametrize("filt", [A.Filter_LINEAR, A.Filter_NEAREST])
def test_gpu_matches_restatement(filt, aliased, cuda_lib, oracle_lib):
    g = fxaa(A.Renderer(cuda_lib, 0), aliased, filt)
    c = fxaa(A.Renderer(oracle_lib, 0), aliased, filt)
    assert_color_bar(g, c, f"fxaa filter {filt}")
