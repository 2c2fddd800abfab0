"""Golden fixtures made from the reference itself (tests/golden/make_golden.py): the scene inputs
are reproduced bit for bit on this host, and the CPU oracle reproduces the reference outputs.
The CUDA renderer is held to the same digests where its colour arithmetic is exact, and to
depth digests everywhere (gpu-marked)."""
import json
import os

import numpy as np
import pytest

from softglrender_gb300 import scenes as S

from golden.cases import CASES
from helpers import render

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "golden.json")) as f:
    GOLDEN = json.load(f)["cases"]

# shading models whose colour has no transcendental arithmetic: the GPU must match bit for bit
EXACT_COLOR = {"base_color", "geometry_stress_20k", "soup_depth_equal", "soup_blend_sub", "soup_17x13"}


def test_fixture_covers_all_cases():
    assert set(GOLDEN) == set(CASES)


@pytest.mark.parametrize("name", sorted(CASES))
def test_scene_inputs_reproducible(name):
    assert CASES[name]().input_digest() == GOLDEN[name]["input"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(name, oracle_lib):
    outs, _ = render(oracle_lib, CASES[name]())
    assert [S.output_digest(o) for o in outs] == GOLDEN[name]["outputs"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_cuda_matches_golden(name, cuda_lib):
    outs, _ = render(cuda_lib, CASES[name]())
    got = [S.output_digest(o) for o in outs]
    for g, ref in zip(got, GOLDEN[name]["outputs"]):
        assert g["depth"] == ref["depth"], f"{name}: depth differs from the reference"
        if name in EXACT_COLOR:
            assert g == ref, f"{name}: colour differs from the reference"
