"""Points, lines and wireframe (Primitive_POINT / Primitive_LINE, PolygonMode_POINT / PolygonMode_LINE;
RendererSoft.cpp:301-321, 409-487, 575-712): the CPU restatement equals the unmodified reference
bit for bit, and the GPU path equals the restatement bit for bit (no texture filtering is involved,
so colour is exact too)."""
import copy

import numpy as np
import pytest

from softglrender_gb300 import api as A
from softglrender_gb300 import scenes as S

from helpers import assert_outputs_match, render

CASES = {
    "msaa1_blend": dict(samples=1, blend=True),
    "msaa1_noblend": dict(samples=1, blend=False),
    "msaa4_blend": dict(samples=4, blend=True),
    "nocull_dense": dict(samples=1, cull=False, lon=40, lat=20, segments=80),
}


def _scene(name):
    return S.config_lines(**CASES[name])


def _draw_only(scene, k):
    s = copy.deepcopy(scene)
    s.passes[0].draws = [scene.passes[0].draws[k]]
    return s


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_equals_reference(name, oracle_lib, reference_lib):
    scene = _scene(name)
    a, _ = render(oracle_lib, scene)
    b, _ = render(reference_lib, scene)
    assert_outputs_match(a, b, name, exact_color=True)


def test_every_draw_draws(oracle_lib, reference_lib):
    """Each of the six draws changes pixels on its own, and equals the reference on its own."""
    scene = _scene("msaa1_noblend")
    bg = render(oracle_lib, S.Scene("bg", [S.PassSpec(640, 400, 1, scene.passes[0].clear, [])]))[0][0]["color"]
    for k in range(6):
        s = _draw_only(scene, k)
        a, _ = render(oracle_lib, s)
        b, _ = render(reference_lib, s)
        assert_outputs_match(a, b, f"draw {k}", exact_color=True)
        assert np.any(a[0]["color"] != bg), f"draw {k} drew nothing"


def test_wireframe_equals_reference(oracle_lib, reference_lib):
    scene = S.config_wireframe(width=480, height=270, lon=96, lat=48)
    a, _ = render(oracle_lib, scene)
    b, _ = render(reference_lib, scene)
    assert_outputs_match(a, b, "wireframe", exact_color=True)
    assert (a[0]["depth"] < 1.0).sum() > 2000


def _points_scene(repeats, size, width=64, height=48):
    rows = np.zeros((1, 16), np.float32)   # one vertex at the origin, identity MVP: the frame centre
    blocks = {"UniformsModel": S.uniforms_model(np.eye(4), np.eye(4), None, False),
              "UniformsMaterial": S.uniforms_material(False, False, False, size, 0.0, [1, 0, 0, 1])}
    d = S.DrawSpec(rows, 64, np.zeros(repeats, np.int32), A.Shading_BaseColor, (),
                   A.RenderStates(primitiveType=A.Primitive_POINT), blocks)
    return S.Scene("points", [S.PassSpec(width, height, 1, A.ClearStates(True, True, (0, 0, 0, 1), 1.0), [d])])


@pytest.mark.parametrize("repeats,size", [(1, 10.0), (4, 10.0), (3, 1.0), (5, 2.5)])
def test_repeated_point_walks(repeats, size, oracle_lib, reference_lib):
    """A stamp leaves the vertex at its last pixel (the reference loops on fragPos), so drawing the
    same index again starts from there: a size-10 point repeated n times covers a diagonal run of
    n stamps 4 pixels apart."""
    scene = _points_scene(repeats, size)
    a, _ = render(oracle_lib, scene)
    b, _ = render(reference_lib, scene)
    assert_outputs_match(a, b, "points", exact_color=True)
    red = a[0]["color"][..., 0] == 255
    if size == 10.0:
        ys, xs = np.nonzero(red)
        # first stamp at [27, 37) x [19, 29); each repeat moves by +4 in x and y
        assert xs.min() == 27 and ys.min() == 19
        assert xs.max() == 36 + 4 * (repeats - 1) and ys.max() == 28 + 4 * (repeats - 1)


def test_derivative_sampler_refused(oracle_lib):
    """A line draw whose shader would take a texture LOD from derivatives is refused (the reference
    has no derivative context outside the triangle quads)."""
    scene = S.config_plain_small(width=64, height=48, lon=8, lat=4, tex=16)
    scene.passes[0].draws[0].states = A.RenderStates(depthTest=True, polygonMode=A.PolygonMode_LINE)
    with pytest.raises(A.SoftGLError) as e:
        render(oracle_lib, scene)
    assert e.value.status == A.SGLC_ERR_UNSUPPORTED


# ---- GPU -----------------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_restatement(name, cuda_lib, oracle_lib):
    scene = _scene(name)
    g, _ = render(cuda_lib, scene)
    c, _ = render(oracle_lib, scene)
    assert_outputs_match(g, c, name, exact_color=True)


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [1, 4])
def test_gpu_wireframe_full_size(samples, cuda_lib, oracle_lib):
    """The viewer's wireframe mode on the 200k-triangle benchmark sphere at 1080p."""
    scene = S.config_wireframe(samples=samples)
    g, st = render(cuda_lib, scene)
    c, _ = render(oracle_lib, scene)
    assert_outputs_match(g, c, "wireframe", exact_color=True)
    assert st["bin_entries"] > 100000


@pytest.mark.gpu
@pytest.mark.parametrize("repeats,size", [(1, 10.0), (4, 10.0), (3, 1.0), (5, 2.5)])
def test_gpu_repeated_point_walks(repeats, size, cuda_lib, oracle_lib):
    scene = _points_scene(repeats, size)
    g, _ = render(cuda_lib, scene)
    c, _ = render(oracle_lib, scene)
    assert_outputs_match(g, c, "points", exact_color=True)


@pytest.mark.gpu
def test_gpu_derivative_sampler_refused(cuda_lib):
    scene = S.config_plain_small(width=64, height=48, lon=8, lat=4, tex=16)
    scene.passes[0].draws[0].states = A.RenderStates(depthTest=True, polygonMode=A.PolygonMode_LINE)
    with pytest.raises(A.SoftGLError) as e:
        render(cuda_lib, scene)
    assert e.value.status == A.SGLC_ERR_UNSUPPORTED
