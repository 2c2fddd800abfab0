"""The synthetic-scene harness: layouts of the reference structs and deterministic generation."""
import numpy as np

from softglrender_gb300 import scenes as S


def test_uniform_block_sizes_match_reference_layout():
    # sizes probed from the reference with GLM aligned types (vec3 = 16 B, mat3 = 48 B)
    assert len(S.uniforms_model(np.eye(4), np.eye(4), None, False)) == 256
    assert len(S.uniforms_scene([0] * 3, [0] * 3, [0] * 3, [0] * 3)) == 64
    assert len(S.uniforms_material(1, 0, 0, 1.0, 0.5, [1, 1, 1, 1])) == 48


def test_vertex_layout_is_view_vertex():
    v, i = S.uv_sphere(8, 4)
    assert v.dtype == np.float32 and v.shape[1] == 16     # View::Vertex, 64 B
    assert i.dtype == np.int32 and i.size % 3 == 0
    assert i.max() < v.shape[0]
    # unit sphere, unit normals
    assert np.allclose(np.linalg.norm(v[:, 0:3], axis=1), 1.0, atol=1e-6)
    assert np.allclose(np.linalg.norm(v[:, 8:11], axis=1), 1.0, atol=1e-6)


def test_uv_sphere_triangle_count():
    _, i = S.uv_sphere(64, 32)
    assert i.size // 3 == 64 * 30 * 2 + 2 * 64


def test_deterministic_math_is_accurate():
    x = np.linspace(-20, 20, 1001)
    assert np.max(np.abs(S.det_sin(x) - np.sin(x))) < 1e-12
    assert np.max(np.abs(S.det_cos(x) - np.cos(x))) < 1e-12
    y = np.linspace(-30, 30, 1001)
    assert np.max(np.abs(S.det_exp(y) / np.exp(y) - 1)) < 1e-13
    z = np.logspace(-20, 20, 1001)
    assert np.max(np.abs(S.det_log(z) - np.log(z))) < 1e-12


def test_generation_is_pure():
    a = S.config_geometry_stress(n_tris=500, width=64, height=48).input_digest()
    b = S.config_geometry_stress(n_tris=500, width=64, height=48).input_digest()
    assert a == b


def test_cube_face_dirs_round_trip():
    # directions of a face's texel centres map back to that face (SamplerSoft.h:311-373)
    for face in range(6):
        d = S.cube_face_dirs(face, 4)
        ax = np.abs(d)
        major = np.argmax(ax, axis=-1)
        expect_axis = face // 2
        assert (major == expect_axis).all()
