"""Headless scene harness: seeded synthetic scenes driven through the Renderer call sequence.

This replaces the interactive viewer (src/Viewer/Viewer.cpp:100-141) with a script that builds
meshes, textures and uniform blocks and then issues exactly the calls Viewer::drawFrame /
Viewer::pipelineDraw issue (Viewer.cpp:388-396): beginRenderPass, setViewPort, then per mesh
setVertexArrayObject / setShaderProgram / setShaderResources / setPipelineStates / draw.

Determinism across machines: every generator below uses integer hashing (splitmix64) and
float64 arithmetic restricted to +, -, *, /, sqrt, floor, frexp and ldexp, which IEEE-754 fixes
bit for bit; sin/cos/exp/log are our own polynomial evaluations. The bytes of a scene are
therefore identical on any host, so fixtures pinned on one machine check outputs on another.

Layouts follow the reference with GLM aligned types (vec3 = 16 B): View::Vertex 64 B
(src/Viewer/Model.h:20-25), UniformsModel 256 B / UniformsScene 64 B / UniformsMaterial 48 B
(src/Viewer/Material.h:63-85). Matrices are column-major like glm::mat4.
"""
from __future__ import annotations

import functools
import hashlib
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import api as A

# ------------------------------------------------------------------------------------------------
# deterministic math (float64)
# ------------------------------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_TWO_PI_HI = 6.28318530717958623200e+00
_TWO_PI_LO = 2.44929359829470635445e-16
_LN2_HI = 6.93147180369123816490e-01
_LN2_LO = 1.90821492927058770002e-10


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def hash_u01(seed: int, stream: int, idx) -> np.ndarray:
    """Uniform [0,1) float64 values, a pure function of (seed, stream, index)."""
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed * 0x10001 + stream) * np.uint64(0x632BE59BD9B4E019) + idx)
    return (key >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def det_sin(x):
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x / _TWO_PI_HI + 0.5)
    r = (x - k * _TWO_PI_HI) - k * _TWO_PI_LO
    r2 = r * r
    term = r.copy()
    acc = r.copy()
    for n in range(1, 18):
        term = term * (-r2) / ((2 * n) * (2 * n + 1))
        acc = acc + term
    return acc


def det_cos(x):
    return det_sin(np.asarray(x, dtype=np.float64) + np.pi / 2)


def det_exp(x):
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x / _LN2_HI + 0.5)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    term = np.ones_like(r)
    acc = np.ones_like(r)
    for n in range(1, 22):
        term = term * r / n
        acc = acc + term
    return np.ldexp(acc, k.astype(np.int64))


def det_log(x):
    x = np.asarray(x, dtype=np.float64)
    m, e = np.frexp(x)
    s = (m - 1.0) / (m + 1.0)
    s2 = s * s
    acc = np.zeros_like(s)
    p = s.copy()
    for n in range(0, 40):
        acc = acc + p / (2 * n + 1)
        p = p * s2
    return 2.0 * acc + e * _LN2_HI + e * _LN2_LO


def dot3(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def normalize(v):
    n = np.sqrt(dot3(v, v))[..., None]
    return v / np.where(n > 0, n, 1.0)


def mm4(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """4x4 product with a fixed summation order (no BLAS)."""
    out = np.zeros((4, 4))
    for i in range(4):
        for j in range(4):
            out[i, j] = ((a[i, 0] * b[0, j] + a[i, 1] * b[1, j]) + a[i, 2] * b[2, j]) + a[i, 3] * b[3, j]
    return out


def mv4(m: np.ndarray, v: np.ndarray) -> np.ndarray:
    """m (4x4) applied to row vectors v (..., 4) with a fixed summation order."""
    return np.stack([((m[i, 0] * v[..., 0] + m[i, 1] * v[..., 1]) + m[i, 2] * v[..., 2]) + m[i, 3] * v[..., 3]
                     for i in range(4)], axis=-1)


def cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def value_noise3(p: np.ndarray, seed: int, octaves: int = 4) -> np.ndarray:
    """Fractal value noise in [-1, 1] at points p (..., 3); smoothstep-interpolated lattice hash."""
    total = np.zeros(p.shape[:-1])
    amp, freq, norm = 1.0, 2.0, 0.0
    for o in range(octaves):
        q = p * freq
        i = np.floor(q)
        f = q - i
        u = f * f * (3.0 - 2.0 * f)
        ii = i.astype(np.int64) + 1024
        acc = np.zeros(p.shape[:-1])
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    key = ((ii[..., 0] + dx) * 73856093) ^ ((ii[..., 1] + dy) * 19349663) ^ ((ii[..., 2] + dz) * 83492791)
                    h = hash_u01(seed, 100 + o, key.astype(np.uint64) & np.uint64(0xFFFFFFFF)) * 2.0 - 1.0
                    wx = u[..., 0] if dx else 1.0 - u[..., 0]
                    wy = u[..., 1] if dy else 1.0 - u[..., 1]
                    wz = u[..., 2] if dz else 1.0 - u[..., 2]
                    acc = acc + h * wx * wy * wz
        total = total + amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


# ------------------------------------------------------------------------------------------------
# camera / matrices (Camera.cpp:26-69 conventions)
# ------------------------------------------------------------------------------------------------
def perspective(fov_rad: float, aspect: float, near: float, reverse_z: bool, far: Optional[float] = None):
    """Camera::projectionMatrix (Camera.cpp:26-44): infinite far plane; optional finite far."""
    t = 1.0 / (det_sin(fov_rad * 0.5) / det_cos(fov_rad * 0.5))
    P = np.zeros((4, 4))
    P[0, 0] = t / aspect
    P[1, 1] = t
    P[3, 2] = -1.0
    if far is None:
        if reverse_z:
            P[2, 2], P[2, 3] = 0.0, near
        else:
            P[2, 2], P[2, 3] = -1.0, -near
    else:
        if reverse_z:
            P[2, 2], P[2, 3] = near / (far - near), near * far / (far - near)
        else:
            P[2, 2], P[2, 3] = -far / (far - near), -near * far / (far - near)
    return P


def look_at(eye, center, up):
    """Camera::viewMatrix (Camera.cpp:46-69)."""
    eye, center, up = (np.asarray(v, dtype=np.float64) for v in (eye, center, up))
    f = normalize(center - eye)
    s = normalize(cross(f, up))
    u = cross(s, f)
    V = np.eye(4)
    V[0, :3], V[0, 3] = s, -dot3(s, eye)
    V[1, :3], V[1, 3] = u, -dot3(u, eye)
    V[2, :3], V[2, 3] = -f, dot3(f, eye)
    return V


def ortho(half_w, half_h, near, far):
    P = np.eye(4)
    P[0, 0] = 1.0 / half_w
    P[1, 1] = 1.0 / half_h
    P[2, 2] = -1.0 / (far - near)      # z_ndc in [0,1] over [near, far]
    P[2, 3] = -near / (far - near)
    return P


def mat4_bytes(M: np.ndarray) -> bytes:
    return np.ascontiguousarray(M.T.astype(np.float32)).tobytes()      # column-major (glm)


def mat3_bytes(M3: np.ndarray) -> bytes:
    out = np.zeros((3, 4), dtype=np.float32)
    out[:, :3] = M3.T.astype(np.float32)                               # 3 columns, vec3 padded to 16 B
    return out.tobytes()


def vec3_bytes(v) -> bytes:
    return struct.pack("<4f", float(v[0]), float(v[1]), float(v[2]), 0.0)


def uniforms_model(model: np.ndarray, mvp: np.ndarray, shadow_mvp: Optional[np.ndarray], reverse_z: bool) -> bytes:
    """UniformsModel (Material.h:70-76), 256 B."""
    if np.any(model[:3, :3] != np.eye(3)):
        raise ValueError("only rigid-identity model matrices are used by the synthetic scenes")
    it = np.eye(3)
    b = struct.pack("<I12x", int(reverse_z)) + mat4_bytes(model) + mat4_bytes(mvp) + mat3_bytes(it)
    b += mat4_bytes(shadow_mvp if shadow_mvp is not None else np.eye(4))
    assert len(b) == 256
    return b


def uniforms_scene(ambient, camera_pos, light_pos, light_color) -> bytes:
    """UniformsScene (Material.h:63-68), 64 B."""
    b = vec3_bytes(ambient) + vec3_bytes(camera_pos) + vec3_bytes(light_pos) + vec3_bytes(light_color)
    assert len(b) == 64
    return b


def uniforms_material(enable_light, enable_ibl, enable_shadow, point_size, k_specular, base_color) -> bytes:
    """UniformsMaterial (Material.h:78-85), 48 B."""
    b = struct.pack("<3I2f12x4f", int(enable_light), int(enable_ibl), int(enable_shadow), point_size, k_specular,
                    *[float(c) for c in base_color])
    assert len(b) == 48
    return b


# ------------------------------------------------------------------------------------------------
# meshes
# ------------------------------------------------------------------------------------------------
def uv_sphere(lon: int, lat: int, radius: float = 1.0, displace_seed: Optional[int] = None,
              amplitude: float = 0.1) -> Tuple[np.ndarray, np.ndarray]:
    """UV sphere as View::Vertex rows (16 float32: pos.xyz_, uv.xy, normal.xyz_, tangent.xyz_) and
    int32 indices, counter-clockwise seen from outside. Pole bands carry one triangle per segment.
    With displace_seed the radius is modulated by 4-octave value noise (amplitude) and normals are
    re-derived from the displaced surface."""
    j = np.arange(lat + 1, dtype=np.float64)[:, None]
    i = np.arange(lon + 1, dtype=np.float64)[None, :]
    theta = j * (np.pi / lat)          # 0 at +y pole
    phi = i * (2.0 * np.pi / lon)
    st, ct = det_sin(theta), det_cos(theta)
    sp, cp = det_sin(phi), det_cos(phi)
    dirs = np.stack([st * sp + 0.0 * cp, ct + 0.0 * sp, st * cp + 0.0 * sp], axis=-1)   # (lat+1, lon+1, 3)
    r = np.full(dirs.shape[:2], radius)
    if displace_seed is not None:
        r = radius + amplitude * value_noise3(dirs * 1.5, displace_seed)
    pos = dirs * r[..., None]
    uv = np.stack([np.broadcast_to(i / lon, r.shape), np.broadcast_to(j / lat, r.shape)], axis=-1)
    zero = 0.0 * st * cp
    tangent = np.stack([cp + zero, zero, -sp + zero], axis=-1)
    if displace_seed is None:
        normal = dirs
    else:
        # central differences over the (theta, phi) grid, wrapping in phi
        dphi = np.roll(pos[:, :-1], -1, axis=1) - np.roll(pos[:, :-1], 1, axis=1)
        dphi = np.concatenate([dphi, dphi[:, :1]], axis=1)
        dth = np.zeros_like(pos)
        dth[1:-1] = pos[2:] - pos[:-2]
        n = normalize(cross(dth, dphi))
        n[0], n[-1] = dirs[0], dirs[-1]
        flip = (dot3(n, dirs) < 0)[..., None]
        normal = np.where(flip, -n, n)
    nv = (lat + 1) * (lon + 1)
    vert = np.zeros((nv, 16), dtype=np.float32)
    vert[:, 0:3] = pos.reshape(-1, 3)
    vert[:, 4:6] = uv.reshape(-1, 2)
    vert[:, 8:11] = normal.reshape(-1, 3)
    vert[:, 12:15] = tangent.reshape(-1, 3)
    idx = []
    row = lon + 1
    for jj in range(lat):
        a = jj * row + np.arange(lon)
        b = a + row
        if jj != 0:
            idx.append(np.stack([a, b, a + 1], axis=-1))
        if jj != lat - 1:
            idx.append(np.stack([a + 1, b, b + 1], axis=-1))
    indices = np.concatenate(idx, axis=0).astype(np.int32).reshape(-1)
    return vert, indices


def triangle_soup(n_tris: int, seed: int, view_proj: np.ndarray, width: int, height: int,
                  median_px: float = 20.0, sigma: float = 1.5) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Random soup for the geometry-stress scene: triangle centres uniform in [-1,1]^3, each
    triangle sized for a log-normal screen area (median, sigma) at its centre's depth. Returns the
    vertex rows (8 float32: pos.xyz_, rgba), int32 indices and a per-triangle opaque flag."""
    t = np.arange(n_tris, dtype=np.uint64)
    c = np.stack([hash_u01(seed, k, t) * 2.0 - 1.0 for k in range(3)], axis=-1)
    u1 = np.maximum(hash_u01(seed, 3, t), 1e-12)
    u2 = hash_u01(seed, 4, t)
    z = np.sqrt(-2.0 * det_log(u1)) * det_cos(2.0 * np.pi * u2)
    area_px = median_px * det_exp(sigma * z)
    clip_c = mv4(view_proj, np.concatenate([c, np.ones((n_tris, 1))], axis=1))
    w = np.abs(clip_c[:, 3]) + 1e-3
    px_world = 2.0 * w / (view_proj[1, 1] * height)          # world length of one pixel at depth w
    edge = np.sqrt(2.3 * area_px) * px_world                 # equilateral-ish triangle of that area
    verts = np.zeros((n_tris, 3, 3))
    for v in range(3):
        d = np.stack([hash_u01(seed, 10 + 3 * v + k, t) * 2.0 - 1.0 for k in range(3)], axis=-1)
        verts[:, v] = c + normalize(d) * (edge[:, None] * 0.66)
    opaque = hash_u01(seed, 20, t) < 0.5
    rgb = np.stack([hash_u01(seed, 21 + k, t) for k in range(3)], axis=-1)
    alpha = np.where(opaque, 1.0, 0.5)
    rows = np.zeros((n_tris * 3, 8), dtype=np.float32)
    rows[:, 0:3] = verts.reshape(-1, 3)
    rows[:, 4:7] = np.repeat(rgb, 3, axis=0)
    rows[:, 7] = np.repeat(alpha, 3)
    indices = np.arange(n_tris * 3, dtype=np.int32)
    return rows, indices, opaque


# ------------------------------------------------------------------------------------------------
# textures
# ------------------------------------------------------------------------------------------------
def checkerboard(size: int, cells: int, seed: int) -> np.ndarray:
    c = np.floor(hash_u01(seed, 200, np.arange(6)) * 256.0).astype(np.uint8).reshape(2, 3)
    y, x = np.mgrid[0:size, 0:size]
    cell = size // cells
    parity = ((x // cell) + (y // cell)) % 2
    img = np.zeros((size, size, 4), dtype=np.uint8)
    img[..., :3] = c[parity]
    img[..., 3] = 255
    return img


@functools.lru_cache(maxsize=None)
def noise_texture(size: int, seed: int, kind: str) -> np.ndarray:
    """Seeded procedural material map (RGBA8). Memoised per process (the 1024^2 maps take seconds to
    make); the returned array is read-only."""
    img = _noise_texture(size, seed, kind)
    img.setflags(write=False)
    return img


def _noise_texture(size: int, seed: int, kind: str) -> np.ndarray:
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    u, v = (x + 0.5) / size, (y + 0.5) / size
    # periodic sampling on a torus so REPEAT is seamless
    p = np.stack([det_cos(2 * np.pi * u) * 1.3, det_sin(2 * np.pi * u) * 1.3, det_cos(2 * np.pi * v) * 1.3 +
                  det_sin(2 * np.pi * v) * 0.7], axis=-1)
    img = np.zeros((size, size, 4), dtype=np.uint8)
    img[..., 3] = 255
    if kind == "albedo":
        for ch in range(3):
            n = value_noise3(p + ch * 3.1, seed + ch, octaves=4)
            img[..., ch] = np.clip(np.floor((0.5 + 0.45 * n) * 255.0), 0, 255).astype(np.uint8)
    elif kind == "normal":
        h = value_noise3(p, seed, octaves=4)
        gx = np.roll(h, -1, axis=1) - np.roll(h, 1, axis=1)
        gy = np.roll(h, -1, axis=0) - np.roll(h, 1, axis=0)
        n = normalize(np.stack([-gx * 4.0, -gy * 4.0, np.ones_like(h)], axis=-1))
        img[..., :3] = np.clip(np.floor((n * 0.5 + 0.5) * 255.0), 0, 255).astype(np.uint8)
    elif kind == "metal_rough":
        rough = 0.05 + 0.95 * (0.5 + 0.5 * value_noise3(p, seed, octaves=3))
        metal = (value_noise3(p + 7.7, seed + 1, octaves=2) > 0.1).astype(np.float64)
        img[..., 0] = 255
        img[..., 1] = np.clip(np.floor(rough * 255.0), 0, 255).astype(np.uint8)
        img[..., 2] = np.clip(np.floor(metal * 255.0), 0, 255).astype(np.uint8)
    else:
        raise ValueError(kind)
    return img


def cube_face_dirs(face: int, size: int) -> np.ndarray:
    """World directions of the texel centres of one cube face, inverting the face selection of
    BaseSamplerCube::convertXYZ2UV (SamplerSoft.h:311-373)."""
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    uc = (x + 0.5) / size * 2.0 - 1.0
    vc = -((y + 0.5) / size * 2.0 - 1.0)          # the sampler flips v
    one = np.ones_like(uc)
    d = {0: (one, vc, -uc), 1: (-one, vc, uc), 2: (uc, one, -vc), 3: (uc, -one, vc),
         4: (uc, vc, one), 5: (-uc, vc, -one)}[face]
    return normalize(np.stack(d, axis=-1))


def sky_radiance(d: np.ndarray, suns: np.ndarray, width: float) -> np.ndarray:
    """Gradient sky plus sun lobes exp((cos - 1) / width); `width` grows with the prefilter level."""
    up = np.clip(d[..., 1], -1.0, 1.0)
    base = np.stack([0.25 + 0.35 * (up * 0.5 + 0.5), 0.30 + 0.40 * (up * 0.5 + 0.5), 0.45 + 0.45 * (up * 0.5 + 0.5)],
                    axis=-1)
    col = base.copy()
    colors = np.array([[1.0, 0.85, 0.6], [0.6, 0.7, 1.0], [1.0, 0.5, 0.4]])
    for k, s in enumerate(suns):
        cosang = dot3(d, s)
        col = col + colors[k][None, None] * det_exp((cosang - 1.0) / width)[..., None] * 0.8
    return col


@functools.lru_cache(maxsize=None)
def ibl_maps(seed: int, prefilter_size: int, irradiance_size: int, levels: int = 5, variant: int = 0):
    """(prefiltered specular chain, irradiance faces) of a seeded environment; memoised per
    process, read-only arrays. `variant` k > 0 rotates the RGB channels k places (another
    environment of the same shape: a differently tinted sky)."""
    pre, irr = _ibl_maps(seed, prefilter_size, irradiance_size, levels)
    if variant % 3:
        k = variant % 3

        def rot(img):
            out = img.copy()
            out[..., :3] = np.roll(img[..., :3], k, axis=-1)
            return out
        pre = [[rot(x) for x in lev] for lev in pre]
        irr = [rot(x) for x in irr]
    for img in [x for lev in pre for x in lev] + list(irr):
        img.setflags(write=False)
    return pre, irr


def _ibl_maps(seed: int, prefilter_size: int, irradiance_size: int, levels: int = 5):
    suns = normalize(np.stack([hash_u01(seed, 300 + k, np.arange(3)) * 2.0 - 1.0 for k in range(3)], axis=-1) +
                     np.array([0.0, 0.6, 0.0]))

    def face_img(face, size, width, scale):
        rad = sky_radiance(cube_face_dirs(face, size), suns, width) * scale
        img = np.zeros((size, size, 4), dtype=np.uint8)
        img[..., :3] = np.clip(np.floor(np.clip(rad, 0.0, 1.0) * 255.0), 0, 255).astype(np.uint8)
        img[..., 3] = 255
        return img

    prefilter = []   # [level][face]
    nlev = int(np.floor(np.log2(prefilter_size))) + 1
    for lev in range(nlev):
        size = max(1, prefilter_size >> lev)
        width = 0.01 * (4.0 ** min(lev, levels))
        prefilter.append([face_img(f, size, width, 0.8) for f in range(6)])
    irradiance = [face_img(f, irradiance_size, 2.0, 0.7) for f in range(6)]
    return prefilter, irradiance


# ------------------------------------------------------------------------------------------------
# scene description + the Viewer-like call sequence
# ------------------------------------------------------------------------------------------------
@dataclass
class TextureSpec:
    name: str                      # uniform sampler name (e.g. "u_albedoMap")
    desc: A.TextureDesc
    sampler: A.SamplerDesc
    layers: Optional[List[np.ndarray]] = None           # level-0 image per layer (setImageData)
    levels: Optional[List[List[np.ndarray]]] = None     # explicit [level][layer] images


@dataclass
class DrawSpec:
    vertexes: np.ndarray           # float32 rows
    stride: int
    indices: np.ndarray
    shading: int
    defines: Tuple[str, ...]
    states: A.RenderStates
    blocks: Dict[str, bytes]       # uniform block name -> bytes
    textures: List[TextureSpec] = field(default_factory=list)


@dataclass
class PassSpec:
    width: int
    height: int
    samples: int                   # 1 or 4
    clear: A.ClearStates
    draws: List[DrawSpec]
    color: bool = True
    depth: bool = True


@dataclass
class Scene:
    name: str
    passes: List[PassSpec]
    meta: Dict[str, object] = field(default_factory=dict)

    def input_digest(self) -> str:
        h = hashlib.sha256()
        for p in self.passes:
            h.update(struct.pack("<4i", p.width, p.height, p.samples, int(p.color)))
            h.update(repr((p.clear.depthFlag, p.clear.colorFlag, tuple(p.clear.clearColor), p.clear.clearDepth)).encode())
            for d in p.draws:
                h.update(repr((d.shading, tuple(d.defines), d.stride, d.states)).encode())
                for t in d.textures:
                    h.update(repr((t.name, t.desc, t.sampler)).encode())
                h.update(np.ascontiguousarray(d.vertexes).tobytes())
                h.update(np.ascontiguousarray(d.indices).tobytes())
                for k in sorted(d.blocks):
                    h.update(k.encode() + d.blocks[k])
                for t in d.textures:
                    for img in (t.layers or []):
                        h.update(np.ascontiguousarray(img).tobytes())
                    for lev in (t.levels or []):
                        for img in lev:
                            h.update(np.ascontiguousarray(img).tobytes())
        return h.hexdigest()[:16]

    @property
    def triangles(self) -> int:
        return sum(len(d.indices) // 3 for p in self.passes for d in p.draws)


_BLOCK_KEYS = {"UniformsScene": 0, "UniformsModel": 1, "UniformsMaterial": 2}   # UniformBlockType


class SceneInstance:
    """Resources of a Scene created on one Renderer; `render()` issues the frame's calls."""

    def __init__(self, renderer: A.Renderer, scene: Scene, layout: int = A.Layout_Linear):
        self.r = renderer
        self.scene = scene
        self.fbos = []
        self.color_tex = []
        self.depth_tex = []
        self.draws = []
        tex_cache: Dict[int, A.Texture] = {}
        for p in scene.passes:
            fbo = renderer.createFrameBuffer(offscreen=True)
            ct = dt = None
            if p.color:
                ct = renderer.createTexture(A.TextureDesc(p.width, p.height, A.TextureType_2D, A.TextureFormat_RGBA8,
                                                          A.TextureUsage_AttachmentColor | A.TextureUsage_RendererOutput,
                                                          False, p.samples > 1))
                ct.initImageData()
                fbo.setColorAttachment(ct, 0)
            if p.depth:
                dt = renderer.createTexture(A.TextureDesc(p.width, p.height, A.TextureType_2D, A.TextureFormat_FLOAT32,
                                                          A.TextureUsage_AttachmentDepth, False, p.samples > 1))
                dt.initImageData()
                fbo.setDepthAttachment(dt)
            self.fbos.append(fbo)
            self.color_tex.append(ct)
            self.depth_tex.append(dt)
            objs = []
            for d in p.draws:
                vao = renderer.createVertexArrayObject(d.vertexes, d.stride, d.indices)
                prog = renderer.createShaderProgram()
                prog.addDefines(d.defines)
                prog.SetShaders(d.shading)
                res = renderer.createShaderResources()
                for name, data in d.blocks.items():
                    ub = renderer.createUniformBlock(name, len(data))
                    ub.setData(data)
                    res.setBlock(_BLOCK_KEYS.get(name, 10 + len(res.blocks)), ub)
                for k, ts in enumerate(d.textures):
                    key = id(ts)
                    tex = tex_cache.get(key)
                    if tex is None:
                        desc = A.TextureDesc(**{**ts.desc.__dict__})
                        if desc.layout == A.Layout_Linear:
                            desc.layout = layout
                        tex = renderer.createTexture(desc)
                        tex.setSamplerDesc(ts.sampler)
                        if ts.levels is not None:
                            tex.initImageData()
                            for lev, imgs in enumerate(ts.levels):
                                for layer, img in enumerate(imgs):
                                    tex.setLevelData(layer, lev, img)
                        else:
                            tex.setImageData(ts.layers)
                        tex_cache[key] = tex
                    us = renderer.createUniformSampler(ts.name, ts.desc)
                    us.setTexture(tex)
                    res.setSampler(k, us)
                ps = renderer.createPipelineStates(d.states)
                objs.append((vao, prog, res, ps))
            self.draws.append(objs)

    def render(self, after_draw=None) -> None:
        """The frame's calls; `after_draw(pass_index, draw_index)`, when given, runs after each draw
        (e.g. to read that draw's statistics)."""
        for pi, (p, fbo, objs) in enumerate(zip(self.scene.passes, self.fbos, self.draws)):
            self.r.beginRenderPass(fbo, p.clear)
            self.r.setViewPort(0, 0, p.width, p.height)
            for di, (vao, prog, res, ps) in enumerate(objs):
                self.r.setVertexArrayObject(vao)
                self.r.setShaderProgram(prog)
                self.r.setShaderResources(res)
                self.r.setPipelineStates(ps)
                self.r.draw()
                if after_draw is not None:
                    after_draw(pi, di)
            self.r.endRenderPass()

    def outputs(self, pass_index: int = -1) -> Dict[str, np.ndarray]:
        p = self.scene.passes[pass_index]
        out = {}
        ct, dt = self.color_tex[pass_index], self.depth_tex[pass_index]
        if ct is not None:
            out["color"] = ct.readImage()
            if p.samples > 1:
                out["resolved"] = ct.readImage(resolved=True)
        if dt is not None:
            out["depth"] = dt.readImage()
        return out


# ------------------------------------------------------------------------------------------------
# the benchmark configurations (sizes parameterised so tests can run small variants)
# ------------------------------------------------------------------------------------------------
def _lambert_states(cull=True, depth_func=A.DepthFunc_LESS) -> A.RenderStates:
    return A.RenderStates(blend=False, depthTest=True, depthMask=True, depthFunc=depth_func, cullFace=cull)


def config_plain_small(seed: int = 1000, width: int = 1024, height: int = 768, lon: int = 64, lat: int = 32,
                       tex: int = 256, filter_min: int = A.Filter_LINEAR_MIPMAP_NEAREST,
                       distance: float = 3.0) -> Scene:
    """UV sphere + checkerboard, directional Blinn-Phong (shininess 32), LESS, cull back, no MSAA."""
    vert, idx = uv_sphere(lon, lat)
    eye = np.array([0.0, 0.0, distance])
    Pm = perspective(np.pi / 3.0, width / height, 0.01, False)
    Vm = look_at(eye, [0, 0, 0], [0, 1, 0])
    Mm = np.eye(4)
    ang = hash_u01(seed, 1, np.arange(2))
    light = normalize(np.array([det_cos(ang[0] * 2 * np.pi) * 0.8, 0.6 + 0.3 * ang[1], det_sin(ang[0] * 2 * np.pi) * 0.3 + 0.7]))
    blocks = {
        "UniformsModel": uniforms_model(Mm, mm4(mm4(Pm, Vm), Mm), None, False),
        "UniformsScene": uniforms_scene([0.15, 0.15, 0.15], eye, light, [1.0, 1.0, 1.0]),
        "UniformsMaterial": uniforms_material(True, False, False, 1.0, 0.6, [1, 1, 1, 1]),
    }
    albedo = TextureSpec("u_albedoMap", A.TextureDesc(tex, tex, A.TextureType_2D, A.TextureFormat_RGBA8,
                                                      A.TextureUsage_Sampler | A.TextureUsage_UploadData, True, False),
                         A.SamplerDesc(filter_min, A.Filter_LINEAR, A.Wrap_REPEAT, A.Wrap_REPEAT, A.Wrap_REPEAT),
                         layers=[checkerboard(tex, 8, seed)])
    draw = DrawSpec(vert, 64, idx, A.Shading_BlinnPhongDir, ("ALBEDO_MAP",), _lambert_states(True), blocks, [albedo])
    clear = A.ClearStates(True, True, (0.05, 0.05, 0.08, 1.0), 1.0)
    return Scene("plain_small", [PassSpec(width, height, 1, clear, [draw])],
                 {"config": 1, "seed": seed, "width": width, "height": height, "samples": 1})


def config_geometry_stress(seed: int = 2000, n_tris: int = 1_000_000, width: int = 1920, height: int = 1080,
                           samples: int = 4) -> Scene:
    """1M-triangle soup with vertex colours: opaque pass, then SRC_ALPHA/ONE_MINUS_SRC_ALPHA pass,
    reversed-Z GREATER, no culling, MSAA 4x; the camera frames the cube so that part of the soup
    crosses the near, far and side planes."""
    aspect = width / height
    eye = np.array([0.35, 0.25, 1.6])
    Pm = perspective(np.deg2rad(75.0), aspect, 0.35, True, far=2.6)
    Vm = look_at(eye, [0.0, 0.0, 0.0], [0, 1, 0])
    VP = mm4(Pm, Vm)
    rows, idx, opaque = triangle_soup(n_tris, seed, VP, width, height)
    tri_rows = rows.reshape(n_tris, 3, 8)

    def sub(mask):
        r = tri_rows[mask].reshape(-1, 8)
        return r, np.arange(r.shape[0], dtype=np.int32)

    r_op, i_op = sub(opaque)
    r_tr, i_tr = sub(~opaque)
    blocks = {
        "UniformsModel": uniforms_model(np.eye(4), VP, None, True),
        "UniformsMaterial": uniforms_material(False, False, False, 1.0, 0.0, [1, 1, 1, 1]),
    }
    opaque_states = A.RenderStates(blend=False, depthTest=True, depthMask=True, depthFunc=A.DepthFunc_GREATER,
                                   cullFace=False)
    blend_params = A.BlendParameters()
    blend_params.SetBlendFactor(A.BlendFactor_SRC_ALPHA, A.BlendFactor_ONE_MINUS_SRC_ALPHA)
    blend_states = A.RenderStates(blend=True, blendParams=blend_params, depthTest=True, depthMask=False,
                                  depthFunc=A.DepthFunc_GREATER, cullFace=False)
    d0 = DrawSpec(r_op, 32, i_op, A.Shading_VertexColor, (), opaque_states, blocks)
    d1 = DrawSpec(r_tr, 32, i_tr, A.Shading_VertexColor, (), blend_states, blocks)
    clear = A.ClearStates(True, True, (0.0, 0.0, 0.0, 1.0), 0.0)
    return Scene("geometry_stress", [PassSpec(width, height, samples, clear, [d0, d1])],
                 {"config": 2, "seed": seed, "width": width, "height": height, "samples": samples})


def pbr_view_blocks(seed: int, view: int, width: int, height: int) -> Dict[str, bytes]:
    """Uniform blocks of one seeded orbit view of the PBR scene (camera and point light follow the
    view; geometry and textures do not depend on it)."""
    yaw = 2.0 * np.pi * hash_u01(seed, 50, view)
    pitch = (hash_u01(seed, 51, view) - 0.5) * 0.8
    dist = 2.7
    eye = np.array([dist * det_cos(pitch) * det_sin(yaw), dist * det_sin(pitch), dist * det_cos(pitch) * det_cos(yaw)])
    Pm = perspective(np.pi / 3.0, width / height, 0.05, False)
    Vm = look_at(eye, [0, 0, 0], [0, 1, 0])
    Mm = np.eye(4)
    light_pos = eye * 0.9 + np.array([1.2, 1.5, 0.3])
    return {
        "UniformsModel": uniforms_model(Mm, mm4(mm4(Pm, Vm), Mm), None, False),
        "UniformsScene": uniforms_scene([0.1, 0.1, 0.1], eye, light_pos, [2.5, 2.4, 2.2]),
        "UniformsMaterial": uniforms_material(True, True, False, 1.0, 0.5, [1, 1, 1, 1]),
    }


def config_pbr(seed: int = 3000, width: int = 1920, height: int = 1080, samples: int = 4, lon: int = 448,
               lat: int = 224, tex: int = 1024, prefilter: int = 512, irradiance: int = 32,
               view: int = 0, ibl_variant: int = 0) -> Scene:
    """Displaced sphere (value noise, amplitude 0.1) with PBR+IBL: albedo / normal / metal-roughness
    maps (trilinear), irradiance + 5-level prefiltered specular cube maps, point light, MSAA 4x.
    `ibl_variant` picks the environment (ibl_maps): another variant is another material."""
    vert, idx = uv_sphere(lon, lat, 1.0, displace_seed=seed, amplitude=0.1)
    blocks = pbr_view_blocks(seed, view, width, height)
    trilinear = A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR, A.Filter_LINEAR, A.Wrap_REPEAT, A.Wrap_REPEAT,
                              A.Wrap_REPEAT)
    tdesc = A.TextureDesc(tex, tex, A.TextureType_2D, A.TextureFormat_RGBA8,
                          A.TextureUsage_Sampler | A.TextureUsage_UploadData, True, False)
    pre, irr = ibl_maps(seed, prefilter, irradiance, variant=ibl_variant)
    cube_pre = TextureSpec("u_prefilterMap",
                           A.TextureDesc(prefilter, prefilter, A.TextureType_CUBE, A.TextureFormat_RGBA8,
                                         A.TextureUsage_Sampler, True, False),
                           A.SamplerDesc(A.Filter_LINEAR_MIPMAP_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE,
                                         A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE),
                           levels=pre)
    cube_irr = TextureSpec("u_irradianceMap",
                           A.TextureDesc(irradiance, irradiance, A.TextureType_CUBE, A.TextureFormat_RGBA8,
                                         A.TextureUsage_Sampler | A.TextureUsage_UploadData, False, False),
                           A.SamplerDesc(A.Filter_LINEAR, A.Filter_LINEAR, A.Wrap_CLAMP_TO_EDGE, A.Wrap_CLAMP_TO_EDGE,
                                         A.Wrap_CLAMP_TO_EDGE),
                           layers=irr)
    textures = [
        TextureSpec("u_albedoMap", tdesc, trilinear, layers=[noise_texture(tex, seed + 10, "albedo")]),
        TextureSpec("u_normalMap", tdesc, trilinear, layers=[noise_texture(tex, seed + 20, "normal")]),
        TextureSpec("u_metalRoughnessMap", tdesc, trilinear, layers=[noise_texture(tex, seed + 30, "metal_rough")]),
        cube_irr, cube_pre,
    ]
    draw = DrawSpec(vert, 64, idx, A.Shading_PBR, ("ALBEDO_MAP", "NORMAL_MAP", "METALROUGHNESS_MAP"),
                    _lambert_states(True), blocks, textures)
    clear = A.ClearStates(True, True, (0.02, 0.02, 0.03, 1.0), 1.0)
    return Scene("pbr", [PassSpec(width, height, samples, clear, [draw])],
                 {"config": 3, "seed": seed, "width": width, "height": height, "samples": samples})


def config_lines(seed: int = 6000, width: int = 640, height: int = 400, samples: int = 1, lon: int = 24,
                 lat: int = 12, segments: int = 40, blend: bool = True, cull: bool = True) -> Scene:
    """Points, lines and wireframe in one pass, as the reference viewer draws them with the
    base-colour shader (Viewer.cpp:244-270; ModelLoader.cpp:40-84), plus vertex-coloured segments:

    d0  a sphere in PolygonMode_LINE (wireframe), partly outside the side planes
    d1  the world-axis grid (Primitive_LINE) on a floor plane that runs behind the camera, so the
        near plane clips it
    d2  seeded vertex-coloured segments, lineWidth 2, alpha blended (per-pixel order matters)
    d3  point lights (Primitive_POINT, pointSize 10) with repeated indices: a stamp leaves the
        vertex at its last pixel, so a repeated point walks
    d4  a small sphere in PolygonMode_POINT (pointSize 3): every shared vertex walks too
    d5  degenerate lines whose two ends fall in one pixel (t = 0 / 0), depth test off
    """
    aspect = width / height
    eye = np.array([0.35, 0.55, 1.75])
    Pm = perspective(np.pi / 3.0, aspect, 0.05, False)
    Vm = look_at(eye, [0.0, 0.0, 0.0], [0, 1, 0])
    VP = mm4(Pm, Vm)
    model = uniforms_model(np.eye(4), VP, None, False)

    def base(point_size, color):
        return {"UniformsModel": model,
                "UniformsMaterial": uniforms_material(False, False, False, point_size, 0.0, color)}

    def rows_of(pos):
        r = np.zeros((len(pos), 16), np.float32)
        r[:, 0:3] = pos
        return r

    depth_less = dict(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS)
    # d0: wireframe sphere
    vert, idx = uv_sphere(lon, lat, 1.0, displace_seed=seed, amplitude=0.1)
    d0 = DrawSpec(vert, 64, idx, A.Shading_BaseColor, (),
                  A.RenderStates(cullFace=cull, polygonMode=A.PolygonMode_LINE, **depth_less),
                  base(1.0, [0.9, 0.9, 0.85, 1.0]))
    # d1: floor grid (ModelLoader::loadWorldAxis layout: lines along x and z, 0.2 apart, to +-3.2)
    g = []
    for i in range(-16, 17, 2):
        g += [[-3.2, -1.1, 0.2 * i], [3.2, -1.1, 0.2 * i], [0.2 * i, -1.1, -3.2], [0.2 * i, -1.1, 3.2]]
    gpos = np.array(g, np.float64)
    d1 = DrawSpec(rows_of(gpos), 64, np.arange(len(gpos), dtype=np.int32), A.Shading_BaseColor, (),
                  A.RenderStates(primitiveType=A.Primitive_LINE, **depth_less), base(1.0, [0.25, 0.25, 0.25, 1.0]))
    # d2: vertex-coloured segments (rows: pos.xyz_, rgba), each at least a few pixels long
    t = np.arange(segments, dtype=np.uint64)
    a = np.stack([hash_u01(seed, 10 + k, t) * 2.4 - 1.2 for k in range(3)], axis=-1)
    d = normalize(np.stack([hash_u01(seed, 20 + k, t) * 2.0 - 1.0 for k in range(3)], axis=-1))
    b = a + d * (0.3 + 1.2 * hash_u01(seed, 30, t))[:, None]
    crow = np.zeros((2 * segments, 8), np.float32)
    crow[0::2, 0:3] = a
    crow[1::2, 0:3] = b
    for k in range(3):
        crow[0::2, 4 + k] = hash_u01(seed, 40 + k, t)
        crow[1::2, 4 + k] = hash_u01(seed, 50 + k, t)
    crow[:, 7] = 0.6
    bp = A.BlendParameters()
    bp.SetBlendFactor(A.BlendFactor_SRC_ALPHA, A.BlendFactor_ONE_MINUS_SRC_ALPHA)
    d2 = DrawSpec(crow, 32, np.arange(2 * segments, dtype=np.int32), A.Shading_VertexColor, (),
                  A.RenderStates(blend=blend, blendParams=bp, primitiveType=A.Primitive_LINE, lineWidth=2.0,
                                 **depth_less), base(1.0, [1, 1, 1, 1]))
    # d3: point lights, some near the frame edges, with repeats
    lp = np.stack([hash_u01(seed, 60 + k, np.arange(12, dtype=np.uint64)) * 3.0 - 1.5 for k in range(3)], axis=-1)
    lp[0] = [1.2, 1.0, 0.5]
    pidx = np.array([0, 0, 0, 1, 2, 3, 3, 4, 5, 6, 7, 8, 9, 10, 11, 11, 11, 11, 5], np.int32)
    d3 = DrawSpec(rows_of(lp), 64, pidx, A.Shading_BaseColor, (),
                  A.RenderStates(primitiveType=A.Primitive_POINT, **depth_less), base(10.0, [1.0, 0.85, 0.3, 1.0]))
    # d4: small sphere drawn as points
    sv, si = uv_sphere(12, 6, 0.35)
    sv = sv.copy()
    sv[:, 0:3] += np.array([-0.9, 0.75, 0.2], np.float32)
    d4 = DrawSpec(sv, 64, si, A.Shading_BaseColor, (),
                  A.RenderStates(cullFace=False, polygonMode=A.PolygonMode_POINT, **depth_less),
                  base(3.0, [0.3, 0.9, 0.4, 1.0]))
    # d5: degenerate lines (both ends in one pixel), depth test off
    q = np.stack([hash_u01(seed, 70 + k, np.arange(6, dtype=np.uint64)) * 1.6 - 0.8 for k in range(3)], axis=-1)
    qq = np.repeat(q, 2, axis=0)
    qq[1::2] += 1e-4
    d5 = DrawSpec(rows_of(qq), 64, np.arange(len(qq), dtype=np.int32), A.Shading_BaseColor, (),
                  A.RenderStates(primitiveType=A.Primitive_LINE), base(1.0, [0.2, 0.5, 1.0, 1.0]))
    clear = A.ClearStates(True, True, (0.05, 0.05, 0.08, 1.0), 1.0)
    return Scene("lines", [PassSpec(width, height, samples, clear, [d0, d1, d2, d3, d4, d5])],
                 {"seed": seed, "width": width, "height": height, "samples": samples})


def config_wireframe(seed: int = 6100, width: int = 1920, height: int = 1080, samples: int = 1, lon: int = 448,
                     lat: int = 224, distance: float = 2.4) -> Scene:
    """The viewer's wireframe mode on the benchmark sphere: base colour, PolygonMode_LINE, back faces
    culled, depth LESS (Viewer.cpp:264-270)."""
    vert, idx = uv_sphere(lon, lat, 1.0, displace_seed=seed, amplitude=0.1)
    eye = np.array([0.0, 0.3, distance])
    Pm = perspective(np.pi / 3.0, width / height, 0.05, False)
    Vm = look_at(eye, [0.0, 0.0, 0.0], [0, 1, 0])
    blocks = {"UniformsModel": uniforms_model(np.eye(4), mm4(Pm, Vm), None, False),
              "UniformsMaterial": uniforms_material(False, False, False, 1.0, 0.0, [0.9, 0.9, 0.9, 1.0])}
    st = A.RenderStates(depthTest=True, depthMask=True, depthFunc=A.DepthFunc_LESS, cullFace=True,
                        polygonMode=A.PolygonMode_LINE)
    draw = DrawSpec(vert, 64, idx, A.Shading_BaseColor, (), st, blocks)
    clear = A.ClearStates(True, True, (0.0, 0.0, 0.0, 1.0), 1.0)
    return Scene("wireframe", [PassSpec(width, height, samples, clear, [draw])],
                 {"seed": seed, "width": width, "height": height, "samples": samples})


def output_digest(arrs: Dict[str, np.ndarray]) -> Dict[str, str]:
    return {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()[:16] for k, v in sorted(arrs.items())}
