"""Seeded synthetic scenes for the rasterisation path.

The reference publishes no benchmark inputs, so these generators define them: a UV
sphere, a value-noise heightfield, a screen-space triangle soup, uniform-noise RGBA8
textures, and the mixed batch of sphere draws. Randomness comes from SplitMix64 (Steele,
Lea & Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) evaluated on
counters, so a scene is a pure function of its seed.

Geometry is computed in float64 and rounded once to float32. The platform's libm is
used for sin/cos, so two machines may differ in the last bit of a generated vertex; the
golden fixtures therefore store their inputs, and parity tests always hand the very same
arrays to the GPU path and to the CPU oracle.

Shader and material conventions (reference include/shaders/shaders.hpp, src/renderer.cpp:76-92):
light direction (0, -1, 0), light colour 0.6; Blinn-Phong and Phong use a specular
exponent of ``specular_exponent * 50``.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

_MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)

SHADER_FLAT = 0
SHADER_PHONG = 1
SHADER_PBR = 2
SHADER_BLINN_PHONG = 3
SHADER_GOURAUD = 4
SHADER_NAMES = {SHADER_FLAT: "flat", SHADER_PHONG: "phong", SHADER_PBR: "pbr",
                SHADER_BLINN_PHONG: "blinn_phong", SHADER_GOURAUD: "gouraud"}


def splitmix64(seed: int, counters: np.ndarray) -> np.ndarray:
    """SplitMix64 output for state ``seed + (i+1) * golden`` at each counter ``i``."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + (counters.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)) & _MASK64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK64
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n float64 values in [0, 1) with 53 random bits each (stream selects a sub-sequence)."""
    c = np.arange(n, dtype=np.uint64) + np.uint64(stream) * np.uint64(1 << 40)
    return (splitmix64(seed, c) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def noise_texture(size_w: int, size_h: Optional[int] = None, seed: int = 1) -> np.ndarray:
    """Uniform RGBA8 noise, shape (H, W, 4), row 0 first."""
    h = size_w if size_h is None else size_h
    n = size_w * h
    words = splitmix64(seed, np.arange((n + 1) // 2, dtype=np.uint64))
    return np.frombuffer(words.tobytes(), dtype=np.uint8)[: n * 4].reshape(h, size_w, 4).copy()


@dataclasses.dataclass
class Material:
    diffuse: Optional[np.ndarray] = None    # (H, W, 4) uint8
    bump: Optional[np.ndarray] = None
    metallic: Optional[np.ndarray] = None
    roughness: Optional[np.ndarray] = None
    ao: Optional[np.ndarray] = None
    specular_exponent: float = 1.0


@dataclasses.dataclass
class Mesh:
    positions: np.ndarray   # (V, 3) float32
    uvs: np.ndarray         # (V, 2) float32
    normals: np.ndarray     # (V, 3) float32
    tangents: np.ndarray    # (V, 3) float32
    bitangents: np.ndarray  # (V, 3) float32
    indices: np.ndarray     # (F, 3) uint32
    groups: np.ndarray      # (G, 3) uint32: start face, face count, material index
    materials: list

    @property
    def num_vertices(self) -> int:
        return int(self.positions.shape[0])

    @property
    def num_faces(self) -> int:
        return int(self.indices.shape[0])


@dataclasses.dataclass
class Camera:
    """Arguments of the reference Camera (src/camera.cpp:30-56) plus setViewport."""
    position: tuple
    target: tuple
    fov_degrees: float
    aspect: float
    viewport: tuple


@dataclasses.dataclass
class Shader:
    kind: int
    light_direction: tuple = (0.0, -1.0, 0.0)
    light_color: tuple = (0.6, 0.6, 0.6)


@dataclasses.dataclass
class Scene:
    name: str
    mesh: Mesh
    camera: Camera
    shader: Shader
    width: int
    height: int
    model: np.ndarray = dataclasses.field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(16))
    clear_bgra: tuple = (0, 0, 0, 255)   # BLACK, reference src/renderer.cpp:113,124


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).astype(np.float32))


def _frame_vectors(n: np.ndarray, t_hint: np.ndarray):
    """Tangent = t_hint made orthogonal to n; bitangent = n x t (unit vectors)."""
    t = t_hint - n * np.sum(n * t_hint, axis=1, keepdims=True)
    ln = np.linalg.norm(t, axis=1, keepdims=True)
    fallback = np.where(np.abs(n[:, :1]) > 0.8, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.where(ln > 1e-8, t / np.maximum(ln, 1e-30), fallback)
    b = np.cross(n, t)
    return t, b


def uv_sphere(lon: int = 64, lat: int = 32, radius: float = 1.0) -> tuple:
    """UV sphere with a duplicated seam column: (lat+1)*(lon+1) vertices, 2*lon*(lat-1)
    counter-clockwise (front-facing from outside) triangles; the degenerate pole
    triangles are omitted. Normals are the unit positions; uv = (j/lon, i/lat)."""
    i = np.arange(lat + 1, dtype=np.float64)[:, None]
    j = np.arange(lon + 1, dtype=np.float64)[None, :]
    theta = math.pi * i / lat                      # 0 at +y
    phi = 2.0 * math.pi * j / lon
    st, ct = np.sin(theta), np.cos(theta)
    sp, cp = np.sin(phi), np.cos(phi)
    n = np.stack(np.broadcast_arrays(st * cp, ct + 0 * cp, -st * sp), axis=-1).reshape(-1, 3)
    pos = radius * n
    uv = np.stack(np.broadcast_arrays(j / lon + 0 * i, i / lat + 0 * j), axis=-1).reshape(-1, 2)
    # tangent along increasing phi: d/dphi (sin t cos p, cos t, -sin t sin p) ~ (-sin p, 0, -cos p)
    t_hint = np.stack(np.broadcast_arrays(-sp + 0 * i, 0 * i + 0 * j, -cp + 0 * i), axis=-1).reshape(-1, 3)
    tan, bit = _frame_vectors(n, t_hint)
    row = lon + 1
    faces = []
    for a in range(lat):
        for b in range(lon):
            v00 = a * row + b
            v01 = a * row + b + 1
            v10 = (a + 1) * row + b
            v11 = (a + 1) * row + b + 1
            if a != 0:
                faces.append((v00, v10, v01))
            if a != lat - 1:
                faces.append((v01, v10, v11))
    idx = np.asarray(faces, dtype=np.uint32)
    return _f32(pos), _f32(uv), _f32(n), _f32(tan), _f32(bit), idx


def value_noise(n: int, seed: int, octaves: int = 4, base_cells: int = 4) -> np.ndarray:
    """Sum of `octaves` layers of smoothstep-interpolated lattice noise on an n x n grid,
    cell count doubling and amplitude halving per octave, normalised to [-1, 1]."""
    coords = np.linspace(0.0, 1.0, n)
    total = np.zeros((n, n))
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        cells = base_cells << o
        lattice = uniform(seed, (cells + 1) * (cells + 1), stream=o).reshape(cells + 1, cells + 1) * 2.0 - 1.0
        x = coords * cells
        i0 = np.minimum(np.floor(x).astype(np.int64), cells - 1)
        f = x - i0
        s = f * f * (3.0 - 2.0 * f)
        a = lattice[i0[:, None], i0[None, :]]
        b = lattice[i0[:, None], i0[None, :] + 1]
        c = lattice[i0[:, None] + 1, i0[None, :]]
        d = lattice[i0[:, None] + 1, i0[None, :] + 1]
        sx, sz = s[None, :], s[:, None]
        total += amp * ((a * (1 - sx) + b * sx) * (1 - sz) + (c * (1 - sx) + d * sx) * sz)
        norm += amp
        amp *= 0.5
    return total / norm


def heightfield(n: int = 1024, seed: int = 2, amplitude: float = 0.2) -> tuple:
    """n x n grid over [-1, 1]^2 in the xz-plane, y = amplitude * value noise, normals by
    central differences, uv = grid index / (n - 1); 2 (n-1)^2 counter-clockwise (seen from
    +y) triangles."""
    g = np.linspace(-1.0, 1.0, n)
    hgt = amplitude * value_noise(n, seed)         # hgt[row=z, col=x]
    X, Z = np.meshgrid(g, g)
    pos = np.stack([X, hgt, Z], axis=-1).reshape(-1, 3)
    step = 2.0 / (n - 1)
    hp = np.pad(hgt, 1, mode="edge")
    dhdx = (hp[1:-1, 2:] - hp[1:-1, :-2]) / (2 * step)
    dhdz = (hp[2:, 1:-1] - hp[:-2, 1:-1]) / (2 * step)
    nrm = np.stack([-dhdx, np.ones_like(dhdx), -dhdz], axis=-1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n))
    uv = np.stack([ii / (n - 1), jj / (n - 1)], axis=-1).reshape(-1, 2)
    tan, bit = _frame_vectors(nrm, np.tile(np.array([[1.0, 0.0, 0.0]]), (n * n, 1)))
    r, c = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    v00 = (r * n + c).ravel()
    v01 = v00 + 1
    v10 = v00 + n
    v11 = v10 + 1
    # seen from +y with x right and z toward the viewer, (v00, v10, v01) is counter-clockwise
    tri = np.empty((2 * v00.size, 3), dtype=np.uint32)
    tri[0::2] = np.stack([v00, v10, v01], axis=1)
    tri[1::2] = np.stack([v01, v10, v11], axis=1)
    return _f32(pos), _f32(uv), _f32(nrm), _f32(tan), _f32(bit), tri


def _single_group(nf: int, material: int = 0) -> np.ndarray:
    return np.asarray([[0, nf, material]], dtype=np.uint32)


def _mesh(parts, materials) -> Mesh:
    pos, uv, nrm, tan, bit, idx = parts
    return Mesh(pos, uv, nrm, tan, bit, np.ascontiguousarray(idx, dtype=np.uint32),
                _single_group(idx.shape[0]), materials)


def orbit_camera(distance: float, elevation_deg: float, azimuth_deg: float, width: int, height: int,
                 fov: float = 60.0) -> Camera:
    el, az = math.radians(elevation_deg), math.radians(azimuth_deg)
    p = (distance * math.cos(el) * math.sin(az), distance * math.sin(el), distance * math.cos(el) * math.cos(az))
    return Camera(tuple(float(np.float32(v)) for v in p), (0.0, 0.0, 0.0), fov, float(np.float32(width / height)),
                  (0, 0, width, height))


# ------------------------------------------------------------------ configurations
def sphere_scene(width: int = 512, height: int = 512, lon: int = 64, lat: int = 32, tex_size: int = 256,
                 tex_seed: int = 1, shader: int = SHADER_BLINN_PHONG, distance: float = 3.0,
                 name: str = "sphere") -> Scene:
    """UV sphere r=1, 64x32 segments, 256^2 noise texture, camera at (0,0,3), fov 60,
    Blinn-Phong, 512^2 (the plain small configuration)."""
    mat = Material(diffuse=noise_texture(tex_size, seed=tex_seed), specular_exponent=1.0)
    if shader in (SHADER_PHONG, SHADER_PBR):
        mat.bump = noise_texture(tex_size, seed=tex_seed + 100)
        mat.metallic = noise_texture(tex_size, seed=tex_seed + 101)
        mat.roughness = noise_texture(tex_size, seed=tex_seed + 102)
        mat.ao = noise_texture(tex_size, seed=tex_seed + 103)
    cam = Camera((0.0, 0.0, float(distance)), (0.0, 0.0, 0.0), 60.0, float(np.float32(width / height)),
                 (0, 0, width, height))
    light = (5.6, 5.6, 5.6) if shader == SHADER_PBR else (0.6, 0.6, 0.6)
    return Scene(name, _mesh(uv_sphere(lon, lat), [mat]), cam, Shader(shader, light_color=light), width, height)


def heightfield_scene(n: int = 1024, width: int = 1920, height: int = 1080, tex_size: int = 2048,
                      shader: int = SHADER_BLINN_PHONG, name: str = "heightfield") -> Scene:
    """1024^2-vertex heightfield (2,093,058 triangles), 2048^2 noise texture (seed 3),
    camera at 30 degrees elevation and distance 2.5, 1920x1080 (the plain large-mesh
    configuration)."""
    mat = Material(diffuse=noise_texture(tex_size, seed=3), specular_exponent=1.0)
    if shader in (SHADER_PHONG, SHADER_PBR):
        mat.bump = noise_texture(tex_size, seed=103)
        mat.metallic = noise_texture(tex_size, seed=104)
        mat.roughness = noise_texture(tex_size, seed=105)
        mat.ao = noise_texture(tex_size, seed=106)
    cam = orbit_camera(2.5, 30.0, 0.0, width, height)
    return Scene(name, _mesh(heightfield(n, seed=2), [mat]), cam, Shader(shader), width, height)


def soup_scene(count: int = 200_000, width: int = 3840, height: int = 2160, seed: int = 4,
               edge_min: float = 0.5, edge_max: float = 4.0, depth_min: float = 0.1, depth_max: float = 100.0,
               name: str = "soup") -> Scene:
    """Independent screen-space triangles: centres uniform over the screen, equilateral
    with edge ~ U[edge_min, edge_max] px and a random rotation, counter-clockwise, at view
    depth ~ U[depth_min, depth_max]; unprojected through a camera at the origin looking
    down -z (fov 60). Per-vertex RGBA8 colour for the Gouraud shader: RGB/255 in the
    normal, A/255 in uv.x (the small-triangle / overdraw stress configuration)."""
    u = uniform(seed, count * 5).reshape(count, 5)
    cx, cy = u[:, 0] * width, u[:, 1] * height
    edge = edge_min + (edge_max - edge_min) * u[:, 2]
    rot = 2.0 * math.pi * u[:, 3]
    depth = depth_min + (depth_max - depth_min) * u[:, 4]
    rad = edge / math.sqrt(3.0)
    ang = rot[:, None] + np.array([0.0, 2.0 * math.pi / 3.0, 4.0 * math.pi / 3.0])[None, :]
    sx = cx[:, None] + rad[:, None] * np.cos(ang)
    sy = cy[:, None] + rad[:, None] * np.sin(ang)
    aspect = float(np.float32(width / height))
    th = math.tan(math.radians(60.0) / 2.0)
    ndc_x = sx / width * 2.0 - 1.0
    ndc_y = sy / height * 2.0 - 1.0
    d = depth[:, None]
    pos = np.stack([ndc_x * d * th * aspect, ndc_y * d * th, -d + 0 * ndc_x], axis=-1).reshape(-1, 3)
    rgba = noise_texture(count * 3, 1, seed=seed + 1000).reshape(-1, 4).astype(np.float64) / 255.0
    nrm = rgba[:, :3]
    uv = np.stack([rgba[:, 3], np.zeros(count * 3)], axis=-1)
    idx = np.arange(count * 3, dtype=np.uint32).reshape(count, 3)
    zeros = np.zeros((count * 3, 3))
    parts = (_f32(pos), _f32(uv), _f32(nrm), _f32(zeros), _f32(zeros), idx)
    cam = Camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 60.0, aspect, (0, 0, width, height))
    return Scene(name, _mesh(parts, [Material()]), cam, Shader(SHADER_GOURAUD), width, height)


BATCH_RESOLUTIONS = ((256, 256), (512, 512), (1024, 1024), (1920, 1080))


@dataclasses.dataclass
class BatchDraw:
    lon: int
    lat: int
    width: int
    height: int
    camera: Camera
    texture: int


def batch_plan(count: int = 512, seed: int = 5) -> list:
    """The mixed batch: UV spheres with lon log-uniform in [8, 256] (lat = lon/2),
    resolution uniform from BATCH_RESOLUTIONS, camera on a random orbit at distance
    U[2, 6] looking at the origin, one of 8 textures."""
    u = uniform(seed, count * 6).reshape(count, 6)
    draws = []
    for k in range(count):
        lon = int(round(2.0 ** (3.0 + 5.0 * u[k, 0])))
        lon = max(8, min(256, lon + (lon & 1)))
        w, h = BATCH_RESOLUTIONS[min(3, int(u[k, 1] * 4))]
        dist = 2.0 + 4.0 * u[k, 2]
        el = -60.0 + 120.0 * u[k, 3]
        az = 360.0 * u[k, 4]
        draws.append(BatchDraw(lon, lon // 2, w, h, orbit_camera(dist, el, az, w, h), min(7, int(u[k, 5] * 8))))
    return draws


def batch_textures(size: int = 1024) -> list:
    return [noise_texture(size, seed=10 + k) for k in range(8)]


def batch_scenes(count: int = 512, seed: int = 5, tex_size: int = 1024, resolution_scale: float = 1.0) -> list:
    """Scenes of the mixed batch (sharing the 8 textures and one mesh per segment count)."""
    texs = batch_textures(tex_size)
    meshes = {}
    scenes = []
    for k, d in enumerate(batch_plan(count, seed)):
        if d.lon not in meshes:
            meshes[d.lon] = uv_sphere(d.lon, d.lat)
        w = max(16, int(d.width * resolution_scale))
        h = max(16, int(d.height * resolution_scale))
        cam = dataclasses.replace(d.camera, viewport=(0, 0, w, h))
        mat = Material(diffuse=texs[d.texture], specular_exponent=1.0)
        scenes.append(Scene(f"batch{k}", _mesh(meshes[d.lon], [mat]), cam, Shader(SHADER_BLINN_PHONG), w, h))
    return scenes


def clear_framebuffer(scene: Scene):
    """Host framebuffer cleared as the reference renderer does each frame
    (src/renderer.cpp:124-125): colour BLACK, depth +inf."""
    b, g, r, a = scene.clear_bgra
    bgra = np.empty((scene.height, scene.width, 4), dtype=np.uint8)
    bgra[...] = (b, g, r, a)
    depth = np.full((scene.height, scene.width), np.inf, dtype=np.float32)
    return bgra, depth
