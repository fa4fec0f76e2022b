"""Python mirror of AxiomR's renderer API over the C ABI (include/axr.h).

Names and argument meaning follow the reference classes:
  Framebuffer     include/framebuffer.hpp  (BGRA8 colour + float depth, row 0 at the bottom)
  Texture         include/texture.hpp      (RGBA8, row 0 first)
  Mesh / Material include/mesh.hpp         (from arrays; OBJ loading is the caller's)
  Camera          include/camera.hpp       (matrices from position/target/fov/aspect)
  FlatShader, PhongShader, PBRShader       include/shaders/shaders.hpp
  BlinnPhongShader, GouraudShader          this library's own shaders
  TiledPipeline   include/tiled_pipeline.hpp (setShader/setCamera/setFramebuffer/drawMesh)
  Renderer.drawMesh                        src/renderer.cpp:16-19
  Draw, Batch, draw_batch, autotune        the batched form (no reference counterpart)
  Graph                                    CUDA-graph capture and replay of a context's work
  Server                                   the serving loop (continuous batching, budgeted residency)
Every call runs the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (AXR_DRAW_CLEAR_COLOR, AXR_DRAW_CLEAR_DEPTH, AXR_TUNE_CLASSES, AxrError, BatchInfo, CameraDesc,
                   DrawDesc, DrawStats, GroupDesc, MaterialDesc, MeshDesc, ShaderDesc, check)

FLAT, PHONG, PBR, BLINN_PHONG, GOURAUD = 0, 1, 2, 3, 4
BATCH_PERSISTENT, BATCH_PHASED, BATCH_BINNED = 0, 1, 2  # launch forms of the batched kernels (AXR_BATCH_*)
DRAW_BINNED, DRAW_KEYED = 0, 1  # forms of the per-draw path (AXR_DRAW_*)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class Context:
    """One CUDA stream, pipeline state and scratch arena on one device (axr_context)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.axr_context_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    @property
    def stream(self) -> int:
        return int(self.lib.axr_context_stream(self.handle) or 0)

    def sync(self) -> None:
        check(self.lib.axr_sync(self.handle), self.handle)

    def reserve(self, max_faces: int) -> None:
        check(self.lib.axr_reserve(self.handle, int(max_faces)), self.handle)

    def stats(self, enable: Optional[bool] = None):
        if enable is not None:
            check(self.lib.axr_stats_enable(self.handle, 1 if enable else 0), self.handle)
            return None
        s = DrawStats()
        check(self.lib.axr_stats_read(self.handle, C.byref(s)), self.handle)
        return {"triangles": s.triangles, "fragments": s.fragments, "large": s.large, "tiles": s.tiles,
                "tested": s.tested, "shaded": s.shaded}

    def profile(self, enable: Optional[bool] = None):
        """Enable/disable stage timing, or (no argument) read and reset it."""
        if enable is not None:
            check(self.lib.axr_profile_enable(self.handle, 1 if enable else 0), self.handle)
            return None
        pr = _lib.Profile()
        check(self.lib.axr_profile_read(self.handle, C.byref(pr)), self.handle)
        return {"draws": pr.draws, "vertex_ms": pr.vertex_ms, "geometry_ms": pr.geometry_ms,
                "large_ms": pr.large_ms, "scan_ms": pr.scan_ms, "shade_ms": pr.shade_ms,
                "clipped_ms": pr.clipped_ms, "kernel_launches": pr.kernel_launches,
                "batch_launches": pr.batch_launches, "batch_vertex_ms": pr.batch_vertex_ms,
                "batch_face_ms": pr.batch_face_ms, "batch_large_ms": pr.batch_large_ms,
                "batch_tile_ms": pr.batch_tile_ms, "batch_clear_ms": pr.batch_clear_ms}

    def fp32_peak_tflops(self) -> float:
        """FP32 issue peak of the device, measured with independent FMA chains."""
        out = C.c_double()
        check(self.lib.axr_measure_fp32_peak(self.handle, C.byref(out)), self.handle)
        return out.value

    def tuning(self) -> list:
        """The batched form's tuning table: per density class, the largest triangle pixel
        box rasterised by one thread."""
        out = (C.c_int32 * AXR_TUNE_CLASSES)()
        check(self.lib.axr_batch_get_tuning(self.handle, out), self.handle)
        return list(out)

    @property
    def batch_form(self) -> int:
        """Launch form of batches planned next (AXR_BATCH_PERSISTENT / AXR_BATCH_PHASED)."""
        return int(self.lib.axr_batch_get_form(self.handle))

    @batch_form.setter
    def batch_form(self, form: int) -> None:
        check(self.lib.axr_batch_set_form(self.handle, int(form)), self.handle)

    def set_tuning(self, small_max_pixels: Sequence[int]) -> None:
        arr = (C.c_int32 * AXR_TUNE_CLASSES)(*[int(v) for v in small_max_pixels])
        check(self.lib.axr_batch_set_tuning(self.handle, arr), self.handle)

    @property
    def draw_form(self) -> int:
        """Form of the per-draw path (DRAW_BINNED, the default, or DRAW_KEYED)."""
        return int(self.lib.axr_get_draw_form(self.handle))

    @draw_form.setter
    def draw_form(self, form: int) -> None:
        check(self.lib.axr_set_draw_form(self.handle, int(form)), self.handle)

    @property
    def bin_params(self) -> dict:
        """Bin parameters of the per-draw binned form (capacity 0: sized per draw)."""
        b = _lib.BinParams()
        check(self.lib.axr_get_bin_params(self.handle, C.byref(b)), self.handle)
        return {"capacity": b.capacity, "tiles_x": b.tiles_x, "tiles_y": b.tiles_y, "thread_pixels": b.thread_pixels}

    @bin_params.setter
    def bin_params(self, v: dict) -> None:
        b = _lib.BinParams(int(v.get("capacity", 0)), int(v.get("tiles_x", 0)), int(v.get("thread_pixels", 64)),
                           int(v.get("tiles_y", 0)))
        check(self.lib.axr_set_bin_params(self.handle, C.byref(b)), self.handle)

    def bin_tuning(self) -> list:
        """The binned batch form's bin parameters per density class."""
        arr = (_lib.BinParams * AXR_TUNE_CLASSES)()
        check(self.lib.axr_batch_get_bin_tuning(self.handle, arr), self.handle)
        return [{"capacity": b.capacity, "tiles_x": b.tiles_x, "tiles_y": b.tiles_y, "thread_pixels": b.thread_pixels}
                for b in arr]

    def set_bin_tuning(self, table: Sequence[dict]) -> None:
        arr = (_lib.BinParams * AXR_TUNE_CLASSES)(
            *[_lib.BinParams(int(v["capacity"]), int(v["tiles_x"]), int(v["thread_pixels"]), int(v.get("tiles_y", 0)))
              for v in table])
        check(self.lib.axr_batch_set_bin_tuning(self.handle, arr), self.handle)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.axr_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Texture:
    """RGBA8 texture (Texture, include/texture.hpp); `rgba` is (H, W, 4) uint8, row 0 first."""

    def __init__(self, ctx: Context, rgba: np.ndarray):
        rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
        if rgba.ndim != 3 or rgba.shape[2] != 4:
            raise ValueError("texture must be (H, W, 4) uint8")
        self.ctx = ctx
        self.height, self.width = rgba.shape[:2]
        h = C.c_void_p()
        check(ctx.lib.axr_texture_create(ctx.handle, rgba.ctypes.data, self.width, self.height, C.byref(h)),
              ctx.handle)
        self.handle = h

    def update(self, rgba: np.ndarray) -> None:
        rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
        self._pending = rgba
        check(self.ctx.lib.axr_texture_update(self.ctx.handle, self.handle, rgba.ctypes.data), self.ctx.handle)

    def sample(self, uv: np.ndarray) -> np.ndarray:
        """Texture::sample at (n, 2) uv -> (n, 4) float32 (runs on the GPU)."""
        uvf = _f32(uv).reshape(-1, 2)
        out = np.zeros((uvf.shape[0], 4), np.float32)
        check(self.ctx.lib.axr_debug_sample(self.ctx.handle, self.handle, uvf.ctypes.data, uvf.shape[0],
                                            out.ctypes.data), self.ctx.handle)
        return out

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.axr_texture_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class Material:
    """Material (include/mesh.hpp:20-34): the textures the shaders read + Ns."""
    diffuse: Optional[Texture] = None
    bump: Optional[Texture] = None
    metallic: Optional[Texture] = None
    roughness: Optional[Texture] = None
    ao: Optional[Texture] = None
    specular_exponent: float = 1.0

    def desc(self) -> MaterialDesc:
        t = lambda x: x.handle if x is not None else None  # noqa: E731
        return MaterialDesc(t(self.diffuse), t(self.bump), t(self.metallic), t(self.roughness), t(self.ao),
                            float(self.specular_exponent))


class Mesh:
    """Device-resident mesh (Mesh, include/mesh.hpp) from vertex/face arrays."""

    def __init__(self, ctx: Context, positions, uvs, normals, indices, groups=None, materials: Sequence = (),
                 tangents=None, bitangents=None):
        self.ctx = ctx
        self._arrays = self._pack(positions, uvs, normals, indices, tangents, bitangents)
        nf = self._arrays["indices"].shape[0]
        self.groups = np.asarray(groups if groups is not None else [[0, nf, 0]], dtype=np.uint32).reshape(-1, 3)
        self.materials = list(materials) if materials else [Material()]
        self.num_faces = nf
        self.num_vertices = self._arrays["positions"].shape[0]
        desc, keep = self._desc(self._arrays)
        h = C.c_void_p()
        check(ctx.lib.axr_mesh_create(ctx.handle, C.byref(desc), C.byref(h)), ctx.handle)
        self.handle = h

    @staticmethod
    def _pack(positions, uvs, normals, indices, tangents, bitangents):
        a = {"positions": _f32(positions).reshape(-1, 3), "uvs": _f32(uvs).reshape(-1, 2),
             "normals": _f32(normals).reshape(-1, 3),
             "indices": np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3),
             "tangents": None if tangents is None else _f32(tangents).reshape(-1, 3),
             "bitangents": None if bitangents is None else _f32(bitangents).reshape(-1, 3)}
        return a

    def _desc(self, a):
        g = (GroupDesc * max(1, len(self.groups)))(*[GroupDesc(int(s), int(c), int(m)) for s, c, m in self.groups])
        mats = (MaterialDesc * max(1, len(self.materials)))(*[m.desc() for m in self.materials])
        d = MeshDesc(a["positions"].shape[0], _ptr(a["positions"]), _ptr(a["uvs"]), _ptr(a["normals"]),
                     _ptr(a["tangents"]), _ptr(a["bitangents"]), a["indices"].shape[0], _ptr(a["indices"]),
                     len(self.groups), C.addressof(g), len(self.materials), C.addressof(mats))
        return d, (g, mats)

    @classmethod
    def from_workload(cls, ctx: Context, mesh, textures: Optional[dict] = None):
        """Build from an axiomr_gb300.workloads.Mesh, uploading its material textures."""
        textures = {} if textures is None else textures
        mats = []
        for m in mesh.materials:
            def tex(img):
                if img is None:
                    return None
                key = id(img)
                if key not in textures:
                    textures[key] = Texture(ctx, img)
                return textures[key]
            mats.append(Material(tex(m.diffuse), tex(m.bump), tex(m.metallic), tex(m.roughness), tex(m.ao),
                                 m.specular_exponent))
        obj = cls(ctx, mesh.positions, mesh.uvs, mesh.normals, mesh.indices, mesh.groups, mats,
                  mesh.tangents, mesh.bitangents)
        obj._textures = textures
        return obj

    def update(self, positions, uvs, normals, indices, tangents=None, bitangents=None) -> None:
        """Re-upload all arrays (same counts), asynchronously on the context stream."""
        a = self._pack(positions, uvs, normals, indices, tangents, bitangents)
        desc, keep = self._desc(a)
        self._pending = (a, keep)
        check(self.ctx.lib.axr_mesh_update(self.ctx.handle, self.handle, C.byref(desc)), self.ctx.handle)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.axr_mesh_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Framebuffer:
    """BGRA8 + float depth framebuffer (Framebuffer, include/framebuffer.hpp)."""

    def __init__(self, ctx: Context, width: int, height: int):
        self.ctx = ctx
        self.width, self.height = int(width), int(height)
        h = C.c_void_p()
        check(ctx.lib.axr_framebuffer_create(ctx.handle, self.width, self.height, C.byref(h)), ctx.handle)
        self.handle = h

    def clearColor(self, r: int, g: int, b: int, a: int) -> None:
        check(self.ctx.lib.axr_framebuffer_clear_color(self.ctx.handle, self.handle, r, g, b, a), self.ctx.handle)

    def clearDepth(self, value: float = float("inf")) -> None:
        check(self.ctx.lib.axr_framebuffer_clear_depth(self.ctx.handle, self.handle, value), self.ctx.handle)

    def read(self, bgra: Optional[np.ndarray] = None, depth: Optional[np.ndarray] = None):
        """(bgra (H, W, 4) uint8, depth (H, W) float32), blocking."""
        bgra = np.empty((self.height, self.width, 4), np.uint8) if bgra is None else bgra
        depth = np.empty((self.height, self.width), np.float32) if depth is None else depth
        check(self.ctx.lib.axr_framebuffer_read(self.ctx.handle, self.handle, bgra.ctypes.data, depth.ctypes.data),
              self.ctx.handle)
        return bgra, depth

    def read_png(self, channels: int = 3) -> bytes:
        """The colour plane as a PNG file (top row first; RGB8 or RGBA8), encoded on the GPU."""
        return read_png(self.ctx, [self], channels)[0]

    def write(self, bgra: Optional[np.ndarray] = None, depth: Optional[np.ndarray] = None) -> None:
        b = None if bgra is None else np.ascontiguousarray(bgra, np.uint8)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        check(self.ctx.lib.axr_framebuffer_write(self.ctx.handle, self.handle, _ptr(b), _ptr(d)), self.ctx.handle)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.axr_framebuffer_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Camera:
    """The reference Camera (include/camera.hpp:6-67, src/camera.cpp:30-205) on the
    library's axr_camera_state: setPosition, setTarget, setFov, setAspectRatio,
    setViewport, handleInput and update(deltaTime) behave as the reference's. The
    constructor also runs update(0), as a frame loop does before its first draw (the
    reference constructor leaves the view matrix at identity until an update); pass
    update=False for the bare constructor."""

    def __init__(self, position=(0.0, 0.0, 0.0), target=(0.0, 0.0, -1.0), fov: float = 60.0,
                 aspect: float = 16.0 / 9.0, viewport=(0, 0, 800, 600), update: bool = True):
        self._lib = _lib.load()
        self.state = _lib.CameraState()
        self.target = tuple(float(v) for v in target)
        self.fov = float(fov)
        self.aspect = float(aspect)
        pos, tgt = _f32(position), _f32(target)
        check(self._lib.axr_camera_init(C.byref(self.state), pos.ctypes.data, tgt.ctypes.data, self.fov, self.aspect))
        self.setViewport(*viewport)
        self._fixed = None
        if update:
            self.update(0.0)

    @classmethod
    def from_workload(cls, cam):
        return cls(cam.position, cam.target, cam.fov_degrees, cam.aspect, cam.viewport)

    @classmethod
    def from_matrices(cls, view_proj, position, viewport=(0, 0, 1, 1)):
        """A camera with a given view-projection matrix (16 floats, column-major) and eye
        position, e.g. matrices computed elsewhere."""
        cam = cls(position, (float(position[0]), float(position[1]), float(position[2]) - 1.0), viewport=viewport,
                  update=False)
        cam._fixed = _f32(view_proj).reshape(16).copy()
        return cam

    # the reference's setters and motion
    def setPosition(self, position) -> None:
        p = _f32(position)
        check(self._lib.axr_camera_set_position(C.byref(self.state), p.ctypes.data))

    def setTarget(self, target) -> None:
        t = _f32(target)
        check(self._lib.axr_camera_set_target(C.byref(self.state), t.ctypes.data))

    def setFov(self, fov: float) -> None:
        check(self._lib.axr_camera_set_fov(C.byref(self.state), float(fov)))

    def setAspectRatio(self, aspect: float) -> None:
        check(self._lib.axr_camera_set_aspect_ratio(C.byref(self.state), float(aspect)))

    def setViewport(self, x: int, y: int, width: int, height: int) -> None:
        check(self._lib.axr_camera_set_viewport(C.byref(self.state), int(x), int(y), int(width), int(height)))

    def handleInput(self, mouse=(0.0, 0.0), right_button: bool = False, keys: str = "") -> None:
        """Camera::handleInput with the window's mouse position, right-button state and the
        keys held down (characters, e.g. "WD")."""
        s = _lib.InputState()
        s.mouse[0], s.mouse[1] = float(mouse[0]), float(mouse[1])
        s.mouse_buttons[1] = 1 if right_button else 0
        for k in keys:
            s.keys[ord(k) & 255] = 1
        check(self._lib.axr_camera_handle_input(C.byref(self.state), C.byref(s)))

    def update(self, delta_time: float) -> None:
        check(self._lib.axr_camera_update(C.byref(self.state), float(delta_time)))

    # accessors
    @property
    def position(self) -> tuple:
        return tuple(float(v) for v in self.state.position)

    @property
    def viewport(self) -> tuple:
        return tuple(int(v) for v in self.state.viewport)

    @property
    def view(self) -> np.ndarray:
        return np.array(self.state.view, np.float32)

    @property
    def projection(self) -> np.ndarray:
        return np.array(self.state.projection, np.float32)

    @property
    def view_proj(self) -> np.ndarray:
        return self._fixed.copy() if self._fixed is not None else np.array(self.state.view_proj, np.float32)

    @property
    def viewport_matrix(self) -> np.ndarray:
        d = CameraDesc()
        check(self._lib.axr_camera_describe(C.byref(self.state), C.byref(d)))
        return np.array(d.viewport, np.float32)

    def desc(self) -> CameraDesc:
        d = CameraDesc()
        check(self._lib.axr_camera_describe(C.byref(self.state), C.byref(d)))
        if self._fixed is not None:
            d.view_proj = (C.c_float * 16)(*self._fixed)
        return d


@dataclasses.dataclass
class Shader:
    kind: int
    lightDirection: tuple = (0.0, -1.0, 0.0)
    lightColor: tuple = (0.6, 0.6, 0.6)

    def desc(self) -> ShaderDesc:
        return ShaderDesc(int(self.kind), (C.c_float * 3)(*self.lightDirection), (C.c_float * 3)(*self.lightColor))


def FlatShader(lightDirection=(0.0, -1.0, 0.0)) -> Shader:
    return Shader(FLAT, lightDirection)


def PhongShader(lightDirection=(0.0, -1.0, 0.0), lightColor=(0.6, 0.6, 0.6)) -> Shader:
    return Shader(PHONG, lightDirection, lightColor)


def PBRShader(lightDirection=(0.0, -1.0, 0.0), lightColor=(5.6, 5.6, 5.6)) -> Shader:
    return Shader(PBR, lightDirection, lightColor)


def BlinnPhongShader(lightDirection=(0.0, -1.0, 0.0), lightColor=(0.6, 0.6, 0.6)) -> Shader:
    return Shader(BLINN_PHONG, lightDirection, lightColor)


def GouraudShader() -> Shader:
    return Shader(GOURAUD)


def _model(m) -> np.ndarray:
    return _f32(np.eye(4) if m is None else m).reshape(16)


class TiledPipeline:
    """TiledPipeline (include/tiled_pipeline.hpp:58-62) on the GPU."""

    def __init__(self, ctx: Context, camera: Optional[Camera] = None, framebuffer: Optional[Framebuffer] = None):
        self.ctx = ctx
        if camera is not None:
            self.setCamera(camera)
        if framebuffer is not None:
            self.setFramebuffer(framebuffer)

    def setShader(self, shader: Optional[Shader]) -> None:
        d = shader.desc() if shader is not None else None
        check(self.ctx.lib.axr_set_shader(self.ctx.handle, C.byref(d) if d is not None else None), self.ctx.handle)

    def setCamera(self, camera: Optional[Camera]) -> None:
        d = camera.desc() if camera is not None else None
        check(self.ctx.lib.axr_set_camera(self.ctx.handle, C.byref(d) if d is not None else None), self.ctx.handle)

    def setFramebuffer(self, fb: Optional[Framebuffer]) -> None:
        check(self.ctx.lib.axr_set_framebuffer(self.ctx.handle, fb.handle if fb is not None else None),
              self.ctx.handle)

    def drawMesh(self, modelMatrix, mesh: Mesh) -> None:
        m = _model(modelMatrix)
        check(self.ctx.lib.axr_draw_mesh(self.ctx.handle, mesh.handle, m.ctypes.data), self.ctx.handle)

    def debugTriangles(self, mesh: Mesh, modelMatrix, view_proj, width: int, height: int,
                       capacity: Optional[int] = None) -> np.ndarray:
        """Clip-stage output records, sorted by draw order: (n, 14) with column 0 the tag."""
        cap = int(capacity if capacity is not None else mesh.num_faces * 8 + 16)
        out = np.zeros((cap, 14), np.float32)
        cnt = C.c_uint32(0)
        m = _model(modelMatrix)
        vp = _f32(view_proj).reshape(16)
        check(self.ctx.lib.axr_debug_triangles(self.ctx.handle, mesh.handle, m.ctypes.data, vp.ctypes.data,
                                               int(width), int(height), out.ctypes.data, cap, C.byref(cnt)),
              self.ctx.handle)
        rec = out[: min(cnt.value, cap)]
        order = np.argsort(rec[:, 0].view(np.uint32), kind="stable")
        return rec[order]


class Renderer:
    """Renderer::drawMesh (src/renderer.cpp:16-19) delegating to its pipeline."""

    def __init__(self, pipeline: TiledPipeline):
        self.pipeline = pipeline

    def drawMesh(self, transMat, mesh: Mesh) -> None:
        self.pipeline.drawMesh(transMat, mesh)


def render_scene(ctx: Context, scene, framebuffer: Optional[Framebuffer] = None, mesh: Optional[Mesh] = None,
                 bgra: Optional[np.ndarray] = None, depth: Optional[np.ndarray] = None, view_proj=None):
    """Draw an axiomr_gb300.workloads.Scene as the reference renderer's frame does
    (clearColor, clearDepth, drawMesh; src/renderer.cpp:124-126) unless an initial
    framebuffer is given; returns (bgra, depth) read back to the host. `view_proj`
    overrides the matrix computed from the scene camera."""
    fb = framebuffer or Framebuffer(ctx, scene.width, scene.height)
    m = mesh or Mesh.from_workload(ctx, scene.mesh)
    if bgra is not None or depth is not None:
        fb.write(bgra, depth)
    else:
        b, g, r, a = scene.clear_bgra
        fb.clearColor(r, g, b, a)
        fb.clearDepth()
    cam = (Camera.from_workload(scene.camera) if view_proj is None
           else Camera.from_matrices(view_proj, scene.camera.position, scene.camera.viewport))
    pipe = TiledPipeline(ctx, cam, fb)
    sh = scene.shader
    pipe.setShader(Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)))
    pipe.drawMesh(scene.model, m)
    out = fb.read()
    ctx.sync()
    return out


# ---------------------------------------------------------------- batched form
@dataclasses.dataclass
class Draw:
    """One draw of a batch (axr_draw_desc): its own mesh, framebuffer, camera and shader.
    clear_color (r, g, b, a) / clear_depth: Framebuffer::clearColor / clearDepth before the
    draw, fused into the batch's tile pass."""
    mesh: "Mesh"
    framebuffer: "Framebuffer"
    camera: "Camera"
    shader: Shader
    model: Optional[np.ndarray] = None
    clear_color: Optional[tuple] = None
    clear_depth: Optional[float] = None

    def desc(self) -> DrawDesc:
        d = DrawDesc()
        d.mesh = self.mesh.handle
        d.framebuffer = self.framebuffer.handle
        d.model = (C.c_float * 16)(*_model(self.model))
        d.camera = self.camera.desc()
        d.shader = self.shader.desc()
        flags = 0
        if self.clear_color is not None:
            flags |= AXR_DRAW_CLEAR_COLOR
            d.clear_rgba = (C.c_uint8 * 4)(*[int(v) for v in self.clear_color])
        if self.clear_depth is not None:
            flags |= AXR_DRAW_CLEAR_DEPTH
            d.clear_depth = float(self.clear_depth)
        d.clear_flags = flags
        return d


def _draw_descs(draws: Sequence[Draw]):
    arr = (DrawDesc * max(1, len(draws)))()
    for i, d in enumerate(draws):
        arr[i] = d.desc()
    return arr


class Batch:
    """A planned batch (axr_batch): launch() enqueues it; the launch can be captured in a Graph."""

    def __init__(self, ctx: Context, draws: Sequence[Draw]):
        self.ctx = ctx
        self.draws = list(draws)
        h = C.c_void_p()
        check(ctx.lib.axr_batch_create(ctx.handle, _draw_descs(self.draws), len(self.draws), C.byref(h)), ctx.handle)
        self.handle = h

    def launch(self) -> None:
        check(self.ctx.lib.axr_batch_launch(self.ctx.handle, self.handle), self.ctx.handle)

    def info(self) -> dict:
        i = BatchInfo()
        check(self.ctx.lib.axr_batch_get_info(self.handle, C.byref(i)))
        return {k: getattr(i, k) for k, _ in BatchInfo._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.axr_batch_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def draw_table(draws: Sequence[Draw]):
    """The draws as the C array of axr_draw_desc that axr_draw_batch takes (built once; a
    host program keeps such a table and edits cameras or model matrices in place)."""
    return _draw_descs(draws)


def draw_batch(ctx: Context, draws) -> None:
    """One-shot batch (axr_draw_batch): the draw list is planned and its table uploaded on
    every call. `draws`: Draw objects, or a table from draw_table()."""
    if isinstance(draws, C.Array):
        check(ctx.lib.axr_draw_batch(ctx.handle, draws, len(draws)), ctx.handle)
        return
    check(ctx.lib.axr_draw_batch(ctx.handle, _draw_descs(draws), len(draws)), ctx.handle)


def autotune(ctx: Context, draws: Sequence[Draw], repeats: int = 3) -> list:
    """Tune the context's per-class raster parameter on these draws; returns the table."""
    out = (C.c_int32 * AXR_TUNE_CLASSES)()
    check(ctx.lib.axr_batch_autotune(ctx.handle, _draw_descs(draws), len(draws), int(repeats), out), ctx.handle)
    return list(out)


def density_class(draw: Draw) -> int:
    d = draw.desc()
    return int(_lib.load().axr_draw_density_class(C.byref(d)))


class Graph:
    """CUDA graph of the work a context enqueued between begin() and end()."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.handle = None

    def begin(self) -> "Graph":
        check(self.ctx.lib.axr_graph_begin(self.ctx.handle), self.ctx.handle)
        return self

    def end(self) -> "Graph":
        h = C.c_void_p()
        check(self.ctx.lib.axr_graph_end(self.ctx.handle, C.byref(h)), self.ctx.handle)
        self.handle = h
        return self

    def launch(self) -> None:
        check(self.ctx.lib.axr_graph_launch(self.ctx.handle, self.handle), self.ctx.handle)

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.axr_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_draws(ctx: Context, scenes, textures: Optional[dict] = None, meshes: Optional[dict] = None,
                framebuffers: Optional[list] = None, clear: bool = True) -> list:
    """Draws for workloads.Scene objects (one framebuffer each; meshes shared by identity of
    the scene's mesh object, textures by identity of the image)."""
    textures = {} if textures is None else textures
    meshes = {} if meshes is None else meshes
    out = []
    for k, sc in enumerate(scenes):
        if id(sc.mesh) not in meshes:
            meshes[id(sc.mesh)] = Mesh.from_workload(ctx, sc.mesh, textures)
        fb = framebuffers[k] if framebuffers is not None else Framebuffer(ctx, sc.width, sc.height)
        b, g, r, a = sc.clear_bgra
        sh = sc.shader
        out.append(Draw(meshes[id(sc.mesh)], fb, Camera.from_workload(sc.camera),
                        Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)), sc.model,
                        (r, g, b, a) if clear else None, float("inf") if clear else None))
    return out


# ---------------------------------------------------------------- serving loop
class Server:
    """The C++ serving loop (axr_server): register mesh assets and textures once, submit
    render requests, wait for their results. Latency is measured on the server clock."""

    def __init__(self, device: int = 0, budget_bytes: int = 40 << 30, max_batch: int = 64, max_inflight: int = 2,
                 per_request: bool = False, overlap_kernels: bool = False):
        self.lib = _lib.load()
        cfg = _lib.ServerConfig(int(device), int(budget_bytes), int(max_batch), int(max_inflight),
                                1 if per_request else 0, 1 if overlap_kernels else 0)
        h = C.c_void_p()
        st = self.lib.axr_server_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise AxrError(st, self.lib.axr_last_error(None).decode(errors="replace"))
        self.handle = h
        self._textures = {}

    def _check(self, st):
        if st != 0:
            msg = self.lib.axr_server_last_error(self.handle) or self.lib.axr_last_error(None)
            raise AxrError(st, msg.decode(errors="replace"))

    def now_ns(self) -> int:
        return int(self.lib.axr_server_now_ns())

    def add_texture(self, rgba: np.ndarray) -> int:
        rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
        out = C.c_int32()
        self._check(self.lib.axr_server_add_texture(self.handle, rgba.ctypes.data, rgba.shape[1], rgba.shape[0],
                                                    C.byref(out)))
        return out.value

    def add_mesh(self, mesh) -> int:
        """Register an axiomr_gb300.workloads.Mesh (its material textures once each)."""
        def tex(img):
            if img is None:
                return -1
            if id(img) not in self._textures:
                self._textures[id(img)] = (self.add_texture(img), img)
            return self._textures[id(img)][0]
        mats = (_lib.ServerMaterial * max(1, len(mesh.materials)))()
        for k, m in enumerate(mesh.materials):
            mats[k] = _lib.ServerMaterial(tex(m.diffuse), tex(m.bump), tex(m.metallic), tex(m.roughness), tex(m.ao),
                                          float(m.specular_exponent))
        pos, uv, nrm = _f32(mesh.positions), _f32(mesh.uvs), _f32(mesh.normals)
        tan = None if mesh.tangents is None else _f32(mesh.tangents)
        bit = None if mesh.bitangents is None else _f32(mesh.bitangents)
        idx = np.ascontiguousarray(mesh.indices, dtype=np.uint32)
        groups = np.ascontiguousarray(mesh.groups, dtype=np.uint32).reshape(-1, 3)
        d = _lib.ServerMeshDesc(pos.shape[0], pos.ctypes.data, uv.ctypes.data, nrm.ctypes.data, _ptr(tan), _ptr(bit),
                                idx.shape[0], idx.ctypes.data, groups.shape[0], groups.ctypes.data,
                                len(mesh.materials), C.cast(mats, C.c_void_p))
        out = C.c_int32()
        self._check(self.lib.axr_server_add_mesh(self.handle, C.byref(d), C.byref(out)))
        return out.value

    def submit(self, mesh_id: int, camera: "Camera", shader: Shader, width: int, height: int, model=None,
               clear_color=(0, 0, 0, 255), clear_depth: float = float("inf"), out_bgra: Optional[np.ndarray] = None,
               out_depth: Optional[np.ndarray] = None, arrival_ns: int = 0, png_channels: int = 0,
               out_png: Optional[np.ndarray] = None) -> int:
        r = _lib.ServerRequest()
        r.mesh = int(mesh_id)
        r.width, r.height = int(width), int(height)
        r.model = (C.c_float * 16)(*_model(model))
        r.camera = camera.desc()
        r.shader = shader.desc()
        flags = 0
        if clear_color is not None:
            flags |= AXR_DRAW_CLEAR_COLOR
            r.clear_rgba = (C.c_uint8 * 4)(*[int(v) for v in clear_color])
        if clear_depth is not None:
            flags |= AXR_DRAW_CLEAR_DEPTH
            r.clear_depth = float(clear_depth)
        r.clear_flags = flags
        r.arrival_ns = int(arrival_ns)
        r.out_bgra = _ptr(out_bgra)
        r.out_depth = _ptr(out_depth)
        r.png_channels = int(png_channels)
        r.out_png = _ptr(out_png)
        r.out_png_capacity = 0 if out_png is None else int(out_png.nbytes)
        t = C.c_uint64()
        self._check(self.lib.axr_server_submit(self.handle, C.byref(r), C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> dict:
        res = _lib.ServerResult()
        self._check(self.lib.axr_server_wait(self.handle, int(ticket), int(timeout_ms), C.byref(res)))
        return {k: getattr(res, k) for k, _ in _lib.ServerResult._fields_}

    def cancel(self, ticket: int) -> None:
        """Cancel a request still in the queue (axr_server_cancel); its wait() then reports
        status AXR_E_CANCELLED (8). Raises for a request already in a batch or done."""
        self._check(self.lib.axr_server_cancel(self.handle, int(ticket)))

    def hold(self, on: bool = True) -> None:
        """Stop admitting (requests queue up) / resume admitting the queue as batches."""
        self._check(self.lib.axr_server_hold(self.handle, 1 if on else 0))

    def stats(self) -> dict:
        st = _lib.ServerStats()
        self._check(self.lib.axr_server_get_stats(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.axr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def png_bound(width: int, height: int, channels: int = 3) -> int:
    """Worst-case PNG file size of a width x height framebuffer (axr_png_bound)."""
    return int(_lib.load().axr_png_bound(width, height, channels))


def read_png(ctx: "Context", framebuffers, channels: int = 3) -> list:
    """PNG files of many framebuffers, encoded by one set of launches and copied back
    (axr_framebuffers_read_png)."""
    n = len(framebuffers)
    if n == 0:
        return []
    fbs = (C.c_void_p * n)(*[fb.handle for fb in framebuffers])
    sizes = (C.c_uint64 * n)()
    bufs = [np.empty(png_bound(fb.width, fb.height, channels), np.uint8) for fb in framebuffers]
    ptrs = (C.c_void_p * n)(*[b.ctypes.data for b in bufs])
    caps = (C.c_uint64 * n)(*[b.nbytes for b in bufs])
    check(ctx.lib.axr_framebuffers_read_png(ctx.handle, n, fbs, channels, ptrs, caps, sizes), ctx.handle)
    return [bufs[i][: int(sizes[i])].tobytes() for i in range(n)]


class PngBatch:
    """Pipelined PNG read-back (axr_png_batch_*): encode() enqueues the encode of a list of
    framebuffers and returns at once; read() waits for it and copies the files to host
    memory on the batch's own streams, so a caller can render and encode the next frames
    while the previous ones come back."""

    def __init__(self, ctx: "Context"):
        self.ctx = ctx
        self.handle = C.c_void_p()
        check(ctx.lib.axr_png_batch_create(ctx.handle, C.byref(self.handle)), ctx.handle)
        self.count = 0

    def encode(self, framebuffers, channels: int = 3) -> None:
        """framebuffers: Framebuffer objects, or a ctypes array of their handles."""
        n = len(framebuffers)
        self._fbs = framebuffers if isinstance(framebuffers, C.Array) else \
            (C.c_void_p * max(1, n))(*[fb.handle for fb in framebuffers])
        check(self.ctx.lib.axr_png_batch_encode(self.ctx.handle, self.handle, n, self._fbs, channels), self.ctx.handle)
        self.count = n

    def sizes(self) -> list:
        out = (C.c_uint64 * max(1, self.count))()
        check(self.ctx.lib.axr_png_batch_sizes(self.ctx.handle, self.handle, out), self.ctx.handle)
        return [int(out[i]) for i in range(self.count)]

    def read_into(self, ptrs, capacities) -> None:
        """Copy the files to host buffers given as ctypes arrays of pointers and sizes."""
        check(self.ctx.lib.axr_png_batch_read(self.ctx.handle, self.handle, ptrs, capacities), self.ctx.handle)

    def read(self) -> list:
        sizes = self.sizes()
        bufs = [np.empty(max(1, k), np.uint8) for k in sizes]
        ptrs = (C.c_void_p * max(1, self.count))(*[b.ctypes.data for b in bufs])
        caps = (C.c_uint64 * max(1, self.count))(*[b.nbytes for b in bufs])
        self.read_into(ptrs, caps)
        return [b[:k].tobytes() for b, k in zip(bufs, sizes)]

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx.lib.axr_png_batch_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
