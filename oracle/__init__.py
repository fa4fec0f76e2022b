"""Oracle test infrastructure: Python drivers for the two CPU oracles.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package, and only as the checker (or as the timed CPU baseline); the product path never
routes through it.

* ``Oracle("port")`` -> oracle/_build/libaxo_port.so, the C restatement (any host).
* ``Oracle("ref")``  -> oracle/_ref/libaxr_ref.so, the reference sources compiled here
  (x86 only, and only where the reference tree exists).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build

HERE = Path(__file__).resolve().parent
CV_FLOATS = 18
TRI_FLOATS = 13


class Texture(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("diffuse", Texture), ("bump", Texture), ("metallic", Texture), ("roughness", Texture),
                ("ao", Texture), ("specular_exponent", C.c_float)]


class Mesh(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", C.c_void_p), ("uvs", C.c_void_p),
                ("normals", C.c_void_p), ("tangents", C.c_void_p), ("bitangents", C.c_void_p),
                ("num_faces", C.c_uint32), ("indices", C.c_void_p), ("num_groups", C.c_uint32),
                ("groups", C.c_void_p), ("num_materials", C.c_uint32), ("materials", C.c_void_p)]


class Shader(C.Structure):
    _fields_ = [("kind", C.c_int32), ("light_direction", C.c_float * 3), ("light_color", C.c_float * 3)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("target", C.c_float * 3), ("fov_degrees", C.c_float),
                ("aspect", C.c_float), ("viewport", C.c_int32 * 4)]


def _ptr(a):
    return None if a is None else a.ctypes.data


class _Keep:
    """Holds numpy arrays alive while C structs point at them."""

    def __init__(self):
        self.refs = []

    def arr(self, a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a


def _texture(keep, img):
    if img is None:
        return Texture(None, 0, 0)
    a = keep.arr(img, np.uint8)
    return Texture(_ptr(a), a.shape[1], a.shape[0])


def make_material(keep, m) -> Material:
    return Material(_texture(keep, m.diffuse), _texture(keep, m.bump), _texture(keep, m.metallic),
                    _texture(keep, m.roughness), _texture(keep, m.ao), float(m.specular_exponent))


def make_mesh(keep, mesh) -> Mesh:
    mats = (Material * max(1, len(mesh.materials)))(*[make_material(keep, m) for m in mesh.materials])
    keep.refs.append(mats)
    f32 = np.float32
    return Mesh(mesh.num_vertices, _ptr(keep.arr(mesh.positions, f32)), _ptr(keep.arr(mesh.uvs, f32)),
                _ptr(keep.arr(mesh.normals, f32)), _ptr(keep.arr(mesh.tangents, f32)),
                _ptr(keep.arr(mesh.bitangents, f32)), mesh.num_faces, _ptr(keep.arr(mesh.indices, np.uint32)),
                int(mesh.groups.shape[0]), _ptr(keep.arr(mesh.groups, np.uint32)), len(mesh.materials),
                C.addressof(mats))


def make_shader(s) -> Shader:
    return Shader(int(s.kind), (C.c_float * 3)(*s.light_direction), (C.c_float * 3)(*s.light_color))


def make_camera(c) -> Camera:
    return Camera((C.c_float * 3)(*c.position), (C.c_float * 3)(*c.target), float(c.fov_degrees),
                  float(c.aspect), (C.c_int32 * 4)(*c.viewport))


class Obj(C.Structure):
    _fields_ = [("num_positions", C.c_uint32), ("positions", C.c_void_p), ("num_uvs", C.c_uint32),
                ("uvs", C.c_void_p), ("num_normals", C.c_uint32), ("normals", C.c_void_p),
                ("num_corners", C.c_uint32), ("corners", C.c_void_p), ("num_polygons", C.c_uint32),
                ("polygon_sizes", C.c_void_p)]


class Oracle:
    """One CPU oracle library (kind "port" or "ref")."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            path = build.build_port()
        elif kind == "ref":
            path = build.build_ref()
            if path is None:
                raise RuntimeError("the reference oracle is only built on x86 hosts with the reference tree")
        else:
            raise ValueError(kind)
        self.lib = C.CDLL(str(path))
        p = kind + "_"
        vp, i32, fp = C.c_void_p, C.c_int, C.c_void_p
        self._camera = getattr(self.lib, p + "camera")
        self._camera.argtypes = [vp, fp]
        self._clip = getattr(self.lib, p + "clip_triangle")
        self._clip.argtypes = [fp, fp, C.POINTER(C.c_int)]
        self._tri = getattr(self.lib, p + "triangle")
        self._tri.argtypes = [fp, i32, i32, fp, C.POINTER(C.c_int)]
        self._sample = getattr(self.lib, p + "sample")
        self._sample.argtypes = [vp, fp, i32, fp]
        self._shade = getattr(self.lib, p + "shade")
        self._shade.argtypes = [vp, vp, fp, fp, fp, fp, fp, fp]
        self._render = getattr(self.lib, p + "render")
        self._render.argtypes = [vp, fp, vp, vp, i32, i32, i32, i32, vp, fp, fp]
        self._draw = getattr(self.lib, p + "draw")
        self._draw.argtypes = [vp, fp, fp, fp, vp, i32, i32, i32, vp, fp]
        for f in (self._camera, self._clip, self._tri, self._sample, self._shade, self._render, self._draw):
            f.restype = C.c_int

    # -- mesh ingest --------------------------------------------------------------------
    def obj_ingest(self, parsed: dict):
        """Port only: de-duplicated vertices (n, 14) and faces (m, 3) of a parsed OBJ
        model (tests/objfile.parse_obj output)."""
        if self.kind != "port":
            raise ValueError("obj_ingest is the port's; the reference loads files (obj_load)")
        pos = np.ascontiguousarray(parsed["positions"], np.float32)
        uv = np.ascontiguousarray(parsed["uvs"], np.float32)
        nrm = np.ascontiguousarray(parsed["normals"], np.float32)
        cor = np.ascontiguousarray(parsed["corners"], np.int32)
        sizes = np.ascontiguousarray(parsed["polygon_sizes"], np.uint32)
        o = Obj(pos.shape[0], pos.ctypes.data, uv.shape[0], uv.ctypes.data, nrm.shape[0], nrm.ctypes.data,
                cor.shape[0], cor.ctypes.data, sizes.shape[0], sizes.ctypes.data)
        nc = max(1, cor.shape[0])
        verts = np.zeros((nc, 14), np.float32)
        faces = np.zeros((nc, 3), np.uint32)
        nv, nf = C.c_uint32(), C.c_uint32()
        f = self.lib.port_obj_ingest
        f.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p, C.POINTER(C.c_uint32)]
        f.restype = C.c_int
        if f(C.addressof(o), verts.ctypes.data, C.byref(nv), faces.ctypes.data, C.byref(nf)) != 0:
            raise RuntimeError("port_obj_ingest failed")
        return verts[: nv.value].copy(), faces[: nf.value].copy()

    def obj_load(self, path: str):
        """Reference only: AR::Mesh(path) -> vertices (n, 14), faces (m, 3), groups (g, 2)."""
        if self.kind != "ref":
            raise ValueError("obj_load runs the reference loader")
        counts = (C.c_uint32 * 3)()
        self.lib.ref_obj_load.argtypes = [C.c_char_p, C.c_void_p]
        if self.lib.ref_obj_load(str(path).encode(), counts) != 0:
            raise RuntimeError("reference Mesh(path) failed")
        verts = np.zeros((max(1, counts[0]), 14), np.float32)
        faces = np.zeros((max(1, counts[1]), 3), np.uint32)
        groups = np.zeros((max(1, counts[2]), 2), np.uint64)
        self.lib.ref_obj_fetch.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        self.lib.ref_obj_fetch(verts.ctypes.data, faces.ctypes.data, groups.ctypes.data)
        return verts[: counts[0]], faces[: counts[1]], groups[: counts[2]]

    def camera_script(self, cam, ops) -> np.ndarray:
        """Reference only: the Camera driven by a script of operations (rows of 6 floats:
        kind, a0..a3, flags; kinds 0 update(dt), 1 handleInput(mouse x, y; flags bit 0 right
        button, bits 1-4 keys W S A D), 2 setPosition, 3 setTarget, 4 setFov,
        5 setAspectRatio, 6 setViewport) -> (n, 51): view, projection, viewProjection and
        position after each operation."""
        if self.kind != "ref":
            raise ValueError("camera_script runs the reference Camera")
        ops = np.ascontiguousarray(ops, np.float32).reshape(-1, 6)
        out = np.zeros((ops.shape[0], 51), np.float32)
        c = make_camera(cam)
        f = self.lib.ref_camera_script
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        f.restype = C.c_int
        if f(C.addressof(c), ops.ctypes.data, ops.shape[0], out.ctypes.data) != 0:
            raise RuntimeError("bad camera script")
        return out

    # -- stages -----------------------------------------------------------------------
    def camera(self, cam) -> np.ndarray:
        """(3, 16) float32: view, projection, viewProjection (column-major)."""
        out = np.zeros(48, np.float32)
        c = make_camera(cam)
        self._camera(C.addressof(c), out.ctypes.data)
        return out.reshape(3, 16)

    def clip_triangle(self, verts3: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(verts3, np.float32).reshape(3 * CV_FLOATS)
        out = np.zeros(24 * CV_FLOATS, np.float32)
        n = C.c_int(0)
        self._clip(v.ctypes.data, out.ctypes.data, C.byref(n))
        return out[: n.value * CV_FLOATS].reshape(n.value, CV_FLOATS)

    def triangle(self, verts3: np.ndarray, width: int, height: int):
        v = np.ascontiguousarray(verts3, np.float32).reshape(3 * CV_FLOATS)
        out = np.zeros(TRI_FLOATS, np.float32)
        bf = C.c_int(0)
        self._tri(v.ctypes.data, width, height, out.ctypes.data, C.byref(bf))
        return out, bool(bf.value)

    def sample(self, img: np.ndarray, uv: np.ndarray) -> np.ndarray:
        keep = _Keep()
        t = _texture(keep, img)
        uvf = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        out = np.zeros((uvf.shape[0], 4), np.float32)
        rc = self._sample(C.addressof(t), uvf.ctypes.data, uvf.shape[0], out.ctypes.data)
        if rc:
            raise RuntimeError(f"{self.kind}_sample failed ({rc})")
        return out

    def shade(self, shader, material, model, view_proj, cam_pos, verts3x14, bar) -> np.ndarray:
        keep = _Keep()
        s = make_shader(shader)
        m = make_material(keep, material)
        arrs = [keep.arr(a, np.float32) for a in (model, view_proj, cam_pos, verts3x14, bar)]
        out = np.zeros(4, np.float32)
        rc = self._shade(C.addressof(s), C.addressof(m), *[a.ctypes.data for a in arrs], out.ctypes.data)
        if rc:
            raise RuntimeError(f"{self.kind}_shade failed ({rc})")
        return out

    # -- whole draw ---------------------------------------------------------------------
    def render(self, scene, bgra=None, depth=None, threads: int = 0, max_faces_per_draw: int = 16384):
        """Draw `scene` into a host framebuffer (cleared as the renderer does unless one is
        given). Returns (bgra (H, W, 4) uint8, depth (H, W) float32, matrices (3, 16))."""
        from axiomr_gb300.workloads import clear_framebuffer

        if bgra is None or depth is None:
            bgra, depth = clear_framebuffer(scene)
        bgra = np.ascontiguousarray(bgra, np.uint8).copy()
        depth = np.ascontiguousarray(depth, np.float32).copy()
        keep = _Keep()
        mesh = make_mesh(keep, scene.mesh)
        cam = make_camera(scene.camera)
        sh = make_shader(scene.shader)
        model = keep.arr(scene.model, np.float32)
        mats = np.zeros(48, np.float32)
        rc = self._render(C.addressof(mesh), model.ctypes.data, C.addressof(cam), C.addressof(sh),
                          scene.width, scene.height, threads, max_faces_per_draw, bgra.ctypes.data,
                          depth.ctypes.data, mats.ctypes.data)
        if rc:
            raise RuntimeError(f"{self.kind}_render failed ({rc})")
        return bgra, depth, mats.reshape(3, 16)


    def draw(self, scene, view_proj, cam_pos=None, bgra=None, depth=None, threads: int = 0):
        """Draw `scene` with an explicit view-projection matrix (16 floats, column-major)
        and eye position (default: the scene camera's). Returns (bgra, depth)."""
        from axiomr_gb300.workloads import clear_framebuffer

        if bgra is None or depth is None:
            bgra, depth = clear_framebuffer(scene)
        bgra = np.ascontiguousarray(bgra, np.uint8).copy()
        depth = np.ascontiguousarray(depth, np.float32).copy()
        keep = _Keep()
        mesh = make_mesh(keep, scene.mesh)
        sh = make_shader(scene.shader)
        model = keep.arr(scene.model, np.float32)
        vp = keep.arr(np.asarray(view_proj, np.float32).reshape(16), np.float32)
        cp = keep.arr(np.asarray(scene.camera.position if cam_pos is None else cam_pos, np.float32), np.float32)
        rc = self._draw(C.addressof(mesh), model.ctypes.data, vp.ctypes.data, cp.ctypes.data, C.addressof(sh),
                        scene.width, scene.height, threads, bgra.ctypes.data, depth.ctypes.data)
        if rc:
            raise RuntimeError(f"{self.kind}_draw failed ({rc})")
        return bgra, depth


def ref_available() -> bool:
    return build.ref_available()
