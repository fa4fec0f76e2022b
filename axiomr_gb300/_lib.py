"""ctypes binding of the C ABI in include/axr.h (axiomr_gb300/_bin/libaxr.so).

The library is the only implementation of the draw path: if it cannot be built or
loaded, every call raises; there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

AXR_OK = 0
STATUS_NAMES = {0: "AXR_OK", 1: "AXR_E_INVALID", 2: "AXR_E_OOM", 3: "AXR_E_BUDGET", 4: "AXR_E_TIMEOUT",
                5: "AXR_E_CUDA", 6: "AXR_E_UNSUPPORTED", 7: "AXR_E_CAPACITY", 8: "AXR_E_CANCELLED"}


class AxrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class MaterialDesc(C.Structure):
    _fields_ = [("diffuse", C.c_void_p), ("bump", C.c_void_p), ("metallic", C.c_void_p),
                ("roughness", C.c_void_p), ("ao", C.c_void_p), ("specular_exponent", C.c_float)]


class GroupDesc(C.Structure):
    _fields_ = [("start_face", C.c_uint32), ("face_count", C.c_uint32), ("material", C.c_uint32)]


class MeshDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", C.c_void_p), ("uvs", C.c_void_p),
                ("normals", C.c_void_p), ("tangents", C.c_void_p), ("bitangents", C.c_void_p),
                ("num_faces", C.c_uint32), ("indices", C.c_void_p), ("num_groups", C.c_uint32),
                ("groups", C.c_void_p), ("num_materials", C.c_uint32), ("materials", C.c_void_p)]


class ShaderDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("light_direction", C.c_float * 3), ("light_color", C.c_float * 3)]


class CameraDesc(C.Structure):
    _fields_ = [("view_proj", C.c_float * 16), ("viewport", C.c_float * 16), ("position", C.c_float * 3)]


AXR_DRAW_CLEAR_COLOR = 1
AXR_DRAW_CLEAR_DEPTH = 2
AXR_TUNE_CLASSES = 6


class DrawDesc(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("framebuffer", C.c_void_p), ("model", C.c_float * 16),
                ("camera", CameraDesc), ("shader", ShaderDesc), ("clear_flags", C.c_uint32),
                ("clear_rgba", C.c_uint8 * 4), ("clear_depth", C.c_float)]


AXR_BATCH_PERSISTENT = 0


class BinParams(C.Structure):
    """axr_bin_params: entries per bin, bin shape (tiles across and down), per-thread raster limit."""
    _fields_ = [("capacity", C.c_int32), ("tiles_x", C.c_int32), ("thread_pixels", C.c_int32), ("tiles_y", C.c_int32)]
AXR_BATCH_PHASED = 1


class BatchInfo(C.Structure):
    _fields_ = [("draws", C.c_uint32), ("launches", C.c_uint32), ("form", C.c_int32), ("pad_", C.c_uint32),
                ("vertices", C.c_uint64), ("faces", C.c_uint64),
                ("pixels", C.c_uint64), ("tiles", C.c_uint64), ("device_bytes", C.c_uint64)]


class ObjDesc(C.Structure):
    _fields_ = [("num_positions", C.c_uint32), ("positions", C.c_void_p), ("num_uvs", C.c_uint32),
                ("uvs", C.c_void_p), ("num_normals", C.c_uint32), ("normals", C.c_void_p),
                ("num_corners", C.c_uint32), ("corners", C.c_void_p), ("num_polygons", C.c_uint32),
                ("polygon_sizes", C.c_void_p), ("num_groups", C.c_uint32), ("groups", C.c_void_p),
                ("num_materials", C.c_uint32), ("materials", C.c_void_p)]


class Profile(C.Structure):
    _fields_ = [("draws", C.c_uint32), ("pad_", C.c_uint32), ("vertex_ms", C.c_double), ("geometry_ms", C.c_double),
                ("large_ms", C.c_double), ("scan_ms", C.c_double), ("shade_ms", C.c_double),
                ("clipped_ms", C.c_double), ("kernel_launches", C.c_uint64), ("batch_launches", C.c_uint64),
                ("batch_vertex_ms", C.c_double), ("batch_face_ms", C.c_double), ("batch_large_ms", C.c_double),
                ("batch_tile_ms", C.c_double), ("batch_clear_ms", C.c_double)]


class CameraState(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("orientation", C.c_float * 4), ("forward", C.c_float * 3),
                ("right", C.c_float * 3), ("up", C.c_float * 3), ("delta_yaw", C.c_float), ("delta_pitch", C.c_float),
                ("velocity", C.c_float * 3), ("fov_degrees", C.c_float), ("aspect_ratio", C.c_float),
                ("near_plane", C.c_float), ("far_plane", C.c_float), ("movement_speed", C.c_float),
                ("mouse_sensitivity", C.c_float), ("last_mouse", C.c_float * 2), ("viewport", C.c_int32 * 4),
                ("view", C.c_float * 16), ("projection", C.c_float * 16), ("view_proj", C.c_float * 16),
                ("view_dirty", C.c_int32), ("projection_dirty", C.c_int32)]


class InputState(C.Structure):
    _fields_ = [("mouse", C.c_float * 2), ("mouse_buttons", C.c_uint8 * 3), ("keys", C.c_uint8 * 256)]


class DrawStats(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("fragments", C.c_uint64), ("large", C.c_uint64), ("tiles", C.c_uint64),
                ("tested", C.c_uint64), ("shaded", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("memory_budget_bytes", C.c_uint64), ("max_batch", C.c_int32),
                ("max_inflight", C.c_int32), ("per_request", C.c_int32), ("overlap_kernels", C.c_int32)]


class ServerMaterial(C.Structure):
    _fields_ = [("diffuse", C.c_int32), ("bump", C.c_int32), ("metallic", C.c_int32), ("roughness", C.c_int32),
                ("ao", C.c_int32), ("specular_exponent", C.c_float)]


class ServerMeshDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", C.c_void_p), ("uvs", C.c_void_p),
                ("normals", C.c_void_p), ("tangents", C.c_void_p), ("bitangents", C.c_void_p),
                ("num_faces", C.c_uint32), ("indices", C.c_void_p), ("num_groups", C.c_uint32),
                ("groups", C.c_void_p), ("num_materials", C.c_uint32), ("materials", C.c_void_p)]


class ServerRequest(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("model", C.c_float * 16),
                ("camera", CameraDesc), ("shader", ShaderDesc), ("clear_flags", C.c_uint32),
                ("clear_rgba", C.c_uint8 * 4), ("clear_depth", C.c_float), ("arrival_ns", C.c_uint64),
                ("out_bgra", C.c_void_p), ("out_depth", C.c_void_p), ("png_channels", C.c_uint32),
                ("out_png", C.c_void_p), ("out_png_capacity", C.c_uint64)]


class ServerResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_uint32), ("arrival_ns", C.c_uint64),
                ("launch_ns", C.c_uint64), ("done_ns", C.c_uint64), ("batch_id", C.c_uint64),
                ("png_bytes", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("batches", C.c_uint64),
                ("uploads", C.c_uint64), ("evictions", C.c_uint64), ("framebuffers", C.c_uint64),
                ("resident_bytes", C.c_uint64), ("peak_bytes", C.c_uint64)]


P = C.c_void_p
FP = C.POINTER(C.c_float)
U8P = C.POINTER(C.c_uint8)
PP = C.POINTER(C.c_void_p)
S = C.c_int

# name -> (restype, argtypes); every function the header declares
SIGNATURES = {
    "axr_context_create": (S, [C.c_int32, PP]),
    "axr_context_destroy": (None, [P]),
    "axr_last_error": (C.c_char_p, [P]),
    "axr_context_stream": (P, [P]),
    "axr_context_set_stream": (S, [P, P]),
    "axr_sync": (S, [P]),
    "axr_reserve": (S, [P, C.c_uint32]),
    "axr_host_alloc": (P, [C.c_size_t]),
    "axr_host_free": (None, [P]),
    "axr_texture_create": (S, [P, P, C.c_int32, C.c_int32, PP]),
    "axr_texture_update": (S, [P, P, P]),
    "axr_texture_destroy": (None, [P, P]),
    "axr_mesh_create": (S, [P, P, PP]),
    "axr_mesh_update": (S, [P, P, P]),
    "axr_mesh_create_from_obj": (S, [P, P, PP]),
    "axr_mesh_read": (S, [P, P, P, P]),
    "axr_mesh_counts": (S, [P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "axr_mesh_destroy": (None, [P, P]),
    "axr_framebuffer_create": (S, [P, C.c_int32, C.c_int32, PP]),
    "axr_framebuffer_destroy": (None, [P, P]),
    "axr_framebuffer_clear_color": (S, [P, P, C.c_uint8, C.c_uint8, C.c_uint8, C.c_uint8]),
    "axr_framebuffer_clear_depth": (S, [P, P, C.c_float]),
    "axr_framebuffer_read": (S, [P, P, P, P]),
    "axr_framebuffer_read_async": (S, [P, P, P, P]),
    "axr_framebuffer_write": (S, [P, P, P, P]),
    "axr_framebuffers_read_async": (S, [P, C.c_int32, P, P, P]),
    "axr_readback_create": (S, [P, PP]),
    "axr_readback_destroy": (None, [P, P]),
    "axr_readback_start": (S, [P, P, C.c_int32, P, P, P]),
    "axr_readback_wait": (S, [P, P]),
    "axr_readback_start_packed": (S, [P, P, C.c_int32, P, C.c_int32, P, C.c_uint64]),
    "axr_framebuffer_size": (S, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "axr_framebuffer_device_pointers": (S, [P, PP, PP]),
    "axr_abi_version": (C.c_int32, []),
    "axr_diag_barrier_timeout": (S, [P, C.c_uint32]),
    "axr_camera_init": (S, [P, P, P, C.c_float, C.c_float]),
    "axr_camera_set_position": (S, [P, P]),
    "axr_camera_set_target": (S, [P, P]),
    "axr_camera_set_fov": (S, [P, C.c_float]),
    "axr_camera_set_aspect_ratio": (S, [P, C.c_float]),
    "axr_camera_set_viewport": (S, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "axr_camera_handle_input": (S, [P, P]),
    "axr_camera_update": (S, [P, C.c_float]),
    "axr_camera_describe": (S, [P, P]),
    "axr_png_bound": (C.c_uint64, [C.c_uint32, C.c_uint32, C.c_uint32]),
    "axr_framebuffers_encode_png": (S, [P, C.c_int32, P, C.c_uint32, P, P, P]),
    "axr_framebuffers_read_png": (S, [P, C.c_int32, P, C.c_uint32, P, P, P]),
    "axr_png_batch_create": (S, [P, PP]),
    "axr_png_batch_destroy": (None, [P, P]),
    "axr_png_batch_encode": (S, [P, P, C.c_int32, P, C.c_uint32]),
    "axr_png_batch_sizes": (S, [P, P, P]),
    "axr_png_batch_read": (S, [P, P, P, P]),
    "axr_set_shader": (S, [P, P]),
    "axr_set_camera": (S, [P, P]),
    "axr_set_framebuffer": (S, [P, P]),
    "axr_draw_mesh": (S, [P, P, P]),
    "axr_draw_mesh_noalloc": (S, [P, P, P]),
    "axr_batch_create": (S, [P, P, C.c_int32, PP]),
    "axr_batch_launch": (S, [P, P]),
    "axr_batch_destroy": (None, [P, P]),
    "axr_batch_get_info": (S, [P, P]),
    "axr_draw_batch": (S, [P, P, C.c_int32]),
    "axr_batch_autotune": (S, [P, P, C.c_int32, C.c_int32, P]),
    "axr_batch_get_tuning": (S, [P, P]),
    "axr_batch_set_tuning": (S, [P, P]),
    "axr_draw_density_class": (C.c_int32, [P]),
    "axr_batch_set_form": (S, [P, C.c_int32]),
    "axr_measure_fp32_peak": (S, [P, C.POINTER(C.c_double)]),
    "axr_server_create": (S, [P, PP]),
    "axr_server_destroy": (None, [P]),
    "axr_server_now_ns": (C.c_uint64, []),
    "axr_server_add_texture": (S, [P, P, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "axr_server_add_mesh": (S, [P, P, C.POINTER(C.c_int32)]),
    "axr_server_submit": (S, [P, P, C.POINTER(C.c_uint64)]),
    "axr_server_wait": (S, [P, C.c_uint64, C.c_int32, P]),
    "axr_server_get_stats": (S, [P, P]),
    "axr_server_hold": (S, [P, C.c_int32]),
    "axr_server_cancel": (S, [P, C.c_uint64]),
    "axr_server_last_error": (C.c_char_p, [P]),
    "axr_batch_get_form": (C.c_int32, [P]),
    "axr_set_draw_form": (S, [P, C.c_int32]),
    "axr_get_draw_form": (C.c_int32, [P]),
    "axr_set_bin_params": (S, [P, P]),
    "axr_get_bin_params": (S, [P, P]),
    "axr_batch_get_bin_tuning": (S, [P, P]),
    "axr_batch_set_bin_tuning": (S, [P, P]),
    "axr_graph_begin": (S, [P]),
    "axr_graph_end": (S, [P, PP]),
    "axr_graph_launch": (S, [P, P]),
    "axr_graph_destroy": (None, [P]),
    "axr_camera_matrices": (S, [P, P, C.c_float, C.c_float, P, P, P]),
    "axr_viewport_matrix": (S, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, P]),
    "axr_stats_enable": (S, [P, C.c_int32]),
    "axr_stats_read": (S, [P, P]),
    "axr_profile_enable": (S, [P, C.c_int32]),
    "axr_profile_read": (S, [P, P]),
    "axr_debug_triangles": (S, [P, P, P, P, C.c_int32, C.c_int32, P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "axr_debug_sample": (S, [P, P, P, C.c_int32, P]),
}

_lib = None
_lock = threading.Lock()


def library_path():
    return _build.LIB


def load(build_if_needed: bool = True):
    """Load libaxr.so (building it first when sources are newer), bind all symbols."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build() if build_if_needed else _build.LIB
            if not path.exists():
                raise OSError(f"{path} not found: the CUDA extension has not been built")
            lib = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status: int, ctx=None) -> None:
    if status != AXR_OK:
        lib = load()
        msg = lib.axr_last_error(ctx).decode(errors="replace") if lib else ""
        raise AxrError(status, msg)
