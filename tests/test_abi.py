"""The C ABI library loads on any host and exports every entry point include/axr.h
declares; the host-side helpers that need no GPU agree with the oracle."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from axiomr_gb300 import _lib
from axiomr_gb300 import workloads as W

HEADER = Path(__file__).resolve().parent.parent / "include" / "axr.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(axr_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_draw_path():
    names = declared_functions()
    for required in ("axr_context_create", "axr_mesh_create", "axr_texture_create", "axr_framebuffer_create",
                     "axr_set_shader", "axr_set_camera", "axr_set_framebuffer", "axr_draw_mesh",
                     "axr_draw_batch", "axr_framebuffer_read"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(_lib.SIGNATURES), "ctypes binding lags the header"


def test_camera_matrices_match_oracle(port):
    lib = _lib.load()
    rng = np.random.default_rng(11)
    cams = [W.orbit_camera(float(rng.uniform(0.5, 10)), float(rng.uniform(-89, 89)), float(rng.uniform(0, 360)),
                           640, 480, fov=float(rng.uniform(20, 120))) for _ in range(100)]
    cams += [W.Camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 60.0, 1.0, (0, 0, 1, 1)),
             W.Camera((0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 60.0, 1.0, (0, 0, 1, 1)),
             W.Camera((0.0, 5.0, 0.0), (0.0, 0.0, 0.0), 200.0, 0.01, (0, 0, 1, 1))]
    for cam in cams:
        out = np.zeros((3, 16), np.float32)
        pos = np.asarray(cam.position, np.float32)
        tgt = np.asarray(cam.target, np.float32)
        assert lib.axr_camera_matrices(pos.ctypes.data, tgt.ctypes.data, cam.fov_degrees, cam.aspect,
                                       out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data) == 0
        exp = port.camera(cam)
        assert np.array_equal(out.view(np.uint32), exp.view(np.uint32)), cam


def test_viewport_matrix():
    lib = _lib.load()
    out = np.zeros(16, np.float32)
    assert lib.axr_viewport_matrix(10, 20, 640, 480, out.ctypes.data) == 0
    m = out.reshape(4, 4)  # m[col, row]
    assert m[0, 0] == 320 and m[1, 1] == -240 and m[2, 2] == 0.5
    assert m[3, 0] == 330 and m[3, 1] == 260 and m[3, 2] == 0.5 and m[3, 3] == 1


def test_null_arguments_are_rejected_without_a_device():
    lib = _lib.load()
    assert lib.axr_context_create(0, None) == 1
    assert lib.axr_camera_matrices(None, None, 60.0, 1.0, None, None, None) == 1
    assert lib.axr_viewport_matrix(0, 0, 1, 1, None) == 1
    assert lib.axr_sync(None) == 1
    assert b"NULL" in lib.axr_last_error(None) or lib.axr_last_error(None)


def test_context_create_reports_missing_gpu():
    lib = _lib.load()
    n = C.c_int(0)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = True
    if has_gpu:
        pytest.skip("a GPU is present; covered by the gpu tests")
    h = C.c_void_p()
    st = lib.axr_context_create(0, C.byref(h))
    assert st == 6  # AXR_E_UNSUPPORTED
    assert h.value is None
    assert lib.axr_last_error(None)
    del n


def test_abi_version_matches_header():
    import re
    from pathlib import Path

    from axiomr_gb300 import _lib

    hdr = (Path(__file__).resolve().parent.parent / "include" / "axr.h").read_text()
    want = int(re.search(r"#define AXR_ABI_VERSION (\d+)", hdr).group(1))
    assert _lib.load().axr_abi_version() == want
