"""The reference Camera's state and motion (src/camera.cpp:30-205) on the host: the
library's axr_camera_* functions against the reference Camera class itself (compiled in
oracle/_ref, driven with a window whose input members are set directly) on seeded scripts
of setters, mouse / keyboard input and updates, and against fixtures made from it."""
import numpy as np
import pytest

import camscript
from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from helpers import GOLDEN, same_bits


def lib_camera(start):
    pos, tgt, fov, aspect = start
    return api.Camera(pos, tgt, fov, aspect, (0, 0, 800, 600), update=False)


def ref_camera(start):
    pos, tgt, fov, aspect = start
    return W.Camera(pos, tgt, fov, aspect, (0, 0, 800, 600))


@pytest.mark.parametrize("k", range(len(camscript.STARTS)))
def test_camera_scripts_match_reference_live(ref, k):
    for seed in range(3):
        ops = camscript.script(100 * k + seed)
        want = ref.camera_script(ref_camera(camscript.STARTS[k]), ops)
        got = camscript.run(lib_camera(camscript.STARTS[k]), ops)
        bad = [i for i in range(len(ops)) if not same_bits(got[i], want[i])]
        assert not bad, f"start {k} seed {seed}: first differing op {bad[0]} {ops[bad[0]].tolist()}"


def test_camera_scripts_match_reference_fixture():
    z = np.load(GOLDEN / "camera_scripts.npz")
    for k in range(len(camscript.STARTS)):
        ops = z[f"ops_{k}"]
        got = camscript.run(lib_camera(camscript.STARTS[k]), ops)
        assert same_bits(got, z[f"out_{k}"]), k


def test_camera_behaviour_kept_from_reference():
    cam = lib_camera(camscript.STARTS[1])
    # the constructor leaves the view at identity (viewProjection = projection)
    assert np.array_equal(cam.view, np.eye(4, dtype=np.float32).reshape(16))
    assert np.array_equal(cam.view_proj, cam.projection)
    cam.update(0.0)
    vp = cam.view_proj
    # setFov / setAspectRatio never reach the matrices
    cam.setFov(20.0)
    cam.setAspectRatio(3.0)
    cam.update(0.5)
    assert np.array_equal(cam.view_proj, vp)
    # a horizontal-only mouse drag does not rotate (both deltas must be non-zero)
    cam.handleInput((100.0, 100.0), True)
    cam.handleInput((140.0, 100.0), True)
    cam.update(0.1)
    assert np.array_equal(cam.view_proj, vp)
    # a diagonal drag does; WASD moves by unit vectors per second
    cam.handleInput((180.0, 130.0), True, "W")
    cam.update(0.1)
    assert not np.array_equal(cam.view_proj, vp)
    p0 = np.array(cam.position)
    cam.handleInput((180.0, 130.0), False, "D")
    cam.update(2.0)
    assert abs(np.linalg.norm(np.array(cam.position) - p0) - 2.0) < 1e-4
