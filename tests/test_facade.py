"""The C++ facade (include/axr.hpp) compiles against the C ABI, and (on a GPU) renders
through Renderer::drawMesh exactly what the CPU oracle renders."""
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from axiomr_gb300 import workloads as W
from helpers import assert_parity

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "facade_render.cpp"


def test_facade_header_compiles(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", "-fsyntax-only",
                    str(SRC)], check=True)


def write_scene(path, sc):
    m = sc.mesh
    tex = m.materials[0].diffuse
    with open(path, "wb") as f:
        f.write(struct.pack("<IIi", sc.width, sc.height, sc.shader.kind))
        f.write(np.asarray(list(sc.shader.light_direction) + list(sc.shader.light_color) + list(sc.camera.position)
                           + list(sc.camera.target) + [sc.camera.fov_degrees, sc.camera.aspect], np.float32).tobytes())
        f.write(np.asarray(sc.model, np.float32).tobytes())
        f.write(struct.pack("<II", m.num_vertices, m.num_faces))
        for a in (m.positions, m.uvs, m.normals):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())
        f.write(np.ascontiguousarray(m.indices, np.uint32).tobytes())
        f.write(struct.pack("<II", tex.shape[1], tex.shape[0]))
        f.write(np.ascontiguousarray(tex, np.uint8).tobytes())
        f.write(struct.pack("<f", m.materials[0].specular_exponent))


@pytest.mark.gpu
def test_facade_renders_like_oracle(tmp_path, port):
    from axiomr_gb300 import build

    lib = build.build()
    exe = tmp_path / "facade_render"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
                    f"-L{lib.parent}", "-laxr", f"-Wl,-rpath,{lib.parent}"], check=True)
    sc = W.sphere_scene(width=240, height=180, lon=48, lat=24, tex_size=128)
    write_scene(tmp_path / "scene.bin", sc)
    subprocess.run([str(exe), str(tmp_path / "scene.bin"), str(tmp_path / "out.bin")], check=True)
    raw = (tmp_path / "out.bin").read_bytes()
    n = sc.width * sc.height
    bgra = np.frombuffer(raw[: 4 * n], np.uint8).reshape(sc.height, sc.width, 4)
    depth = np.frombuffer(raw[4 * n:], np.float32).reshape(sc.height, sc.width)
    exp = port.render(sc)[:2]
    assert_parity((bgra, depth), exp, "C++ facade")


def test_facade_camera_matches_reference_fixture(tmp_path):
    """The camera behind axr::Camera (axr_camera_*), driven from C++, reproduces the
    reference Camera's matrices after every operation of the fixture scripts; the facade
    class itself equals the Python binding's camera."""
    import camscript
    from axiomr_gb300 import api, build

    if not shutil.which("g++"):
        pytest.skip("no g++")
    lib = build.build()
    exe = tmp_path / "facade_camera"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "facade_camera.cpp"), "-o", str(exe), f"-L{lib.parent}", "-laxr",
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    z = np.load(ROOT / "tests" / "golden" / "camera_scripts.npz")
    for k, (pos, tgt, fov, aspect) in enumerate(camscript.STARTS):
        ops = z[f"ops_{k}"]
        script = tmp_path / f"s{k}.bin"
        with open(script, "wb") as f:
            f.write(np.asarray([*pos, *tgt, fov, aspect], np.float32).tobytes())
            f.write(struct.pack("<I", ops.shape[0]))
            f.write(np.ascontiguousarray(ops, np.float32).tobytes())
        out = tmp_path / f"o{k}.bin"
        subprocess.run([str(exe), str(script), str(out)], check=True)
        got = np.fromfile(out, np.float32)
        n = ops.shape[0]
        assert np.array_equal(got[: 51 * n].reshape(n, 51).view(np.uint32), z[f"out_{k}"].view(np.uint32)), k
        cam = api.Camera(pos, tgt, fov, aspect)
        cam.handleInput((10.0, 10.0), True)
        cam.handleInput((40.0, 25.0), True, "W")
        cam.update(0.1)
        assert np.array_equal(got[51 * n:].view(np.uint32), cam.view_proj.view(np.uint32)), k
