"""The reference-side binding (include/axr_gpu_pipeline.hpp): an AR::Pipeline subclass that
overrides drawMesh (include/pipeline.hpp:25) and forwards to the C ABI. It is compiled here
against the reference's own headers (with the oracle's shims for glm, Tracy and windows.h),
linked with the reference objects of oracle/_ref and with libaxr.so, and run: the mesh it
would upload must be the reference Mesh's (groups and materials in order, texels byte for
byte as the PNG holds them), and without a GPU the pipeline stays inert and leaves the
framebuffer as the renderer cleared it."""
import struct
import subprocess
import zlib
from pathlib import Path

import numpy as np
import pytest

from oracle import build as ob
from objfile import sphere_obj

ROOT = Path(__file__).resolve().parent.parent


def png_rgba(img: np.ndarray) -> bytes:
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


@pytest.fixture(scope="module")
def binding_exe(tmp_path_factory):
    ref = ob.build_ref()
    if ref is None:
        pytest.skip("the reference objects build only on x86 hosts with the reference tree")
    from axiomr_gb300 import build as pb

    lib = pb.build()
    root = ob.reference_root()
    shim = ob.HERE / "shim"
    out = tmp_path_factory.mktemp("binding") / "binding_check"
    cmd = ["g++", "-std=c++23", "-O1", "-ffp-contract=off", "-w", "-include", str(shim / "std_prelude.hpp"),
           f"-I{ob.REF_OUT_DIR / 'aliases'}", f"-I{shim}", f"-I{root / 'include'}", f"-I{root / 'src'}",
           f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "binding_check.cpp"), "-o", str(out),
           str(ref), str(lib), f"-Wl,-rpath,{ref.parent}", f"-Wl,-rpath,{lib.parent}", "-pthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_binding_compiles_links_and_converts_the_reference_mesh(binding_exe, tmp_path):
    tex = (np.arange(4 * 3 * 4, dtype=np.uint32) * 37 % 256).astype(np.uint8).reshape(3, 4, 4)
    (tmp_path / "tex.png").write_bytes(png_rgba(tex))
    (tmp_path / "model.obj").write_text(sphere_obj(12, 6))
    (tmp_path / "model.mtl").write_text("newmtl body\nNs 2.5\nmap_Kd tex.png\n\nnewmtl lower\nNs 7\n")
    res = subprocess.run([str(binding_exe), str(tmp_path / "model.obj")], capture_output=True, text=True,
                         check=True, timeout=120)
    lines = res.stdout.splitlines()
    counts = lines[0].split()
    faces = int(counts[3])
    assert faces == 2 * 12 * 6 and int(counts[5]) == 3 * faces  # quads fan into two triangles
    assert int(counts[7]) == 2 and int(counts[9]) == 2
    groups = [tuple(map(int, ln.split()[1:])) for ln in lines if ln.startswith("group")]
    assert groups == [(0, faces // 2, 0), (faces // 2, faces // 2, 1)]
    mats = [ln for ln in lines if ln.startswith("material")]
    assert mats == ["material Ns 2.5 diffuse 1", "material Ns 7 diffuse 0"]
    texl = [ln for ln in lines if ln.startswith("texels")][0].split()
    assert texl[1] == "4x3"
    assert np.array_equal(np.asarray(list(map(int, texl[2:])), np.uint8), tex.reshape(-1))
    last = lines[-1].split()
    if last[1] == "0":  # no GPU here: the pipeline is inert, the framebuffer as cleared
        assert int(last[3]) != 0
        assert last[5:9] == ["30", "20", "10", "255"]  # B, G, R, A of clearColor(10, 20, 30, 255)
