"""Oracle test infrastructure: build recipes for the two CPU oracles.

* ``build_port()`` compiles the C restatement in ``oracle/port`` into
  ``oracle/_build/libaxo_port.so``. It builds on any host (x86 here, aarch64 on the GPU
  box) and is the checker the GPU parity tests and the CPU baseline use.
* ``build_ref()`` compiles the AxiomR reference sources *where they lie* (the reference
  tree: ``AXR_REFERENCE``, else ``reference`` beside the repository root) together with the
  project's shims in ``oracle/shim`` and ``oracle/ref_harness.cpp`` into
  ``oracle/_ref/libaxr_ref.so``. No reference source is copied. The reference's
  rasteriser uses AVX2 (and contains unused AVX-512 variants), so this build is x86-only;
  on other hosts, or when the reference tree is absent, it is skipped.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use these
libraries; the product never links them.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
PORT_SRC = HERE / "port"
PORT_OUT = HERE / "_build" / "libaxo_port.so"
REF_OUT_DIR = HERE / "_ref"
REF_OUT = REF_OUT_DIR / "libaxr_ref.so"

# Reference translation units on the drawMesh path (plus what they link against).
# window*.cpp, renderer.cpp and main.cpp are Win32 / application code and are left out.
REF_TUS = [
    "src/tiled_pipeline.cpp",
    "src/pipeline.cpp",
    "src/framebuffer.cpp",
    "src/texture.cpp",
    "src/thread_pool.cpp",
    "src/camera.cpp",
    "src/mesh.cpp",
    "external/stb_image/stb_image.cpp",
]

# The reference includes several headers by Windows paths ("glm\glm.hpp",
# <tracy\Tracy.hpp>) and one with different case ("Framebuffer.hpp"). On Linux a
# backslash is an ordinary filename character, so these one-line forwarding files are
# generated into the build directory rather than kept in the repository.
ALIASES = {
    "glm\\glm.hpp": '#include "glm/glm.hpp"\n',
    "glm\\gtc\\matrix_transform.hpp": '#include "glm/gtc/matrix_transform.hpp"\n',
    "tracy\\Tracy.hpp": '#include "tracy/Tracy.hpp"\n',
    "Framebuffer.hpp": '#include "framebuffer.hpp"\n',
}


def reference_root() -> Path:
    env = os.environ.get("AXR_REFERENCE")
    return Path(env) if env else HERE.parent.parent / "reference"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def build_port(force: bool = False) -> Path:
    srcs = sorted(PORT_SRC.glob("*.c"))
    deps = srcs + sorted(PORT_SRC.glob("*.h")) + [HERE / "axo.h"]
    if not force and not _stale(PORT_OUT, deps):
        return PORT_OUT
    PORT_OUT.parent.mkdir(parents=True, exist_ok=True)
    objdir = PORT_OUT.parent / "port_obj"
    objdir.mkdir(exist_ok=True)
    # -ffp-contract=off: every float operation rounds on its own, as in the reference
    # build; no -ffast-math; portable code only (no -march flags).
    cflags = ["-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
              "-Wall", "-Wextra", "-Wno-unused-parameter", "-D_GNU_SOURCE", f"-I{HERE}", f"-I{PORT_SRC}"]

    def cc(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        _run(["gcc", *cflags, "-c", str(src), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        objs = list(ex.map(cc, srcs))
    tmp = PORT_OUT.with_suffix(".so.tmp")
    _run(["gcc", "-shared", "-pthread", *map(str, objs), "-o", str(tmp), "-lm"])
    tmp.replace(PORT_OUT)
    return PORT_OUT


def ref_available() -> bool:
    root = reference_root()
    return platform.machine() in ("x86_64", "AMD64") and all((root / t).exists() for t in REF_TUS)


def build_ref(force: bool = False) -> Path | None:
    """Build oracle/_ref/libaxr_ref.so, or return None where it cannot be built."""
    if not ref_available():
        return None
    root = reference_root()
    harness = HERE / "ref_harness.cpp"
    shim = HERE / "shim"
    inputs = [root / t for t in REF_TUS] + [harness, HERE / "axo.h", Path(__file__)]
    inputs += [p for p in shim.rglob("*") if p.is_file()]
    inputs += [p for p in (root / "include").rglob("*.hpp")]
    if not force and not _stale(REF_OUT, inputs):
        return REF_OUT
    REF_OUT_DIR.mkdir(parents=True, exist_ok=True)
    alias_dir = REF_OUT_DIR / "aliases"
    if alias_dir.exists():
        shutil.rmtree(alias_dir)
    alias_dir.mkdir()
    for name, body in ALIASES.items():
        (alias_dir / name).write_text("// generated forwarding header (oracle build)\n#pragma once\n" + body)
    objdir = REF_OUT_DIR / "obj"
    objdir.mkdir(exist_ok=True)
    # The reference's own flags are MSVC "/O2 /arch:AVX2" (CMakeLists.txt:17-19). GCC
    # needs -mavx2 for the live rasteriser and -mavx512f for the unused AVX-512 variant
    # in the same file; -ffp-contract=off keeps every multiply and add separately rounded.
    cxxflags = ["-std=c++23", "-O2", "-fPIC", "-mavx2", "-mavx512f", "-ffp-contract=off", "-pthread", "-w",
                "-include", str(shim / "std_prelude.hpp"), f"-I{alias_dir}", f"-I{shim}", f"-I{root / 'include'}", f"-I{root / 'src'}",
                f"-I{root / 'external' / 'stb_image'}", f"-I{HERE}"]

    def cxx(src: Path) -> Path:
        obj = objdir / (src.parent.name + "_" + src.stem + ".o")
        _run(["g++", *cxxflags, "-c", str(src), "-o", str(obj)])
        return obj

    srcs = [root / t for t in REF_TUS] + [harness]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(cxx, srcs))
    tmp = REF_OUT.with_suffix(".so.tmp")
    _run(["g++", "-shared", "-pthread", *map(str, objs), "-o", str(tmp)])
    tmp.replace(REF_OUT)
    return REF_OUT


if __name__ == "__main__":
    print("port:", build_port(force=True))
    print("ref :", build_ref(force=True))
