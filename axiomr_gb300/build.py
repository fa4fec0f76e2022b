"""Build recipe for the in-tree CUDA library ``axiomr_gb300/_bin/libaxr.so``.

nvcc compiles the kernels for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``)
with ``--fmad=false`` (no multiply-add contraction anywhere in device code) and
``-lineinfo``; the host API is compiled with ``-ffp-contract=off`` for the same reason.
The CUDA runtime is linked statically and its symbols are kept private to the library.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_bin"
LIB = OUT_DIR / "libaxr.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    return Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{proc.stdout}\n{proc.stderr}")
    return proc.stdout + proc.stderr


def _sources():
    return sorted(CSRC.glob("*.cu")), sorted(CSRC.glob("*.cpp"))


def _deps():
    return sorted(CSRC.glob("*")) + [ROOT / "include" / "axr.h", Path(__file__)]


def _digest() -> str:
    """Content hash of every input of the library (sources, headers, this recipe, the extra
    compiler flags and the host architecture): the library is rebuilt when it changes."""
    h = hashlib.sha256()
    for p in _deps():
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(os.environ.get("AXR_NVCC_FLAGS", "").encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _stale(out: Path) -> bool:
    stamp = out.with_suffix(".sha256")
    return not out.exists() or not stamp.exists() or stamp.read_text().strip() != _digest()


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale(LIB):
        return LIB
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    objdir = OUT_DIR / "obj"
    objdir.mkdir(exist_ok=True)
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    cu, cpp = _sources()
    logs = []
    # tuning builds: e.g. AXR_NVCC_FLAGS="-DAXR_GEOMETRY_MIN_BLOCKS=6"
    extra = os.environ.get("AXR_NVCC_FLAGS", "").split()

    def compile_cu(src: Path) -> Path:
        obj = objdir / (src.stem + ".cu.o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v", *inc, *extra, "-c", str(src), "-o", str(obj)]
        logs.append(_run(cmd))
        return obj

    def compile_cpp(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
               "-Wno-unused-parameter", f"-I{home / 'include'}", *inc, "-c", str(src), "-o", str(obj)]
        logs.append(_run(cmd))
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(cu) + len(cpp))) as ex:
        futs = [ex.submit(compile_cu, s) for s in cu] + [ex.submit(compile_cpp, s) for s in cpp]
        objs = [f.result() for f in futs]
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static",
          "-Xlinker", "--exclude-libs,ALL", "-Xlinker", f"--version-script={CSRC / 'exports.map'}",
          "-lpthread", "-ldl", "-lrt"])
    tmp.replace(LIB)
    LIB.with_suffix(".sha256").write_text(_digest() + "\n")
    (OUT_DIR / "ptxas.log").write_text("\n".join(logs))
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
