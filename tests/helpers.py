"""Test helpers: golden-fixture loading and frame comparison with the parity bar
(depth bit-exact, hence coverage and depth-test winners; 8-bit colour within 1 LSB)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from axiomr_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"
COLOR_TOLERANCE_LSB = 1


def same_bits(a, b) -> bool:
    """Float arrays equal bit for bit, except that any NaN matches any NaN: the bit pattern
    of a NaN that an operation creates is the machine's default NaN (x86, Arm and the GPU
    differ), and the reference makes NaNs on degenerate input (a tangent frame of a
    zero-area triangle)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


def golden_names():
    return sorted(p.stem[len("scene_"):] for p in GOLDEN.glob("scene_*.npz"))


def load_golden(name):
    """(scene, view_proj, bgra_in, depth_in, bgra_expected, depth_expected)."""
    z = np.load(GOLDEN / f"scene_{name}.npz")
    mats = []
    for k in range(int(z["num_materials"])):
        get = lambda f: z[f"mat{k}_{f}"] if f"mat{k}_{f}" in z.files else None  # noqa: E731
        mats.append(W.Material(get("diffuse"), get("bump"), get("metallic"), get("roughness"), get("ao"),
                               float(z[f"mat{k}_ns"])))
    mesh = W.Mesh(z["positions"], z["uvs"], z["normals"], z["tangents"], z["bitangents"], z["indices"],
                  z["groups"], mats)
    w, h = int(z["width"]), int(z["height"])
    cam = W.Camera(tuple(float(v) for v in z["cam_pos"]), (0.0, 0.0, 0.0), 60.0, w / h, (0, 0, w, h))
    shader = W.Shader(int(z["shader_kind"]), tuple(float(v) for v in z["light_direction"]),
                      tuple(float(v) for v in z["light_color"]))
    scene = W.Scene(str(z["name"]), mesh, cam, shader, w, h, model=z["model"])
    return scene, z["view_proj"], z["bgra_in"], z["depth_in"], z["bgra"], z["depth"]


def frame_diff(got, exp):
    """Compare (bgra, depth) pairs; returns a dict of counts."""
    gb, gd = got
    eb, ed = exp
    gdu, edu = np.ascontiguousarray(gd).view(np.uint32), np.ascontiguousarray(ed).view(np.uint32)
    depth_mismatch = int((gdu != edu).sum())
    cdiff = np.abs(gb.astype(np.int16) - eb.astype(np.int16))
    return {
        "pixels": int(gd.size),
        "depth_mismatch": depth_mismatch,
        "coverage_mismatch": int((np.isfinite(gd) != np.isfinite(ed)).sum()),
        "color_max_lsb": int(cdiff.max()) if cdiff.size else 0,
        "color_differing_pixels": int((cdiff.max(axis=-1) > 0).sum()),
    }


def assert_parity(got, exp, what=""):
    d = frame_diff(got, exp)
    print(f"{what}: {d}")
    assert d["depth_mismatch"] == 0, f"{what}: depth differs at {d['depth_mismatch']} pixels ({d})"
    assert d["color_max_lsb"] <= COLOR_TOLERANCE_LSB, f"{what}: colour differs by more than 1 LSB ({d})"
    return d
