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


def _const_tex(rgba, size=8):
    return np.broadcast_to(np.array(rgba, np.uint8), (size, size, 4)).copy()


# Lighting at its sharpest: specular exponent 50 * Ns of 0, 1, 1000 and 50,000 (a highlight a
# few pixels wide), and PBR on a flat normal map with roughness 0, 1/255 (the distribution
# term a spike that depends on n.h to the last bits) and 40/255, metallic 0 and 1.
SHADING_EXTREMES = {
    **{f"blinn_ns{ns:g}": (W.SHADER_BLINN_PHONG, dict(specular_exponent=ns)) for ns in (0.0, 0.02, 20.0, 1000.0)},
    **{f"phong_ns{ns:g}": (W.SHADER_PHONG, dict(specular_exponent=ns, bump=(128, 128, 255, 255)))
       for ns in (0.0, 20.0, 1000.0)},
    **{f"pbr_r{r}_m{m}": (W.SHADER_PBR, dict(bump=(128, 128, 255, 255), roughness=(r, r, r, 255),
                                             metallic=(m, m, m, 255), ao=(255, 255, 255, 255)))
       for r in (0, 1, 40) for m in (0, 255)},
}


def shading_extreme_scene(name):
    """A dense smooth sphere (192x96 segments, 320x240) lit for a highlight in view, with the
    material of SHADING_EXTREMES[name]."""
    kind, opts = SHADING_EXTREMES[name]
    sc = W.sphere_scene(width=320, height=240, lon=192, lat=96, shader=kind, name=name)
    ld = np.array([-0.3, -0.4, -1.0], np.float32)
    sc.shader = W.Shader(kind, light_direction=tuple(map(float, ld / np.linalg.norm(ld))),
                         light_color=sc.shader.light_color)
    mat = sc.mesh.materials[0]
    for k, v in opts.items():
        setattr(mat, k, _const_tex(v) if isinstance(v, tuple) else v)
    return sc
