"""Generate the golden fixtures in this directory from the AxiomR reference itself.

The reference ships no tests or golden data, so the fixtures are outputs of its own
TiledPipeline::drawMesh and stage functions, compiled here by oracle/build.py (x86 with
the reference tree present) and driven through oracle/ref_harness.cpp. Each fixture
stores its inputs (mesh arrays, textures, matrices) next to the reference's outputs, so
tests on another machine feed exactly the same bytes to the code under test.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
    python tests/golden/make_golden.py obj    # rewrites only the mesh-ingest fixtures
    python tests/golden/make_golden.py camera # rewrites only the camera-script fixture
"""
from __future__ import annotations

import dataclasses
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from axiomr_gb300 import workloads as W  # noqa: E402
from oracle import Oracle  # noqa: E402


def scene_list():
    s = []
    for k in range(5):
        s.append(W.sphere_scene(width=112, height=96, lon=24, lat=12, tex_size=32, shader=k, name=f"sphere_{W.SHADER_NAMES[k]}"))
    # clipping against the side planes and the near plane
    s.append(W.sphere_scene(width=100, height=75, lon=32, lat=16, tex_size=16, distance=1.3, name="sphere_close"))
    s.append(W.soup_scene(count=2500, width=160, height=120, seed=11, edge_min=0.5, edge_max=12.0,
                          depth_min=0.1, depth_max=0.35, name="soup_near"))
    s.append(W.soup_scene(count=3000, width=144, height=80, seed=12, edge_min=1.0, edge_max=30.0,
                          depth_min=0.1, depth_max=100.0, name="soup_mixed"))
    s.append(W.heightfield_scene(n=40, width=160, height=90, tex_size=32, shader=W.SHADER_PHONG, name="height_phong"))
    s.append(W.heightfield_scene(n=40, width=96, height=54, tex_size=32, shader=W.SHADER_PBR, name="height_pbr"))
    # two material groups listed out of face order
    sc = W.sphere_scene(width=96, height=96, lon=16, lat=8, tex_size=16, name="sphere_groups")
    nf = sc.mesh.num_faces
    m2 = W.Material(diffuse=W.noise_texture(16, seed=99), specular_exponent=0.5)
    mesh = dataclasses.replace(sc.mesh, groups=np.asarray([[nf // 2, nf - nf // 2, 1], [0, nf // 2, 0]], np.uint32),
                               materials=[sc.mesh.materials[0], m2])
    s.append(dataclasses.replace(sc, mesh=mesh))
    return s


def prefilled(scene, seed):
    """A framebuffer that was not cleared: random colour and depth in [-1, 1] (the merge
    keeps existing pixels unless the new depth is strictly smaller)."""
    u = W.uniform(seed, scene.width * scene.height * 2).reshape(2, scene.height, scene.width)
    depth = (u[0] * 2.0 - 1.0).astype(np.float32)
    depth[u[1] < 0.2] = np.inf
    bgra = W.noise_texture(scene.width, scene.height, seed=seed)
    return bgra, depth


def save_scene(path, sc, view_proj, bgra_in, depth_in, bgra, depth):
    m = sc.mesh
    mats = {}
    for k, mat in enumerate(m.materials):
        for f in ("diffuse", "bump", "metallic", "roughness", "ao"):
            img = getattr(mat, f)
            if img is not None:
                mats[f"mat{k}_{f}"] = img
        mats[f"mat{k}_ns"] = np.float32(mat.specular_exponent)
    np.savez_compressed(
        path, name=sc.name, positions=m.positions, uvs=m.uvs, normals=m.normals, tangents=m.tangents,
        bitangents=m.bitangents, indices=m.indices, groups=m.groups, num_materials=len(m.materials),
        model=np.asarray(sc.model, np.float32), view_proj=np.asarray(view_proj, np.float32),
        cam_pos=np.asarray(sc.camera.position, np.float32), shader_kind=sc.shader.kind,
        light_direction=np.asarray(sc.shader.light_direction, np.float32),
        light_color=np.asarray(sc.shader.light_color, np.float32), width=sc.width, height=sc.height,
        bgra_in=bgra_in, depth_in=depth_in, bgra=bgra, depth=depth, **mats)


def obj_cases():
    """OBJ texts for the mesh-ingest fixtures (tests/objfile.py)."""
    sys.path.insert(0, str(HERE.parent))
    import objfile

    cases = [("sphere", objfile.sphere_obj(24, 12)), ("sphere_fine", objfile.sphere_obj(96, 48))]
    cases += [(f"tricky{k}", objfile.tricky_obj(k)) for k in range(3)]
    return cases


def make_obj_goldens(ref):
    """The reference's Mesh(path) on each OBJ text: vertices (position, uv, normal,
    tangent, bitangent), faces and material groups, stored with the text."""
    import tempfile

    for old in HERE.glob("obj_*.npz"):
        old.unlink()
    with tempfile.TemporaryDirectory() as d:
        for name, text in obj_cases():
            path = Path(d) / f"{name}.obj"
            path.write_text(text)
            verts, faces, groups = ref.obj_load(str(path))
            np.savez_compressed(HERE / f"obj_{name}.npz", text=np.asarray(text), vertices=verts, faces=faces,
                                groups=groups)
            print(f"obj_{name:12s} vertices={verts.shape[0]} faces={faces.shape[0]} groups={groups.tolist()}")


def make_camera_goldens(ref):
    """The reference Camera driven by seeded scripts (tests/camscript.py): matrices and
    position after every operation."""
    sys.path.insert(0, str(HERE.parent))
    import camscript

    arrays = {}
    for k, (pos, tgt, fov, aspect) in enumerate(camscript.STARTS):
        ops = camscript.script(7000 + k, n=120)
        arrays[f"ops_{k}"] = ops
        arrays[f"out_{k}"] = ref.camera_script(W.Camera(pos, tgt, fov, aspect, (0, 0, 800, 600)), ops)
    np.savez_compressed(HERE / "camera_scripts.npz", **arrays)
    print("camera scripts:", len(camscript.STARTS))


def main():
    ref = Oracle("ref")
    if sys.argv[1:] == ["obj"]:
        make_obj_goldens(ref)
        return
    if sys.argv[1:] == ["camera"]:
        make_camera_goldens(ref)
        return
    for old in HERE.glob("*.npz"):
        old.unlink()
    make_obj_goldens(ref)
    make_camera_goldens(ref)
    for i, sc in enumerate(scene_list()):
        vp = ref.camera(sc.camera)[2]
        if sc.name == "sphere_close":
            bgra_in, depth_in = prefilled(sc, 1234)
        else:
            bgra_in, depth_in = W.clear_framebuffer(sc)
        bgra, depth = ref.draw(sc, vp, bgra=bgra_in, depth=depth_in)
        save_scene(HERE / f"scene_{sc.name}.npz", sc, vp, bgra_in, depth_in, bgra, depth)
        print(f"{sc.name:16s} covered={int(np.isfinite(depth).sum())}")

    # stage fixtures
    rng = np.random.default_rng(2024)
    clip_in = rng.normal(size=(400, 3, 18)).astype(np.float32)
    clip_in[:, :, 17] = (np.abs(clip_in[:, :, 17]) + rng.choice([0.0, -0.4], size=(400, 1))).astype(np.float32)
    clip_out = np.zeros((400, 24, 18), np.float32)
    clip_n = np.zeros(400, np.int32)
    setup_out = np.zeros((400, 13), np.float32)
    setup_bf = np.zeros(400, np.int32)
    for k in range(400):
        o = ref.clip_triangle(clip_in[k])
        clip_n[k] = o.shape[0]
        clip_out[k, : o.shape[0]] = o
        setup_out[k], setup_bf[k] = ref.triangle(clip_in[k], 320, 200)
    tex = W.noise_texture(23, 17, seed=77)
    uv = rng.uniform(-0.25, 1.25, size=(2000, 2)).astype(np.float32)
    uv[:200] = rng.integers(0, 5, size=(200, 2)) / 4.0  # texel-boundary coordinates
    samples = ref.sample(tex, uv)
    cams = [W.orbit_camera(float(rng.uniform(0.5, 10)), float(rng.uniform(-89, 89)), float(rng.uniform(0, 360)),
                           640, 480, fov=float(rng.uniform(20, 120))) for _ in range(64)]
    cams += [W.Camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), 60.0, 1.0, (0, 0, 1, 1)),
             W.Camera((0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 60.0, 1.0, (0, 0, 1, 1)),
             W.Camera((0.0, 5.0, 0.0), (0.0, 0.0, 0.0), 60.0, 1.0, (0, 0, 1, 1))]
    cam_params = np.asarray([[*c.position, *c.target, c.fov_degrees, c.aspect] for c in cams], np.float32)
    cam_out = np.stack([ref.camera(c) for c in cams])
    np.savez_compressed(HERE / "stages.npz", clip_in=clip_in, clip_out=clip_out, clip_n=clip_n, setup_out=setup_out,
                        setup_backface=setup_bf, tex=tex, uv=uv, samples=samples, cam_params=cam_params,
                        cam_out=cam_out)
    print("stages: clip counts", np.bincount(clip_n // 3))


if __name__ == "__main__":
    main()
