"""Device-side mesh ingest (axr_mesh_create_from_obj): vertex de-duplication, fan
triangulation and tangent frames on the GPU give the reference's Mesh(path) bit for bit
(fixtures made from the reference by tests/golden/make_golden.py), and the ingested mesh
draws the same frame as the same arrays uploaded with axr_mesh_create."""
import ctypes as C

import numpy as np
import pytest

import objfile
from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import ObjDesc, check
from helpers import GOLDEN, same_bits

pytestmark = pytest.mark.gpu


def ingest(ctx, parsed, materials=()):
    pos = np.ascontiguousarray(parsed["positions"], np.float32)
    uv = np.ascontiguousarray(parsed["uvs"], np.float32)
    nrm = np.ascontiguousarray(parsed["normals"], np.float32)
    cor = np.ascontiguousarray(parsed["corners"], np.int32)
    sizes = np.ascontiguousarray(parsed["polygon_sizes"], np.uint32)
    nf = int(parsed["num_faces"])
    groups = np.ascontiguousarray([[0, nf, 0]] if nf else np.zeros((0, 3)), np.uint32)
    mats = (api.MaterialDesc * 1)(*[m.desc() for m in materials] or [api.MaterialDesc()])
    d = ObjDesc(pos.shape[0], pos.ctypes.data, uv.shape[0], uv.ctypes.data, nrm.shape[0], nrm.ctypes.data,
                cor.shape[0], cor.ctypes.data, sizes.shape[0], sizes.ctypes.data, groups.shape[0],
                groups.ctypes.data, 1, C.cast(mats, C.c_void_p))
    h = C.c_void_p()
    check(ctx.lib.axr_mesh_create_from_obj(ctx.handle, C.byref(d), C.byref(h)), ctx.handle)
    return h


def read(ctx, h):
    nv, nf, nd = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(ctx.lib.axr_mesh_counts(h, C.byref(nv), C.byref(nf), C.byref(nd)))
    verts = np.zeros((max(1, nv.value), 14), np.float32)
    faces = np.zeros((max(1, nf.value), 3), np.uint32)
    check(ctx.lib.axr_mesh_read(ctx.handle, h, verts.ctypes.data, faces.ctypes.data), ctx.handle)
    return verts[: nv.value], faces[: nf.value]


@pytest.mark.parametrize("name", sorted(p.stem[len("obj_"):] for p in GOLDEN.glob("obj_*.npz")))
def test_ingest_matches_reference(ctx, name):
    z = np.load(GOLDEN / f"obj_{name}.npz")
    parsed = objfile.parse_obj(str(z["text"]))
    h = ingest(ctx, parsed)
    verts, faces = read(ctx, h)
    ctx.lib.axr_mesh_destroy(ctx.handle, h)
    assert verts.shape == z["vertices"].shape and faces.shape == z["faces"].shape
    ref = z["vertices"]
    bad = np.argwhere((verts.view(np.uint32) != ref.view(np.uint32)) & ~(np.isnan(verts) & np.isnan(ref)))
    assert bad.size == 0, f"{len(bad)} vertex floats differ, first {bad[:5].tolist()}"
    assert np.array_equal(faces, z["faces"])


def test_ingest_matches_port_on_larger_models(ctx, port):
    for text in (objfile.sphere_obj(256, 128), objfile.tricky_obj(99)):
        parsed = objfile.parse_obj(text)
        h = ingest(ctx, parsed)
        verts, faces = read(ctx, h)
        ctx.lib.axr_mesh_destroy(ctx.handle, h)
        pv, pf = port.obj_ingest(parsed)
        assert same_bits(verts, pv) and np.array_equal(faces, pf)


def test_ingested_mesh_draws_like_uploaded_arrays(ctx):
    z = np.load(GOLDEN / "obj_sphere.npz")
    parsed = objfile.parse_obj(str(z["text"]))
    tex = api.Texture(ctx, W.noise_texture(64, seed=5))
    mat = api.Material(tex, tex, tex, tex, tex, 1.0)
    h = ingest(ctx, parsed, [mat])
    v = z["vertices"]
    up = api.Mesh(ctx, v[:, 0:3], v[:, 3:5], v[:, 5:8], z["faces"], None, [mat], v[:, 8:11], v[:, 11:14])
    for shader in (api.PhongShader(), api.PBRShader(), api.BlinnPhongShader()):
        frames = []
        for mesh_handle in (h, up.handle):
            fb = api.Framebuffer(ctx, 160, 120)
            fb.clearColor(0, 0, 0, 255)
            fb.clearDepth()
            pipe = api.TiledPipeline(ctx, api.Camera((0.3, 0.4, 2.6), (0.0, 0.0, 0.0), 60.0, 160 / 120), fb)
            pipe.setShader(shader)
            check(ctx.lib.axr_draw_mesh(ctx.handle, mesh_handle, np.eye(4, dtype=np.float32).ctypes.data), ctx.handle)
            frames.append(fb.read())
        assert np.array_equal(frames[0][0], frames[1][0])
        assert np.array_equal(frames[0][1].view(np.uint32), frames[1][1].view(np.uint32))
        assert np.isfinite(frames[0][1]).sum() > 1000
    ctx.lib.axr_mesh_destroy(ctx.handle, h)


def test_ingest_rejects_bad_input(ctx):
    parsed = objfile.parse_obj(objfile.tricky_obj(1))
    bad = dict(parsed)
    bad["polygon_sizes"] = parsed["polygon_sizes"] + 1  # sizes no longer add up
    with pytest.raises(api.AxrError):
        ingest(ctx, bad)
    bad = dict(parsed)
    c = parsed["corners"].copy()
    c[0, 0] = 10_000  # position index past the pool
    bad["corners"] = c
    with pytest.raises(api.AxrError):
        ingest(ctx, bad)
