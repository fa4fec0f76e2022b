"""GPU behaviour of the C ABI beyond single-frame parity: sequential draws into one
framebuffer, draws into an uncleared framebuffer, unset pipeline state, material groups,
mesh and texture updates, CUDA-graph replay, statistics and argument errors."""
import ctypes as C

import numpy as np
import pytest

from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import AxrError
from helpers import assert_parity, frame_diff

pytestmark = pytest.mark.gpu


def test_two_draws_into_one_framebuffer(ctx, port):
    """Renderer::render draws meshes one after another into one cleared framebuffer."""
    a = W.sphere_scene(width=200, height=150, lon=24, lat=12)
    b = W.soup_scene(count=3000, width=200, height=150, seed=3, edge_min=2, edge_max=30, depth_min=0.5,
                     depth_max=2.0)
    vp_a = port.camera(a.camera)[2]
    vp_b = port.camera(b.camera)[2]
    eb, ed = port.draw(a, vp_a)
    eb, ed = port.draw(b, vp_b, bgra=eb, depth=ed)
    fb = api.Framebuffer(ctx, 200, 150)
    gb, gd = api.render_scene(ctx, a, framebuffer=fb, view_proj=vp_a)
    gb, gd = api.render_scene(ctx, b, framebuffer=fb, bgra=gb, depth=gd, view_proj=vp_b)
    assert_parity((gb, gd), (eb, ed), "two draws")


def test_redraw_same_mesh_keeps_framebuffer(ctx, port):
    """Drawing the same mesh twice: the second draw changes nothing (strict less-than)."""
    sc = W.sphere_scene(width=160, height=160, lon=32, lat=16)
    vp = port.camera(sc.camera)[2]
    fb = api.Framebuffer(ctx, sc.width, sc.height)
    mesh = api.Mesh.from_workload(ctx, sc.mesh)
    first = api.render_scene(ctx, sc, framebuffer=fb, mesh=mesh, view_proj=vp)
    pipe = api.TiledPipeline(ctx, api.Camera.from_matrices(vp, sc.camera.position), fb)
    pipe.setShader(api.BlinnPhongShader())
    pipe.drawMesh(None, mesh)
    second = fb.read()
    assert np.array_equal(first[0], second[0]) and np.array_equal(first[1], second[1])


def test_unset_state_is_a_noop(ctx):
    fb = api.Framebuffer(ctx, 32, 32)
    sc = W.sphere_scene(width=32, height=32, lon=8, lat=4, tex_size=8)
    mesh = api.Mesh.from_workload(ctx, sc.mesh)
    fb.clearColor(1, 2, 3, 4)
    before = fb.read()
    pipe = api.TiledPipeline(ctx)
    pipe.setShader(None)
    pipe.setCamera(api.Camera.from_workload(sc.camera))
    pipe.setFramebuffer(fb)
    pipe.drawMesh(None, mesh)  # no shader: nothing happens (src/tiled_pipeline.cpp:146)
    after = fb.read()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert (before[0][..., 0] == 3).all() and (before[0][..., 2] == 1).all() and (before[0][..., 3] == 4).all()
    assert np.isinf(before[1]).all()


def test_material_groups(ctx, port):
    sc = W.sphere_scene(width=128, height=128, lon=16, lat=8, tex_size=16)
    nf = sc.mesh.num_faces
    import dataclasses

    mesh = dataclasses.replace(sc.mesh, groups=np.asarray([[nf // 3, nf - nf // 3, 1], [0, nf // 3, 0]], np.uint32),
                               materials=[sc.mesh.materials[0], W.Material(W.noise_texture(16, seed=5), None, None,
                                                                           None, None, 0.3)])
    sc = dataclasses.replace(sc, mesh=mesh)
    vp = port.camera(sc.camera)[2]
    assert_parity(api.render_scene(ctx, sc, view_proj=vp), port.draw(sc, vp), "groups")


def test_mesh_and_texture_update(ctx, port):
    a = W.sphere_scene(width=96, height=96, lon=16, lat=8, tex_size=16)
    b = W.sphere_scene(width=96, height=96, lon=16, lat=8, tex_size=16, tex_seed=9, distance=2.5)
    vp = port.camera(b.camera)[2]
    textures = {}
    mesh = api.Mesh.from_workload(ctx, a.mesh, textures)
    tex = next(iter(textures.values()))
    m = b.mesh
    mesh.update(m.positions * np.float32(1.0), m.uvs, m.normals, m.indices, m.tangents, m.bitangents)
    tex.update(b.mesh.materials[0].diffuse)
    got = api.render_scene(ctx, b, mesh=mesh, view_proj=vp)
    assert_parity(got, port.draw(b, vp), "updated mesh")


def test_graph_replay_equals_direct(ctx, port):
    sc = W.soup_scene(count=5000, width=256, height=192, seed=14, edge_min=0.5, edge_max=40)
    vp = port.camera(sc.camera)[2]
    fb = api.Framebuffer(ctx, sc.width, sc.height)
    mesh = api.Mesh.from_workload(ctx, sc.mesh)
    pipe = api.TiledPipeline(ctx, api.Camera.from_matrices(vp, sc.camera.position), fb)
    pipe.setShader(api.GouraudShader())
    ctx.reserve(sc.mesh.num_faces)
    lib = ctx.lib
    assert lib.axr_graph_begin(ctx.handle) == 0
    fb.clearColor(0, 0, 0, 255)
    fb.clearDepth()
    pipe.drawMesh(None, mesh)
    g = C.c_void_p()
    assert lib.axr_graph_end(ctx.handle, C.byref(g)) == 0
    for _ in range(3):
        assert lib.axr_graph_launch(ctx.handle, g) == 0
    got = fb.read()
    lib.axr_graph_destroy(g)
    assert_parity(got, port.draw(sc, vp), "graph replay")


def test_stats_count_fragments(ctx, port):
    sc = W.soup_scene(count=2000, width=200, height=200, seed=15, edge_min=1, edge_max=10, depth_min=1,
                      depth_max=2)
    ctx.stats(True)
    ctx.stats()  # reset
    api.render_scene(ctx, sc)
    s = ctx.stats()
    ctx.stats(False)
    # all 2000 faces are front-facing; the ones crossing a screen edge are split by the
    # clipper into several triangles
    assert s["triangles"] >= 2000
    assert s["fragments"] > 0 and s["tiles"] > 0


def test_invalid_arguments(ctx):
    lib = ctx.lib
    h = C.c_void_p()
    assert lib.axr_framebuffer_create(ctx.handle, 0, 10, C.byref(h)) == 1
    assert lib.axr_texture_create(ctx.handle, None, 4, 4, C.byref(h)) == 1
    with pytest.raises(AxrError):
        api.Mesh(ctx, np.zeros((3, 3)), np.zeros((3, 2)), np.zeros((3, 3)), np.array([[0, 1, 5]]))
    with pytest.raises(AxrError):
        api.Mesh(ctx, np.zeros((3, 3)), np.zeros((3, 2)), np.zeros((3, 3)), np.array([[0, 1, 2]]),
                 groups=[[0, 2, 0]])
    pipe = api.TiledPipeline(ctx)
    with pytest.raises(AxrError):
        pipe.setShader(api.Shader(42))
    assert b"" != lib.axr_last_error(ctx.handle)


def test_empty_and_offscreen_meshes(ctx, port):
    sc = W.sphere_scene(width=64, height=64, lon=8, lat=4, tex_size=8)
    fb = api.Framebuffer(ctx, 64, 64)
    import dataclasses

    empty = dataclasses.replace(sc.mesh, groups=np.zeros((0, 3), np.uint32))
    got = api.render_scene(ctx, dataclasses.replace(sc, mesh=empty), framebuffer=fb)
    assert np.isinf(got[1]).all()
    behind = dataclasses.replace(sc, camera=W.Camera((0.0, 0.0, 3.0), (0.0, 0.0, 6.0), 60.0, 1.0, (0, 0, 64, 64)))
    got = api.render_scene(ctx, behind, framebuffer=fb)
    assert np.isinf(got[1]).all()


def test_clipped_winner_pass_skipped_only_when_nothing_can_clip(ctx, port):
    """A mesh whose bounding sphere lies inside all six clip planes cannot have clipped
    triangles: its draw runs without the clipped-winner pass (one launch fewer). The same
    mesh crossing the near plane runs it, and both frames match the oracle."""
    sc = W.sphere_scene(width=160, height=120, lon=24, lat=12)
    near = W.sphere_scene(width=160, height=120, lon=24, lat=12)
    near.camera = W.orbit_camera(1.05, 0.0, 0.0, 160, 120)  # the unit sphere reaches the near plane
    launches = []
    for s in (sc, near):
        ctx.sync()
        k0 = ctx.profile()["kernel_launches"]
        got = api.render_scene(ctx, s)
        launches.append(ctx.profile()["kernel_launches"] - k0)
        assert_parity(got, port.draw(s, port.camera(s.camera)[2]), "sphere")
    assert launches[0] == launches[1] - 1, launches
