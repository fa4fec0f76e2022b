"""The no-allocation draw (axr_draw_mesh_noalloc) against the regular draw.

Some callers cannot let a library allocate device memory: a renderer that records its
frame into a CUDA graph (an allocation during stream capture breaks the capture), a
real-time loop that forbids allocator calls after start-up, or a host application that
owns the device-memory budget. axr_draw_mesh_noalloc serves them by keeping its scratch in
a fixed array inside the library. These tests call it through the C ABI and require the
same frame as axr_draw_mesh (depth bit-exact, colour within the 1 LSB tolerance of the
other parity tests) on two calls in a row, the second running on whatever the first left
in the shared array, and that a draw above its limits is refused."""
import ctypes as C

import numpy as np
import pytest

from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from helpers import COLOR_TOLERANCE_LSB, frame_diff

pytestmark = pytest.mark.gpu

AXR_E_CAPACITY = 7


def draw(ctx, scene, entry):
    fb = api.Framebuffer(ctx, scene.width, scene.height)
    mesh = api.Mesh.from_workload(ctx, scene.mesh)
    b, g, r, a = scene.clear_bgra
    fb.clearColor(r, g, b, a)
    fb.clearDepth()
    pipe = api.TiledPipeline(ctx, api.Camera.from_workload(scene.camera), fb)
    sh = scene.shader
    pipe.setShader(api.Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)))
    model = np.ascontiguousarray(scene.model, np.float32)
    status = getattr(ctx.lib, entry)(ctx.handle, mesh.handle, model.ctypes.data)
    assert status == 0, ctx.lib.axr_last_error(ctx.handle)
    return fb.read()


def test_noalloc_draw_matches_regular_draw_twice():
    ctx = api.Context(0)
    scenes = [
        # near-plane triangles: exercises the clipped-winner list in the shared array
        W.soup_scene(count=4000, width=400, height=300, seed=10, edge_min=1, edge_max=50, depth_min=0.1,
                     depth_max=0.3),
        W.sphere_scene(),  # the 512x512 sphere configuration
    ]
    for sc in scenes:
        expected = draw(ctx, sc, "axr_draw_mesh")
        got = draw(ctx, sc, "axr_draw_mesh_noalloc")
        d = frame_diff(got, expected)
        print(sc.name, d)
        assert d["depth_mismatch"] == 0
        assert d["color_max_lsb"] <= COLOR_TOLERANCE_LSB
        assert np.isfinite(got[1]).sum() > 0
    ctx.close()


def test_noalloc_draw_rejects_oversized_target():
    ctx = api.Context(0)
    sc = W.sphere_scene(width=2048, height=1024, lon=8, lat=4, tex_size=8)
    fb = api.Framebuffer(ctx, sc.width, sc.height)
    mesh = api.Mesh.from_workload(ctx, sc.mesh)
    pipe = api.TiledPipeline(ctx, api.Camera.from_workload(sc.camera), fb)
    pipe.setShader(api.BlinnPhongShader())
    model = np.eye(4, dtype=np.float32)
    status = ctx.lib.axr_draw_mesh_noalloc(ctx.handle, mesh.handle, model.ctypes.data)
    assert status == AXR_E_CAPACITY
    assert b"limited to" in ctx.lib.axr_last_error(ctx.handle)
    ctx.close()


def test_noalloc_draw_reports_statistics_and_allocates_nothing():
    """The no-allocation draw's statistics reach axr_stats_read (the same triangle and
    fragment counts as the keyed per-draw path, which runs the same kernels; the kernel
    that adds them to the context's counters carries the error bits the same way), and
    after one warm-up call further calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    ctx = api.Context(0)
    sc = W.sphere_scene(width=320, height=240, lon=96, lat=48, tex_size=64)
    ctx.draw_form = api.DRAW_KEYED
    ctx.stats(True)
    ctx.stats()
    draw(ctx, sc, "axr_draw_mesh")
    regular = ctx.stats()
    draw(ctx, sc, "axr_draw_mesh_noalloc")
    noalloc = ctx.stats()
    assert noalloc["triangles"] == regular["triangles"] > 0
    assert noalloc["fragments"] == regular["fragments"] > 0
    ctx.stats(False)
    # free device memory across the calls (the framebuffer and mesh are made first)
    fb = api.Framebuffer(ctx, sc.width, sc.height)
    mesh = api.Mesh.from_workload(ctx, sc.mesh)
    pipe = api.TiledPipeline(ctx, api.Camera.from_workload(sc.camera), fb)
    pipe.setShader(api.BlinnPhongShader())
    model = np.ascontiguousarray(sc.model, np.float32)
    assert ctx.lib.axr_draw_mesh_noalloc(ctx.handle, mesh.handle, model.ctypes.data) == 0
    ctx.sync()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        assert ctx.lib.axr_draw_mesh_noalloc(ctx.handle, mesh.handle, model.ctypes.data) == 0
    ctx.sync()
    assert torch.cuda.mem_get_info(0)[0] == free0
    ctx.close()
