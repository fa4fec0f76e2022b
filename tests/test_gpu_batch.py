"""Batched form (axr_batch_* / axr_draw_batch): every draw of a batch must give the frame
that the per-draw path gives for it (the same device functions compute every value, so
the comparison is exact), and the oracle's frame within the parity bar. Covers the
fused clears (both, one, none), framebuffers whose width is not a multiple of 4 (no TMA
tile stores), all shader kinds in one batch (one launch per kind), clipped triangles,
CUDA-graph replay, the one-shot entry point, the autotuner and argument errors."""
import numpy as np
import pytest

from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import AxrError
from helpers import assert_parity

pytestmark = pytest.mark.gpu


def small_batch(count=24, seed=5, scale=0.25, tex=64):
    return W.batch_scenes(count=count, seed=seed, tex_size=tex, resolution_scale=scale)


def plain_frames(ctx, scenes, draws):
    """Each draw through the per-draw path into a fresh framebuffer (clear, clear, drawMesh)."""
    out = []
    for sc, d in zip(scenes, draws):
        fb = api.Framebuffer(ctx, sc.width, sc.height)
        if d.clear_color is not None:
            fb.clearColor(*d.clear_color)
        if d.clear_depth is not None:
            fb.clearDepth(d.clear_depth)
        pipe = api.TiledPipeline(ctx, d.camera, fb)
        pipe.setShader(d.shader)
        pipe.drawMesh(d.model, d.mesh)
        out.append(fb.read())
        fb.close()
    return out


def assert_same(got, exp, what):
    gb, gd = got
    eb, ed = exp
    dd = int((np.ascontiguousarray(gd).view(np.uint32) != np.ascontiguousarray(ed).view(np.uint32)).sum())
    cd = int((gb != eb).any(axis=-1).sum())
    assert dd == 0 and cd == 0, f"{what}: {dd} depth and {cd} colour pixels differ from the per-draw path"


def test_batch_equals_per_draw_path_and_oracle(ctx, port):
    scenes = small_batch()
    draws = api.batch_draws(ctx, scenes)
    batch = api.Batch(ctx, draws)
    batch.launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, scenes, draws)
    for k, (g, e) in enumerate(zip(got, exp)):
        assert_same(g, e, f"draw {k}")
    for k in range(0, len(scenes), 6):  # the oracle on a subset (its CPU time dominates)
        sc = scenes[k]
        assert_parity(got[k], port.draw(sc, port.camera(sc.camera)[2]), f"batch draw {k} vs oracle")
    info = batch.info()
    assert info["draws"] == len(scenes) and info["launches"] == 1
    assert info["faces"] == sum(sc.mesh.indices.shape[0] for sc in scenes)
    batch.close()


def test_batch_relaunch_and_graph_replay(ctx):
    scenes = small_batch(count=12, seed=7)
    draws = api.batch_draws(ctx, scenes)
    batch = api.Batch(ctx, draws)
    batch.launch()
    first = [d.framebuffer.read() for d in draws]
    for d in draws:  # scribble, so that the replay has to rewrite everything
        d.framebuffer.clearColor(9, 9, 9, 9)
        d.framebuffer.clearDepth(-1.0)
    g = api.Graph(ctx).begin()
    batch.launch()
    g.end()
    for _ in range(2):
        g.launch()
    ctx.sync()
    for k, d in enumerate(draws):
        assert_same(d.framebuffer.read(), first[k], f"graph replay draw {k}")
    g.close()
    batch.close()


def test_one_shot_batch_and_clear_variants(ctx):
    scenes = small_batch(count=9, seed=11)
    draws = api.batch_draws(ctx, scenes)
    # draws 0-2 clear both planes, 3-5 colour only, 6-8 nothing; the framebuffers start
    # from a known non-clear state
    for k, d in enumerate(draws):
        d.framebuffer.clearColor(10, 20, 30, 40)
        d.framebuffer.clearDepth(0.999)
        if 3 <= k < 6:
            d.clear_depth = None
        elif k >= 6:
            d.clear_color = None
            d.clear_depth = None
    api.draw_batch(ctx, draws)
    got = [d.framebuffer.read() for d in draws]
    exp = []
    for sc, d in zip(scenes, draws):
        fb = api.Framebuffer(ctx, sc.width, sc.height)
        fb.clearColor(10, 20, 30, 40)
        fb.clearDepth(0.999)
        if d.clear_color is not None:
            fb.clearColor(*d.clear_color)
        if d.clear_depth is not None:
            fb.clearDepth(d.clear_depth)
        pipe = api.TiledPipeline(ctx, d.camera, fb)
        pipe.setShader(d.shader)
        pipe.drawMesh(d.model, d.mesh)
        exp.append(fb.read())
    for k in range(len(draws)):
        assert_same(got[k], exp[k], f"one-shot draw {k}")
    # a second one-shot batch of another size re-plans into the same context batch
    api.draw_batch(ctx, draws[:4])
    ctx.sync()


def test_batch_odd_widths_without_tma(ctx):
    """Widths that are not a multiple of 4 have no tensor map: plain tile stores."""
    scenes = [W.sphere_scene(width=w, height=h, lon=lon, lat=lon // 2, tex_size=32)
              for (w, h, lon) in ((250, 131, 24), (97, 203, 40), (33, 17, 8), (1001, 64, 64))]
    draws = api.batch_draws(ctx, scenes)
    api.Batch(ctx, draws).launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, scenes, draws)
    for k in range(len(scenes)):
        assert_same(got[k], exp[k], f"odd width draw {k}")


def test_phased_clears_with_and_without_tensor_maps(ctx):
    """The phased form's fused clears: framebuffers with tensor maps get their key-less
    tiles from TMA stores of a cleared tile in the tile pass, the others from the clear
    kernel; both in one batch, over framebuffers scribbled beforehand, with partial edge
    tiles and a draw whose mesh covers little of its frame, equal the per-draw path."""
    sizes = ((256, 131, 32), (250, 131, 24), (100, 37, 16), (97, 203, 40), (512, 64, 8), (36, 300, 64))
    scenes = [W.sphere_scene(width=w, height=h, lon=lon, lat=lon // 2, tex_size=32) for (w, h, lon) in sizes]
    scenes[4].camera = W.orbit_camera(12.0, 10.0, 30.0, 512, 64)  # far away: mostly key-less tiles
    draws = api.batch_draws(ctx, scenes)
    for d in draws:
        d.clear_color = (10, 20, 30, 40)
        d.clear_depth = 0.75
        d.framebuffer.clearColor(200, 1, 2, 3)
        d.framebuffer.clearDepth(-5.0)
    saved = ctx.batch_form
    try:
        ctx.batch_form = api.BATCH_PHASED
        b = api.Batch(ctx, draws)
    finally:
        ctx.batch_form = saved
    b.launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, scenes, draws)
    for k in range(len(scenes)):
        assert_same(got[k], exp[k], f"draw {k} ({sizes[k][0]}x{sizes[k][1]})")
    b.close()


def test_batch_all_shader_kinds(ctx, port):
    """Flat, Phong, PBR, Blinn-Phong and Gouraud draws in one batch: one launch per kind."""
    scenes = []
    for k, kind in enumerate((W.SHADER_FLAT, W.SHADER_PHONG, W.SHADER_PBR, W.SHADER_BLINN_PHONG, W.SHADER_GOURAUD)):
        if kind == W.SHADER_GOURAUD:
            sc = W.soup_scene(count=2000, width=128, height=96, seed=20 + k, edge_min=2, edge_max=20,
                              depth_min=0.5, depth_max=5.0)
        else:
            sc = W.sphere_scene(width=128, height=96, lon=32, lat=16, tex_size=32, shader=kind)
        scenes.append(sc)
    draws = api.batch_draws(ctx, scenes)
    batch = api.Batch(ctx, draws)
    assert batch.info()["launches"] == 5
    batch.launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, scenes, draws)
    for k, sc in enumerate(scenes):
        assert_same(got[k], exp[k], f"shader kind {sc.shader.kind}")
        assert_parity(got[k], port.draw(sc, port.camera(sc.camera)[2]), f"batch shader {sc.shader.kind} vs oracle")


def test_batch_clipped_triangles(ctx):
    """Cameras inside the near/side planes of the spheres exercise the clipped-winner path."""
    scenes = []
    for k, dist in enumerate((1.05, 1.3, 1.6)):
        sc = W.batch_scenes(count=1, seed=5, tex_size=32, resolution_scale=0.25)[0]
        cam = W.orbit_camera(dist, 10.0 * k, 30.0 * k, sc.width, sc.height)
        scenes.append(W.Scene(f"clip{k}", sc.mesh, cam, sc.shader, sc.width, sc.height))
    draws = api.batch_draws(ctx, scenes)
    api.Batch(ctx, draws).launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, scenes, draws)
    for k in range(len(scenes)):
        assert_same(got[k], exp[k], f"clipped draw {k}")


def test_autotune_table(ctx):
    scenes = small_batch(count=16, seed=13)
    draws = api.batch_draws(ctx, scenes)
    classes = {api.density_class(d) for d in draws}
    assert all(0 <= c < 6 for c in classes)
    before = ctx.tuning()
    table = api.autotune(ctx, draws, repeats=1)
    assert len(table) == 6 and all(v in (16, 32, 64, 128, 256) for v in table)
    assert ctx.tuning() == table
    for c in range(6):
        if c not in classes:
            assert table[c] == before[c]
    # a batch planned with the tuned table gives the same frames
    batch = api.Batch(ctx, draws)
    batch.launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, scenes, draws)
    for k in range(len(scenes)):
        assert_same(got[k], exp[k], f"tuned draw {k}")
    ctx.set_tuning(before)


def test_batch_argument_errors(ctx):
    scenes = small_batch(count=2, seed=3)
    draws = api.batch_draws(ctx, scenes)
    dup = [draws[0], api.Draw(draws[1].mesh, draws[0].framebuffer, draws[1].camera, draws[1].shader)]
    with pytest.raises(AxrError) as ei:
        api.Batch(ctx, dup)
    assert "distinct" in ei.value.message
    bad = api.Draw(draws[0].mesh, draws[0].framebuffer, draws[0].camera, api.Shader(17))
    with pytest.raises(AxrError):
        api.draw_batch(ctx, [bad])
    api.draw_batch(ctx, [])  # empty batch: nothing to do
    ctx.sync()


def test_framebuffers_read_async_matches_single_reads(ctx):
    import ctypes as C

    scenes = small_batch(count=6, seed=17)
    draws = api.batch_draws(ctx, scenes)
    api.draw_batch(ctx, draws)
    single = [d.framebuffer.read() for d in draws]
    n = len(draws)
    outs = [(np.zeros((d.framebuffer.height, d.framebuffer.width, 4), np.uint8),
             np.zeros((d.framebuffer.height, d.framebuffer.width), np.float32)) for d in draws]
    fbs = (C.c_void_p * n)(*[d.framebuffer.handle.value for d in draws])
    bgra = (C.c_void_p * n)(*[o[0].ctypes.data for o in outs])
    depth = (C.c_void_p * n)(*[o[1].ctypes.data if k % 2 == 0 else None for k, o in enumerate(outs)])
    assert ctx.lib.axr_framebuffers_read_async(ctx.handle, n, fbs, bgra, depth) == 0
    ctx.sync()
    for k in range(n):
        assert np.array_equal(outs[k][0], single[k][0])
        if k % 2 == 0:
            assert np.array_equal(outs[k][1].view(np.uint32), single[k][1].view(np.uint32))
        else:
            assert not outs[k][1].any()  # depth not requested


def test_detached_readback_pipeline(ctx):
    """axr_readback_start / wait: copies on the read-back's own streams while the next batch
    renders into another framebuffer set; each set comes back as its own frames."""
    import ctypes as C

    scenes = small_batch(count=5, seed=23)
    sets = [api.batch_draws(ctx, scenes), api.batch_draws(ctx, scenes[::-1])]
    n = len(scenes)
    expect = []
    for st in sets:
        api.draw_batch(ctx, st)
        expect.append([d.framebuffer.read()[0] for d in st])
    for st in sets:  # clear them again
        for d in st:
            d.framebuffer.clearColor(0, 0, 0, 0)
    ctx.sync()
    rbs = []
    for _ in sets:
        h = C.c_void_p()
        api.check(ctx.lib.axr_readback_create(ctx.handle, C.byref(h)), ctx.handle)
        rbs.append(h)
    outs = [[np.zeros((d.framebuffer.height, d.framebuffer.width, 4), np.uint8) for d in st] for st in sets]
    for k, st in enumerate(sets):
        api.draw_batch(ctx, st)
        fbs = (C.c_void_p * n)(*[d.framebuffer.handle.value for d in st])
        bgra = (C.c_void_p * n)(*[o.ctypes.data for o in outs[k]])
        api.check(ctx.lib.axr_readback_start(ctx.handle, rbs[k], n, fbs, bgra, None), ctx.handle)
    for k in range(2):
        api.check(ctx.lib.axr_readback_wait(ctx.handle, rbs[k]), ctx.handle)
        for got, want in zip(outs[k], expect[k]):
            assert np.array_equal(got, want)
    for h in rbs:
        ctx.lib.axr_readback_destroy(ctx.handle, h)


def test_packed_readback_formats(ctx):
    """axr_readback_start_packed: all colour planes in one host buffer, image after image,
    as stored (BGRA, row 0 first) or as the window shows them (RGB, top row first)."""
    import ctypes as C

    scenes = small_batch(count=5, seed=29)
    draws = api.batch_draws(ctx, scenes)
    api.draw_batch(ctx, draws)
    planes = [d.framebuffer.read()[0] for d in draws]
    n = len(draws)
    fbs = (C.c_void_p * n)(*[d.framebuffer.handle.value for d in draws])
    h = C.c_void_p()
    api.check(ctx.lib.axr_readback_create(ctx.handle, C.byref(h)), ctx.handle)
    pixels = sum(p.shape[0] * p.shape[1] for p in planes)
    for fmt, bpp in ((0, 4), (1, 3)):
        buf = np.zeros(pixels * bpp + 7, np.uint8)
        api.check(ctx.lib.axr_readback_start_packed(ctx.handle, h, n, fbs, fmt, buf.ctypes.data, buf.nbytes),
                  ctx.handle)
        api.check(ctx.lib.axr_readback_wait(ctx.handle, h), ctx.handle)
        at = 0
        for p in planes:
            k = p.shape[0] * p.shape[1] * bpp
            img = buf[at:at + k].reshape(p.shape[0], p.shape[1], bpp)
            want = p if fmt == 0 else p[::-1][:, :, [2, 1, 0]]
            assert np.array_equal(img, want)
            at += k
        assert not buf[at:].any()
    small = np.zeros(16, np.uint8)
    assert ctx.lib.axr_readback_start_packed(ctx.handle, h, n, fbs, 1, small.ctypes.data, small.nbytes) != 0
    ctx.lib.axr_readback_destroy(ctx.handle, h)


def test_grid_barrier_timeout_reports_and_context_survives(ctx):
    """Failure path of the persistent form's grid barrier, without a GPU fault: one CTA waits
    at a barrier the other never reaches; the bounded wait gives up after 50 ms, the next
    sync reports AXR_E_TIMEOUT, and the same context then renders a persistent batch that
    equals the phased one."""
    import time

    t0 = time.perf_counter()
    st = int(ctx.lib.axr_diag_barrier_timeout(ctx.handle, 50))
    took = time.perf_counter() - t0
    assert st == 4, (st, ctx.lib.axr_last_error(ctx.handle))
    assert 0.04 < took < 5.0
    assert int(ctx.lib.axr_diag_barrier_timeout(ctx.handle, 0)) == 1  # argument check
    ctx.sync()  # the error bit was cleared by the report
    scenes = small_batch(count=8, seed=23)
    frames = {}
    saved = ctx.batch_form
    try:
        for form in (api.BATCH_PERSISTENT, api.BATCH_PHASED):
            ctx.batch_form = form
            draws = api.batch_draws(ctx, scenes)
            api.draw_batch(ctx, draws)
            ctx.sync()
            frames[form] = [d.framebuffer.read() for d in draws]
    finally:
        ctx.batch_form = saved
    for k in range(len(scenes)):
        assert_same(frames[api.BATCH_PERSISTENT][k], frames[api.BATCH_PHASED][k], f"draw {k} after the timeout")


def test_split_phased_batch_equals_unsplit(ctx):
    """A phased batch of 128+ draws runs as two launch sets (context stream and a side
    stream, own counters and lists): its frames and statistics equal those of the
    persistent form (one launch set) on the same draws, eagerly and replayed from a graph."""
    scenes = W.batch_scenes(count=130, seed=29, tex_size=64, resolution_scale=0.1)
    draws = api.batch_draws(ctx, scenes)
    saved = ctx.batch_form
    frames, stats = {}, {}
    try:
        for form in (api.BATCH_PERSISTENT, api.BATCH_PHASED):
            ctx.batch_form = form
            batch = api.Batch(ctx, draws)
            for d in draws:
                d.framebuffer.clearColor(7, 7, 7, 7)
            ctx.stats(True)
            ctx.stats()  # reset
            batch.launch()
            stats[form] = ctx.stats()
            ctx.stats(False)
            frames[form] = [d.framebuffer.read() for d in draws]
            if form == api.BATCH_PHASED:
                assert batch.info()["launches"] == 2  # one shader kind, two launch sets
                for d in draws:
                    d.framebuffer.clearColor(9, 9, 9, 9)
                    d.framebuffer.clearDepth(-1.0)
                g = api.Graph(ctx).begin()
                batch.launch()
                g.end()
                g.launch()
                ctx.sync()
                for k, d in enumerate(draws):
                    assert_same(d.framebuffer.read(), frames[form][k], f"graph replay of the split batch, draw {k}")
                g.close()
                for d in draws:  # the one-shot entry point plans and launches the same split
                    d.framebuffer.clearColor(5, 5, 5, 5)
                api.draw_batch(ctx, draws)
                ctx.sync()
                for k, d in enumerate(draws):
                    assert_same(d.framebuffer.read(), frames[form][k], f"one-shot split batch, draw {k}")
            batch.close()
    finally:
        ctx.batch_form = saved
    for k in range(len(draws)):
        assert_same(frames[api.BATCH_PHASED][k], frames[api.BATCH_PERSISTENT][k], f"split vs persistent, draw {k}")
    assert stats[api.BATCH_PHASED] == stats[api.BATCH_PERSISTENT] and stats[api.BATCH_PHASED]["shaded"] > 0


def test_mesh_update_refreshes_bounds_for_planning(ctx):
    """axr_mesh_update of a mesh above 8,192 vertices computes the new positions' bounding
    sphere on the device (no host pass over the arrays): a draw of the updated mesh falls in the same density class as
    one of a mesh created from the same arrays, over model scales that cross every class
    boundary; the frames of the two agree exactly."""
    a = W.sphere_scene(width=96, height=96, lon=128, lat=64).mesh  # 8,385 vertices: the device path
    b = W.heightfield_scene(n=100, width=96, height=96, tex_size=16).mesh
    n = a.positions.shape[0]
    pos = (b.positions[:n] * np.float32(2.5) + np.float32([0.3, -0.2, 0.1])).astype(np.float32)
    mesh_a = api.Mesh(ctx, a.positions, a.uvs, a.normals, a.indices)
    mesh_a.update(pos, a.uvs, a.normals, a.indices)
    mesh_b = api.Mesh(ctx, pos, a.uvs, a.normals, a.indices)
    fb_a, fb_b = api.Framebuffer(ctx, 96, 96), api.Framebuffer(ctx, 96, 96)
    fb_big = api.Framebuffer(ctx, 2048, 2048)  # the classes need large screen areas per triangle
    cam = api.Camera((0.0, 0.0, 6.0), (0.0, 0.0, 0.0), 60.0, 1.0)
    seen = set()
    for s in np.geomspace(0.02, 5.0, 40):
        model = np.diag([s, s, s, 1.0]).astype(np.float32).reshape(16)
        da = api.Draw(mesh_a, fb_big, cam, api.BlinnPhongShader(), model)
        db = api.Draw(mesh_b, fb_big, cam, api.BlinnPhongShader(), model)
        ca, cb = api.density_class(da), api.density_class(db)
        assert ca == cb, (s, ca, cb)
        seen.add(ca)
    assert len(seen) >= 4
    model = np.diag([0.3, 0.3, 0.3, 1.0]).astype(np.float32).reshape(16)
    draws = [api.Draw(mesh_a, fb_a, cam, api.BlinnPhongShader(), model, (0, 0, 0, 255), float("inf")),
             api.Draw(mesh_b, fb_b, cam, api.BlinnPhongShader(), model, (0, 0, 0, 255), float("inf"))]
    api.draw_batch(ctx, draws)
    assert_same(fb_a.read(), fb_b.read(), "updated vs created mesh")


def test_split_batch_mixed_kinds_and_clears(ctx):
    """A phased batch of 150 draws of all five shader kinds (five groups, each run as two
    launch sets) with mixed clear requests (both planes, colour only, none) over
    framebuffers that start from a known state: every frame equals the persistent form's."""
    kinds = (W.SHADER_FLAT, W.SHADER_PHONG, W.SHADER_PBR, W.SHADER_BLINN_PHONG, W.SHADER_GOURAUD)
    base = {kind: W.sphere_scene(width=64, height=48, lon=24, lat=12, tex_size=16, shader=kind) for kind in kinds}
    scenes = []
    for k in range(150):
        kind = kinds[k % 5]
        sc = base[kind]
        cam = W.orbit_camera(2.0 + 0.02 * k, 10.0 + k % 40, 7.0 * k, sc.width, sc.height)
        scenes.append(W.Scene(f"mix{k}", sc.mesh, cam, sc.shader, sc.width, sc.height))
    draws = api.batch_draws(ctx, scenes)
    for k, d in enumerate(draws):
        if k % 3 == 1:
            d.clear_depth = None
        elif k % 3 == 2:
            d.clear_color = None
            d.clear_depth = None
    saved = ctx.batch_form
    frames = {}
    try:
        for form in (api.BATCH_PERSISTENT, api.BATCH_PHASED):
            ctx.batch_form = form
            batch = api.Batch(ctx, draws)
            if form == api.BATCH_PHASED:
                assert batch.info()["launches"] == 10  # five kinds, two launch sets each
            for d in draws:
                d.framebuffer.clearColor(40, 50, 60, 70)
                d.framebuffer.clearDepth(0.9)
            batch.launch()
            ctx.sync()
            frames[form] = [d.framebuffer.read() for d in draws]
            batch.close()
    finally:
        ctx.batch_form = saved
    for k in range(len(draws)):
        assert_same(frames[api.BATCH_PHASED][k], frames[api.BATCH_PERSISTENT][k], f"mixed split draw {k}")


def test_full_mixed_batch_split_equals_persistent(ctx):
    """The benchmark's 512-draw mixed batch (framebuffers at half scale, 1024² textures):
    the phased form, split into two launch sets, gives every frame of the persistent form
    bit for bit; compared through per-frame digests of colour and depth."""
    import hashlib

    scenes = W.batch_scenes(count=512, tex_size=1024, resolution_scale=0.5)
    draws = api.batch_draws(ctx, scenes)
    saved = ctx.batch_form
    digests = {}
    try:
        for form in (api.BATCH_PERSISTENT, api.BATCH_PHASED):
            ctx.batch_form = form
            batch = api.Batch(ctx, draws)
            assert batch.info()["launches"] == (2 if form == api.BATCH_PHASED else 1)
            batch.launch()
            ctx.sync()
            out = []
            for d in draws:
                bgra, depth = d.framebuffer.read()
                out.append(hashlib.sha1(bgra.tobytes() + np.ascontiguousarray(depth).view(np.uint32).tobytes()).digest())
            digests[form] = out
            batch.close()
    finally:
        ctx.batch_form = saved
    bad = [k for k in range(len(draws)) if digests[api.BATCH_PHASED][k] != digests[api.BATCH_PERSISTENT][k]]
    assert not bad, f"{len(bad)} draws differ, first {bad[:5]}"
