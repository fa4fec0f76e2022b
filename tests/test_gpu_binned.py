"""The binned forms (bins of 8 tiles rasterised in shared memory, TMA tile loads and
stores): the per-draw binned path (AXR_DRAW_BINNED) must give exactly the frame of
the keyed path (visibility keys in device memory), whatever the bin shape, per-thread raster
limit or bin capacity (a full bin spills into the key plane), whether the framebuffer is
cleared, pre-filled or drawn into several times, and whether its width allows tensor maps;
and the binned batch form must give exactly the per-draw frames, including its fused clears,
and the oracle's frames within the parity bar."""
import numpy as np
import pytest

from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import AxrError
from helpers import assert_parity, golden_names, load_golden

pytestmark = pytest.mark.gpu


def same(got, exp, what):
    gb, gd = got
    eb, ed = exp
    dd = int((np.ascontiguousarray(gd).view(np.uint32) != np.ascontiguousarray(ed).view(np.uint32)).sum())
    cd = int((gb != eb).any(axis=-1).sum())
    assert dd == 0 and cd == 0, f"{what}: {dd} depth and {cd} colour pixels differ"


def render(ctx, form, scene, params=None, **kw):
    ctx.draw_form = form
    if params is not None:
        ctx.bin_params = params
    try:
        return api.render_scene(ctx, scene, **kw)
    finally:
        ctx.draw_form = api.DRAW_KEYED
        ctx.bin_params = {"capacity": 0, "tiles_x": 0, "tiles_y": 0, "thread_pixels": 64}


def scenes():
    out = [W.sphere_scene(width=256, height=192, lon=64, lat=32, tex_size=64),
           W.sphere_scene(width=250, height=131, lon=24, lat=12, tex_size=32),  # width % 4 != 0: no tensor map
           W.soup_scene(count=6000, width=320, height=240, seed=41, edge_min=0.5, edge_max=60.0, depth_min=0.1,
                        depth_max=100.0),  # clipped triangles, large and tiny ones
           W.heightfield_scene(n=96, width=300, height=170, tex_size=64)]
    close = W.sphere_scene(width=200, height=160, lon=48, lat=24, tex_size=32, shader=W.SHADER_PHONG)
    close.camera = W.orbit_camera(1.2, 15.0, 40.0, 200, 160)  # inside the near/side planes
    out.append(close)
    return out


def test_binned_equals_keyed_and_oracle(ctx, port):
    for k, sc in enumerate(scenes()):
        keyed = render(ctx, api.DRAW_KEYED, sc)
        binned = render(ctx, api.DRAW_BINNED, sc)
        same(binned, keyed, f"scene {k} {sc.name}")
        assert_parity(binned, port.draw(sc, port.camera(sc.camera)[2]), f"binned {sc.name} vs oracle")


@pytest.mark.parametrize("name", golden_names())
def test_binned_matches_golden_prefilled(ctx, name):
    """The goldens include pre-filled framebuffers: tiles loaded with TMA and merged into."""
    scene, vp, bgra_in, depth_in, bgra, depth = load_golden(name)
    got = render(ctx, api.DRAW_BINNED, scene, bgra=bgra_in, depth=depth_in, view_proj=vp)
    assert_parity(got, (bgra, depth), f"binned vs golden {name}")


@pytest.mark.parametrize("shape", [(8, 1), (4, 2), (2, 4), (1, 8), (4, 1), (2, 2), (1, 2), (1, 1)])
@pytest.mark.parametrize("thread_pixels", [1, 64, 2048])
def test_bin_shapes_and_thread_limits(ctx, shape, thread_pixels):
    for k, sc in enumerate(scenes()[:3]):
        keyed = render(ctx, api.DRAW_KEYED, sc)
        got = render(ctx, api.DRAW_BINNED, sc, {"capacity": 0, "tiles_x": shape[0], "tiles_y": shape[1],
                                                "thread_pixels": thread_pixels})
        same(got, keyed, f"scene {k}, bins of {shape} tiles, thread limit {thread_pixels}")


def test_full_bins_spill_into_the_key_plane(ctx):
    """Capacity 16 overflows most bins of a dense mesh: the excess goes through the key
    plane, which the bin pass folds in; the frame is unchanged and the key plane is left
    empty for the next draw (checked by drawing twice)."""
    dense = W.sphere_scene(width=320, height=240, lon=192, lat=96, tex_size=64)
    keyed = render(ctx, api.DRAW_KEYED, dense)
    for shape in ((8, 1), (2, 4), (1, 1)):
        got = render(ctx, api.DRAW_BINNED, dense, {"capacity": 16, "tiles_x": shape[0], "tiles_y": shape[1],
                                                   "thread_pixels": 64})
        same(got, keyed, f"capacity 16, bins of {shape} tiles")
    got = render(ctx, api.DRAW_KEYED, dense)
    same(got, keyed, "keyed after spills")


def test_several_draws_into_one_framebuffer(ctx):
    """Draws merge into what earlier draws left (strict less-than against the loaded depth)."""
    a = W.sphere_scene(width=256, height=256, lon=48, lat=24, tex_size=64)
    b = W.soup_scene(count=3000, width=256, height=256, seed=9, edge_min=2, edge_max=40, depth_min=0.5,
                     depth_max=20.0)
    results = {}
    for form in (api.DRAW_KEYED, api.DRAW_BINNED):
        ctx.draw_form = form
        fb = api.Framebuffer(ctx, 256, 256)
        fb.clearColor(5, 6, 7, 255)
        fb.clearDepth()
        for sc in (a, b, a):
            pipe = api.TiledPipeline(ctx, api.Camera.from_workload(sc.camera), fb)
            sh = sc.shader
            pipe.setShader(api.Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)))
            pipe.drawMesh(sc.model, api.Mesh.from_workload(ctx, sc.mesh))
        results[form] = fb.read()
        fb.close()
    ctx.draw_form = api.DRAW_KEYED
    same(results[api.DRAW_BINNED], results[api.DRAW_KEYED], "three draws into one framebuffer")


def test_bin_parameter_errors(ctx):
    for bad in ({"capacity": 8, "tiles_x": 8, "thread_pixels": 64}, {"capacity": 0, "tiles_x": 3, "thread_pixels": 64},
                {"capacity": 0, "tiles_x": 8, "thread_pixels": 0}, {"capacity": 1 << 17, "tiles_x": 8,
                                                                     "thread_pixels": 64},
                {"capacity": 0, "tiles_x": 4, "tiles_y": 4, "thread_pixels": 64}):
        with pytest.raises(AxrError):
            ctx.bin_params = bad
    with pytest.raises(AxrError):
        ctx.draw_form = 7
    table = ctx.bin_tuning()
    with pytest.raises(AxrError):  # capacity and shape 0 are for single draws only
        ctx.set_bin_tuning([{**t, "capacity": 0} for t in table])
    with pytest.raises(AxrError):
        ctx.set_bin_tuning([{**t, "tiles_x": 0} for t in table])
    ctx.set_bin_tuning([{**t, "capacity": 512, "tiles_x": 4, "tiles_y": 1} for t in table])
    assert all(t["capacity"] == 512 and t["tiles_x"] == 4 and t["tiles_y"] == 1 for t in ctx.bin_tuning())
    ctx.set_bin_tuning(table)


# ------------------------------------------------------------------ batched binned form
def plain_frames(ctx, scenes_, draws, prefill=None):
    out = []
    for sc, d in zip(scenes_, draws):
        fb = api.Framebuffer(ctx, sc.width, sc.height)
        if prefill:
            fb.clearColor(*prefill[0])
            fb.clearDepth(prefill[1])
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


@pytest.fixture
def binned_batches(ctx):
    before = ctx.batch_form
    ctx.batch_form = api.BATCH_BINNED
    yield
    ctx.batch_form = before


def test_batch_binned_equals_per_draw_and_oracle(ctx, port, binned_batches):
    sc = W.batch_scenes(count=24, seed=5, tex_size=64, resolution_scale=0.25)
    draws = api.batch_draws(ctx, sc)
    for d in draws:
        d.framebuffer.clearColor(9, 9, 9, 9)
        d.framebuffer.clearDepth(-1.0)
    batch = api.Batch(ctx, draws)
    assert batch.info()["form"] == api.BATCH_BINNED
    batch.launch()
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, sc, draws)
    for k in range(len(sc)):
        same(got[k], exp[k], f"binned batch draw {k}")
    for k in range(0, len(sc), 6):
        assert_parity(got[k], port.draw(sc[k], port.camera(sc[k].camera)[2]), f"binned batch draw {k} vs oracle")
    # recorded into a graph and replayed
    for d in draws:
        d.framebuffer.clearColor(1, 2, 3, 4)
        d.framebuffer.clearDepth(0.5)
    g = api.Graph(ctx).begin()
    batch.launch()
    g.end()
    g.launch()
    g.launch()
    ctx.sync()
    for k, d in enumerate(draws):
        same(d.framebuffer.read(), got[k], f"replayed binned batch draw {k}")
    g.close()
    batch.close()


def test_batch_binned_clear_variants_and_odd_widths(ctx, binned_batches):
    sc = W.batch_scenes(count=9, seed=11, tex_size=32, resolution_scale=0.25)
    sc += [W.sphere_scene(width=w, height=h, lon=lon, lat=lon // 2, tex_size=32)
           for (w, h, lon) in ((250, 131, 24), (97, 203, 40), (33, 17, 8))]
    draws = api.batch_draws(ctx, sc)
    for k, d in enumerate(draws):
        d.framebuffer.clearColor(10, 20, 30, 40)
        d.framebuffer.clearDepth(0.999)
        if k % 3 == 1:
            d.clear_depth = None
        elif k % 3 == 2:
            d.clear_color = None
            d.clear_depth = None
    api.draw_batch(ctx, draws)
    got = [d.framebuffer.read() for d in draws]
    exp = plain_frames(ctx, sc, draws, prefill=((10, 20, 30, 40), 0.999))
    for k in range(len(draws)):
        same(got[k], exp[k], f"binned clear variant draw {k}")


def test_batch_binned_shader_kinds_and_split_sets(ctx, port, binned_batches):
    """All five shader kinds (one launch set each) and a batch large enough for two launch
    sets on two streams."""
    kinds = []
    for k, kind in enumerate((W.SHADER_FLAT, W.SHADER_PHONG, W.SHADER_PBR, W.SHADER_BLINN_PHONG, W.SHADER_GOURAUD)):
        if kind == W.SHADER_GOURAUD:
            s = W.soup_scene(count=2000, width=128, height=96, seed=20 + k, edge_min=2, edge_max=20, depth_min=0.5,
                             depth_max=5.0)
        else:
            s = W.sphere_scene(width=128, height=96, lon=32, lat=16, tex_size=32, shader=kind)
        kinds.append(s)
    big = W.batch_scenes(count=140, seed=17, tex_size=32, resolution_scale=0.125)
    for group in (kinds, big):
        draws = api.batch_draws(ctx, group)
        batch = api.Batch(ctx, draws)
        batch.launch()
        got = [d.framebuffer.read() for d in draws]
        exp = plain_frames(ctx, group, draws)
        for k in range(len(group)):
            same(got[k], exp[k], f"draw {k} of a batch of {len(group)}")
        batch.close()
    for sc in kinds:
        draws = api.batch_draws(ctx, [sc])
        api.Batch(ctx, draws).launch()
        assert_parity(draws[0].framebuffer.read(), port.draw(sc, port.camera(sc.camera)[2]), f"kind {sc.shader.kind}")


def test_batch_binned_tuning_table_changes_nothing(ctx, binned_batches):
    sc = W.batch_scenes(count=12, seed=23, tex_size=32, resolution_scale=0.25)
    draws = api.batch_draws(ctx, sc)
    exp = plain_frames(ctx, sc, draws)
    before = ctx.bin_tuning()
    try:
        for table in ([{"capacity": 16, "tiles_x": 2, "tiles_y": 4, "thread_pixels": 1}] * 6,
                      [{"capacity": 4096, "tiles_x": 4, "tiles_y": 2, "thread_pixels": 2048}] * 6,
                      [{"capacity": 64, "tiles_x": 1, "tiles_y": 1, "thread_pixels": 64}] * 6):
            ctx.set_bin_tuning(table)
            api.Batch(ctx, draws).launch()
            for k, d in enumerate(draws):
                same(d.framebuffer.read(), exp[k], f"draw {k} with bins {table[0]}")
    finally:
        ctx.set_bin_tuning(before)
