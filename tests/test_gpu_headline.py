"""Parity at the configurations the benchmark numbers are quoted on.

* The mixed batch exactly as `bench.py` renders it by default: 512 draws at full
  resolution with the eight 1024^2 textures, planned after the autotuner, drawn by the
  batched form. Every draw is compared with the oracle (depth bit-exact, colour within
  1 LSB) and the per-draw differing-pixel counts are printed.
* The binned and persistent launch forms on the same 512-draw batch, against the phased
  form bit for bit.
* The served mix at full size: a 200,000-triangle soup at 3840x2160 and a 2,093,058-
  triangle heightfield at 1920x1080 among small requests, each the same alone and in the
  mix, and the two large requests against the oracle.
"""
import numpy as np
import pytest

from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import AXR_OK
from helpers import frame_diff

pytestmark = pytest.mark.gpu


def test_full_mixed_batch_against_oracle(ctx, port):
    scenes = W.batch_scenes()
    assert len(scenes) == 512
    draws = api.batch_draws(ctx, scenes)
    api.autotune(ctx, draws, repeats=1)
    batch = api.Batch(ctx, draws)
    for d in draws:  # scribble, so that the batch has to write every pixel
        d.framebuffer.clearColor(7, 7, 7, 7)
        d.framebuffer.clearDepth(-1.0)
    batch.launch()
    ctx.sync()
    worst = {"depth_mismatch": 0, "color_max_lsb": 0}
    differing = []
    for k, (sc, d) in enumerate(zip(scenes, draws)):
        got = d.framebuffer.read()
        exp = port.draw(sc, port.camera(sc.camera)[2])
        r = frame_diff(got, exp)
        differing.append(r["color_differing_pixels"])
        worst["depth_mismatch"] = max(worst["depth_mismatch"], r["depth_mismatch"])
        worst["color_max_lsb"] = max(worst["color_max_lsb"], r["color_max_lsb"])
        assert r["depth_mismatch"] == 0, f"draw {k} ({sc.width}x{sc.height}): {r}"
        assert r["color_max_lsb"] <= 1, f"draw {k} ({sc.width}x{sc.height}): {r}"
    print(f"512 draws vs oracle: worst {worst}; colour-differing pixels per draw: total {sum(differing)}, "
          f"max {max(differing)}, draws with any {sum(1 for x in differing if x)}")
    batch.close()
    for d in draws:
        d.framebuffer.close()


@pytest.mark.parametrize("form", [api.BATCH_BINNED, api.BATCH_PERSISTENT])
def test_full_mixed_batch_forms_agree(ctx, form):
    """The other launch forms on the same 512-draw batch give the phased form's frames bit
    for bit (the phased form being the one checked against the oracle above when the
    autotuner picks it; either way every form is pinned at the headline configuration)."""
    scenes = W.batch_scenes()
    textures, meshes = {}, {}
    ref = api.batch_draws(ctx, scenes, textures, meshes)
    alt = api.batch_draws(ctx, scenes, textures, meshes)
    saved = ctx.batch_form
    try:
        ctx.batch_form = api.BATCH_PHASED
        b_ref = api.Batch(ctx, ref)
        ctx.batch_form = form
        b_alt = api.Batch(ctx, alt)
    finally:
        ctx.batch_form = saved
    for d in alt:
        d.framebuffer.clearColor(7, 7, 7, 7)
        d.framebuffer.clearDepth(-1.0)
    b_ref.launch()
    b_alt.launch()
    ctx.sync()
    for k, (dr, da) in enumerate(zip(ref, alt)):
        cr, zr = dr.framebuffer.read()
        ca, za = da.framebuffer.read()
        assert np.array_equal(cr, ca), f"draw {k}: colour differs in {int((cr != ca).any(axis=2).sum())} pixels"
        assert np.array_equal(zr.view(np.uint32), za.view(np.uint32)), f"draw {k}: depth differs"
    b_ref.close()
    b_alt.close()
    for d in ref + alt:
        d.framebuffer.close()


def _request(srv, mid, sc):
    bgra = np.zeros((sc.height, sc.width, 4), np.uint8)
    depth = np.zeros((sc.height, sc.width), np.float32)
    sh = sc.shader
    b, g, r, a = sc.clear_bgra
    t = srv.submit(mid, api.Camera.from_workload(sc.camera),
                   api.Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)), sc.width, sc.height,
                   sc.model, (r, g, b, a), float("inf"), bgra, depth)
    return t, bgra, depth


def test_full_size_served_mix(port):
    soup = W.soup_scene(seed=1000)
    hf = W.heightfield_scene()
    hf.camera = W.orbit_camera(2.5, 30.0, 130.0, 1920, 1080)
    small = [W.sphere_scene(width=w, height=h, lon=lon, lat=lon // 2, tex_size=64, tex_seed=3 + k)
             for k, (w, h, lon) in enumerate(((256, 256, 64), (512, 512, 128), (1024, 1024, 256)))]
    scenes = [soup, hf] + small
    srv = api.Server(0, budget_bytes=40 << 30, max_batch=16, max_inflight=2)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    alone = []
    for k, sc in enumerate(scenes):
        t, bgra, depth = _request(srv, ids[k], sc)
        res = srv.wait(t, 120000)
        assert res["status"] == AXR_OK and res["batch_size"] == 1, res
        alone.append((bgra, depth))
    order = [0, 2, 1, 3, 0, 4, 1, 2, 0, 3]
    srv.hold(True)
    pending = [(k,) + _request(srv, ids[k], scenes[k]) for k in order]
    srv.hold(False)
    sizes = []
    for k, t, bgra, depth in pending:
        res = srv.wait(t, 120000)
        assert res["status"] == AXR_OK, res
        sizes.append(res["batch_size"])
        assert np.array_equal(bgra, alone[k][0]), f"request kind {k}: colour differs between alone and the mix"
        assert np.array_equal(depth.view(np.uint32), alone[k][1].view(np.uint32)), \
            f"request kind {k}: depth differs between alone and the mix"
    assert max(sizes) > 1, "the mix was never batched"
    srv.close()
    for k in (0, 1):
        sc = scenes[k]
        r = frame_diff(alone[k], port.draw(sc, port.camera(sc.camera)[2]))
        print(f"served {sc.name} {sc.width}x{sc.height} vs oracle: {r}")
        assert r["depth_mismatch"] == 0 and r["color_max_lsb"] <= 1, r
