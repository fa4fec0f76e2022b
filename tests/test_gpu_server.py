"""Serving loop (axr_server_*): results are the same rendered alone and in a mix of
concurrent requests (exactly: the same device functions compute every value), equal to
the per-draw path and within the parity bar of the oracle; assets are evicted and
re-uploaded under a small device-memory budget without changing results; per-request
mode gives the same frames, and so do slots rendering side by side on their own streams;
oversized requests and bad arguments are rejected."""
import numpy as np
import pytest

from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import AXR_OK, AxrError
from helpers import assert_parity

pytestmark = pytest.mark.gpu


def scenes_mix():
    out = []
    for k in range(4):
        out.append(W.soup_scene(count=3000, width=160 + 8 * k, height=120, seed=40 + k, edge_min=1, edge_max=12,
                                depth_min=0.2, depth_max=50.0))
    for k, (w, h, lon) in enumerate(((128, 128, 32), (200, 100, 16), (96, 160, 48))):
        sc = W.sphere_scene(width=w, height=h, lon=lon, lat=lon // 2, tex_size=64, tex_seed=7 + k)
        out.append(sc)
    return out


def request(srv, ids, sc, k):
    bgra = np.zeros((sc.height, sc.width, 4), np.uint8)
    depth = np.zeros((sc.height, sc.width), np.float32)
    sh = sc.shader
    b, g, r, a = sc.clear_bgra
    t = srv.submit(ids[k], api.Camera.from_workload(sc.camera), api.Shader(sh.kind, tuple(sh.light_direction),
                   tuple(sh.light_color)), sc.width, sc.height, sc.model, (r, g, b, a), float("inf"), bgra, depth)
    return t, bgra, depth


def per_draw(ctx, sc):
    return api.render_scene(ctx, sc)


def test_same_alone_and_in_mix(ctx, port):
    scenes = scenes_mix()
    srv = api.Server(0, budget_bytes=2 << 30, max_batch=8, max_inflight=2)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    # alone
    alone = []
    for k, sc in enumerate(scenes):
        t, bgra, depth = request(srv, ids, sc, k)
        res = srv.wait(t, 60000)
        assert res["status"] == AXR_OK and res["batch_size"] == 1
        alone.append((bgra, depth))
    # in a mix: every scene three times, queued while the loop holds, then released
    order = [k % len(scenes) for k in range(3 * len(scenes))]
    srv.hold(True)
    pending = [(k,) + request(srv, ids, scenes[k], k) for k in order]
    srv.hold(False)
    sizes = []
    for k, t, bgra, depth in pending:
        res = srv.wait(t, 60000)
        assert res["status"] == AXR_OK
        sizes.append(res["batch_size"])
        assert np.array_equal(bgra, alone[k][0]) and np.array_equal(depth.view(np.uint32), alone[k][1].view(np.uint32)), \
            f"scene {k} differs between alone and mixed (batch of {res['batch_size']})"
    assert max(sizes) > 1, "the mix was never batched"
    st = srv.stats()
    assert st["completed"] == len(scenes) + len(order) and st["batches"] < st["completed"]
    assert max(sizes) == 8  # max_batch
    srv.close()
    # equal to the per-draw path, and to the oracle within the parity bar
    for k, sc in enumerate(scenes):
        got = per_draw(ctx, sc)
        assert np.array_equal(got[0], alone[k][0]) and np.array_equal(got[1].view(np.uint32), alone[k][1].view(np.uint32))
        if k % 3 == 0:
            assert_parity(alone[k], port.draw(sc, port.camera(sc.camera)[2]), f"served scene {k} vs oracle")


def test_eviction_under_small_budget(ctx):
    scenes = scenes_mix()
    # room for about two framebuffers and a few meshes: assets must come and go
    srv = api.Server(0, budget_bytes=3 << 20, max_batch=4, max_inflight=2)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    expect = [per_draw(ctx, sc) for sc in scenes]
    pending = []
    for rep in range(3):
        for k, sc in enumerate(scenes):
            pending.append((k,) + request(srv, ids, sc, k))
    for k, t, bgra, depth in pending:
        res = srv.wait(t, 60000)
        assert res["status"] == AXR_OK, res
        assert np.array_equal(bgra, expect[k][0]) and np.array_equal(depth.view(np.uint32), expect[k][1].view(np.uint32))
    st = srv.stats()
    assert st["evictions"] > 0 and st["uploads"] > len(scenes)
    assert st["peak_bytes"] <= 3 << 20
    srv.close()


def test_per_request_mode_matches(ctx):
    scenes = scenes_mix()[:4]
    srv = api.Server(0, budget_bytes=1 << 30, max_batch=8, max_inflight=2, per_request=True)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    pending = [(k,) + request(srv, ids, sc, k) for k, sc in enumerate(scenes)]
    for k, t, bgra, depth in pending:
        res = srv.wait(t, 60000)
        assert res["status"] == AXR_OK
        exp = per_draw(ctx, scenes[k])
        assert np.array_equal(bgra, exp[0]) and np.array_equal(depth.view(np.uint32), exp[1].view(np.uint32))
    srv.close()


@pytest.mark.parametrize("per_request", [False, True])
@pytest.mark.parametrize("budget", [1 << 30, 3 << 20])
def test_overlapping_slots_match(ctx, per_request, budget):
    """overlap_kernels: each in-flight slot renders on its own stream and scratch. Frames
    equal the per-draw path with a roomy budget and with one that forces framebuffers and
    assets to be freed and reallocated between the slots' streams."""
    scenes = scenes_mix()
    srv = api.Server(0, budget_bytes=budget, max_batch=4, max_inflight=2, per_request=per_request,
                     overlap_kernels=True)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    expect = [per_draw(ctx, sc) for sc in scenes]
    srv.hold(True)
    pending = [(k % len(scenes),) + request(srv, ids, scenes[k % len(scenes)], k % len(scenes))
               for k in range(3 * len(scenes))]
    srv.hold(False)
    for k, t, bgra, depth in pending:
        res = srv.wait(t, 60000)
        assert res["status"] == AXR_OK, res
        assert np.array_equal(bgra, expect[k][0]) and np.array_equal(depth.view(np.uint32), expect[k][1].view(np.uint32)), \
            f"scene {k} differs (batch of {res['batch_size']})"
    st = srv.stats()
    if budget < (1 << 30):
        assert st["evictions"] > 0
    srv.close()


def test_oversized_request_and_bad_arguments():
    sc = W.sphere_scene(width=64, height=64, lon=8, lat=4, tex_size=8)
    srv = api.Server(0, budget_bytes=1 << 20, max_batch=4, max_inflight=1)
    mid = srv.add_mesh(sc.mesh)
    cam = api.Camera.from_workload(sc.camera)
    t = srv.submit(mid, cam, api.BlinnPhongShader(), 4096, 4096)  # 4096^2 framebuffer > 1 MiB
    res = srv.wait(t, 60000)
    assert res["status"] == 3  # AXR_E_BUDGET
    t = srv.submit(mid, cam, api.BlinnPhongShader(), 64, 64)
    assert srv.wait(t, 60000)["status"] == AXR_OK
    with pytest.raises(AxrError):
        srv.submit(mid + 5, cam, api.BlinnPhongShader(), 64, 64)
    with pytest.raises(AxrError):
        srv.submit(mid, cam, api.Shader(9), 64, 64)
    with pytest.raises(AxrError):
        srv.wait(123456, 10)
    srv.close()


@pytest.mark.parametrize("per_request", [0, 1])
def test_png_outputs(ctx, per_request):
    """Requests that ask for PNG files (RGB or RGBA) beside or instead of the raw planes, in
    mixed batches: every file decodes to the request's colour plane; a buffer too small for
    its file gives AXR_E_CAPACITY with the needed size."""
    import pngfile

    scenes = scenes_mix()
    srv = api.Server(0, budget_bytes=2 << 30, max_batch=8, max_inflight=2, per_request=per_request)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    srv.hold(True)
    pend = []
    for k, sc in enumerate(scenes + scenes[:3]):
        ch = (3, 4, 0)[k % 3]
        bgra = np.zeros((sc.height, sc.width, 4), np.uint8)
        png = np.zeros(api.png_bound(sc.width, sc.height, ch or 3), np.uint8) if ch else None
        sh = sc.shader
        b, g, r, a = sc.clear_bgra
        t = srv.submit(ids[k % len(scenes)], api.Camera.from_workload(sc.camera),
                       api.Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)), sc.width, sc.height,
                       sc.model, (r, g, b, a), float("inf"), bgra, None, png_channels=ch, out_png=png)
        pend.append((t, ch, bgra, png))
    small = np.zeros(64, np.uint8)
    sc = scenes[0]
    t_small = srv.submit(ids[0], api.Camera.from_workload(sc.camera), api.BlinnPhongShader(), sc.width, sc.height,
                         sc.model, png_channels=3, out_png=small)
    srv.hold(False)
    for t, ch, bgra, png in pend:
        res = srv.wait(t, 60000)
        assert res["status"] == AXR_OK
        if ch:
            data = png[: res["png_bytes"]].tobytes()
            img, c, _ = pngfile.decode(data)
            assert c == ch and np.array_equal(img, pngfile.expected(bgra, ch))
        else:
            assert res["png_bytes"] == 0
    res = srv.wait(t_small, 60000)
    assert res["status"] == 7 and res["png_bytes"] > 64  # AXR_E_CAPACITY
    srv.close()


def test_cancel_queued_request():
    """Host-side fault injection: with admission held, a queued request is cancelled; it
    completes with AXR_E_CANCELLED and its host buffers stay untouched, the others render
    normally once admission resumes. Cancelling an unknown or finished ticket fails."""
    sc = W.sphere_scene(width=96, height=80, lon=16, lat=8, tex_size=16)
    srv = api.Server(0, budget_bytes=1 << 30, max_batch=8, max_inflight=1)
    ids = [srv.add_mesh(sc.mesh)]
    srv.hold(True)
    reqs = [request(srv, ids, sc, 0) for _ in range(3)]
    srv.cancel(reqs[1][0])
    with pytest.raises(AxrError):
        srv.cancel(reqs[1][0] + 1000)  # unknown ticket
    srv.hold(False)
    res = [srv.wait(t, 60000) for t, _, _ in reqs]
    assert [r["status"] for r in res] == [AXR_OK, 8, AXR_OK]  # AXR_E_CANCELLED
    assert not reqs[1][1].any() and not reqs[1][2].any()
    assert np.array_equal(reqs[0][1], reqs[2][1]) and reqs[0][1].any()
    t, bgra, depth = request(srv, ids, sc, 0)  # the host buffers must outlive the request
    srv.wait(t, 60000)
    with pytest.raises(AxrError):
        srv.cancel(t)  # waited for, so no longer known
    srv.close()
    assert bgra.any()


def test_slow_consumer_results_are_kept(ctx):
    """Host-side fault injection: a consumer that collects results late and out of order.
    The loop keeps running, every result is held until it is waited for, and each equals
    the per-draw path's frame."""
    scenes = scenes_mix()
    srv = api.Server(0, budget_bytes=1 << 30, max_batch=4, max_inflight=2)
    ids = [srv.add_mesh(sc.mesh) for sc in scenes]
    reqs = [(k % len(scenes),) + request(srv, ids, scenes[k % len(scenes)], k % len(scenes)) for k in range(21)]
    order = list(range(len(reqs)))[::-1][:7] + list(range(len(reqs)))[:14]  # the last ones first
    for i in order:
        k, t, bgra, depth = reqs[i]
        assert srv.wait(t, 60000)["status"] == AXR_OK
    exp = [per_draw(ctx, sc) for sc in scenes]
    for k, t, bgra, depth in reqs:
        assert np.array_equal(bgra, exp[k][0])
        assert np.array_equal(depth.view(np.uint32), exp[k][1].view(np.uint32))
    assert srv.stats()["completed"] == len(reqs)
    srv.close()
