"""Output encoding on the GPU (axr_framebuffers_encode_png / axr_framebuffers_read_png):
each file is read back by an independent PNG reader (tests/pngfile.py: chunk CRCs checked
with zlib.crc32, the stream inflated by CPython's zlib, which checks the Adler-32) and must
hold exactly what the reference's window shows for the framebuffer: the colour plane top
row first (framebuffer row 0 is the bottom row), RGB with alpha dropped, or RGBA."""
import ctypes as C

import numpy as np
import pytest

import pngfile
from axiomr_gb300 import api
from axiomr_gb300 import workloads as W
from axiomr_gb300._lib import AxrError

pytestmark = pytest.mark.gpu


def fb_with(ctx, bgra):
    h, w = bgra.shape[:2]
    fb = api.Framebuffer(ctx, w, h)
    fb.write(np.ascontiguousarray(bgra, np.uint8), np.zeros((h, w), np.float32))
    return fb


def check_file(data, bgra, channels):
    img, ch, seen = pngfile.decode(data)
    assert ch == channels and seen == {0}
    assert np.array_equal(img, pngfile.expected(bgra, channels))


def patterns(rng, w, h):
    noise = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    flat = np.broadcast_to(np.array([10, 200, 30, 255], np.uint8), (h, w, 4)).copy()
    hstripes = np.repeat(rng.integers(0, 256, (h, 1, 4), dtype=np.uint8), w, axis=1)  # rows constant
    vstripes = np.repeat(rng.integers(0, 256, (1, w, 4), dtype=np.uint8), h, axis=0)  # rows repeat
    blocks = np.kron(rng.integers(0, 4, (h // 7 + 1, w // 5 + 1, 1)) * 60, np.ones((7, 5, 4)))[:h, :w].astype(np.uint8)
    alpha = flat.copy()
    alpha[..., 3] = rng.integers(0, 256, (h, w), dtype=np.uint8)  # equal RGB, varying alpha
    return {"noise": noise, "flat": flat, "hstripes": hstripes, "vstripes": vstripes, "blocks": blocks, "alpha": alpha}


@pytest.mark.parametrize("channels", [3, 4])
def test_rendered_frame_round_trips(ctx, channels):
    sc = W.sphere_scene(width=256, height=192, lon=32, lat=16)
    fb = api.Framebuffer(ctx, sc.width, sc.height)
    bgra, _ = api.render_scene(ctx, sc, framebuffer=fb)
    data = fb.read_png(channels)
    check_file(data, bgra, channels)
    assert len(data) < 0.5 * sc.width * sc.height * channels  # the background compresses


@pytest.mark.parametrize("shape", [(1, 1), (1, 40), (40, 1), (23, 37), (5, 31), (7, 33), (3, 64), (2, 65), (200, 300)])
def test_patterns_and_odd_sizes(ctx, shape):
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    h, w = shape
    pats = patterns(rng, w, h)
    fbs = [fb_with(ctx, p) for p in pats.values()]
    for channels in (3, 4):
        files = api.read_png(ctx, fbs, channels)
        for (name, p), data in zip(pats.items(), files):
            check_file(data, p, channels)


def test_several_idat_chunks_and_sizes(ctx):
    """Noise does not compress: the stream spans several 64 KiB IDAT chunks; flat and
    striped images shrink to a few percent."""
    rng = np.random.default_rng(7)
    w, h = 512, 300
    pats = patterns(rng, w, h)
    fbs = [fb_with(ctx, p) for p in pats.values()]
    files = api.read_png(ctx, fbs, 3)
    sizes = dict(zip(pats, map(len, files)))
    raw = h * (1 + 3 * w)
    assert raw < sizes["noise"] <= api.png_bound(w, h, 3)
    assert len([c for c in pngfile.chunks(files[0]) if c[0] == b"IDAT"]) >= 6
    # runs are cut every 32 pixels: a flat step costs ~13 bits against 96 bytes of RGB
    assert sizes["flat"] < raw / 30 and sizes["hstripes"] < raw / 20 and sizes["vstripes"] < raw / 15
    for (name, p), data in zip(pats.items(), files):
        check_file(data, p, 3)


def test_wide_rows_beyond_match_distance(ctx):
    """Scanlines longer than deflate's 32 KiB window: no row-above matches, still exact."""
    rng = np.random.default_rng(11)
    w, h = 11000, 3
    img = np.repeat(rng.integers(0, 256, (1, w, 4), dtype=np.uint8), h, axis=0)
    img[1, ::97] = 0
    fb = fb_with(ctx, img)
    for channels in (3, 4):
        check_file(fb.read_png(channels), img, channels)


def test_batched_encode_of_rendered_batch(ctx):
    """The frames of one batch, encoded by one call into device buffers."""
    scenes = W.batch_scenes(count=12, tex_size=64, resolution_scale=0.25)
    draws = api.batch_draws(ctx, scenes)
    api.draw_batch(ctx, draws)
    fbs = [d.framebuffer for d in draws]
    n = len(fbs)
    caps = [api.png_bound(fb.width, fb.height, 3) for fb in fbs]
    import torch

    bufs = [torch.empty((c + 255) // 256 * 256, dtype=torch.uint8, device="cuda:0") for c in caps]
    sizes = torch.zeros(n, dtype=torch.int64, device="cuda:0")
    torch.cuda.synchronize()
    arr = (C.c_void_p * n)(*[fb.handle for fb in fbs])
    outs = (C.c_void_p * n)(*[b.data_ptr() for b in bufs])
    capa = (C.c_uint64 * n)(*caps)
    api.check(ctx.lib.axr_framebuffers_encode_png(ctx.handle, n, arr, 3, outs, capa, C.c_void_p(sizes.data_ptr())),
              ctx.handle)
    ctx.sync()
    sz = sizes.cpu().numpy()
    for i, fb in enumerate(fbs):
        bgra, _ = fb.read()
        check_file(bufs[i][: int(sz[i])].cpu().numpy().tobytes(), bgra, 3)


def test_encode_argument_errors(ctx):
    fb = fb_with(ctx, np.zeros((8, 8, 4), np.uint8))
    n = 1
    arr = (C.c_void_p * n)(fb.handle)
    sizes = (C.c_uint64 * n)()
    with pytest.raises(AxrError):  # channels
        api.check(ctx.lib.axr_framebuffers_read_png(ctx.handle, 1, arr, 2, None, None, sizes), ctx.handle)
    small = np.empty(16, np.uint8)
    ptrs = (C.c_void_p * n)(small.ctypes.data)
    caps = (C.c_uint64 * n)(16)
    with pytest.raises(AxrError):  # host buffer too small; the size is still reported
        api.check(ctx.lib.axr_framebuffers_read_png(ctx.handle, 1, arr, 3, ptrs, caps, sizes), ctx.handle)
    assert sizes[0] > 16
    import torch

    dev = torch.empty(64, dtype=torch.uint8, device="cuda:0")
    outs = (C.c_void_p * n)(dev.data_ptr())
    dsz = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    with pytest.raises(AxrError):  # device buffer below the bound
        api.check(ctx.lib.axr_framebuffers_encode_png(ctx.handle, 1, arr, 3, outs, caps, C.c_void_p(dsz.data_ptr())),
                  ctx.handle)


def test_many_images_in_one_call(ctx):
    """More images than the CRC pass keeps per tile (1024), of mixed small sizes."""
    rng = np.random.default_rng(13)
    imgs = []
    for k in range(1100):
        h, w = int(rng.integers(1, 12)), int(rng.integers(1, 40))
        img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        if k % 3 == 0:
            img[:] = img[0, 0]  # flat
        imgs.append(img)
    fbs = [fb_with(ctx, im) for im in imgs]
    for channels in (3, 4):
        files = api.read_png(ctx, fbs, channels)
        for im, data in zip(imgs, files):
            check_file(data, im, channels)


def test_png_batch_pipeline(ctx):
    """Two PngBatch objects in flight: encode A, encode B, read A, read B; a batch re-used
    after its read encodes the framebuffers' new contents."""
    rng = np.random.default_rng(17)
    shapes = [(31, 45), (64, 64), (7, 300)]
    a_imgs = [rng.integers(0, 256, (h, w, 4), dtype=np.uint8) for h, w in shapes]
    b_imgs = [np.kron(rng.integers(0, 3, (h // 4 + 1, w // 4 + 1, 4)), np.ones((4, 4, 1)))[:h, :w].astype(np.uint8) * 80
              for h, w in shapes]
    fa = [fb_with(ctx, im) for im in a_imgs]
    fb = [fb_with(ctx, im) for im in b_imgs]
    pa, pb = api.PngBatch(ctx), api.PngBatch(ctx)
    pa.encode(fa, 3)
    pb.encode(fb, 4)
    for im, data in zip(a_imgs, pa.read()):
        check_file(data, im, 3)
    for im, data in zip(b_imgs, pb.read()):
        check_file(data, im, 4)
    new = [255 - im for im in a_imgs]
    for f, im in zip(fa, new):
        f.write(im, np.zeros(im.shape[:2], np.float32))
    pa.encode(fa, 3)
    for im, data in zip(new, pa.read()):
        check_file(data, im, 3)
    pa.close()
    pb.close()


def test_read_png_from_two_threads(ctx):
    """Calls on one context from two threads are serialised: each gets its own files."""
    import threading

    rng = np.random.default_rng(31)
    sets = [[rng.integers(0, 256, (40 + 7 * k, 60, 4), dtype=np.uint8) for k in range(6)] for _ in range(2)]
    fbs = [[fb_with(ctx, im) for im in s] for s in sets]
    out = [None, None]
    errors = []

    def run(i):
        try:
            for _ in range(5):
                out[i] = api.read_png(ctx, fbs[i], 3)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(e)

    ts = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for i in range(2):
        for im, data in zip(sets[i], out[i]):
            check_file(data, im, 3)
