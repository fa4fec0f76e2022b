"""Host-side checks of the PNG output path (no GPU): the worst-case size bound and the
test reader itself on files written by CPython's zlib."""
import numpy as np
import pytest

import pngfile
from axiomr_gb300 import api


def test_png_bound_covers_worst_case():
    for w, h, ch in [(1, 1, 3), (1, 1, 4), (37, 23, 3), (3840, 2160, 3), (1920, 1080, 4), (11000, 3, 3)]:
        b = api.png_bound(w, h, ch)
        raw = h * (1 + w * ch)
        # 9 bits per byte, zlib and PNG framing, 12 bytes per 64 KiB chunk
        assert b >= raw * 9 // 8 + 8 + 33 + 39 + 12 + 12 * (raw * 9 // 8 // 65524 + 1)
        assert b < raw * 9 // 8 + 2 * 65536 + 1024
    assert api.png_bound(0, 5, 3) == 0 and api.png_bound(5, 0, 3) == 0 and api.png_bound(5, 5, 2) == 0


def test_reader_on_reference_files():
    rng = np.random.default_rng(3)
    for shape in [(1, 1, 3), (5, 7, 4), (64, 33, 3)]:
        px = rng.integers(0, 256, shape, dtype=np.uint8)
        img, ch, seen = pngfile.decode(pngfile.encode_reference(px))
        assert ch == shape[2] and seen == {0} and np.array_equal(img, px)


def test_reader_rejects_corruption():
    px = np.zeros((4, 4, 3), np.uint8)
    data = bytearray(pngfile.encode_reference(px))
    data[40] ^= 1
    with pytest.raises(AssertionError):
        pngfile.decode(bytes(data))
