"""A strict PNG reader for the encoder tests: checks the signature, every chunk's CRC-32
(zlib.crc32), IHDR, chunk order and IEND, inflates the IDAT stream with CPython's zlib
(which checks the Adler-32) and undoes the scanline filters. An implementation apart from
the one under test, so a decoded image equal to the framebuffer proves the file lossless
and well formed."""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89PNG\r\n\x1a\n"


def chunks(data: bytes):
    assert data[:8] == SIGNATURE, "bad signature"
    at = 8
    out = []
    while at < len(data):
        (n,) = struct.unpack(">I", data[at:at + 4])
        kind = data[at + 4:at + 8]
        body = data[at + 8:at + 8 + n]
        (crc,) = struct.unpack(">I", data[at + 8 + n:at + 12 + n])
        assert len(body) == n, "truncated chunk"
        assert zlib.crc32(kind + body) & 0xFFFFFFFF == crc, f"CRC of {kind!r} chunk {len(out)}"
        out.append((kind, body))
        at += 12 + n
    assert at == len(data), "bytes after the last chunk"
    return out


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def decode(data: bytes):
    """-> (pixels (H, W, C) uint8, channels, filter types seen)."""
    cs = chunks(data)
    assert cs[0][0] == b"IHDR" and cs[-1] == (b"IEND", b""), "IHDR first, IEND last"
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", cs[0][1])
    assert depth == 8 and ctype in (2, 6) and comp == 0 and filt == 0 and inter == 0
    ch = 3 if ctype == 2 else 4
    kinds = [k for k, _ in cs]
    first = kinds.index(b"IDAT")
    last = len(kinds) - 1 - kinds[::-1].index(b"IDAT")
    assert all(k == b"IDAT" for k in kinds[first:last + 1]), "IDAT chunks must be consecutive"
    stream = b"".join(b for k, b in cs if k == b"IDAT")
    d = zlib.decompressobj()
    raw = d.decompress(stream)
    assert d.eof and not d.unused_data, "zlib stream must end exactly at the data end"
    stride = 1 + w * ch
    assert len(raw) == h * stride, f"{len(raw)} inflated bytes, expected {h * stride}"
    rows = np.frombuffer(raw, np.uint8).reshape(h, stride)
    img = np.zeros((h, w * ch), np.uint8)
    seen = set()
    for y in range(h):
        f = int(rows[y, 0])
        seen.add(f)
        line = rows[y, 1:].astype(np.int32)
        up = img[y - 1].astype(np.int32) if y else np.zeros(w * ch, np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + up) & 255
        elif f in (1, 3, 4):
            cur = np.zeros(w * ch, np.int32)
            for i in range(w * ch):
                a = cur[i - ch] if i >= ch else 0
                c = up[i - ch] if i >= ch else 0
                pred = a if f == 1 else ((a + up[i]) // 2 if f == 3 else _paeth(a, up[i], c))
                cur[i] = (line[i] + pred) & 255
        else:
            raise AssertionError(f"filter type {f}")
        img[y] = cur.astype(np.uint8)
    return img.reshape(h, w, ch), ch, seen


def expected(bgra: np.ndarray, channels: int) -> np.ndarray:
    """What the file must hold for a framebuffer's colour plane (H, W, 4) BGRA8 with row 0
    at the bottom: the top row first, RGB (alpha dropped) or RGBA."""
    order = [2, 1, 0] if channels == 3 else [2, 1, 0, 3]
    return np.ascontiguousarray(bgra[::-1][:, :, order])


def encode_reference(pixels: np.ndarray) -> bytes:
    """A PNG written with CPython's zlib (filter None), to test this reader."""
    h, w, ch = pixels.shape
    raw = b"".join(b"\x00" + pixels[y].tobytes() for y in range(h))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, 8, 2 if ch == 3 else 6, 0, 0, 0)
    return SIGNATURE + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
