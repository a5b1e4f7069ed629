"""The PNG decoder of the glTF importer (tinytrace_gb300/png.py) on files written by the test
with every colour type, bit depth and scanline filter, and with Adam7 interlacing; all decode
to the 8-bit RGBA the reference's importer asks its decoder for."""
import struct
import zlib

import numpy as np
import pytest

from tinytrace_gb300 import png

CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _pack_rows(samples, depth):
    """(h, w, c) integer samples -> (h, stride) bytes."""
    h, w, c = samples.shape
    flat = samples.reshape(h, w * c)
    if depth == 16:
        return np.stack([flat >> 8, flat & 0xFF], -1).reshape(h, -1).astype(np.uint8)
    if depth == 8:
        return flat.astype(np.uint8)
    bits = ((flat[..., None] >> np.arange(depth - 1, -1, -1)) & 1).reshape(h, -1).astype(np.uint8)
    return np.packbits(bits, axis=1)


def _filter(rows, bpp, ftypes):
    out = []
    prev = np.zeros(rows.shape[1], np.int32)
    for y, row in enumerate(rows.astype(np.int32)):
        f = ftypes[y % len(ftypes)]
        left = np.concatenate([np.zeros(bpp, np.int32), row[:-bpp]])[:len(row)]
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])[:len(row)]
        if f == 0:
            enc = row
        elif f == 1:
            enc = row - left
        elif f == 2:
            enc = row - prev
        elif f == 3:
            enc = row - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            enc = row - pred
        out.append(bytes([f]) + (enc & 0xFF).astype(np.uint8).tobytes())
        prev = row
    return b"".join(out)


def _write(samples, ctype, depth, palette=None, trns=None, interlace=False, ftypes=(0, 1, 2, 3, 4)):
    h, w, c = samples.shape
    bpp = max(1, c * depth // 8)
    if not interlace:
        raw = _filter(_pack_rows(samples, depth), bpp, ftypes)
    else:
        raw = b""
        for x0, y0, dx, dy in png.ADAM7:
            sub = samples[y0::dy, x0::dx]
            if sub.size:
                raw += _filter(_pack_rows(sub, depth), bpp, ftypes)
    body = png.SIGNATURE + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    if palette is not None:
        body += _chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        body += _chunk(b"tRNS", trns)
    return body + _chunk(b"IDAT", zlib.compress(raw)) + _chunk(b"IEND", b"")


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("ctype,depth", [(6, 8), (2, 8), (6, 16), (2, 16), (0, 1), (0, 2), (0, 4), (0, 8), (0, 16),
                                         (4, 8), (4, 16), (3, 1), (3, 2), (3, 4), (3, 8)])
def test_decode(ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth)
    h, w = 13, 11
    c = CHANNELS[ctype]
    hi = (1 << depth) - 1
    samples = rng.integers(0, hi + 1, (h, w, c))
    palette = None
    if ctype == 3:
        palette = rng.integers(0, 256, ((1 << depth), 3))
    got = png.decode(_write(samples, ctype, depth, palette, interlace=interlace))
    assert got.shape == (h, w, 4) and got.dtype == np.uint8
    if ctype == 3:
        want = np.concatenate([palette[samples[..., 0]], np.full((h, w, 1), 255)], -1)
    else:
        to8 = (lambda v: v >> 8) if depth == 16 else ((lambda v: v * 255 // hi) if depth < 8 else (lambda v: v))
        s8 = to8(samples)
        rgb = np.repeat(s8[..., :1], 3, -1) if ctype in (0, 4) else s8[..., :3]
        alpha = s8[..., -1:] if ctype in (4, 6) else np.full((h, w, 1), 255)
        want = np.concatenate([rgb, alpha], -1)
    assert np.array_equal(got, want.astype(np.uint8))


def test_transparency_chunks():
    rng = np.random.default_rng(1)
    idx = rng.integers(0, 4, (5, 6, 1))
    pal = rng.integers(0, 256, (4, 3))
    got = png.decode(_write(idx, 3, 8, pal, trns=bytes([0, 128])))
    assert np.array_equal(got[..., 3], np.array([0, 128, 255, 255])[idx[..., 0]])
    rgb = rng.integers(0, 3, (5, 6, 3))
    key = rgb[0, 0]
    got = png.decode(_write(rgb, 2, 8, trns=struct.pack(">HHH", *key)))
    assert np.array_equal(got[..., 3] == 0, (rgb == key).all(-1))


def test_errors():
    with pytest.raises(png.PngError):
        png.decode(b"GIF89a....")
    good = _write(np.zeros((4, 4, 3), np.int64), 2, 8)
    with pytest.raises(png.PngError):
        png.decode(good.replace(b"IHDR" + struct.pack(">II", 4, 4), b"IHDR" + struct.pack(">II", 4, 40)))
