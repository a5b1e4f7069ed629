"""PNG decoding for the glTF importer (the reference decodes with the `png` crate,
src/asset/gltf.rs:122-137, asking for 8-bit samples with an alpha channel).

Reads every standard PNG: colour types 0 (grey), 2 (RGB), 3 (palette, with tRNS alpha),
4 (grey + alpha) and 6 (RGBA); bit depths 1, 2, 4, 8 and 16; the five scanline filters;
Adam7 interlacing.  The result is always (height, width, 4) uint8 RGBA: 16-bit samples keep
their high byte, grey values below 8 bits scale to 0..255 (v * 255 / (2^depth - 1)), grey is
replicated to RGB, and alpha is 255 where the image has none (tRNS gives palette alpha and
the one transparent grey or RGB colour).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89PNG\r\n\x1a\n"
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


class PngError(ValueError):
    pass


def _unfilter(raw: memoryview, at: int, rows: int, stride: int, bpp: int) -> tuple[np.ndarray, int]:
    """Reverses the per-row filters of `rows` scanlines of `stride` bytes starting at `at`."""
    out = np.zeros((rows, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(rows):
        if at + 1 + stride > len(raw):
            raise PngError("image data is truncated")
        ftype = raw[at]
        line = np.frombuffer(raw[at + 1:at + 1 + stride], np.uint8).astype(np.int32)
        at += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 1:  # Sub: a running sum along each byte lane
            cur = line.copy()
            for k in range(min(bpp, stride)):
                cur[k::bpp] = np.cumsum(line[k::bpp]) & 0xFF
        elif ftype == 2:  # Up
            cur = (line + prev) & 0xFF
        elif ftype == 3:  # Average
            cur = line.copy()
            for i in range(stride):
                left = cur[i - bpp] if i >= bpp else 0
                cur[i] = (cur[i] + ((left + prev[i]) >> 1)) & 0xFF
        elif ftype == 4:  # Paeth
            cur = line.copy()
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (cur[i] + pred) & 0xFF
        else:
            raise PngError(f"unknown filter type {ftype}")
        out[y] = cur
        prev = cur
    return out, at


def _samples(rows: np.ndarray, width: int, depth: int, channels: int) -> np.ndarray:
    """Unpacked samples (rows, width, channels) as integers of the image's depth."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :width * channels].reshape(h, width, channels).astype(np.int32)
    if depth == 16:
        v = rows[:, :2 * width * channels].reshape(h, width * channels, 2).astype(np.int32)
        return ((v[..., 0] << 8) | v[..., 1]).reshape(h, width, channels)
    bits = np.unpackbits(rows, axis=1)  # depths 1, 2, 4: samples packed MSB first
    n = width * channels
    bits = bits[:, :n * depth].reshape(h, n, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.int32)
    return (bits.astype(np.int32) * weights).sum(-1).reshape(h, width, channels)


def _to_rgba8(s: np.ndarray, ctype: int, depth: int, palette, trns) -> np.ndarray:
    h, w = s.shape[:2]
    out = np.full((h, w, 4), 255, np.uint8)
    if ctype == 3:
        if palette is None:
            raise PngError("palette image without PLTE")
        idx = s[..., 0]
        if idx.max(initial=0) >= len(palette):
            raise PngError("palette index out of range")
        out[..., :3] = palette[idx]
        if trns is not None:
            alpha = np.full(len(palette), 255, np.uint8)
            alpha[:len(trns)] = np.frombuffer(trns, np.uint8)[:len(palette)]
            out[..., 3] = alpha[idx]
        return out

    def to8(v):
        if depth == 16:
            return (v >> 8).astype(np.uint8)
        if depth < 8:
            return (v * 255 // ((1 << depth) - 1)).astype(np.uint8)
        return v.astype(np.uint8)

    if ctype in (0, 4):
        g = to8(s[..., 0])
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if ctype == 4:
            out[..., 3] = to8(s[..., 1])
        elif trns is not None and len(trns) >= 2:
            key = struct.unpack(">H", trns[:2])[0]
            out[..., 3] = np.where(s[..., 0] == key, 0, 255)
    else:
        out[..., :3] = to8(s[..., :3])
        if ctype == 6:
            out[..., 3] = to8(s[..., 3])
        elif trns is not None and len(trns) >= 6:
            key = np.array(struct.unpack(">HHH", trns[:6]))
            out[..., 3] = np.where((s[..., :3] == key).all(-1), 0, 255)
    return out


def decode(data: bytes) -> np.ndarray:
    """(height, width, 4) uint8 RGBA of a PNG file's bytes."""
    if data[:8] != SIGNATURE:
        raise PngError("not a PNG file")
    at = 8
    ihdr = None
    palette = trns = None
    idat = []
    while at + 8 <= len(data):
        length, kind = struct.unpack(">I4s", data[at:at + 8])
        body = data[at + 8:at + 8 + length]
        at += 12 + length
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = bytes(body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if ihdr is None:
        raise PngError("missing IHDR")
    width, height, depth, ctype, _, _, interlace = ihdr
    if ctype not in CHANNELS or depth not in (1, 2, 4, 8, 16):
        raise PngError(f"unsupported colour type {ctype} / depth {depth}")
    channels = CHANNELS[ctype]
    bpp = max(1, channels * depth // 8)
    raw = memoryview(zlib.decompress(b"".join(idat)))
    if not interlace:
        stride = (width * channels * depth + 7) // 8
        rows, _ = _unfilter(raw, 0, height, stride, bpp)
        s = _samples(rows, width, depth, channels)
    else:
        s = np.zeros((height, width, channels), np.int32)
        pos = 0
        for x0, y0, dx, dy in ADAM7:
            pw = (width - x0 + dx - 1) // dx if width > x0 else 0
            ph = (height - y0 + dy - 1) // dy if height > y0 else 0
            if pw == 0 or ph == 0:
                continue
            stride = (pw * channels * depth + 7) // 8
            rows, pos = _unfilter(raw, pos, ph, stride, bpp)
            s[y0::dy, x0::dx] = _samples(rows, pw, depth, channels)
    return _to_rgba8(s, ctype, depth, palette, trns)
