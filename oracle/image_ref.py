"""CPU restatement of the image-output step (test infrastructure only).

Tonemap: RTCamp8/Main.cpp:669-682 (v -> clamp((int)(pow(v * 0.3, 1 / 2.2) * 255),
0, 255) per channel). Error map: VisualizeError/Main.cpp:64-82 (squared
luminance difference over a maximum, rgbToLuminance weights of Vector.h:828-830,
Jet colormap of tinycolormap: clamp(1.5 - 4 |t - m|, 0, 1), m = 0.75 / 0.5 /
0.25 for r / g / b). FP32 arithmetic as in the reference; a NaN maps to 0.
Also a minimal PNG reader (stored or compressed IDAT, filter type 0 rows) for
checking written files.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _to_byte(v):
    v = np.asarray(v, np.float32)
    s = v * np.float32(255.0)
    out = np.where(np.isnan(s), 0, np.clip(np.trunc(np.nan_to_num(s, nan=0.0)), 0, 255))
    return out.astype(np.uint8)


def tonemap(film_sum, scale=1.0, exposure=0.3, gamma=2.2):
    v = np.asarray(film_sum, np.float32) * np.float32(scale)
    with np.errstate(invalid="ignore"):
        t = np.power(v * np.float32(exposure), np.float32(1.0) / np.float32(gamma), dtype=np.float32)
    return _to_byte(t)


def luminance(rgb):
    rgb = np.asarray(rgb, np.float32)
    return (np.float32(0.298912) * rgb[..., 0] + np.float32(0.586611) * rgb[..., 1]) + np.float32(0.114478) * rgb[..., 2]


def error_map(a, scale_a, b, scale_b, max_value):
    la = luminance(np.asarray(a, np.float32) * np.float32(scale_a))
    lb = luminance(np.asarray(b, np.float32) * np.float32(scale_b))
    d = np.abs(la - lb)
    t = np.clip(d * d * (np.float32(1.0) / np.float32(max_value)), 0, 1).astype(np.float32)
    out = np.empty(t.shape + (3,), np.uint8)
    for c, m in enumerate((0.75, 0.5, 0.25)):
        out[..., c] = _to_byte(np.clip(np.float32(1.5) - np.float32(4.0) * np.abs(t - np.float32(m)), 0, 1))
    return out


def read_png(path):
    """RGB8 PNG -> uint8 [H, W, 3]; checks the signature and every chunk CRC."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    w = h = None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == crc, typ
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 2
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 3 * w + 1)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3).copy()
