"""A small PNG writer for test fixtures: every colour type, bit depth, filter
type, tRNS form and Adam7 interlacing (W3C PNG specification), so that the
decoder is exercised on files that common encoders do not produce.  Python's
zlib does the compression."""
from __future__ import annotations

import struct
import zlib

import numpy as np

CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def pack_row(samples: np.ndarray, depth: int) -> bytes:
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    bits = "".join(format(int(v), f"0{depth}b") for v in samples)
    bits += "0" * (-len(bits) % 8)
    return bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def filter_rows(rows: list[bytes], bpp: int, filters: list[int]) -> bytes:
    out = b""
    prev = bytes(len(rows[0])) if rows else b""
    for i, row in enumerate(rows):
        f = filters[i % len(filters)]
        enc = bytearray(len(row))
        for k in range(len(row)):
            a = row[k - bpp] if k >= bpp else 0
            b = prev[k]
            c = prev[k - bpp] if k >= bpp else 0
            pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[f]
            enc[k] = (row[k] - pred) & 255
        out += bytes([f]) + bytes(enc)
        prev = row
    return out


def make_png(samples: np.ndarray, depth: int, color: int, palette: bytes | None = None, trns: bytes | None = None,
             interlace: int = 0, filters=(0, 1, 2, 3, 4)) -> bytes:
    """samples: (H, W) or (H, W, channels) integer array of raw sample values."""
    h, w = samples.shape[:2]
    ch = CHANNELS[color]
    s = samples.reshape(h, w, ch)
    bpp = max(1, ch * depth // 8)
    if interlace:
        data = b""
        for x0, y0, dx, dy in ADAM7:
            sub = s[y0::dy, x0::dx]
            if sub.size == 0:
                continue
            data += filter_rows([pack_row(sub[j].reshape(-1), depth) for j in range(sub.shape[0])], bpp, list(filters))
    else:
        data = filter_rows([pack_row(s[j].reshape(-1), depth) for j in range(h)], bpp, list(filters))
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, interlace))
    if palette is not None:
        out += chunk(b"PLTE", palette)
    if trns is not None:
        out += chunk(b"tRNS", trns)
    out += chunk(b"tEXt", b"Comment\x00fixture")
    z = zlib.compress(data, 6)
    return out + chunk(b"IDAT", z[:len(z) // 2]) + chunk(b"IDAT", z[len(z) // 2:]) + chunk(b"IEND", b"")
