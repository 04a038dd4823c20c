"""Headless image files of the path-tracer pass.

PNG: 8-bit RGBA (the R8G8B8A8_UNORM pixels of Context.tonemap), filter type
0, zlib stream from the standard library. PFM: linear float RGB, rows stored
bottom to top. Frames are arrays of shape (height, width, channels), top row
first.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"


def _chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def write_png(path: str, rgba) -> None:
    a = np.ascontiguousarray(rgba, np.uint8)
    h, w, c = a.shape
    if c != 4:
        raise ValueError("write_png takes (height, width, 4) uint8")
    raw = np.concatenate([np.zeros((h, 1), np.uint8), a.reshape(h, 4 * w)], 1).tobytes()
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(_SIG + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))


def read_png(path: str) -> np.ndarray:
    """8-bit RGBA, non-interlaced PNG with filter types 0..4 -> (h, w, 4) uint8."""
    data = open(path, "rb").read()
    if data[:8] != _SIG:
        raise ValueError(f"{path} is not a PNG file")
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise ValueError(f"bad CRC in chunk {kind!r}")
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body)
            if (depth, ctype, inter) != (8, 6, 0):
                raise ValueError("only 8-bit RGBA, non-interlaced")
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    out = np.zeros((h, 4 * w), np.int32)
    for y in range(h):
        ft, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        prev = out[y - 1] if y else np.zeros(4 * w, np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(4 * w, np.int32)
            for x in range(4 * w):
                left = cur[x - 4] if x >= 4 else 0
                up, ul = prev[x], (prev[x - 4] if x >= 4 else 0)
                if ft == 1:
                    pred = left
                elif ft == 3:
                    pred = (left + up) // 2
                else:
                    p = left + up - ul
                    pa, pb, pc = abs(p - left), abs(p - up), abs(p - ul)
                    pred = left if pa <= pb and pa <= pc else (up if pb <= pc else ul)
                cur[x] = (line[x] + pred) & 255
        out[y] = cur
    return out.astype(np.uint8).reshape(h, w, 4)


def write_pfm(path: str, rgb) -> None:
    a = np.ascontiguousarray(rgb, np.float32)
    h, w, _ = a.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(a[::-1]).astype("<f4").tobytes())


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        if f.readline().strip() != b"PF":
            raise ValueError(f"{path} is not a colour PFM file")
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        a = np.frombuffer(f.read(12 * w * h), "<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return np.ascontiguousarray(a[::-1]).astype(np.float32)
