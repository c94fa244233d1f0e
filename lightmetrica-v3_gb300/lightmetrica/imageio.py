"""Image files for film::bitmap and texture::bitmap, with the reference's conventions
(src/film/film_bitmap.cpp:156-274, src/texture/texture_bitmap.cpp:49-66).

* Films keep row 0 at the bottom. .png and .hdr are written top row first (the film flipped),
  .pfm bottom row first (unflipped, as the PFM convention is). .png stores
  clamp(int(256 * v^(1/2.2)), 0, 255) per channel.
* .hdr is Radiance RGBE (Ward, "Real pixels", Graphics Gems II): a shared exponent e with
  v = m * 2^(e - 136). Written as flat scanlines; read flat or with the per-channel run-length
  encoding of newer writers.
* Textures load with row 0 at the bottom (the reference flips on load by default), so an .hdr
  read here is flipped; a .pfm already stores its bottom row first.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


def _parent(path: str) -> None:
    d = os.path.dirname(path)
    if d and not os.path.exists(d):
        os.makedirs(d, exist_ok=True)


def write_pfm(path: str, img: np.ndarray) -> None:
    """img: (h, w, 3) with row 0 at the bottom."""
    _parent(path)
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1\n".encode())
        f.write(np.ascontiguousarray(img[..., :3], dtype="<f4").tobytes())


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        kind = f.readline().strip()
        w, h = map(int, f.readline().split())
        s = float(f.readline())
        ch = 3 if kind == b"PF" else 1
        data = np.frombuffer(f.read(), dtype="<f4" if s < 0 else ">f4")[:w * h * ch].reshape(h, w, ch).astype(np.float32)
    return np.ascontiguousarray(np.repeat(data, 3, axis=2) if ch == 1 else data)


def write_png(path: str, img: np.ndarray) -> None:
    """8-bit RGB PNG of a film (row 0 at the bottom), gamma 1/2.2."""
    _parent(path)
    h, w = img.shape[:2]
    with np.errstate(invalid="ignore"):
        t = np.power(np.asarray(img[..., :3], np.float64), 1.0 / 2.2) * 256.0
    t = np.nan_to_num(t, nan=0.0, posinf=255.0, neginf=0.0)
    px = np.clip(np.floor(t), 0, 255).astype(np.uint8)[::-1]
    raw = b"".join(b"\x00" + px[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def _to_rgbe(img: np.ndarray) -> np.ndarray:
    v = np.maximum(np.asarray(img[..., :3], np.float64), 0.0)
    m = v.max(axis=-1)
    mant, e = np.frexp(m)
    out = np.zeros(v.shape[:-1] + (4,), np.uint8)
    ok = m >= 1e-32
    scale = np.where(ok, mant * 256.0 / np.where(ok, m, 1.0), 0.0)
    out[..., :3] = np.clip(np.floor(v * scale[..., None]), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(ok, e + 128, 0).astype(np.uint8)
    return out


def write_hdr(path: str, img: np.ndarray) -> None:
    """Radiance .hdr of a film (row 0 at the bottom), top row first."""
    _parent(path)
    h, w = img.shape[:2]
    rgbe = _to_rgbe(img)[::-1]
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n")
        f.write(f"-Y {h} +X {w}\n".encode())
        f.write(np.ascontiguousarray(rgbe).tobytes())


def read_hdr(path: str, flip: bool = True) -> np.ndarray:
    """(h, w, 3) float32 from a Radiance .hdr; flip=True puts the file's last row at row 0."""
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    header = []
    while True:
        end = data.index(b"\n", pos)
        line = data[pos:end]
        pos = end + 1
        if line.strip() == b"" and header:
            break
        header.append(line)
    if not header or not header[0].startswith(b"#?"):
        raise ValueError("not a Radiance .hdr file")
    end = data.index(b"\n", pos)
    res = data[pos:end].split()
    pos = end + 1
    if len(res) != 4 or res[0] != b"-Y" or res[2] != b"+X":
        raise ValueError("unsupported .hdr orientation (only -Y h +X w)")
    h, w = int(res[1]), int(res[3])
    buf = np.frombuffer(data, np.uint8, offset=pos)
    out = np.zeros((h, w, 4), np.uint8)
    p = 0
    for y in range(h):
        if 8 <= w < 32768 and p + 4 <= buf.size and buf[p] == 2 and buf[p + 1] == 2 and (int(buf[p + 2]) << 8 | int(buf[p + 3])) == w:
            p += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = int(buf[p])
                    p += 1
                    if n > 128:
                        n -= 128
                        out[y, x:x + n, c] = buf[p]
                        p += 1
                    else:
                        out[y, x:x + n, c] = buf[p:p + n]
                        p += n
                    x += n
        else:
            out[y] = buf[p:p + 4 * w].reshape(w, 4)
            p += 4 * w
    e = out[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)
    img = (out[..., :3].astype(np.float64) * f[..., None]).astype(np.float32)
    return np.ascontiguousarray(img[::-1] if flip else img)
