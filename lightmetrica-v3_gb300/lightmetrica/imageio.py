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
* .png textures (texture_bitmap.cpp:56-58 loads every format through stb_image's stbi_loadf):
  decoded per the PNG specification (ISO/IEC 15948: zlib stream of filtered scanlines, filter
  types 0-4, Adam7 interlacing, bit depths 1-16, gray / RGB / palette / alpha), 16-bit samples
  reduced to their high byte and sub-byte gray scaled to 0-255 as stb_image does, then turned
  into linear floats the way stbi_loadf converts any 8-bit image: colour channels
  (v / 255)^2.2, alpha v / 255.
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


# ---------------------------------------------------------------------------------------------
# PNG decoding (ISO/IEC 15948)

_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _unfilter(data: bytes, pos: int, w: int, h: int, bpp: int, row_bytes: int) -> tuple[np.ndarray, int]:
    """Reverses the per-scanline filters of one (sub-)image: returns (h, row_bytes) uint8 and the
    position after it. bpp: bytes per complete pixel (at least 1)."""
    out = np.zeros((h, row_bytes), np.uint8)
    prev = np.zeros(row_bytes, np.int32)
    for y in range(h):
        if pos + 1 + row_bytes > len(data):
            raise ValueError("truncated PNG image data")
        ft = data[pos]
        raw = np.frombuffer(data, np.uint8, row_bytes, pos + 1).astype(np.int32)
        pos += 1 + row_bytes
        if ft == 0:
            cur = raw
        elif ft == 1:    # Sub: each byte adds the byte bpp to its left (a running sum per lane)
            pad = (-row_bytes) % bpp
            lanes = np.concatenate([raw, np.zeros(pad, np.int32)]).reshape(-1, bpp)
            cur = (np.cumsum(lanes, axis=0) & 0xFF).reshape(-1)[:row_bytes]
        elif ft == 2:    # Up
            cur = (raw + prev) & 0xFF
        elif ft in (3, 4):
            r = raw.tolist()
            up = prev.tolist()
            c = [0] * row_bytes
            for i in range(row_bytes):
                a = c[i - bpp] if i >= bpp else 0
                b = up[i]
                if ft == 3:  # Average
                    c[i] = (r[i] + ((a + b) >> 1)) & 0xFF
                else:        # Paeth
                    cc = up[i - bpp] if i >= bpp else 0
                    p = a + b - cc
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - cc)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else cc)
                    c[i] = (r[i] + pr) & 0xFF
            cur = np.asarray(c, np.int32)
        else:
            raise ValueError(f"bad PNG filter type {ft}")
        out[y] = cur
        prev = cur
    return out, pos


def _samples(rows: np.ndarray, w: int, channels: int, depth: int) -> np.ndarray:
    """Unfiltered scanlines -> (h, w, channels) integer samples at the file's bit depth."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :w * channels].reshape(h, w, channels).astype(np.int32)
    if depth == 16:
        v = rows[:, :2 * w * channels].reshape(h, w * channels, 2).astype(np.int32)
        return (v[..., 0] << 8 | v[..., 1]).reshape(h, w, channels)
    bits = np.unpackbits(rows, axis=1)[:, :w * depth].reshape(h, w, depth)
    weights = 1 << np.arange(depth - 1, -1, -1)
    return (bits.astype(np.int32) * weights).sum(axis=2).reshape(h, w, 1)


def read_png(path: str, flip: bool = True) -> np.ndarray:
    """(h, w, c) float32 from a PNG as stbi_loadf returns it (c = 3 or 4; gray is widened to RGB);
    flip=True puts the file's last row at row 0."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos = 8
    ihdr = None
    plte = None
    trns = None
    idat = []
    while pos + 8 <= len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if len(body) != n:
            raise ValueError("truncated PNG chunk")
        pos += 12 + n
        if tag == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3).astype(np.int32)
        elif tag == b"tRNS":
            trns = body
        elif tag == b"IDAT":
            idat.append(body)
        elif tag == b"IEND":
            break
    if ihdr is None or not idat:
        raise ValueError("PNG without IHDR or IDAT")
    w, h, depth, ctype, comp, filt, interlace = ihdr
    if ctype not in _CHANNELS or comp != 0 or filt != 0 or interlace not in (0, 1) or w == 0 or h == 0:
        raise ValueError(f"unsupported PNG (colour type {ctype}, interlace {interlace})")
    if depth not in ((1, 2, 4, 8, 16) if ctype == 0 else (1, 2, 4, 8) if ctype == 3 else (8, 16)):
        raise ValueError(f"bad PNG bit depth {depth} for colour type {ctype}")
    if ctype == 3 and plte is None:
        raise ValueError("palette PNG without PLTE")
    ch = _CHANNELS[ctype]
    raw = zlib.decompress(b"".join(idat))
    bpp = max(1, ch * depth // 8)
    samples = np.zeros((h, w, ch), np.int32)
    p = 0
    passes = _ADAM7 if interlace else ((0, 0, 1, 1),)
    for x0, y0, dx, dy in passes:
        pw, ph = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
        if pw <= 0 or ph <= 0:
            continue
        rows, p = _unfilter(raw, p, pw, ph, bpp, (pw * ch * depth + 7) // 8)
        samples[y0::dy, x0::dx] = _samples(rows, pw, ch, depth)
    # to 8 bits as stb_image does: 16-bit -> high byte, sub-byte gray scaled (palette indices not)
    if depth == 16:
        samples = samples >> 8
    elif depth < 8 and ctype == 0:
        samples = samples * (255 // ((1 << depth) - 1))
    if ctype == 3:
        idx = np.clip(samples[..., 0], 0, plte.shape[0] - 1)
        rgb = plte[idx]
        alpha = None
        if trns is not None:
            ta = np.full(plte.shape[0], 255, np.int32)
            t = np.frombuffer(trns, np.uint8)[:plte.shape[0]]
            ta[:t.size] = t
            alpha = ta[idx][..., None]
        px = rgb if alpha is None else np.concatenate([rgb, alpha], axis=2)
    elif ctype in (0, 4):
        px = np.concatenate([np.repeat(samples[..., :1], 3, axis=2), samples[..., 1:]], axis=2)
    else:
        px = samples
    v = px.astype(np.float64) / 255.0
    v[..., :3] = np.power(v[..., :3], 2.2)
    img = v.astype(np.float32)
    return np.ascontiguousarray(img[::-1] if flip else img)
