"""Film and texture files (film_bitmap.cpp:156-274, texture_bitmap.cpp:49-66): row conventions,
the .png encoding (gamma 1/2.2, 8 bits, flipped), Radiance RGBE (flat and run-length scanlines)."""
import struct
import zlib

import numpy as np


def _film(h=5, w=9, seed=1):
    rng = np.random.default_rng(seed)
    img = rng.lognormal(-1.0, 1.2, (h, w, 3)).astype(np.float32)
    img[0, 0] = [0, 0, 0]
    return img


def test_pfm_round_trip(tmp_path):
    from lightmetrica import imageio
    img = _film()
    p = str(tmp_path / "sub" / "a.pfm")   # the directory is created
    imageio.write_pfm(p, img)
    assert np.array_equal(imageio.read_pfm(p), img)
    raw = open(p, "rb").read()
    assert raw.startswith(b"PF\n9 5\n-1\n")
    # bottom row (film row 0) first, unflipped
    assert np.array_equal(np.frombuffer(raw[len(b"PF\n9 5\n-1\n"):][:12], "<f4"), img[0, 0])


def test_hdr_round_trip_and_flip(tmp_path):
    from lightmetrica import imageio
    img = _film()
    p = str(tmp_path / "a.hdr")
    imageio.write_hdr(p, img)
    back = imageio.read_hdr(p)                      # flipped back: row 0 at the bottom
    m = img.max(axis=2, keepdims=True)
    assert np.all(np.abs(back - img) <= m / 128 + 1e-30)
    top_first = imageio.read_hdr(p, flip=False)
    assert np.array_equal(top_first, back[::-1])
    assert open(p, "rb").read().startswith(b"#?RADIANCE")


def test_hdr_reads_run_length_scanlines(tmp_path):
    from lightmetrica import imageio
    w = 10
    # one scanline, RLE: per channel a run of 10 (R=128, G=64), literals (B), a run (E=129)
    line = bytes([2, 2, 0, w])
    line += bytes([128 + 10, 128])
    line += bytes([128 + 10, 64])
    line += bytes([10]) + bytes(range(10))
    line += bytes([128 + 10, 129])
    p = tmp_path / "r.hdr"
    p.write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X 10\n" + line)
    img = imageio.read_hdr(str(p))
    f = 2.0 ** (129 - 136)
    assert img.shape == (1, 10, 3)
    assert np.allclose(img[0, :, 0], 128 * f) and np.allclose(img[0, :, 1], 64 * f)
    assert np.allclose(img[0, :, 2], np.arange(10) * f)


def test_png_encoding(tmp_path):
    from lightmetrica import imageio
    img = _film(3, 4)
    p = str(tmp_path / "a.png")
    imageio.write_png(p, img)
    raw = open(p, "rb").read()
    assert raw[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(raw):
        n = struct.unpack(">I", raw[pos:pos + 4])[0]
        tag = raw[pos + 4:pos + 8]
        body = raw[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", raw[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(tag + body) & 0xFFFFFFFF
        chunks[tag] = chunks.get(tag, b"") + body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (w, h, depth, ctype) == (4, 3, 8, 2)
    rows = zlib.decompress(chunks[b"IDAT"])
    px = np.frombuffer(rows, np.uint8).reshape(3, 1 + 4 * 3)
    assert (px[:, 0] == 0).all()
    got = px[:, 1:].reshape(3, 4, 3)
    want = np.clip(np.floor(256.0 * np.power(img.astype(np.float64), 1 / 2.2)), 0, 255).astype(np.uint8)[::-1]
    assert np.array_equal(got, want)


def test_texture_loads_hdr_bottom_row_first(tmp_path, lm):
    from lightmetrica import imageio
    img = _film(4, 6)
    p = str(tmp_path / "env.hdr")
    imageio.write_hdr(p, img)
    tex = lm.load_texture("io_tex", "bitmap", path=p)
    assert tex.data.shape == (4, 6, 3)
    assert np.all(np.abs(tex.data - img) <= img.max(axis=2, keepdims=True) / 128 + 1e-30)
