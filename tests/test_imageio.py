"""Film and texture files (film_bitmap.cpp:156-274, texture_bitmap.cpp:49-66): row conventions,
the .png encoding (gamma 1/2.2, 8 bits, flipped), Radiance RGBE (flat and run-length scanlines)."""
import struct
import zlib

import numpy as np
import pytest


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


# ---------------------------------------------------------------------------------------------
# .png textures: a test-side encoder (ISO/IEC 15948) that applies every filter type, Adam7 and each
# colour type / bit depth; the decoder must give back the samples, reduced to 8 bits and made
# linear as stbi_loadf does ((v / 255)^2.2 for colour, v / 255 for alpha).

_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _pack(sub, depth):
    ph, pw, ch = sub.shape
    if depth == 8:
        return sub.astype(np.uint8).reshape(ph, pw * ch)
    if depth == 16:
        v = sub.astype(np.uint16).reshape(ph, pw * ch)
        return np.stack([v >> 8, v & 0xFF], axis=2).astype(np.uint8).reshape(ph, 2 * pw * ch)
    bits = ((sub.reshape(ph, pw * ch, 1) >> np.arange(depth - 1, -1, -1)) & 1).astype(np.uint8).reshape(ph, -1)
    return np.packbits(bits, axis=1)


def _filter_rows(rows, bpp, filters):
    out = []
    prior = np.zeros(rows.shape[1], np.int32)
    for y, r in enumerate(rows.astype(np.int32)):
        ft = filters[y % len(filters)]
        left = np.concatenate([np.zeros(bpp, np.int32), r[:-bpp]]) if r.size > bpp else np.zeros_like(r)
        ul = np.concatenate([np.zeros(bpp, np.int32), prior[:-bpp]]) if r.size > bpp else np.zeros_like(r)
        if ft == 0:
            f = r
        elif ft == 1:
            f = r - left
        elif ft == 2:
            f = r - prior
        elif ft == 3:
            f = r - (left + prior) // 2
        else:
            p = left + prior - ul
            pa, pb, pc = np.abs(p - left), np.abs(p - prior), np.abs(p - ul)
            f = r - np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prior, ul))
        out.append(bytes([ft]) + (f & 0xFF).astype(np.uint8).tobytes())
        prior = r
    return b"".join(out)


def _encode_png(path, samples, ctype, depth, interlace=False, filters=(0, 1, 2, 3, 4), plte=None, trns=None):
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    raw = b""
    for x0, y0, dx, dy in (_ADAM7 if interlace else ((0, 0, 1, 1),)):
        sub = samples[y0::dy, x0::dx]
        if sub.size:
            raw += _filter_rows(_pack(sub, depth), bpp, filters)

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    body = chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if plte is not None:
        body += chunk(b"PLTE", plte.astype(np.uint8).tobytes())
    if trns is not None:
        body += chunk(b"tRNS", trns)
    comp = zlib.compress(raw, 9)
    body += chunk(b"IDAT", comp[:len(comp) // 2]) + chunk(b"IDAT", comp[len(comp) // 2:])   # split IDAT
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + body + chunk(b"IEND", b""))


def _linear(px8):
    v = px8.astype(np.float64) / 255.0
    v[..., :3] = v[..., :3] ** 2.2
    return v.astype(np.float32)


@pytest.mark.parametrize("ctype,depth,interlace", [(2, 8, False), (2, 8, True), (6, 16, False), (6, 16, True), (0, 1, False),
                                                   (0, 2, True), (0, 4, False), (0, 16, True), (4, 8, True), (2, 16, False)])
def test_png_decoder_colour_types_filters_interlace(tmp_path, ctype, depth, interlace):
    from lightmetrica import imageio
    rng = np.random.default_rng(depth * 10 + ctype)
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    h, w = 11, 13
    samples = rng.integers(0, 1 << depth, (h, w, ch))
    p = str(tmp_path / f"t{ctype}_{depth}_{int(interlace)}.png")
    _encode_png(p, samples, ctype, depth, interlace)
    got = imageio.read_png(p, flip=False)
    s8 = samples >> 8 if depth == 16 else (samples * (255 // ((1 << depth) - 1)) if depth < 8 else samples)
    if ctype in (0, 4):
        s8 = np.concatenate([np.repeat(s8[..., :1], 3, axis=2), s8[..., 1:]], axis=2)
    assert got.shape == s8.shape
    assert np.array_equal(got, _linear(s8))
    assert np.array_equal(imageio.read_png(p), got[::-1])      # default: flipped, row 0 at the bottom


@pytest.mark.parametrize("depth", [1, 2, 4, 8])
def test_png_decoder_palette_and_transparency(tmp_path, depth):
    from lightmetrica import imageio
    rng = np.random.default_rng(depth)
    n = 1 << depth
    plte = rng.integers(0, 256, (n, 3))
    idx = rng.integers(0, n, (9, 10, 1))
    p = str(tmp_path / f"pal{depth}.png")
    _encode_png(p, idx, 3, depth, interlace=depth == 4, plte=plte)
    assert np.array_equal(imageio.read_png(p, flip=False), _linear(plte[idx[..., 0]]))
    alpha = rng.integers(0, 256, max(1, n // 2)).astype(np.uint8)   # shorter than the palette: the rest opaque
    _encode_png(p, idx, 3, depth, plte=plte, trns=alpha.tobytes())
    full = np.full(n, 255)
    full[:alpha.size] = alpha
    want = np.concatenate([plte[idx[..., 0]], full[idx[..., 0]][..., None]], axis=2)
    assert np.array_equal(imageio.read_png(p, flip=False), _linear(want))


def test_png_known_answer_paeth(tmp_path):
    """A 2 x 2 RGB image, both rows Paeth-filtered, bytes written out by hand."""
    from lightmetrica import imageio
    # pixels: row 0 (10,20,30) (40,50,60); row 1 (70,80,90) (100,110,120)
    # row 0: prior row 0, so Paeth predicts the left pixel: (10,20,30) (30,30,30)
    # row 1: first pixel predicts up (10,20,30) -> (60,60,60); second: a=(70,80,90), b=(40,50,60),
    # c=(10,20,30), p=a+b-c=(100,110,120), pa=|p-a|=30, pb=60, pc=90 -> a -> (30,30,30)
    rows = bytes([4, 10, 20, 30, 30, 30, 30, 4, 60, 60, 60, 30, 30, 30])

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    p = str(tmp_path / "ka.png")
    with open(p, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 2, 2, 8, 2, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(rows)) + chunk(b"IEND", b""))
    want = np.array([[[10, 20, 30], [40, 50, 60]], [[70, 80, 90], [100, 110, 120]]])
    assert np.array_equal(imageio.read_png(p, flip=False), _linear(want))


def test_png_film_round_trip_and_texture(tmp_path, lm):
    """write_png's film (gamma 1/2.2, top row first) read back as a texture: the quantised film,
    linear again, row 0 at the bottom; an env light loads it from envmap_path."""
    from lightmetrica import imageio
    img = _film(6, 8)
    p = str(tmp_path / "film.png")
    imageio.write_png(p, img)
    q = np.clip(np.floor(256.0 * np.power(img.astype(np.float64), 1 / 2.2)), 0, 255)
    tex = lm.load_texture("io_png", "bitmap", path=p)
    assert np.array_equal(tex.data, _linear(q))
    env = lm.load_light("io_env_png", "env", envmap_path=p)
    assert np.array_equal(env.data, tex.data)


def test_png_errors(tmp_path, lm):
    p = str(tmp_path / "bad.png")
    with open(p, "wb") as f:
        f.write(b"not a png at all")
    with pytest.raises(lm.LmGpuError):
        lm.load_texture("io_bad", "bitmap", path=p)
    _encode_png(p, np.zeros((2, 2, 3), np.int64), 2, 8)
    data = open(p, "rb").read()
    with open(p, "wb") as f:
        f.write(data[:-30])    # cut inside the image data
    with pytest.raises(lm.LmGpuError):
        lm.load_texture("io_cut", "bitmap", path=p)
