"""The oracle pinned to the reference's own texture, environment-light, OBJ and model code (CPU).

oracle/_ref/liblmref.so also compiles src/texture/texture_bitmap.cpp, src/light/light_env.cpp,
src/objloader/objloader{,_simple}.cpp, src/model/model_wavefrontobj.cpp (the model with its OBJ
mesh and material::mixture_wavefrontobj), src/material/material_proxy.cpp and
src/renderer/renderer_raycast.cpp unmodified.
stb_image, which texture_bitmap.cpp decodes image files with, is third-party and not among the
reference's sources: the library's stand-in takes images already decoded (oracle/ref.py
register_image), so these tests pin everything after the decode -- texel lookup with wrapping and
clamping, the vertical flip, alpha, the environment map's sampling distribution and its
direct/emission sampling, the OBJ parser, the model's material conversion and mesh grouping --
and the renderers over scenes made of them, bit for bit.
"""
import os
import struct
import zlib

import numpy as np
import pytest


def _same_bits(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return a.shape == b.shape and bool(((a == b) | (np.isnan(a) & np.isnan(b))).all())


def _bad_rows(a, b):
    return np.nonzero(~((a == b) | (np.isnan(a) & np.isnan(b))).all(1))[0][:5]


def _image(rng, h, w, c):
    t = rng.random((h, w, c)).astype(np.float32) * 2.0
    if c == 4:
        t[..., 3] = rng.choice([0.0, 0.25, 1.0], size=(h, w))
    return t


def _uv(rng, n=6000):
    uv = rng.uniform(-2.5, 3.5, (n, 2))
    edges = np.array([0.0, 1.0, -1.0, 0.5, 1 - 1e-16, -1e-300, 2.0, 0.999999])
    uv[: len(edges) ** 2] = np.stack(np.meshgrid(edges, edges), -1).reshape(-1, 2)
    return uv


@pytest.mark.parametrize("h,w,c", [(5, 7, 3), (3, 13, 4), (1, 1, 3), (16, 8, 4)])
@pytest.mark.parametrize("flip", [True, False])
def test_textures_match_reference(ref_mod, oracle_mod, h, w, c, flip):
    """texture_bitmap.cpp: eval and eval_alpha (coordinates wrapped to [0, 1), texel index
    clamped) and has_alpha, for RGB and RGBA images loaded flipped and unflipped."""
    rng = np.random.default_rng(h * 100 + w + c)
    img = _image(rng, h, w, c)                   # top row first, as the image file holds it
    path = f"pin_tex/{h}x{w}x{c}_{int(flip)}.img"
    ref_mod.register_image(path, img)
    S = ref_mod.RefScene()
    t = S.texture(path, flip=flip)
    O = oracle_mod.OracleScene(True)
    o = O.add_texture(img[::-1] if flip else img)  # the oracle takes row 0 at the bottom
    uv = _uv(rng)
    a = S.texture_query(t, uv)
    b = O.texture_query(o, uv)
    assert a[:, 4].min() == (1 if c == 4 else 0)
    assert _same_bits(a, b), f"rows {_bad_rows(a, b)}"


def _material_records(rng, n=20000):
    def unit(x):
        return x / np.linalg.norm(x, axis=1, keepdims=True)
    nn = unit(rng.normal(size=(n, 3)))
    rec = np.zeros((n, 26))
    rec[:, 0:3] = rng.normal(size=(n, 3))
    rec[:, 3:6] = nn
    rec[:, 6:9] = nn
    rec[:, 9:11] = rng.uniform(-1.5, 2.5, (n, 2))
    rec[:, 11:14] = unit(rng.normal(size=(n, 3)))
    rec[:, 14:17] = unit(rng.normal(size=(n, 3)))
    rec[: n // 10, 14:17] = -rec[: n // 10, 11:14]
    rec[:, 17] = rng.integers(0, 2, n)
    rec[:, 18] = rng.integers(0, 2, n)
    rec[:, 19] = rng.integers(0, 2, n)
    rec[:, 20:26] = rng.random((n, 6))
    return rec


@pytest.mark.parametrize("case", ["diffuse_rgb", "mixture_rgba_mask", "mixture_rgba_no_mask", "mixture_rgb",
                                  "mixture_plain"])
def test_textured_materials_match_reference(ref_mod, oracle_mod, case):
    """material_diffuse.cpp with mapKd, and model_wavefrontobj.cpp's
    material::mixture_wavefrontobj (a diffuse and a glossy lobe picked by the alpha of mapKd
    unless no_alpha_mask): every Material query, bit for bit."""
    rng = np.random.default_rng(len(case))
    c = 4 if "rgba" in case else 3
    img = _image(rng, 6, 9, c)
    path = f"pin_mat/{case}.img"
    ref_mod.register_image(path, img)
    S = ref_mod.RefScene()
    O = oracle_mod.OracleScene(True)
    Kd, Ks, ax, ay = [0.6, 0.5, 0.4], [0.7, 0.65, 0.5], 0.15, 0.4
    tex_r = S.texture(path) if case != "mixture_plain" else -1
    tex_o = O.add_texture(img[::-1]) if case != "mixture_plain" else -1
    if case == "diffuse_rgb":
        a_mat = S.material_tex("material::diffuse", Kd, tex_r)
        o_mat = O.add_material(oracle_mod.MAT["material::diffuse"], Kd)
        O.set_material_textures(o_mat, tex_o, -1)
    else:
        no_mask = case == "mixture_rgba_no_mask"
        a_mat = S.material_tex("material::mixture_wavefrontobj", Kd + Ks + [ax, ay, no_mask], tex_r)
        o_mat = O.add_material(oracle_mod.MAT["material::mixture_wavefrontobj"], Kd + Ks + [ax, ay])
        mask = tex_o if (c == 4 and not no_mask) else -1
        if tex_o >= 0:
            O.set_material_textures(o_mat, tex_o, mask)
    rec = _material_records(rng)
    a = S.material_query(a_mat, rec)
    b = O.material_query(o_mat, rec)
    assert _same_bits(a, b), f"rows {_bad_rows(a, b)}"
    if case == "mixture_rgba_mask":   # the alpha picks the lobe: both components occur
        assert 0 < a[:, 11].mean() < 1


def _env_image(rng, h=16, w=32):
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    img = 0.2 + 0.5 * (y / h) + 0.3 * rng.random((h, w)).astype(np.float32)
    img = np.stack([img, img * 0.9, img * 1.1], -1)
    img[3, 5] = [40.0, 35.0, 30.0]        # a sun a few texels wide
    img[3, 6] = [20.0, 18.0, 15.0]
    img[h - 1, :] = 0.0                   # a black row: zero-probability texels
    return img.astype(np.float32)


@pytest.mark.parametrize("rot,scale", [(0.0, 1.0), (37.5, 1.7), (-200.0, 0.5)])
def test_env_light_matches_reference(ref_mod, oracle_mod, rot, scale):
    """light_env.cpp: the luminance distribution over the map (Dist2 of max component x sin
    theta), sample_direct toward random shading points with its pdf_direct and eval, and
    sample_ray from the scene's bounding sphere, rotated and scaled, bit for bit."""
    from lightmetrica import synthetic as syn
    rng = np.random.default_rng(int(rot) + 500)
    img = _env_image(rng)
    path = f"pin_env/{rot}_{scale}.img"
    ref_mod.register_image(path, img)
    gp, _, gf = syn.ground_grid(4, 3.0)
    nrm1 = np.array([[0, 1, 0]], np.float32)
    S = ref_mod.RefScene()
    m0 = S.add_mesh_raw(gp, nrm1, gf.reshape(-1), np.zeros(gf.size, np.int32))
    S.add_child(0, S.primitive(m0))
    light = S.light_env(path, rot, scale)
    S.add_child(0, S.primitive(light=light))
    S.build()
    O = oracle_mod.OracleScene(True)
    mat = O.add_material(oracle_mod.MAT["material::diffuse"], [0.5, 0.5, 0.5])
    o0 = O.add_mesh(gp, nrm1, gf.reshape(-1), np.zeros(gf.size, np.int32))
    O.add_child(0, O.primitive(o0, mat, -1, -1))
    O.add_child(0, O.primitive(-1, -1, O.add_env(img[::-1], rot, scale), -1))
    O.build()
    n = 8000
    rec = np.zeros((n, 14))
    rec[:, 0:3] = rng.uniform(-3, 3, (n, 3))
    nn = rng.normal(size=(n, 3))
    nn /= np.linalg.norm(nn, axis=1, keepdims=True)
    rec[:, 3:6] = nn
    rec[:, 6:9] = nn
    rec[:, 9:14] = rng.random((n, 5))
    a = S.light_query(light, np.eye(4), rec)
    b = O.light_query(rec)
    assert a[:, 0].sum() > n // 2 and a[:, 20].sum() == n
    assert _same_bits(a, b), f"rows {_bad_rows(a, b)}"


# -- whole renders over env maps, textures and OBJ models -----------------------------------------

def _write_png_rgba(path, img_top_first_u8):
    """An 8-bit RGBA PNG (colour type 6, filter 0 on every row)."""
    h, w, _ = img_top_first_u8.shape
    raw = b"".join(b"\x00" + img_top_first_u8[r].tobytes() for r in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


# Coordinates are exact in float32: the reference parses them with atof into doubles, the GPU
# mirror keeps vertices in float32, and the two agree bit for bit only where that rounding is exact.
_OBJ = """# test scene
mtllib scene.mtl
v -2 0 -2
v 2 0 -2
v 2 0 2
v -2 0 2
vt 0 0
vt 2.5 0
vt 2.5 2.5
vt 0 2.5
vn 0 1 0
g ground
usemtl tex_alpha
f 1/1/1 4/4/1 3/3/1 2/2/1
v -0.625 0.0 -0.375
v 0.25 0.0 -0.375
v 0.25 0.75 -0.375
v -0.625 0.75 -0.375
v -0.625 0.0 0.375
v 0.25 0.0 0.375
v 0.25 0.75 0.375
v -0.625 0.75 0.375
g box
usemtl glossy
f 5 6 7
f 5 7 8
f 9 11 10
f 9 12 11
f 5 9 10
f 5 10 6
f 8 7 11
f 8 11 12
f 5 8 12
f 5 12 9
f 6 10 11
f 6 11 7
v 0.625 0.125 0.625
v 1.25 0.125 0.625
v 0.875 0.75 0.875
vt 0.125 0.125
vt 0.875 0.125
vt 0.5 0.875
g glass
usemtl glass
f -3/-3 -2/-2 -1/-1
v 1.0 0.0 -1.0
v 1.625 0.0 -1.0
v 1.625 0.875 -1.25
g mirror
usemtl mirror
f 16 17 18
v -0.5 2.25 -0.5
v 0.5 2.25 -0.5
v 0.5 2.25 0.5
v -0.5 2.25 0.5
vn 0 -1 0
g light
usemtl emitter
f 19//2 20//2 21//2 22//2
"""

_MTL = """newmtl tex_alpha
illum 2
Kd 0.8 0.8 0.8
Ks 0.3 0.3 0.3
Ns 40
map_Kd tex.png

newmtl glossy
illum 2
Kd 0.2 0.3 0.5
Ks 0.6 0.5 0.4
Ns 200
aniso 0.5

newmtl glass
illum 7
Ni 1.45

newmtl mirror
illum 5

newmtl emitter
illum 2
Kd 0 0 0
Ke 6 5 4
"""


def _obj_scenes(lm, ref_mod, tmp_path, prefix, env):
    rng = np.random.default_rng(3)
    tex = (rng.random((6, 8, 4)) * 255).astype(np.uint8)
    tex[..., 3] = np.where(rng.random((6, 8)) < 0.3, 0, 255)
    _write_png_rgba(os.path.join(tmp_path, "tex.png"), tex)
    with open(os.path.join(tmp_path, "scene.obj"), "w") as f:
        f.write(_OBJ)
    with open(os.path.join(tmp_path, "scene.mtl"), "w") as f:
        f.write(_MTL)
    obj = os.path.join(tmp_path, "scene.obj")
    w, h = 24, 18
    cam = dict(position=[0.3, 1.6, 4.2], center=[0.2, 0.4, 0.0], up=[0, 1, 0], vfov=45.0, aspect=w / h)
    env_img = _env_image(np.random.default_rng(8)) if env else None

    # the GPU mirror's scene: camera, the model (one group node each, as lm::primitive makes them)
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", "sahbvh"))
    scene.add_primitive(camera=lm.load_camera(prefix + "camera", "pinhole", **cam))
    scene.add_primitive(model=lm.load_model(prefix + "model", "wavefrontobj", path=obj))
    if env:
        scene.add_primitive(light=lm.load_light(prefix + "env", "env", envmap=env_img[::-1], rot=25.0, scale=0.8))

    # the reference's: the same nodes, the model read and converted by its own loader
    from lightmetrica import imageio
    ref_mod.register_image(os.path.join(tmp_path, "tex.png"), imageio.read_png(os.path.join(tmp_path, "tex.png"),
                                                                                 flip=False))
    S = ref_mod.RefScene()
    g = S.group()
    S.add_child(g, S.primitive(camera=S.camera(cam["position"], cam["center"], cam["up"], cam["vfov"], cam["aspect"])))
    S.add_child(0, g)
    model = S.model(obj)
    g = S.group()
    assert S.add_child_from_model(g, model) == 5
    S.add_child(0, g)
    if env:
        path = os.path.join(tmp_path, "env.img")
        ref_mod.register_image(path, env_img)
        g = S.group()
        S.add_child(g, S.primitive(light=S.light_env(path, 25.0, 0.8)))
        S.add_child(0, g)
    f = S.film(w, h)
    S.build()
    return scene, S, f, w, h


@pytest.mark.parametrize("env", [False, True])
@pytest.mark.parametrize("sampling_mode", ["naive", "mis"])
def test_obj_model_pt_matches_reference(ref_mod, oracle_mod, lm, tmp_path, env, sampling_mode):
    """An OBJ scene read by the reference's objloader::simple and model::wavefrontobj (polygon
    fans, negative and position-only indices, faces without normals, the MTL's illum / Ns /
    aniso / Ke / map_Kd conversions, an RGBA texture's alpha mask, an area light from Ke) and
    rendered by its renderer::pt, with and without an environment map, against the restatement
    over the same file as the GPU mirror's objloader reads it, every pixel bit for bit."""
    scene, S, f, w, h = _obj_scenes(lm, ref_mod, str(tmp_path), f"objpin_{env}_{sampling_mode}_", env)
    a = S.render_pt(f, 4, 7, seed=3, sampling_mode=sampling_mode)
    O = oracle_mod.from_lm_scene(scene, double=True)
    O.build()
    b, _, _, _ = O.render_pt(w, h, 4, 7, seed=3, sampling_mode=sampling_mode, rng="mt19937", nthreads=1)
    assert np.nansum(a) > 0
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))).all(axis=2))
    assert bad.size == 0, f"{len(bad)} pixels differ, first {bad[:4].tolist()}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"


@pytest.mark.parametrize("key", ["renderer::lt", "renderer::bdpt"])
def test_obj_model_light_tracing_matches_reference(ref_mod, oracle_mod, lm, tmp_path, key):
    """renderer::lt and renderer::bdpt over the OBJ scene with its environment map, bit for bit."""
    scene, S, f, w, h = _obj_scenes(lm, ref_mod, str(tmp_path), f"objpin_{key.split('::')[1]}_", True)
    n = 3 * w * h
    a = S.render_spi(key, f, n, 6, seed=4)
    O = oracle_mod.from_lm_scene(scene, double=True)
    O.build()
    if key == "renderer::lt":
        b, _, _ = O.render_lt(w, h, n, 6, seed=4, rng="mt19937", nthreads=1)
    else:
        b, _, _ = O.render_bdpt(w, h, n, 6, seed=4, rng="mt19937", nthreads=1, mode="bdpt")
    assert np.nansum(a) > 0
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))).all(axis=2))
    assert bad.size == 0, f"{len(bad)} pixels differ, first {bad[:4].tolist()}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"


def test_textured_env_scene_from_lm_scene_matches_reference(ref_mod, oracle_mod, lm):
    """from_lm_scene's own mapping of textured diffuse and mixture materials, a proxy and an
    environment map (the spheres scene with its constant environment replaced), rendered by the
    reference's renderer::pt and the restatement, bit for bit."""
    from lightmetrica import synthetic as syn
    p = "pin_texenv_"
    scene, film, _ = syn.spheres_scene(n_spheres=5, subdiv=3, ground_quads=8, w=20, h=12, prefix=p)
    rng = np.random.default_rng(9)
    env = _env_image(rng)
    for n in scene.nodes:
        if n["type"] == "primitive" and n["light"] is not None and n["light"].key_name == "light::envconst":
            n["light"] = lm.load_light(p + "env", "env", envmap=env[::-1], rot=-60.0, scale=1.3)
    tex_rgb = lm.load_texture(p + "t3", "bitmap", data=_image(rng, 4, 5, 3))
    tex_rgba = lm.load_texture(p + "t4", "bitmap", data=_image(rng, 5, 4, 4))
    prims = [n for n in scene.nodes if n["type"] == "primitive" and n["mesh"] is not None and n["light"] is None]
    prims[0]["material"] = lm.load_material(p + "d", "diffuse", Kd=[0.5, 0.5, 0.5], mapKd=tex_rgb)
    mix = lm.load_material(p + "mx", "mixture_wavefrontobj", Kd=[0.4, 0.5, 0.6], Ks=[0.5, 0.5, 0.5], ax=0.2, ay=0.3,
                           mapKd=tex_rgba, no_alpha_mask=False)
    prims[1]["material"] = mix
    prims[2]["material"] = lm.load_material(p + "px", "proxy", ref=mix)
    S = ref_mod.from_lm_scene(scene)
    f = S.film(film.w, film.h)
    S.build()
    a = S.render_pt(f, 3, 6, seed=2, sampling_mode="mis")
    O = oracle_mod.from_lm_scene(scene, double=True)
    O.build()
    b, _, _, _ = O.render_pt(film.w, film.h, 3, 6, seed=2, sampling_mode="mis", rng="mt19937", nthreads=1)
    assert np.nansum(a) > 0
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))).all(axis=2))
    assert bad.size == 0, f"{len(bad)} pixels differ, first {bad[:4].tolist()}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"


@pytest.mark.parametrize("which", ["box", "spheres_env"])
@pytest.mark.parametrize("mode", ["shaded", "normal", "constant", "color"])
def test_raycast_images_match_reference_renderer(ref_mod, oracle_mod, lm, which, mode):
    """renderer_raycast.cpp (primary rays at pixel centres, reflectance times 0.2 + 0.8 |n . d|, the
    environment's radiance where a ray escapes, the background where nothing is hit): its
    shaded, normal-visualising, constant-colour and colour-override images against the
    restatement's, every pixel bit for bit; the spheres carry a textured diffuse and a mixture
    material under an env map."""
    from lightmetrica import synthetic as syn
    p = f"pin_rc_{which}_{mode}_"
    if which == "box":
        scene, film = syn.box_scene(w=32, h=24, prefix=p)
    else:
        scene, film, _ = syn.spheres_scene(n_spheres=5, subdiv=3, ground_quads=8, w=30, h=18, prefix=p)
        rng = np.random.default_rng(4)
        for n in scene.nodes:
            if n["type"] == "primitive" and n["light"] is not None and n["light"].key_name == "light::envconst":
                n["light"] = lm.load_light(p + "env", "env", envmap=_env_image(rng)[::-1], rot=15.0, scale=1.2)
        prims = [n for n in scene.nodes if n["type"] == "primitive" and n["mesh"] is not None and n["light"] is None]
        prims[0]["material"] = lm.load_material(p + "d", "diffuse", Kd=[0.5, 0.5, 0.5],
                                                 mapKd=lm.load_texture(p + "t", "bitmap", data=_image(rng, 4, 5, 3)))
        prims[1]["material"] = lm.load_material(p + "mx", "mixture_wavefrontobj", Kd=[0.4, 0.5, 0.6], Ks=[0.5, 0.5, 0.5],
                                                ax=0.2, ay=0.3, mapKd="", no_alpha_mask=False)
    kw = {"shaded": {}, "normal": {"visualize_normal": True}, "constant": {"use_constant_color": True},
          "color": {"color": (0.25, 0.5, 0.75)}}[mode]
    bg = (0.1, 0.2, 0.3)
    S = ref_mod.from_lm_scene(scene)
    f = S.film(film.w, film.h)
    S.build()
    a = S.render_raycast(f, bg=bg, **kw)
    O = oracle_mod.from_lm_scene(scene, double=True)
    O.build()
    b, _ = O.render_raycast(film.w, film.h, bg=bg, nthreads=1, **kw)
    assert np.abs(a).sum() > 0
    assert _same_bits(a, b), f"{int((a != b).any(axis=2).sum())} pixels differ"
