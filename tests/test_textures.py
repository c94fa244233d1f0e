"""Image textures: texture::bitmap as material::diffuse's mapKd (material_diffuse.cpp:36-40, 70-88),
as material::mixture_wavefrontobj's mapKd and alpha mask (model_wavefrontobj.cpp:361-517), and
OBJ map_Kd (model_wavefrontobj.cpp:133-214). Lookup: the nearest texel of the wrapped texture
coordinate, row 0 at the bottom (texture_bitmap.cpp:68-85); coordinates are interpolated with
mix_barycentric (mesh_raw.cpp:97).

CPU: the oracle's lookup and orientation on a textured quad seen head-on (raycast colors are the
texels), and the alpha mask's component rules. GPU: raycast and path-traced images against the
oracle (matched random streams), an OBJ whose MTL names a PNG with an alpha channel, and the
renderers that do not take image textures refusing them."""
import os
import struct
import zlib

import numpy as np
import pytest

CHECKER = np.array([[[0.9, 0.1, 0.1], [0.1, 0.9, 0.1]],
                    [[0.1, 0.1, 0.9], [0.8, 0.8, 0.2]]], np.float32)  # row 0 = bottom


def _quad_scene(lm, tex_data, material="diffuse", prefix="tq_", w=32, h=32, env=0.5, extra_light=True, quad_on=True):
    """A unit quad [-1, 1]^2 at z = 0 facing +z, texture coordinates (0, 0) .. (1, 1), seen head-on
    by a pinhole camera, under a constant environment; behind it (z = -1) a grey back wall."""
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    cam = lm.load_camera(prefix + "cam", "pinhole", position=[0, 0, 4], center=[0, 0, 0], up=[0, 1, 0], vfov=30,
                         aspect=w / h)
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", "sahbvh"))
    scene.add_primitive(camera=cam)
    tex = lm.load_texture(prefix + "tex", "bitmap", data=tex_data)
    ps = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    ts = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    f = np.array([0, 1, 2, 0, 2, 3], np.int32)
    quad = lm.load_mesh(prefix + "quad", "raw", ps=ps, ns=[[0, 0, 1]], ts=ts, fs={"p": f, "n": np.zeros(6, np.int32), "t": f})
    if material == "diffuse":
        mat = lm.load_material(prefix + "mat", "diffuse", Kd=[0, 1, 0], mapKd=tex)
    else:
        mat = lm.load_material(prefix + "mat", "mixture_wavefrontobj", Kd=[0.5, 0.5, 0.5], Ks=[0.2, 0.2, 0.2], ax=0.3,
                               ay=0.3, mapKd=tex)
    if quad_on:
        scene.add_primitive(mesh=quad, material=mat)
    back = lm.load_mesh(prefix + "back", "raw", ps=ps * [3, 3, 1] + [0, 0, -1], ns=[[0, 0, 1]], ts=[0, 0],
                        fs={"p": f, "n": np.zeros(6, np.int32), "t": np.zeros(6, np.int32)})
    scene.add_primitive(mesh=back, material=lm.load_material(prefix + "grey", "diffuse", Kd=[0.5, 0.5, 0.5]))
    if extra_light:
        lq = np.array([[-0.5, 2, 0.5], [0.5, 2, 0.5], [0.5, 2, 1.5], [-0.5, 2, 1.5]], np.float32)
        lmesh = lm.load_mesh(prefix + "lmesh", "raw", ps=lq, ns=[[0, -1, 0]], ts=[0, 0],
                             fs={"p": f, "n": np.zeros(6, np.int32), "t": np.zeros(6, np.int32)})
        scene.add_primitive(mesh=lmesh, material=lm.load_material(prefix + "black", "diffuse", Kd=[0, 0, 0]),
                            light=lm.load_light(prefix + "area", "area", Ke=[6, 6, 6], mesh=lmesh))
    scene.add_primitive(light=lm.load_light(prefix + "env", "envconst", Le=[env, env, env]))
    return scene, film, mat


def _regions(img):
    """Mean color of the four texel regions of the quad in a 32 x 32 head-on image (pixels well
    inside each quadrant), in texel order (row 0 = bottom row of the image)."""
    h, w = img.shape[:2]
    c = w // 2
    # the quad spans about +-7.5 pixels around the center at vfov 30 and distance 4
    q = 3
    return {(0, 0): img[c - 1 - q:c - 1, c - 1 - q:c - 1].reshape(-1, 3),
            (0, 1): img[c - 1 - q:c - 1, c + 1:c + 1 + q].reshape(-1, 3),
            (1, 0): img[c + 1:c + 1 + q, c - 1 - q:c - 1].reshape(-1, 3),
            (1, 1): img[c + 1:c + 1 + q, c + 1:c + 1 + q].reshape(-1, 3)}


def test_oracle_texture_lookup_and_orientation(lm, oracle_mod):
    """Raycast with constant colors (renderer_raycast.cpp:84-93): every pixel of the quad is the
    texel under it; texel row 0 is at the bottom of the image (row 0 of the film)."""
    scene, _, _ = _quad_scene(lm, CHECKER, prefix="tqo_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    img, _ = S.render_raycast(32, 32, use_constant_color=True)
    for (ty, tx), px in _regions(img).items():
        assert np.allclose(px, CHECKER[ty, tx], atol=1e-6), ((ty, tx), px[:2])


def test_oracle_alpha_mask_rules(lm, oracle_mod):
    """A mixture whose mapKd has alpha 0 is a pure pass-through (the back wall shows through as if
    the quad were absent); alpha 1 is the textured surface."""
    from lightmetrica import _native  # noqa: F401  (the lm fixture needs the library)
    rgba0 = np.concatenate([CHECKER, np.zeros((2, 2, 1), np.float32)], 2)
    scene, _, mat = _quad_scene(lm, rgba0, material="mixture", prefix="tqa0_")
    assert mat.mask is not None
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    img, _, _, _ = S.render_pt(32, 32, 64, 6, seed=3, rng="philox")
    # without the quad
    scene2, _, _ = _quad_scene(lm, rgba0, material="mixture", prefix="tqa1_", quad_on=False)
    S2 = oracle_mod.from_lm_scene(scene2, double=True)
    S2.build()
    ref, _, _, _ = S2.render_pt(32, 32, 64, 6, seed=3, rng="philox")
    c = 16
    a, b = img[c - 4:c + 4, c - 4:c + 4], ref[c - 4:c + 4, c - 4:c + 4]
    assert abs(a.mean() - b.mean()) / b.mean() < 0.1


@pytest.mark.gpu
def test_raycast_textured_matches_oracle(lm, oracle_mod):
    scene, film, _ = _quad_scene(lm, CHECKER, prefix="tqg_")
    scene.build()
    for kw in ({"use_constant_color": True}, {}):
        lm.load_renderer("tqg_rc", "raycast", scene=scene, output=film, **kw).render()
        gpu = film.buffer()
        S = oracle_mod.from_lm_scene(scene, double=False)
        S.build(robust=True)
        ref, _ = S.render_raycast(32, 32, **kw)
        bad = np.abs(gpu - ref).max(axis=2) > 1e-4
        assert bad.mean() < 0.01, bad.sum()  # texel boundaries may round either way in fp32
    for (ty, tx), px in _regions(film.buffer()).items():
        assert np.all(np.abs(px - CHECKER[ty, tx]) < 1.0), (ty, tx)


@pytest.mark.gpu
@pytest.mark.parametrize("material", ["diffuse", "mixture"])
def test_pt_textured_matches_oracle(lm, oracle_mod, material):
    """renderer::pt on a textured diffuse quad, and on a mixture whose RGBA mapKd is also its alpha
    mask (alpha 1, 0.5 and 0 texels: surface, half and pass-through), against the fp64 oracle on
    matched random streams."""
    data = CHECKER
    if material == "mixture":
        data = np.concatenate([CHECKER, np.array([[[1.0], [0.0]], [[0.5], [1.0]]], np.float32)], 2)
    scene, film, _ = _quad_scene(lm, data, material=material, prefix=f"tqp{material}_")
    scene.build()
    lm.load_renderer(f"tqp_pt{material}", "pt", scene=scene, output=film, max_verts=6, seed=7, spp=32,
                     scheduler="sample").render()
    gpu = film.buffer()
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _, _ = S.render_pt(32, 32, 32, 6, seed=7, rng="philox")
    assert ref.sum() > 0
    rel = np.abs(gpu - ref).sum() / np.abs(ref).sum()
    assert rel < 3e-3, rel


def _write_rgba_png(path, rgba8):
    """An 8-bit RGBA PNG, top row first (the file's order)."""
    h, w = rgba8.shape[:2]
    raw = b"".join(b"\x00" + rgba8[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw)))
        f.write(chunk(b"IEND", b""))


def _textured_obj(tmp_path):
    """A floor and a wall, the wall's material with map_Kd = an RGBA PNG (a cut-out pattern), an
    emissive ceiling quad."""
    rng = np.random.default_rng(3)
    rgba = rng.integers(0, 256, (8, 8, 4)).astype(np.uint8)
    rgba[..., 3] = np.where(rng.random((8, 8)) < 0.4, 0, 255)
    _write_rgba_png(str(tmp_path / "cut.png"), rgba)
    (tmp_path / "t.mtl").write_text(
        "newmtl floor\nKd 0.6 0.6 0.6\n"
        "newmtl wall\nKd 1 1 1\nKs 0.1 0.1 0.1\nNs 20\nmap_Kd cut.png\n"
        "newmtl lamp\nKd 0 0 0\nKe 10 10 10\n")
    (tmp_path / "t.obj").write_text(
        "mtllib t.mtl\n"
        "v -2 0 -2\nv 2 0 -2\nv 2 0 2\nv -2 0 2\n"
        "v -1 0 -0.5\nv 1 0 -0.5\nv 1 2 -0.5\nv -1 2 -0.5\n"
        "v -0.5 2.5 -0.5\nv 0.5 2.5 -0.5\nv 0.5 2.5 0.5\nv -0.5 2.5 0.5\n"
        "vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
        "vn 0 1 0\nvn 0 0 1\nvn 0 -1 0\n"
        "usemtl floor\nf 1//1 4//1 3//1 2//1\n"
        "usemtl wall\nf 5/1/2 6/2/2 7/3/2 8/4/2\n"
        "usemtl lamp\nf 9//3 10//3 11//3 12//3\n")
    return str(tmp_path / "t.obj")


def test_obj_map_kd_assets(lm, tmp_path):
    model = lm.load_model("tobj", "wavefrontobj", path=_textured_obj(tmp_path))
    tex = model.assets["texture_cut"]
    assert tex.key_name == "texture::bitmap" and tex.has_alpha() and tex.texels().shape == (8, 8, 4)
    wall = model.assets["wall"]
    assert wall.mapKd is tex and wall.mask is tex
    alpha = tex.texels()[..., 3]
    assert set(np.unique(alpha).tolist()) <= {0.0, 1.0}
    # skip_specular_mat turns the alpha mask off (model_wavefrontobj.cpp:214)
    model2 = lm.load_model("tobj2", "wavefrontobj", path=_textured_obj(tmp_path), skip_specular_mat=True)
    assert model2.assets["wall"].mask is None and model2.assets["wall"].mapKd is not None


@pytest.mark.gpu
def test_obj_map_kd_scene_matches_oracle(lm, oracle_mod, tmp_path):
    model = lm.load_model("tobjg", "wavefrontobj", path=_textured_obj(tmp_path))
    film = lm.load_film("tobj_film", "bitmap", w=40, h=32)
    cam = lm.load_camera("tobj_cam", "pinhole", position=[0, 1.2, 4], center=[0, 0.8, 0], up=[0, 1, 0], vfov=40,
                         aspect=40 / 32)
    scene = lm.load_scene("tobj_scene", "default", accel=lm.load_accel("tobj_accel", "sahbvh"))
    scene.add_primitive(camera=cam)
    scene.add_primitive(model=model)
    scene.add_primitive(light=lm.load_light("tobj_env", "envconst", Le=[0.3, 0.3, 0.3]))
    scene.build()
    lm.load_renderer("tobj_pt", "pt", scene=scene, output=film, max_verts=7, seed=2, spp=32, scheduler="sample").render()
    gpu = film.buffer()
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _, _ = S.render_pt(40, 32, 32, 7, seed=2, rng="philox")
    assert ref.sum() > 0
    rel = np.abs(gpu - ref).sum() / np.abs(ref).sum()
    assert rel < 3e-3, rel
    # renderers without image textures refuse the scene instead of ignoring the texture
    with pytest.raises(lm.LmGpuError):
        lm.load_renderer("tobj_lt", "lt", scene=scene, output=film, max_verts=5, seed=1, scheduler="sample",
                         num_samples=1000).render()
    with pytest.raises(lm.LmGpuError):
        lm.load_renderer("tobj_bd", "bdpt", scene=scene, output=film, max_verts=5, seed=1, scheduler="sample",
                         num_samples=1000).render()
