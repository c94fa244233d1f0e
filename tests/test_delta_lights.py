"""light::point (src/light/light_point.cpp) and light::directional (src/light/light_directional.cpp).

Known answers (a diffuse plane z = 0 of albedo rho under one light, seen by a pinhole camera on
the z axis; max_verts = 3 keeps direct light only): a point light of Le = I at height h gives
radiance rho / pi * I * h / r^3 at distance r from the light; a directional light of Le = E gives
rho / pi * E * |cos| everywhere. Path tracing samples these with next-event estimation alone and,
as renderer_pt.cpp:166-180 has it, a light that BSDF sampling cannot reach keeps the MIS weight 1,
so the 'mis' image equals the 'nee' image. Light tracing and BDPT estimate the same images
(the point light connects through s = 1 and s = 2; the directional light is neither connectable
nor reachable, so only s >= 2 remains). Mixed scenes (the Cornell box with an area and a point
light; spheres with glass and glossy materials under an environment and a directional light):
BDPT and light tracing agree with path tracing in expectation.
GPU (through the C-ABI): the same samples as the oracle with matched Philox streams for pt, lt and
bdpt; the plane known answers."""
import numpy as np
import pytest


def _plane_scene(lm, prefix, light, w=32, h=32, **lprop):
    camera = lm.load_camera(prefix + "camera", "pinhole", position=[0, 0, 5], center=[0, 0, 0], up=[0, 1, 0], vfov=30,
                            aspect=w / h)
    mesh = lm.load_mesh(prefix + "plane", "raw", ps=[-2, -2, 0, 2, -2, 0, 2, 2, 0, -2, 2, 0], ns=[0, 0, 1],
                        ts=[0, 0, 1, 0, 1, 1, 0, 1], fs={"p": [0, 1, 2, 0, 2, 3], "n": [0] * 6, "t": [0, 1, 2, 0, 2, 3]})
    mat = lm.load_material(prefix + "white", "diffuse", Kd=[0.8, 0.8, 0.8])
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", "sahbvh"))
    scene.add_primitive(camera=camera)
    scene.add_primitive(mesh=mesh, material=mat)
    scene.add_primitive(light=lm.load_light(prefix + "light", light, **lprop))
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    return scene, film


def _point_answer(w, h, height, le, rho=0.8, sub=8):
    """Per pixel the mean over a sub x sub grid of rho / pi * Le * h / r^3 on the plane; the pinhole
    at z = 5 (vfov 30, aspect w / h) sees the plane point 5 tan(15 deg) (aspect (2 rx - 1), 2 ry - 1)
    (the answer is symmetric, so the row order does not matter)."""
    tf = np.tan(np.radians(15.0))
    aspect = w / h
    ox = (np.arange(w * sub) + 0.5) / (w * sub)
    oy = (np.arange(h * sub) + 0.5) / (h * sub)
    X = 5 * tf * aspect * (2 * ox[None, :] - 1)
    Y = 5 * tf * (2 * oy[:, None] - 1)
    r2 = X * X + Y * Y + height * height
    L = rho / np.pi * le * height / r2 ** 1.5
    return L.reshape(h, sub, w, sub).mean(axis=(1, 3))


def _blocks(a, k=4):
    h, w = a.shape[:2]
    return a.reshape(k, h // k, k, w // k, -1).sum(axis=(1, 3))


def test_light_props(lm):
    p = lm.load_light("dl_p", "point", Le=[1, 2, 3], position=[0, 1, 2])
    assert np.allclose(p.Le, [1, 2, 3]) and np.allclose(p.position, [0, 1, 2])
    d = lm.load_light("dl_d", "directional", Le=2, direction=[0, 0, -3])
    assert np.allclose(d.direction, [0, 0, -1]) and np.allclose(d.Le, [2, 2, 2])
    with pytest.raises(lm.LmGpuError):
        lm.load_light("dl_z", "directional", Le=1, direction=[0, 0, 0])
    with pytest.raises(lm.LmGpuError):
        lm.load_light("dl_m", "point", Le=1)   # no position


def test_flattened_light_rows(lm):
    scene, _ = _plane_scene(lm, "dfl_", "directional", Le=[2, 2, 2], direction=[0.3, 0.2, -1])
    rows = scene._flatten(geometry=False)["lights"]
    assert len(rows) == 1 and rows[0].type == 4
    d = np.array(rows[0].vec[:])
    assert abs(np.linalg.norm(d) - 1) < 1e-6 and d[2] < 0
    scene, _ = _plane_scene(lm, "dfp_", "point", Le=[1, 1, 1], position=[0, 0, 1])
    rows = scene._flatten(geometry=False)["lights"]
    assert rows[0].type == 3 and list(rows[0].vec[:]) == [0, 0, 1]


def test_oracle_point_light_plane_known_answer(lm, oracle_mod):
    scene, _ = _plane_scene(lm, "dpp_", "point", Le=[1, 1, 1], position=[0, 0, 1])
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    nee, _, _, _ = S.render_pt(32, 32, 16, 3, seed=1, sampling_mode="nee")
    mis, _, _, _ = S.render_pt(32, 32, 16, 3, seed=1, sampling_mode="mis")
    # weight 1: BSDF sampling never reaches a point light (equal up to the threads' summation order)
    assert np.allclose(nee, mis, rtol=1e-12, atol=0)
    ans = _point_answer(32, 32, 1.0, 1.0)
    rel = np.abs(nee[..., 0] - ans) / ans
    assert rel.mean() < 0.01 and rel.max() < 0.05, (rel.mean(), rel.max())
    # more vertices add nothing (no other surface); two vertices see no light
    more, _, _, _ = S.render_pt(32, 32, 16, 6, seed=1, sampling_mode="nee")
    assert np.allclose(more, nee, rtol=1e-12, atol=0)
    two, _, _, _ = S.render_pt(32, 32, 4, 2, seed=1)
    assert not two.any()


def test_oracle_directional_light_plane_known_answer(lm, oracle_mod):
    d = np.array([0.3, 0.2, -1.0])
    scene, _ = _plane_scene(lm, "ddp_", "directional", Le=[2, 2, 2], direction=d.tolist())
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    nee, _, _, _ = S.render_pt(32, 32, 4, 3, seed=1, sampling_mode="nee")
    mis, _, _, _ = S.render_pt(32, 32, 4, 3, seed=1, sampling_mode="mis")
    assert np.allclose(nee, mis, rtol=1e-12, atol=0)
    ans = 0.8 / np.pi * 2 / np.linalg.norm(d)
    assert np.allclose(nee, ans, rtol=1e-9)


@pytest.mark.parametrize("light,prop", [("point", {"Le": [1, 1, 1], "position": [0, 0, 1]}),
                                        ("directional", {"Le": [2, 2, 2], "direction": [0.3, 0.2, -1]})])
def test_oracle_lt_bdpt_plane_known_answer(lm, oracle_mod, light, prop):
    scene, _ = _plane_scene(lm, f"dlb_{light}_", light, **prop)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt, _, _, _ = S.render_pt(32, 32, 64, 3, seed=1)
    lt, _, _ = S.render_lt(32, 32, 2_000_000, 3, seed=3)
    # min_verts 3: without the camera -> light paths (the point light seen directly, below)
    bd, _, _ = S.render_bdpt(32, 32, 400_000, 3, seed=3, min_verts=3)
    b0 = _blocks(pt)
    for img in (lt, bd):
        assert (np.abs(_blocks(img) - b0) / b0).max() < 0.03, (np.abs(_blocks(img) - b0) / b0).max()


def test_oracle_point_light_seen_directly(lm, oracle_mod):
    """BDPT's s = 1, t = 1 strategy connects the camera to a point light (both endpoints are
    connectable, bidir.h:200-214), as path tracing's next-event estimation from the camera vertex
    does in image mode (renderer_pt.cpp:123-131): one pixel receives num_pixels * Le * We / r^2,
    We = 1 / (4 tan^2(fov / 2) aspect cos^3) the pinhole's importance (camera_pinhole.cpp:150-170)."""
    scene, _ = _plane_scene(lm, "dsd_", "point", Le=[1, 1, 1], position=[0.1, 0.05, 1])
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    bd, _, _ = S.render_bdpt(32, 32, 100_000, 2, seed=3)
    pim, _, _, _ = S.render_pt(32, 32, 16, 2, seed=1, primary_mode="image")
    tf = np.tan(np.radians(15.0))
    r2 = 0.1 ** 2 + 0.05 ** 2 + 4.0 ** 2
    we = 1 / (4 * tf * tf * (4 / np.sqrt(r2)) ** 3)
    for img in (bd, pim):
        assert (img[..., 0] > 0).sum() == 1
        assert abs(img[..., 0].sum() / (32 * 32 * we / r2) - 1) < 1e-9
    pix, _, _, _ = S.render_pt(32, 32, 16, 2, seed=1)   # pixel mode: no NEE from the camera
    assert not pix.any()


def _box_point(lm, prefix, w=16, h=16):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=w, h=h, prefix=prefix)
    scene.add_primitive(light=lm.load_light(prefix + "point", "point", Le=[0.6, 0.5, 0.4], position=[0.8, 0.7, 0.75]))
    return scene, film


def _spheres_directional(lm, prefix, w=16, h=12):
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.spheres_scene(n_spheres=10, subdiv=3, ground_quads=8, w=w, h=h, prefix=prefix)
    scene.add_primitive(light=lm.load_light(prefix + "sun", "directional", Le=[3, 2.8, 2.5], direction=[0.4, -1, 0.3]))
    return scene, film


def test_oracle_box_point_light_bdpt_lt_match_pt(lm, oracle_mod):
    scene, _ = _box_point(lm, "dbx_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt, _, _, _ = S.render_pt(16, 16, 2048, 6, seed=1)
    pt2, _, _, _ = S.render_pt(16, 16, 256, 2, seed=1)
    # image mode: next-event estimation from the camera sees the point light, as BDPT does
    pti, _, _, _ = S.render_pt(16, 16, 2048, 6, seed=1, primary_mode="image")
    bd, _, _ = S.render_bdpt(16, 16, 200_000, 6, seed=3)
    assert abs(bd.sum() / pti.sum() - 1) < 0.01
    assert (np.abs(_blocks(bd) - _blocks(pti)) / _blocks(pti)).max() < 0.06
    lt, _, _ = S.render_lt(16, 16, 2_000_000, 6, seed=3)
    assert abs(lt.sum() / (pt - pt2).sum() - 1) < 0.02
    # the point light adds light: the box without it is darker
    from lightmetrica import synthetic as syn
    plain, _ = syn.box_scene(w=16, h=16, prefix="dbx0_")
    S0 = oracle_mod.from_lm_scene(plain, double=True)
    S0.build()
    pt0, _, _, _ = S0.render_pt(16, 16, 512, 6, seed=1)
    assert pt.sum() > 1.05 * pt0.sum()


def test_oracle_spheres_directional_bdpt_lt_match_pt(lm, oracle_mod):
    """Glossy and glass spheres, six area lights, a constant environment and a directional light."""
    scene, _ = _spheres_directional(lm, "dsp_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt, _, _, _ = S.render_pt(16, 12, 4096, 7, seed=1)
    pt2, _, _, _ = S.render_pt(16, 12, 256, 2, seed=1)
    # sunlight reaches BDPT through light subpaths only (s >= 2), which mostly land outside the
    # view: more samples than the scene without the sun needs
    bd, _, _ = S.render_bdpt(16, 12, 4_000_000, 7, seed=3)
    assert abs(bd.mean() / pt.mean() - 1) < 0.01, bd.mean() / pt.mean()
    b1, b2 = _blocks(pt), _blocks(bd)
    assert (np.abs(b1 - b2) / b1).max() < 0.08, (np.abs(b1 - b2) / b1).max()
    lt, _, _ = S.render_lt(16, 12, 4_000_000, 7, seed=3)
    assert abs(lt.sum() / (pt - pt2).sum() - 1) < 0.03


# ---------------------------------------------------------------------------------------------
# GPU

def _rel_l1(a, b):
    return np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mis", "nee"])
def test_pt_delta_lights_match_oracle(lm, oracle_mod, mode):
    for scene, film, w, h in ((*_box_point(lm, f"gdb_{mode}_", 32, 32), 32, 32),
                              (*_spheres_directional(lm, f"gds_{mode}_", 32, 24), 32, 24)):
        scene.build()
        lm.load_renderer("gd_pt", "pt", scene=scene, output=film, max_verts=8, seed=9, sampling_mode=mode,
                         scheduler="sample", spp=16).render()
        gpu = film.buffer().astype(np.float64)
        S = oracle_mod.from_lm_scene(scene, double=True)
        S.build()
        ref, _, _, _ = S.render_pt(w, h, 16, 8, seed=9, sampling_mode=mode, rng="philox")
        assert ref.sum() > 0
        assert _rel_l1(gpu, ref) < 2e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("renderer", ["lt", "bdpt"])
def test_lt_bdpt_delta_lights_match_oracle(lm, oracle_mod, renderer):
    for scene, film, w, h in ((*_box_point(lm, f"gdl_{renderer}_", 32, 32), 32, 32),
                              (*_spheres_directional(lm, f"gdk_{renderer}_", 32, 24), 32, 24)):
        scene.build()
        n = 1 << 20 if renderer == "lt" else 1 << 18
        lm.load_renderer("gd_r", renderer, scene=scene, output=film, max_verts=8, seed=5, scheduler="sample",
                         num_samples=n).render()
        gpu = film.buffer().astype(np.float64)
        S = oracle_mod.from_lm_scene(scene, double=True)
        S.build()
        if renderer == "lt":
            ref, _, _ = S.render_lt(w, h, n, 8, seed=5)
        else:
            ref, _, _ = S.render_bdpt(w, h, n, 8, seed=5)
        assert ref.sum() > 0
        tol = 1e-3 if renderer == "lt" else 2e-3
        assert _rel_l1(gpu, ref) < tol, _rel_l1(gpu, ref)


@pytest.mark.gpu
def test_delta_lights_plane_known_answer_gpu(lm):
    scene, film = _plane_scene(lm, "gpp_", "point", Le=[1, 1, 1], position=[0, 0, 1])
    scene.build()
    lm.load_renderer("gpp_r", "pt", scene=scene, output=film, max_verts=3, seed=1, scheduler="sample", spp=64).render()
    ans = _point_answer(32, 32, 1.0, 1.0)
    rel = np.abs(film.buffer()[..., 0] - ans) / ans
    assert rel.mean() < 0.005 and rel.max() < 0.03, (rel.mean(), rel.max())
    lm.load_renderer("gpp_b", "bdpt", scene=scene, output=film, min_verts=3, max_verts=3, seed=1, scheduler="sample",
                     num_samples=1 << 21).render()
    assert (np.abs(_blocks(film.buffer()[..., :1]) - _blocks(ans[..., None])) / _blocks(ans[..., None])).max() < 0.03
    d = np.array([0.3, 0.2, -1.0])
    scene, film = _plane_scene(lm, "gdp_", "directional", Le=[2, 2, 2], direction=d.tolist())
    scene.build()
    lm.load_renderer("gdp_r", "pt", scene=scene, output=film, max_verts=3, seed=1, scheduler="sample", spp=4).render()
    assert np.allclose(film.buffer(), 0.8 / np.pi * 2 / np.linalg.norm(d), rtol=1e-5)
    lm.load_renderer("gdp_l", "lt", scene=scene, output=film, max_verts=3, seed=1, scheduler="sample",
                     num_samples=1 << 22).render()
    assert abs(film.buffer().mean() / (0.8 / np.pi * 2 / np.linalg.norm(d)) - 1) < 0.01


@pytest.mark.gpu
def test_scene_create_refuses_bad_delta_lights(lm):
    """lmgpu_scene_create checks the rows it receives: a directional light needs a nonzero
    direction, a point light a finite position (the Python components check their props too)."""
    scene, _ = _plane_scene(lm, "gbd_", "directional", Le=[1, 1, 1], direction=[0, 0, -1])
    scene.nodes[-1]["light"].direction = np.zeros(3)
    with pytest.raises(lm.LmGpuError):
        scene.build()
    scene, _ = _plane_scene(lm, "gbp_", "point", Le=[1, 1, 1], position=[0, 0, 1])
    scene.nodes[-1]["light"].position = np.array([0.0, np.nan, 1.0])
    with pytest.raises(lm.LmGpuError):
        scene.build()
