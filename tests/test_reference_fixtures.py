"""Scenes of the reference's own functests, built with the same scene-graph calls:

* functest/lmscene.py:29-65 (plane_emitter): one 2x2 area light (Ke = 1, black material) facing a
  pinhole camera. Known answer: the path tracer sees radiance exactly 1 where the light covers a
  pixel and 0 elsewhere; light tracing samples no camera -> light path, so its image is 0; BDPT
  recovers the light through its s = 0 and s = 1 strategies.
* functest/func_render_instancing.py:62-190: a 10x20 UV sphere placed 10x10 times three ways
  (plain translation groups, one instance group, nested instance groups), rendered by
  renderer::raycast with visualize_normal and a white background. The three forms and both accel
  kinds (flattened, two-level) give the same image.
"""
import numpy as np
import pytest


def _plane_emitter(lm, w, h, prefix):
    # lmscene.py:29-65
    camera = lm.load_camera(prefix + "camera", "pinhole", position=[0, 0, 5], center=[0, 0, 0], up=[0, 1, 0], vfov=30,
                            aspect=16 / 9)
    mesh = lm.load_mesh(prefix + "mesh", "raw", ps=[-1, -1, -1, 1, -1, -1, 1, 1, -1, -1, 1, -1], ns=[0, 0, 1],
                        ts=[0, 0, 1, 0, 1, 1, 0, 1], fs={"p": [0, 1, 2, 0, 2, 3], "n": [0, 0, 0, 0, 0, 0], "t": [0, 1, 2, 0, 2, 3]})
    material = lm.load_material(prefix + "mat_black", "diffuse", Kd=[0, 0, 0])
    light = lm.load_light(prefix + "light", "area", Ke=[1, 1, 1], mesh=mesh)
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", "sahbvh"))
    scene.add_primitive(camera=camera)
    scene.add_primitive(mesh=mesh, material=material, light=light)
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    return scene, film


def _plane_coverage(w, h):
    """Per pixel: 1 if the whole pixel sees the light quad, 0 if none of it does, else -1 (the
    pinhole's rays meet the plane z = -1 at 6 * tan(15 deg) * (aspect * (2 rx - 1), 2 ry - 1))."""
    tf = np.tan(np.radians(15.0))
    aspect = 16 / 9

    def inside(rx, ry):
        return (np.abs(6 * tf * aspect * (2 * rx - 1)) < 1) & (np.abs(6 * tf * (2 * ry - 1)) < 1)
    cov = np.full((h, w), -1)
    for y in range(h):
        for x in range(w):
            corners = [inside((x + a) / w, (y + b) / h) for a in (0, 1) for b in (0, 1)]
            cov[y, x] = 1 if all(corners) else (0 if not any(corners) else -1)
    return cov


def test_plane_emitter_oracle_known_answer(lm, oracle_mod):
    scene, film = _plane_emitter(lm, 32, 18, "pe_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    img, _, _, _ = S.render_pt(32, 18, 4, 5, seed=1)
    cov = _plane_coverage(32, 18)
    assert (cov == 1).sum() > 50 and (cov == 0).sum() > 50
    assert np.allclose(img[cov == 1], 1.0, atol=1e-12)
    assert not img[cov == 0].any()
    lt, _, _ = S.render_lt(32, 18, 100_000, 5, seed=1)
    assert not lt.any()


def _uv_sphere(n_theta=10):
    """Vertices on rings of constant theta (n_theta + 1 rings of 2 n_theta vertices, poles
    repeated), two triangles per quad except at the poles, unit radius
    (func_render_instancing.py:62-93)."""
    n_phi = 2 * n_theta
    th = np.repeat(np.arange(n_theta + 1) * np.pi / n_theta, n_phi)
    ph = np.tile(np.arange(n_phi) * 2 * np.pi / n_phi, n_theta + 1)
    ns = np.stack([np.sin(th) * np.sin(ph), np.cos(th), np.sin(th) * np.cos(ph)], axis=1)
    faces = []
    for i in range(1, n_theta + 1):
        for j in range(1, n_phi + 1):
            p00, p01 = (i - 1) * n_phi + j - 1, (i - 1) * n_phi + j % n_phi
            p10, p11 = i * n_phi + j - 1, i * n_phi + j % n_phi
            if i > 1:
                faces.append([p10, p01, p00])
            if i < n_theta:
                faces.append([p11, p01, p10])
    return ns.copy(), ns, np.zeros((ns.shape[0], 2)), np.asarray(faces, np.int32)


def _instancing_scene(lm, form, accel, prefix, w=96, h=54):
    vs, ns, ts, fs = _uv_sphere()
    mesh = lm.load_mesh(prefix + "mesh_sphere", "raw", ps=vs.flatten().tolist(), ns=ns.flatten().tolist(), ts=ts.flatten().tolist(),
                        fs={"p": fs.flatten().tolist(), "t": fs.flatten().tolist(), "n": fs.flatten().tolist()})
    camera = lm.load_camera(prefix + "camera_main", "pinhole", position=[0, 0, 50], center=[0, 0, 0], up=[0, 1, 0], vfov=30,
                            aspect=16 / 9)
    material = lm.load_material(prefix + "material_white", "diffuse", Kd=[1, 1, 1])
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", accel))
    scene.add_primitive(camera=camera)
    grid = np.linspace(-10, 10, 10)
    if form == "plain":            # func_render_instancing.py:124-134
        for y in grid:
            for x in grid:
                p = scene.create_primitive_node(mesh=mesh, material=material)
                t = scene.create_group_node(lm.translate(np.array([x, y, 0])))
                scene.add_child(t, p)
                scene.add_child(scene.root_node(), t)
    elif form == "single":         # :147-160
        g = scene.create_instance_group_node()
        scene.add_child(g, scene.create_primitive_node(mesh=mesh, material=material))
        for y in grid:
            for x in grid:
                t = scene.create_group_node(lm.translate(np.array([x, y, 0])))
                scene.add_child(t, g)
                scene.add_child(scene.root_node(), t)
    else:                          # :172-190, nested instance groups
        g1 = scene.create_instance_group_node()
        scene.add_child(g1, scene.create_primitive_node(mesh=mesh, material=material))
        g2 = scene.create_instance_group_node()
        for y in grid:
            t = scene.create_group_node(lm.translate(np.array([0, y, 0])))
            scene.add_child(t, g1)
            scene.add_child(g2, t)
        for x in grid:
            t = scene.create_group_node(lm.translate(np.array([x, 0, 0])))
            scene.add_child(t, g2)
            scene.add_child(scene.root_node(), t)
    film = lm.load_film(prefix + "film_output", "bitmap", w=w, h=h)
    return scene, film


def test_instancing_forms_flatten_alike(lm):
    """The three scene-graph forms hold the same 100 spheres in world space (as sets of triangles)."""
    worlds = []
    for form in ("plain", "single", "nested"):
        scene, _ = _instancing_scene(lm, form, "sahbvh", f"if_{form}_")
        p = scene._flatten()["positions"].astype(np.float64).reshape(-1, 9)
        worlds.append(p[np.lexsort(p.T[::-1])])
    assert worlds[0].shape == (100 * 360, 9)
    assert np.allclose(worlds[0], worlds[1], atol=1e-5) and np.allclose(worlds[0], worlds[2], atol=1e-5)


@pytest.mark.gpu
def test_plane_emitter_gpu_known_answer(lm):
    scene, film = _plane_emitter(lm, 32, 18, "peg_")
    scene.build()
    cov = _plane_coverage(32, 18)
    lm.load_renderer("peg_pt", "pt", scene=scene, output=film, max_verts=5, seed=1, spp=4, scheduler="sample").render()
    img = film.buffer()
    assert np.allclose(img[cov == 1], 1.0, atol=1e-6) and not img[cov == 0].any()
    lm.load_renderer("peg_lt", "lt", scene=scene, output=film, max_verts=5, seed=1, num_samples=100_000, scheduler="sample").render()
    assert not film.buffer().any()
    lm.load_renderer("peg_bd", "bdpt", scene=scene, output=film, max_verts=5, seed=1, num_samples=1 << 20,
                     scheduler="sample").render()
    bd = film.buffer()
    assert abs(bd[cov == 1].mean() - 1) < 0.02 and bd[cov == 0].max() < 1e-6


@pytest.mark.gpu
def test_instancing_forms_render_alike(lm):
    imgs = {}
    for form in ("plain", "single", "nested"):
        for accel in ("sahbvh", "embreeinstanced"):
            scene, film = _instancing_scene(lm, form, accel, f"ig_{form}_{accel}_")
            scene.build()
            lm.load_renderer(f"ig_r_{form}_{accel}", "raycast", scene=scene, output=film, visualize_normal=True,
                             bg_color=[1, 1, 1]).render()
            imgs[(form, accel)] = film.buffer().copy()
    ref = imgs[("plain", "sahbvh")]
    assert (ref < 1).any() and (ref == 1).any()   # spheres and background
    for k, img in imgs.items():
        bad = (np.abs(img - ref).max(axis=2) > 1e-3).mean()
        assert bad < 0.005, (k, bad)
