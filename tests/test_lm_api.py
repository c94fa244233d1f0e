"""The drop-in `lightmetrica` API (host side, no GPU): component keys, scene-graph rules
(src/scene.cpp:72-156), and flattening that agrees bit for bit with the oracle's fp32 mode."""
import numpy as np
import pytest


def test_registered_keys(lm):
    keys = lm.registered_components()
    for k in ["accel::sahbvh", "accel::nanort", "accel::embree", "accel::embreeinstanced", "accel::gpu",
              "renderer::pt", "renderer::lt", "renderer::raycast", "film::bitmap", "camera::pinhole", "mesh::raw",
              "model::wavefrontobj", "material::mixture_wavefrontobj", "renderer::bdpt", "renderer::bdptopt",
              "renderer::pt_naive_path", "renderer::pt_nee_path", "renderer::lt_nee_path", "renderer::blank",
              "material::diffuse", "material::glossy", "material::glass", "material::mirror",
              "light::area", "light::envconst", "light::env", "scene::default"]:
        assert k in keys


def test_locators_and_missing_keys(lm):
    m = lm.load_material("mat", "diffuse", Kd=[0.5, 0.5, 0.5])
    assert m.loc() == "$.assets.mat"
    assert lm.get("$.assets.mat") is m
    with pytest.raises(lm.LmGpuError):
        lm.load_material("x", "nonexistent")
    with pytest.raises(lm.LmGpuError):
        lm.load_material("g", "glossy", Ks=[1, 1, 1])  # missing ax/ay


def _tri_mesh(lm, name="tri"):
    return lm.load_mesh(name, "raw", ps=[0, 0, 0, 1, 0, 0, 0, 1, 0], ns=[0, 0, 1], ts=[0, 0],
                        fs={"p": [0, 1, 2], "n": [0, 0, 0], "t": [0, 0, 0]})


def test_scene_graph_rules(lm):
    scene = lm.load_scene("scene", "default", accel=lm.load_accel("accel", "sahbvh"))
    mesh = _tri_mesh(lm)
    mat = lm.load_material("mat", "diffuse")
    cam = lm.load_camera("cam", "pinhole", position=[0, 0, 5], center=[0, 0, 0], up=[0, 1, 0], vfov=30, aspect=1)
    light = lm.load_light("l", "area", Ke=[1, 1, 1], mesh=mesh)
    with pytest.raises(lm.LmGpuError):
        scene.create_primitive_node()                                # no assets
    with pytest.raises(lm.LmGpuError):
        scene.create_primitive_node(mesh=mesh)                       # mesh without material
    with pytest.raises(lm.LmGpuError):
        scene.create_primitive_node(camera=cam, light=light)         # camera and light
    scene.add_primitive(light=lm.load_light("e1", "envconst", Le=[1, 1, 1]))
    with pytest.raises(lm.LmGpuError):
        scene.add_primitive(light=lm.load_light("e2", "envconst", Le=[1, 1, 1]))  # second env light
    scene.add_primitive(camera=cam)
    scene.add_primitive(mesh=mesh, material=mat, light=light)
    assert scene.camera_node() >= 0 and scene.env_light_node() >= 0
    assert scene.num_lights() == 2
    flat = scene._flatten()
    # lights in traversal order (scene.cpp:279-286): env first here, then the area light
    assert [L.type for L in flat["lights"]] == [1, 0]
    assert flat["prim_light"].tolist() == [1]


def _instanced_scene(lm):
    """Nested groups with rotation, translation and scale, plus an instance group."""
    scene = lm.load_scene("scene", "default", accel=lm.load_accel("accel", "embree"))
    rng = np.random.default_rng(3)
    ps = rng.random((30, 3)).astype(np.float32)
    mesh = lm.load_mesh("m", "raw", ps=ps, ns=[0, 0, 1], ts=[0, 0],
                        fs={"p": np.arange(30), "n": np.zeros(30, int), "t": np.zeros(30, int)})
    mat = lm.load_material("mat", "diffuse")
    scene.add_transformed_primitive(lm.rotate(0.3, [1, 2, 3]) @ lm.scale([1.5, 0.5, 2.0]), mesh=mesh, material=mat)
    g = scene.create_instance_group_node()
    scene.add_child(g, scene.create_primitive_node(mesh=mesh, material=mat))
    for k in range(3):
        t = scene.create_group_node(lm.translate([k * 1.5, 0.25, -k]) @ lm.rotate(0.7 * k, [0, 1, 0]))
        scene.add_child(t, g)
        scene.add_child(scene.root_node(), t)
    return scene


def test_flatten_bitexact_with_oracle_fp32(lm, oracle_mod):
    """World-space triangles (the accel input) equal the oracle's fp32 flattening bit for bit,
    including nested group transforms and instance groups (accel_sahbvh.cpp:132-151)."""
    scene = _instanced_scene(lm)
    pos = scene._flatten()["positions"]
    S = oracle_mod.from_lm_scene(scene, double=False)
    S.build()
    assert S.num_tris == pos.shape[0] == 40
    p = pos.reshape(-1, 3, 3)
    mine = np.concatenate([p[:, 0], p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]], 1)  # fp32 subtraction
    assert np.array_equal(S.triangles(), mine)


def test_flatten_close_to_oracle_fp64(lm, oracle_mod):
    scene = _instanced_scene(lm)
    pos = scene._flatten()["positions"]
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    p = pos.reshape(-1, 3, 3).astype(np.float64)
    mine = np.concatenate([p[:, 0], p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]], 1)
    assert np.allclose(S.triangles(), mine, atol=1e-5)


def test_synthetic_box_geometry(lm):
    """The benchmark box: 10 wall quads (20 triangles), two 12-triangle boxes, a 2-triangle light;
    every triangle's winding agrees with its shading normal (a mismatch would zero its shading)."""
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene()
    flat = scene._flatten()
    assert flat["positions"].shape[0] == 20 + 24 + 2
    p = flat["positions"].reshape(-1, 3, 3)
    gn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    sn = flat["normals"].reshape(-1, 3, 3).sum(1)
    assert np.all(np.sum(gn * sn, axis=1) > 0)


def test_synthetic_spheres_counts(lm):
    from lightmetrica import synthetic as syn
    scene, film, info = syn.spheres_scene(n_spheres=3, subdiv=2, ground_quads=8, w=32, h=18)
    flat = scene._flatten()
    assert flat["positions"].shape[0] == info["triangles"] == 3 * 320 + 2 * 64 + 12
    kinds = sorted({m.key_name for m in flat["materials"]})
    assert "material::diffuse" in kinds
    # icosphere subdivision counts: 20 * 4^s faces
    v, f = syn.icosphere(6)
    assert f.shape[0] == 81920 and v.shape[0] == 40962


def test_sphere_rays_unit_directions():
    from lightmetrica import synthetic as syn
    r = syn.sphere_rays(1000, [0, 1, 0])
    assert r.shape == (1000, 8) and r.dtype == np.float32
    assert np.allclose(np.linalg.norm(r[:, 4:7], axis=1), 1, atol=1e-6)


def test_render_server_never_evicts_the_scene_it_admits(monkeypatch):
    """Admitting a request on a resident but idle scene may evict other idle scenes, never that one
    (host logic only: the batch and footprint calls are stubbed)."""
    from lightmetrica import serving

    class FakeBatch:
        def __init__(self, *a, **k):
            self.n = 0

        def submit(self, *a, **k):
            self.n += 1
            return self.n - 1

    monkeypatch.setattr(serving, "BatchRenderer", FakeBatch)
    monkeypatch.setattr(serving, "scene_footprint", lambda s: 100)
    monkeypatch.setattr(serving, "_release_scene", lambda s: None)
    import lightmetrica as lm
    monkeypatch.setattr(lm, "load_film", lambda *a, **k: object())
    srv = serving.RenderServer(lambda k: f"scene{k}", hbm_budget=2 * 100 + 2 * 96, build_threads=0)  # two scenes + two films
    for rid, key in ((0, "a"), (1, "b")):
        srv.submit(serving.Request(rid=rid, arrival=0.0, scene_key=key, w=2, h=2, spp=1, max_verts=2, seed=0))
        assert srv._try_admit(srv.pending.pop())
        srv.scene_users[key] = 0          # finished: both scenes idle, budget full
    srv.scene_last_use = {"a": 1.0, "b": 0.5}
    req = serving.Request(rid=2, arrival=0.0, scene_key="b", w=2, h=2, spp=1, max_verts=2, seed=0)
    assert srv._try_admit(req)            # evicts "a" (older use time does not matter: "b" is needed)
    assert "b" in srv.scenes and "a" not in srv.scenes and srv.evictions == 1


def test_render_server_does_not_rebuild_a_scene_that_cannot_fit(monkeypatch):
    """A scene whose measured footprint does not fit is built once and then waits; nothing is
    evicted for a request that eviction cannot make room for (host logic; device calls stubbed)."""
    from lightmetrica import serving

    class FakeBatch:
        def __init__(self, *a, **k):
            self.n = 0

        def submit(self, *a, **k):
            self.n += 1
            return self.n - 1

    builds = []
    monkeypatch.setattr(serving, "BatchRenderer", FakeBatch)
    monkeypatch.setattr(serving, "scene_footprint", lambda s: 1000 if s == "big" else 100)
    monkeypatch.setattr(serving, "_release_scene", lambda s: None)
    import lightmetrica as lm
    monkeypatch.setattr(lm, "load_film", lambda *a, **k: object())

    def make(k):
        builds.append(k)
        return k
    srv = serving.RenderServer(make, hbm_budget=500, build_threads=0)
    small = serving.Request(rid=0, arrival=0.0, scene_key="small", w=2, h=2, spp=1, max_verts=2, seed=0)
    assert srv._try_admit(small)
    srv.scene_users["small"] = 0
    big = serving.Request(rid=1, arrival=0.0, scene_key="big", w=2, h=2, spp=1, max_verts=2, seed=0)
    for _ in range(5):
        assert not srv._try_admit(big)
    assert builds.count("big") == 1 and "small" in srv.scenes and srv.evictions == 0


def test_render_server_builds_scenes_on_a_worker(monkeypatch):
    """With build threads, admission starts the build and returns; the request is admitted once
    the scene is ready, and the scene is built once."""
    import threading
    import time
    from lightmetrica import serving

    class FakeBatch:
        def __init__(self, *a, **k):
            pass

        def submit(self, *a, **k):
            return 0

        def close(self):
            pass

    monkeypatch.setattr(serving, "BatchRenderer", FakeBatch)
    monkeypatch.setattr(serving, "scene_footprint", lambda s: 100)
    import lightmetrica as lm
    monkeypatch.setattr(lm, "load_film", lambda *a, **k: object())
    gate = threading.Event()
    builds = []

    def make(k):
        gate.wait(5)
        builds.append(k)
        return k
    srv = serving.RenderServer(make, hbm_budget=10**6, build_threads=1)
    req = serving.Request(rid=0, arrival=0.0, scene_key="s", w=2, h=2, spp=1, max_verts=2, seed=0)
    assert not srv._try_admit(req) and not srv._try_admit(req)   # building
    gate.set()
    for _ in range(500):
        if srv._try_admit(req):
            break
        time.sleep(0.01)
    assert req.job is not None and builds == ["s"] and srv.scene_builds == 1
    srv.close()


def test_material_proxy_and_constant_texture(lm, oracle_mod):
    """material::proxy renders as the material it refers to (material_proxy.cpp); a diffuse
    mapKd that is a texture::constant is its color (texture_constant.cpp); a constant texture is
    a 1 x 1 environment map."""
    from lightmetrica import synthetic as syn
    base, _ = syn.box_scene(w=8, h=8, prefix="px0_")
    S0 = oracle_mod.from_lm_scene(base, double=True)
    S0.build()
    ref, _, _, _ = S0.render_pt(8, 8, 8, 5, seed=2)
    # the same box with its grey walls through a proxy, and a red wall Kd given as a constant texture
    scene, _ = syn.box_scene(w=8, h=8, prefix="px1_")
    proxy = lm.load_material("px1_proxy", "proxy", ref="px1_grey")
    tex = lm.load_texture("px1_tex", "constant", color=[0.75, 0.25, 0.25])
    red = lm.load_material("px1_red_tex", "diffuse", mapKd=tex, Kd=[0, 1, 0])
    for n in scene.nodes:
        if n["type"] == "primitive" and n["material"] is not None:
            if n["material"].key_name == "material::diffuse" and np.allclose(n["material"].Kd, [0.75, 0.75, 0.75]):
                n["material"] = proxy
            elif np.allclose(getattr(n["material"], "Kd", [0, 0, 0]), [0.75, 0.25, 0.25]):
                n["material"] = red
    rows = [m.native() for m in scene._flatten()["materials"]]
    assert any(r.type == 0 and np.allclose(list(r.color), [0.75, 0.75, 0.75]) for r in rows)
    assert any(r.type == 0 and np.allclose(list(r.color), [0.75, 0.25, 0.25]) for r in rows)
    S1 = oracle_mod.from_lm_scene(scene, double=True)
    S1.build()
    img, _, _, _ = S1.render_pt(8, 8, 8, 5, seed=2)
    assert np.allclose(img, ref, rtol=1e-12, atol=1e-15)
    assert np.array_equal(tex.data, np.array([[[0.75, 0.25, 0.25]]], np.float32)) and not tex.has_alpha()
    env = lm.load_light("px1_env", "env", envmap=tex)
    assert env.data.shape == (1, 1, 3)
    with pytest.raises(lm.LmGpuError):
        lm.load_material("px1_bad", "proxy", ref="px1_tex")    # not a material
    bmp = lm.load_texture("px1_bmp", "bitmap", data=np.ones((2, 2, 3)))
    img_mat = lm.load_material("px1_img", "diffuse", mapKd=bmp)   # an image texture, looked up per point
    assert img_mat.mapKd is bmp and bmp.texels().shape == (2, 2, 3)
    with pytest.raises(lm.LmGpuError):
        lm.load_material("px1_notex", "diffuse", mapKd="px1_red_tex")  # a material is not a texture


def test_asset_group_and_script_stubs(lm):
    """lm.load_asset_group (src/assetgroup.cpp): children under $.assets.<group>.<name>, usable as
    references; the subsystem calls example scripts make (log, progress, objloader, debug) exist."""
    g = lm.load_asset_group("ag_room", "default")
    cam = g.load_camera("camera1", "pinhole", position=[0, 0, 5], center=[0, 0, 0], up=[0, 1, 0], vfov=30, aspect=1)
    assert cam.loc() == "$.assets.ag_room.camera1"
    assert lm.get("$.assets.ag_room.camera1") is cam
    sub = g.load_asset_group("sub")
    mat = sub.load_material("m", "diffuse", Kd=[0.5, 0.5, 0.5])
    assert mat.loc() == "$.assets.ag_room.sub.m"
    proxy = lm.load_material("ag_proxy", "proxy", ref="$.assets.ag_room.sub.m")
    assert proxy.underlying() is mat
    film = g.load_film("film", "bitmap", w=4, h=4)
    assert lm.get_film("$.assets.ag_room.film") is film
    with pytest.raises(lm.LmGpuError):
        g.save_to_file("x.serialized")
    lm.log.init("logger::default")
    lm.progress.init("progress::default")
    lm.objloader.init("tinyobjloader")
    lm.debug.print_asset_tree()
    assert lm.log.LogLevel.Warn > lm.log.LogLevel.Info and lm.FloatT in (lm.Float32, lm.Float64)
