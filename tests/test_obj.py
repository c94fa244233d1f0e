"""model::wavefrontobj and material::mixture_wavefrontobj.

CPU: the OBJ/MTL rules of the reference's objloader::simple (quads, negative indices, missing
normals, groups, per-face materials, default material); the model's assets (names, lights for
Ke > 0, material mapping); scene.add_primitive(model=...); the oracle's mixture material equals
the diffuse / glossy material it reduces to. GPU: an OBJ scene with a mixture material against
the oracle with matched random streams."""
import os

import numpy as np
import pytest

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
OBJ = os.path.join(DATA, "cornell_quads.obj")


def test_objloader_rules():
    from lightmetrica import objloader
    m = objloader.load_obj(OBJ)
    assert m.ps.shape == (16, 3) and m.ns.shape == (5, 3)
    assert [x.name for x in m.materials] == ["white", "red", "green", "lamp", "shiny"]
    assert [(p.material, len(p.faces) // 3) for p in m.primitives] == [(0, 2), (0, 2), (0, 2), (1, 2), (2, 2), (3, 2), (4, 2)]
    floor = m.primitives[0].faces
    assert floor == [(0, -1, 0), (3, -1, 0), (2, -1, 0), (0, -1, 0), (2, -1, 0), (1, -1, 0)]  # quad -> (0,1,2), (0,2,3)
    right = m.primitives[4].faces
    assert [f[0] for f in right] == [1, 2, 6, 1, 6, 5]                                       # negative indices
    assert all(f[2] == -1 for f in right)                                                     # no normals
    shiny = m.materials[4]
    assert shiny.Ks == (0.3, 0.3, 0.3) and shiny.Ns == 80 and shiny.an == pytest.approx(0.4)
    assert m.materials[3].Ke == (17.0, 17.0, 17.0)


def test_objloader_default_material_and_errors(tmp_path):
    from lightmetrica import objloader
    p = tmp_path / "t.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    m = objloader.load_obj(str(p))
    assert [x.name for x in m.materials] == ["default"] and m.materials[0].Kd == (1.0, 1.0, 1.0)
    assert len(m.primitives) == 1 and m.primitives[0].material == 0
    q = tmp_path / "u.obj"
    q.write_text("v 0 0 0\nusemtl nope\nf 1 1 1\n")
    with pytest.raises(ValueError):
        objloader.load_obj(str(q))


def test_model_assets_and_scene(lm):
    model = lm.load_model("obj_box", "wavefrontobj", path=OBJ)
    names = sorted(model.assets)
    assert "white" in names and "mesh_5" in names            # 5 materials come first
    assert "mesh_10_light" in names                            # the lamp group (6th mesh) emits
    assert lm._resolve("$.assets.obj_box.mesh_10_light").key_name == "light::area"
    mats = {k: v.key_name for k, v in model.assets.items() if k in ("white", "shiny")}
    assert mats == {"white": "material::mixture_wavefrontobj", "shiny": "material::mixture_wavefrontobj"}
    shiny = model.assets["shiny"]
    r, a = 2.0 / 82.0, np.sqrt(1 - 0.4 * 0.9)
    assert shiny.ax == pytest.approx(max(1e-3, r / a)) and shiny.ay == pytest.approx(max(1e-3, r * a))
    scene = lm.load_scene("obj_scene", "default", accel=lm.load_accel("obj_accel", "sahbvh"))
    scene.add_primitive(model=model)
    flat = scene._flatten()
    assert flat["positions"].shape[0] == 14
    assert len(flat["lights"]) == 1
    # faces without normals shade with their geometric normal
    right = 8  # first triangle of the right wall
    assert np.allclose(flat["normals"][right].reshape(3, 3), [[-1, 0, 0]] * 3)


def _oracle_img(oracle_mod, scene, spp=32):
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    img, _, _, _ = S.render_pt(16, 16, spp, 6, seed=5, rng="philox")
    return img


@pytest.mark.parametrize("which", ["diffuse", "glossy"])
def test_oracle_mixture_reduces_to_its_lobe(lm, oracle_mod, which):
    """mixture(Kd, 0) is material::diffuse(Kd) and mixture(0, Ks) is material::glossy(Ks): with the
    same random streams the oracle gives the same image up to rounding."""
    from lightmetrica import synthetic as syn
    imgs = []
    for mix in (False, True):
        scene, _ = syn.box_scene(w=16, h=16, prefix=f"mx{which}{mix}_")
        if which == "diffuse":
            m = (lm.load_material(f"m{mix}", "mixture_wavefrontobj", Kd=[0.6, 0.5, 0.4], Ks=[0, 0, 0], ax=0.2, ay=0.2)
                 if mix else lm.load_material(f"m{mix}", "diffuse", Kd=[0.6, 0.5, 0.4]))
        else:
            m = (lm.load_material(f"g{mix}", "mixture_wavefrontobj", Kd=[0, 0, 0], Ks=[0.7, 0.7, 0.6], ax=0.2, ay=0.3)
                 if mix else lm.load_material(f"g{mix}", "glossy", Ks=[0.7, 0.7, 0.6], ax=0.2, ay=0.3))
        for n in scene.nodes:  # every surface of the box gets the material under test (not the light)
            if n["type"] == "primitive" and n["mesh"] is not None and n["light"] is None:
                n["material"] = m
        imgs.append(_oracle_img(oracle_mod, scene))
    a, b = imgs
    assert a.sum() > 0
    assert np.abs(a - b).max() <= 1e-6 * max(1.0, np.abs(a).max())


@pytest.mark.gpu
def test_obj_scene_matches_oracle(lm, oracle_mod):
    model = lm.load_model("obj_box_g", "wavefrontobj", path=OBJ)
    film = lm.load_film("obj_film", "bitmap", w=32, h=32)
    cam = lm.load_camera("obj_cam", "pinhole", position=[0.5, 0.5, 2.6], center=[0.5, 0.5, 0.0], up=[0, 1, 0],
                         vfov=30, aspect=1.0)
    scene = lm.load_scene("obj_scene_g", "default", accel=lm.load_accel("obj_accel_g", "sahbvh"))
    scene.add_primitive(camera=cam)
    scene.add_primitive(model=model)
    scene.add_primitive(light=lm.load_light("obj_env", "envconst", Le=[0.2, 0.2, 0.2]))
    scene.build()
    lm.load_renderer("obj_pt", "pt", scene=scene, output=film, max_verts=8, seed=4, spp=32, scheduler="sample").render()
    gpu = film.buffer()
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _, _ = S.render_pt(32, 32, 32, 8, seed=4, rng="philox")
    assert ref.sum() > 0
    rel = np.abs(gpu - ref).sum() / np.abs(ref).sum()
    assert rel < 3e-3, rel
