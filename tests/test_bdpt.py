"""renderer::bdpt (src/renderer/renderer_bdpt.cpp:297-413 over include/lm/bidir.h): bidirectional
path tracing with every strategy weighted by the power heuristic.

CPU (oracle): BDPT and path tracing estimate the same image (Cornell box in both random streams;
spheres with glossy and glass materials, area lights and a constant environment); the white
furnace (known answer 1 everywhere); max_verts = 2 keeps only the camera's direct view of the
lights. Host: the renderer::bdpt props and argument checks.
GPU (through the C-ABI): the same samples as the oracle with matched Philox streams; the furnace;
a render split into calls with consecutive first_path equals one call; a two-level (instanced)
scene renders as its flattened build."""
import ctypes as C

import numpy as np
import pytest


def _blocks(a, by, bx):
    h, w = a.shape[:2]
    return a.reshape(by, h // by, bx, w // bx, 3).sum(axis=(1, 3))


def test_oracle_bdpt_matches_pt_box(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, _ = syn.box_scene(w=16, h=16, prefix="bdb_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt, _, _, _ = S.render_pt(16, 16, 2048, 6, seed=1)
    bd, rays, _ = S.render_bdpt(16, 16, 200_000, 6, seed=3)
    assert rays > 400_000
    assert abs(bd.sum() / pt.sum() - 1) < 0.01
    b1, b2 = _blocks(pt, 4, 4), _blocks(bd, 4, 4)
    assert (np.abs(b1 - b2) / b1).max() < 0.06
    bdm, _, _ = S.render_bdpt(16, 16, 200_000, 6, seed=3, rng="mt19937")   # the reference's own stream
    assert abs(bdm.sum() / pt.sum() - 1) < 0.01


def test_oracle_bdpt_matches_pt_spheres(lm, oracle_mod):
    """Glossy and glass vertices (specular vertices are never connected), six area lights and a
    constant environment (light subpaths from the bounding disk)."""
    from lightmetrica import synthetic as syn
    scene, _, _ = syn.spheres_scene(n_spheres=10, subdiv=3, ground_quads=8, w=16, h=12, prefix="bds_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt, _, _, _ = S.render_pt(16, 12, 4096, 7, seed=1)
    bd, _, _ = S.render_bdpt(16, 12, 400_000, 7, seed=3)
    assert abs(bd.mean() / pt.mean() - 1) < 0.01
    b1, b2 = _blocks(pt, 4, 4), _blocks(bd, 4, 4)
    assert (np.abs(b1 - b2) / b1).max() < 0.05


def test_oracle_bdpt_white_furnace(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, _ = syn.furnace_scene(w=32, h=32, prefix="bdf_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    bd, _, _ = S.render_bdpt(32, 32, 200_000, 5, seed=3)
    assert abs(bd.mean() - 1) < 0.01
    # max_verts 2: only camera -> light (s = 0, t = 2): the environment seen directly, 0 on the sphere
    direct, _, _ = S.render_bdpt(32, 32, 200_000, 2, seed=3)
    bg, _, _, _ = S.render_pt(32, 32, 64, 2, seed=1)
    assert abs(direct[bg.min(axis=2) == 1].mean() - 1) < 0.02
    assert direct[bg.max(axis=2) == 0].mean() < 0.01   # silhouette pixels may see some environment


@pytest.mark.parametrize("mode,n", [("bdptopt", 200_000), ("pt_naive_path", 2_000_000), ("pt_nee_path", 400_000),
                                    ("lt_nee_path", 1_000_000)])
def test_oracle_bidir_renderers_match_pt_box(lm, oracle_mod, mode, n):
    """The path-structure renderers (renderer_bdpt.cpp:63-288) and renderer::bdptopt estimate the
    path tracer's image where their strategies cover all transport: the closed box, one area
    light not seen directly, diffuse walls."""
    from lightmetrica import synthetic as syn
    scene, _ = syn.box_scene(w=16, h=16, prefix="bdm_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt, _, _, _ = S.render_pt(16, 16, 2048, 6, seed=1)
    img, _, _ = S.render_bdpt(16, 16, n, 6, seed=3, mode=mode)
    assert abs(img.mean() / pt.mean() - 1) < 0.02, img.mean() / pt.mean()


def test_renderer_bdpt_props(lm):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=8, h=8, prefix="bdp_")
    r = lm.load_renderer("bdp_r", "bdpt", scene=scene, output=film, max_verts=6, seed=2, scheduler="sample", num_samples=10)
    assert (r.num_samples, r.max_verts, r.min_verts, r.seed) == (10, 6, 2, 2)
    t = lm.load_renderer("bdp_t", "bdpt", scene=scene, output=film, min_verts=3, max_verts=6, scheduler="time", render_time=1)
    assert t.min_verts == 3 and t.samples_per_iter == 100000
    with pytest.raises(lm.LmGpuError):
        lm.load_renderer("bdp_x", "bdpt", scene=scene, output=film, max_verts=6, scheduler="spp", num_samples=1)


def test_bdpt_entry_refuses_bad_arguments(lm):
    from lightmetrica import _native as N
    p = N.BDPTParams()
    p.num_samples, p.max_verts = 10, 6
    assert N.lib().lmgpu_render_bdpt(None, None, C.byref(p), None, None) != 0


# ---------------------------------------------------------------------------------------------
# GPU

def _render_bdpt(lm, scene, film, n, max_verts, seed, name, **kw):
    lm.load_renderer(name, "bdpt", scene=scene, output=film, max_verts=max_verts, seed=seed, scheduler="sample",
                     num_samples=n, **kw).render()
    return film.buffer().astype(np.float64)


def _rel_l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


@pytest.mark.gpu
def test_bdpt_box_matches_oracle(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=32, h=32, prefix="bdg_")
    scene.build()
    gpu = _render_bdpt(lm, scene, film, 1 << 18, 8, 5, "bdg_r")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_bdpt(32, 32, 1 << 18, 8, seed=5)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 2e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
def test_bdpt_spheres_env_glass_matches_oracle(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.spheres_scene(n_spheres=10, subdiv=3, ground_quads=8, w=32, h=24, prefix="bdsg_")
    scene.build()
    gpu = _render_bdpt(lm, scene, film, 1 << 18, 8, 9, "bdsg_r", min_verts=2)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_bdpt(32, 24, 1 << 18, 8, seed=9)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 2e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["bdptopt", "pt_naive_path", "pt_nee_path", "lt_nee_path"])
def test_bidir_renderers_match_oracle(lm, oracle_mod, mode):
    """Each strategy mode against the oracle with matched streams on the spheres scene (glass
    vertices trigger pt_nee_path's s = 0 replacement; the environment and the glass are what
    pt_nee_path and lt_nee_path cannot reach, identically on both sides)."""
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.spheres_scene(n_spheres=10, subdiv=3, ground_quads=8, w=32, h=24, prefix="bdmg_")
    scene.build()
    lm.load_renderer("bdmg_" + mode, mode, scene=scene, output=film, max_verts=8, seed=9, scheduler="sample",
                     num_samples=1 << 18).render()
    gpu = film.buffer().astype(np.float64)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_bdpt(32, 24, 1 << 18, 8, seed=9, mode=mode)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 2e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
def test_bdpt_furnace_known_answer(lm, oracle_mod):
    """Only an environment light: light subpaths start on the bounding disk and s = 0 paths end on
    the environment."""
    from lightmetrica import synthetic as syn
    scene, film = syn.furnace_scene(w=32, h=32, prefix="bdfg_")
    scene.build()
    img = _render_bdpt(lm, scene, film, 1 << 20, 5, 3, "bdfg_r")
    assert abs(img.mean() - 1) < 0.01
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_bdpt(32, 32, 1 << 20, 5, seed=3)
    assert _rel_l1(img, ref) < 2e-3, _rel_l1(img, ref)


@pytest.mark.gpu
def test_bdpt_textured_env_instanced_matches_oracle(lm, oracle_mod):
    """A textured environment (light::env), area lights and a two-level accel against the oracle's
    flattened scene with the same random streams."""
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.instanced_scene(n_instances=6, n_lat=10, n_lon=14, n_lights=3, w=32, h=24, env_w=32, env_h=16,
                                         seed=11, spread=3.0, accel="embreeinstanced", prefix="bdo_")
    scene.build()
    gpu = _render_bdpt(lm, scene, film, 1 << 18, 6, 7, "bdo_r")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_bdpt(32, 24, 1 << 18, 6, seed=7)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 5e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
def test_bdpt_split_calls_equal_one_call(lm):
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=24, h=24, prefix="bdc_")
    scene.build()

    def call(n, first, acc):
        p = N.BDPTParams()
        p.num_samples, p.first_path, p.min_verts, p.max_verts, p.seed, p.accumulate = n, first, 2, 7, 11, acc
        st = N.RenderStats()
        N.check(N.lib().lmgpu_render_bdpt(scene._h, film._h, C.byref(p), None, C.byref(st)))
        return st

    st = call(100_000, 0, 0)
    assert st.paths == 100_000 and st.rays == st.extension_rays + st.shadow_rays > 200_000
    one = film.buffer().astype(np.float64)
    call(30_000, 0, 0)
    call(50_000, 30_000, 1)
    call(20_000, 80_000, 1)
    three = film.buffer().astype(np.float64)
    assert np.abs(one - three).max() <= 1e-5 * np.abs(one).max()


@pytest.mark.gpu
def test_bdpt_instanced_matches_flattened(lm):
    from lightmetrica import synthetic as syn
    out = []
    for accel, pre in (("embreeinstanced", "bdi_"), ("sahbvh", "bdj_")):
        scene, film, _ = syn.instanced_scene(n_instances=6, n_lat=10, n_lon=14, n_lights=3, w=32, h=24, env_w=32, env_h=16,
                                             seed=11, spread=3.0, accel=accel, prefix=pre)
        scene.build()
        out.append(_render_bdpt(lm, scene, film, 1 << 18, 7, 4, pre + "r"))
    a, b = out
    assert b.sum() > 0
    assert _rel_l1(a, b) < 0.02, _rel_l1(a, b)
    assert abs(a.sum() / b.sum() - 1) < 0.01
