"""renderer::lt (src/renderer/renderer_lt.cpp:18-160): light tracing with connections to the camera.

CPU (oracle): light tracing and path tracing estimate the same image, so the oracle's light tracer
equals its path tracer minus the paths it cannot sample (camera -> light, two vertices) on the
Cornell box, in both random streams; the white furnace (a diffuse sphere of albedo 1 under a
constant environment of radiance 1, a known answer of 1 per covered pixel) pins the environment
light's rays from the scene's bounding disk (light_envconst.cpp:47-68); max_verts <= 2 gives no
connection. Host: the renderer::lt props (scheduler::spi::sample / time).
GPU (through the C-ABI): the same light paths as the oracle with matched Philox streams (area,
environment and textured environment lights, glossy and glass vertices in transport direction
LE); a render split into calls with consecutive first_path equals the single call; a two-level
(instanced) scene renders as its flattened build."""
import ctypes as C

import numpy as np
import pytest


def _blocks(a, k=4):
    h, w = a.shape[:2]
    return a.reshape(k, h // k, k, w // k, 3).sum(axis=(1, 3))


def test_oracle_lt_matches_pt_in_expectation(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, _ = syn.box_scene(w=16, h=16, prefix="ltpt_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pt6, _, _, _ = S.render_pt(16, 16, 1024, 6, seed=1)
    pt2, _, _, _ = S.render_pt(16, 16, 1024, 2, seed=1)
    ref = pt6 - pt2                     # paths of 3..6 vertices: what light tracing samples
    lt, rays, _ = S.render_lt(16, 16, 2_000_000, 6, seed=3)
    assert rays > 2_000_000
    assert abs(lt.sum() / ref.sum() - 1) < 0.02
    b1, b2 = _blocks(ref), _blocks(lt)
    assert (np.abs(b1 - b2) / b1).max() < 0.08
    lt_mt, _, _ = S.render_lt(16, 16, 2_000_000, 6, seed=3, rng="mt19937")   # the reference's own stream
    assert abs(lt_mt.sum() / ref.sum() - 1) < 0.02


def test_oracle_lt_white_furnace(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, _ = syn.furnace_scene(w=32, h=32, prefix="ltf_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    lt, _, _ = S.render_lt(32, 32, 4_000_000, 5, seed=3)
    bg, _, _, _ = S.render_pt(32, 32, 64, 2, seed=1)   # 1 where the environment is seen directly
    inside = bg.max(axis=2) == 0
    assert inside.sum() > 300
    assert abs(lt[inside].mean() - 1) < 0.01
    assert lt[bg.min(axis=2) == 1].mean() < 0.01


def test_oracle_lt_needs_three_vertices(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, _ = syn.box_scene(w=8, h=8, prefix="lt2_")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    lt, _, _ = S.render_lt(8, 8, 20000, 2, seed=3)
    assert not lt.any()


def test_renderer_lt_props(lm):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=8, h=8, prefix="ltp_")
    r = lm.load_renderer("ltp_r", "lt", scene=scene, output=film, max_verts=5, seed=2, scheduler="sample", num_samples=10)
    assert r.num_samples == 10 and r.max_verts == 5 and r.seed == 2
    t = lm.load_renderer("ltp_t", "lt", scene=scene, output=film, max_verts=5, scheduler="time", render_time=0.5)
    assert t.samples_per_iter == 100000 and t.render_time == 0.5
    with pytest.raises(lm.LmGpuError):
        lm.load_renderer("ltp_x", "lt", scene=scene, output=film, max_verts=5, scheduler="pixel", num_samples=1)
    with pytest.raises(lm.LmGpuError):
        lm.load_renderer("ltp_y", "lt", scene=scene, output=film, max_verts=5, scheduler="sample")  # no num_samples


def test_lt_entry_refuses_bad_arguments(lm):
    from lightmetrica import _native as N
    L = N.lib()
    p = N.LTParams()
    p.num_samples, p.max_verts = 10, 5
    assert L.lmgpu_render_lt(None, None, C.byref(p), None, None) != 0


# ---------------------------------------------------------------------------------------------
# GPU

def _render_lt(lm, scene, film, n, max_verts, seed, name):
    lm.load_renderer(name, "lt", scene=scene, output=film, max_verts=max_verts, seed=seed, scheduler="sample",
                     num_samples=n).render()
    return film.buffer().astype(np.float64)


def _rel_l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


@pytest.mark.gpu
def test_lt_box_matches_oracle(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=32, h=32, prefix="ltg_")
    scene.build()
    gpu = _render_lt(lm, scene, film, 1 << 20, 8, 5, "ltg_r")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_lt(32, 32, 1 << 20, 8, seed=5)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 1e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
def test_lt_spheres_env_glass_matches_oracle(lm, oracle_mod):
    """Area lights, a constant environment (rays from the bounding disk), glossy and glass
    spheres: glass refraction in transport direction LE has no eta^2."""
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.spheres_scene(n_spheres=10, subdiv=3, ground_quads=8, w=32, h=24, prefix="lts_")
    scene.build()
    gpu = _render_lt(lm, scene, film, 1 << 21, 8, 9, "lts_r")
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, _ = S.render_lt(32, 24, 1 << 21, 8, seed=9)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 1e-3, _rel_l1(gpu, ref)


@pytest.mark.gpu
def test_lt_furnace_known_answer(lm):
    from lightmetrica import synthetic as syn
    scene, film = syn.furnace_scene(w=32, h=32, prefix="ltfg_")
    scene.build()
    img = _render_lt(lm, scene, film, 1 << 22, 5, 3, "ltfg_r")
    lm.load_renderer("ltfg_pt", "pt", scene=scene, output=film, max_verts=2, spp=16, seed=1, scheduler="sample").render()
    bg = film.buffer()
    inside = bg.max(axis=2) == 0
    assert inside.sum() > 300
    assert abs(img[inside].mean() - 1) < 0.01


@pytest.mark.gpu
def test_lt_split_calls_equal_one_call(lm):
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=24, h=24, prefix="ltc_")
    scene.build()
    L = N.lib()

    def call(n, first, acc):
        p = N.LTParams()
        p.num_samples, p.first_path, p.max_verts, p.seed, p.accumulate = n, first, 7, 11, acc
        st = N.RenderStats()
        N.check(L.lmgpu_render_lt(scene._h, film._h, C.byref(p), None, C.byref(st)))
        return st

    st = call(300_000, 0, 0)
    assert st.paths == 300_000 and st.rays == st.extension_rays + st.shadow_rays > 300_000
    one = film.buffer().astype(np.float64)
    call(100_000, 0, 0)
    call(120_000, 100_000, 1)
    call(80_000, 220_000, 1)
    three = film.buffer().astype(np.float64)
    assert np.abs(one - three).max() <= 1e-5 * np.abs(one).max()
    # a different first_path is a different set of light paths
    call(300_000, 300_000, 0)
    other = film.buffer().astype(np.float64)
    assert np.abs(other - one).max() > 1e-3 * np.abs(one).max()


@pytest.mark.gpu
def test_lt_instanced_matches_flattened(lm):
    from lightmetrica import synthetic as syn
    out = []
    for accel, pre in (("embreeinstanced", "lti_"), ("sahbvh", "ltj_")):
        scene, film, _ = syn.instanced_scene(n_instances=6, n_lat=10, n_lon=14, n_lights=3, w=32, h=24, env_w=32, env_h=16,
                                             seed=11, spread=3.0, accel=accel, prefix=pre)
        scene.build()
        out.append(_render_lt(lm, scene, film, 1 << 20, 7, 4, pre + "r"))
    a, b = out
    assert b.sum() > 0
    # the same light paths on geometry that differs only by fp32 rounding
    assert _rel_l1(a, b) < 0.02, _rel_l1(a, b)
    assert abs(a.sum() / b.sum() - 1) < 0.01
