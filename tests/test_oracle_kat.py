"""Pins the CPU oracle (the checker of the CUDA path) to known answers.

The reference holds no golden vectors for this path (its accel/renderer tests are visual
notebooks), so the oracle is pinned by: the published Philox4x32-10 known-answer vectors,
hand-built ray/triangle cases whose answers follow from geometry, agreement between the
restated SAH BVH and an exhaustive triangle test, and white-furnace renders whose expected pixel
value is known in closed form.
"""
import ctypes as C
import math

import numpy as np
import pytest


def _philox(O, c, k):
    L = O.lib()
    L.lmo_philox4x32.argtypes = [C.c_uint] * 6 + [C.POINTER(C.c_uint)]
    out = (C.c_uint * 4)()
    L.lmo_philox4x32(*c, *k, out)
    return list(out)


def test_philox_known_answers(oracle_mod):
    # Random123 kat_vectors for philox4x32 with 10 rounds
    assert _philox(oracle_mod, [0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert _philox(oracle_mod, [0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert _philox(oracle_mod, [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_philox_uniforms_in_unit_interval(oracle_mod):
    us = np.array([oracle_mod.philox_uniform(7, p, v, s) for p in range(64) for v in range(1, 4) for s in range(16)])
    assert us.min() >= 0.0 and us.max() < 1.0
    assert abs(us.mean() - 0.5) < 0.03


def _single_tri_scene(O, double, p):
    S = O.OracleScene(double)
    m = S.add_mesh(np.asarray(p, np.float32).reshape(3, 3), [[0, 0, 1]], [0, 1, 2], [0, 0, 0])
    mat = S.add_material(0, [1, 1, 1])
    S.add_child(0, S.primitive(m, mat))
    S.build(nthreads=1)
    return S


@pytest.mark.parametrize("double", [True, False])
def test_triangle_known_answers(oracle_mod, double):
    """Moller-Trumbore as accel_sahbvh.cpp:58-75: interior, edges, vertex, outside, parallel,
    behind, and the t == tmax boundary (accepted) / t < tmin (rejected)."""
    S = _single_tri_scene(oracle_mod, double, [0, 0, 0, 1, 0, 0, 0, 1, 0])

    def ray(ox, oy, dz=-1.0, tmin=1e-3, tmax=1e10, oz=1.0):
        return [ox, oy, oz, tmin, 0, 0, dz, tmax]
    rays = np.array([
        ray(0.25, 0.25),            # interior
        ray(0.5, 0.0),              # on edge v = 0
        ray(0.0, 0.5),              # on edge u = 0
        ray(0.5, 0.5),              # on edge u + v = 1
        ray(0.0, 0.0),              # vertex p1
        ray(0.6, 0.6),              # outside
        ray(0.25, 0.25, dz=1.0),    # pointing away: t = -1
        ray(0.25, 0.25, tmax=1.0),  # t == tmax: accepted
        ray(0.25, 0.25, tmin=1.5),  # t < tmin: rejected
        [0.25, 0.25, 1.0, 1e-3, 1.0, 0.0, 0.0, 1e10],  # parallel to the plane: |det| < 1e-8
    ], np.float32)
    t, uv, tri, _ = S.intersect(rays, nthreads=1)
    expect_hit = [True, True, True, True, True, False, False, True, False, False]
    assert list(tri >= 0) == expect_hit
    hit = tri >= 0
    assert np.allclose(t[hit], 1.0)
    assert np.allclose(uv[0], [0.25, 0.25])
    assert np.allclose(uv[1], [0.5, 0.0]) and np.allclose(uv[2], [0.0, 0.5])


def _random_soup(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    e = rng.uniform(-0.05, 0.05, (n, 2, 3))
    return np.stack([c, c + e[:, 0], c + e[:, 1]], 1).astype(np.float32)


def _soup_scene(O, tris, double, robust=False):
    S = O.OracleScene(double)
    ps = tris.reshape(-1, 3)
    n = len(tris)
    m = S.add_mesh(ps, [[0, 0, 1]], np.arange(3 * n, dtype=np.int32), np.zeros(3 * n, np.int32))
    mat = S.add_material(0, [1, 1, 1])
    S.add_child(0, S.primitive(m, mat))
    S.build(robust=robust)
    return S


@pytest.mark.parametrize("double,robust", [(True, False), (False, True)])
def test_sahbvh_matches_exhaustive(oracle_mod, double, robust):
    """The restated SAH BVH finds the same closest hit as testing every triangle (ties aside)."""
    tris = _random_soup(3000, 1)
    S = _soup_scene(oracle_mod, tris, double, robust)
    rng = np.random.default_rng(2)
    n = 4000
    o = rng.random((n, 3)) * 1.4 - 0.2
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, np.full((n, 1), 1e-3), d, np.full((n, 1), 1e10)], 1).astype(np.float32)
    t1, _, i1, _ = S.intersect(rays)
    t2, _, i2, _ = S.intersect(rays, brute=True)
    same = (i1 == i2) | ((i1 >= 0) & (i2 >= 0) & (t1 == t2))
    assert same.mean() == 1.0, f"{(~same).sum()} mismatches"
    assert (i1 >= 0).sum() > 500


def test_flatten_matches_transform_order(oracle_mod):
    """The oracle flattens group transforms as traverse_primitive_nodes does (scene.cpp:216-230):
    a translated instance lands at the translated position."""
    S = oracle_mod.OracleScene(True)
    m = S.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), [[0, 0, 1]], [0, 1, 2], [0, 0, 0])
    mat = S.add_material(0, [1, 1, 1])
    g = S.group(np.array([[1, 0, 0, 2], [0, 1, 0, 3], [0, 0, 1, 4], [0, 0, 0, 1]], np.float64))
    S.add_child(g, S.primitive(m, mat))
    S.add_child(0, g)
    S.build(nthreads=1)
    assert np.allclose(S.triangles()[0], [2, 3, 4, 1, 0, 0, 0, 1, 0])


@pytest.mark.parametrize("material", ["diffuse", "glass"])
def test_white_furnace(oracle_mod, lm, material):
    """Albedo-1 convex sphere (or lossless glass) under a constant environment of radiance 1: every
    pixel converges to 1 (renderer_pt.cpp with NEE + MIS)."""
    from lightmetrica import synthetic as syn
    scene, film = syn.furnace_scene(material, w=16, h=16, subdiv=3)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    img, _, rays, _ = S.render_pt(16, 16, 256, 64 if material == "glass" else 8, seed=3, rng="philox")
    assert rays > 0
    assert abs(img.mean() - 1.0) < 0.02, img.mean()


def test_reference_rng_stream_is_deterministic_single_thread(oracle_mod, lm):
    """With one thread and a seed the restated mt19937 stream is reproducible, as the reference is
    under num_threads=1."""
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=8, h=8)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build(nthreads=1)
    a, _, _, _ = S.render_pt(8, 8, 4, 9, seed=5, rng="mt19937", nthreads=1)
    b, _, _, _ = S.render_pt(8, 8, 4, 9, seed=5, rng="mt19937", nthreads=1)
    assert np.array_equal(a, b)
    assert a.sum() > 0


def test_sampling_modes_agree_in_expectation(oracle_mod, lm):
    """naive, NEE and MIS are unbiased estimators of the same image (renderer_pt.cpp:127-271)."""
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=8, h=8)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    means = {}
    for mode, spp in (("naive", 4096), ("nee", 512), ("mis", 512)):
        img, _, _, _ = S.render_pt(8, 8, spp, 9, seed=11, sampling_mode=mode, rng="philox")
        means[mode] = img.mean()
    assert abs(means["nee"] - means["mis"]) / means["mis"] < 0.03, means
    assert abs(means["naive"] - means["mis"]) / means["mis"] < 0.08, means


def test_primary_modes_agree_in_expectation(oracle_mod, lm):
    """Pixel and image primary-ray sampling estimate the same image: image mode's w*h*spp paths are
    rescaled by w*h / (paths) (renderer_pt.cpp:307-312 with scheduler::spi), i.e. by 1 / spp."""
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=8, h=8)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    pix, _, _, _ = S.render_pt(8, 8, 512, 9, seed=11, rng="philox")
    img, _, _, _ = S.render_pt(8, 8, 512, 9, seed=11, primary_mode="image", rng="philox")
    assert abs(img.mean() / pix.mean() - 1) < 0.03, (img.mean(), pix.mean())
