"""Parity of the CUDA path with the oracle (run on a GPU; every call goes through liblmgpu's C-ABI).

Bars:
* accel hits: bit-exact (triangle index, t, u, v) against the fp32 restatement of
  accel_sahbvh.cpp; exact-t ties (two triangles at identical t) are the only exemption. Against the
  fp64 faithful restatement: t within 1e-5 relative, and every index mismatch classified as a
  near-tie or an edge-grazing hit.
* renderer::raycast: pixel colors within 1e-4 absolute of the fp32 restatement.
* renderer::pt with the same Philox stream as the oracle (matched paths): image relative L1 error
  below 2e-3 against the fp64 restatement, per mode, material and light type.
* renderer::pt against the reference's own random stream (std::mt19937 per thread): per-pixel
  z-test at matched spp and normalized MSE = sum((x - ref)^2) / sum(ref^2) <= 1e-3 against the
  committed 16k-spp oracle image.
"""
import ctypes as C

import numpy as np
import pytest
from parity_util import classify_fp64_mismatches, compare_bitexact

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device(native_lib):
    from lightmetrica import _native as N
    N.check(native_lib.lmgpu_set_device(0))


def _soup_scene(lm, n, seed):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    e = rng.uniform(-0.03, 0.03, (n, 2, 3))
    tris = np.stack([c, c + e[:, 0], c + e[:, 1]], 1).astype(np.float32).reshape(-1, 3)
    scene = lm.load_scene("scene", "default", accel=lm.load_accel("accel", "sahbvh"))
    mesh = lm.load_mesh("soup", "raw", ps=tris, ns=[0, 0, 1], ts=[0, 0],
                        fs={"p": np.arange(3 * n), "n": np.zeros(3 * n, int), "t": np.zeros(3 * n, int)})
    scene.add_primitive(mesh=mesh, material=lm.load_material("m", "diffuse"))
    return scene


def _rays(n, seed, lo=-0.2, hi=1.2):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.concatenate([o, np.full((n, 1), 1e-3), d, np.full((n, 1), 1e10)], 1).astype(np.float32)
    r[:6, 4:7] = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, -0.0, -1]]
    return r


def test_intersect_bitexact_soup(lm, oracle_mod):
    scene = _soup_scene(lm, 20000, 1)
    scene._accel.build(scene)
    rays = _rays(200000, 2)
    gpu = scene._accel.intersect_batch(rays)
    S = oracle_mod.from_lm_scene(scene, double=False)
    S.build(robust=True)
    t, uv, ids, _ = S.intersect(rays, refine_t=True)
    assert (ids >= 0).mean() > 0.3
    ties = compare_bitexact(gpu, t, uv, ids, rays, S.triangles())
    assert ties <= 10


def test_intersect_edge_cases(lm, oracle_mod):
    """Rays through shared edges and vertices of a grid, grazing and axis-aligned rays."""
    from lightmetrica import synthetic as syn
    ps, ns, f = syn.ground_grid(16, 1.0)
    scene = lm.load_scene("scene", "default", accel=lm.load_accel("accel", "sahbvh"))
    mesh = lm.load_mesh("g", "raw", ps=ps, ns=ns, ts=[0, 0],
                        fs={"p": f.reshape(-1), "n": np.zeros(f.size, int), "t": np.zeros(f.size, int)})
    scene.add_primitive(mesh=mesh, material=lm.load_material("m", "diffuse"))
    scene._accel.build(scene)
    xs = np.linspace(-1, 1, 33).astype(np.float32)  # every vertex and edge midpoint line
    gx, gz = np.meshgrid(xs, xs)
    n = gx.size
    down = np.stack([gx.ravel(), np.full(n, 1.0), gz.ravel(), np.full(n, 1e-3), np.zeros(n), -np.ones(n), np.zeros(n),
                     np.full(n, 1e10)], 1).astype(np.float32)
    graze = down.copy()
    graze[:, 1] = 0.0          # origin in the plane, direction along it
    graze[:, 4:7] = [1, 0, 0]
    rays = np.concatenate([down, graze, _rays(2000, 3, -1.5, 1.5)])
    gpu = scene._accel.intersect_batch(rays)
    S = oracle_mod.from_lm_scene(scene, double=False)
    S.build(robust=True)
    t, uv, ids, _ = S.intersect(rays, brute=True, refine_t=True)
    compare_bitexact(gpu, t, uv, ids, rays, S.triangles())
    assert (gpu["prim"][:n] >= 0).all(), "every downward ray hits the closed grid"


def test_intersect_spheres_vs_fp32_and_fp64(lm, oracle_mod):
    """Uniform-sphere rays from a point inside a displaced-sphere scene (the raycast probe of the
    plain drop-in benchmark, at reduced size)."""
    from lightmetrica import synthetic as syn
    scene, film, info = syn.spheres_scene(n_spheres=6, subdiv=5, ground_quads=64, w=64, h=36)
    scene._accel.build(scene)
    rays = syn.sphere_rays(400000, [0.0, 1.0, 0.5], seed=5)
    gpu = scene._accel.intersect_batch(rays)
    S32 = oracle_mod.from_lm_scene(scene, double=False)
    S32.build(robust=True)
    t, uv, ids, _ = S32.intersect(rays, refine_t=True)
    compare_bitexact(gpu, t, uv, ids, rays, S32.triangles())
    # against the reference precision
    S64 = oracle_mod.from_lm_scene(scene, double=True)
    S64.build()
    t64, uv64, ids64, _ = S64.intersect(rays)
    g = gpu["prim"].astype(np.int64)
    both = (g >= 0) & (g == ids64)
    rel = np.abs(gpu["t"][both] - t64[both]) / t64[both]
    assert rel.max() <= 1e-5, rel.max()
    assert (g != ids64).mean() < 1e-3
    tri = scene._flatten()["positions"].reshape(-1, 3, 3).astype(np.float64)
    _, _, unexplained = classify_fp64_mismatches(rays, g, ids64, tri)
    assert not unexplained, unexplained[:10]


def test_occluded_matches_closest_hit(lm):
    scene = _soup_scene(lm, 5000, 4)
    scene._accel.build(scene)
    from lightmetrica import _native as N
    rays = _rays(50000, 6)
    rays[:, 7] = np.random.default_rng(7).uniform(0.01, 2.0, len(rays))  # finite tmax like shadow rays
    closest = scene._accel.intersect_batch(rays)
    import ctypes as C2
    L = N.lib()
    cudart = _cudart()
    d_rays = _dev_alloc(cudart, rays.nbytes)
    d_occ = _dev_alloc(cudart, len(rays))
    try:
        _h2d(cudart, d_rays, rays)
        N.check(L.lmgpu_accel_occluded_device(scene._accel._h, d_rays, len(rays), d_occ, None))
        occ = np.zeros(len(rays), np.uint8)
        _d2h(cudart, occ, d_occ)
    finally:
        cudart.cudaFree(d_rays)
        cudart.cudaFree(d_occ)
    assert np.array_equal(occ.astype(bool), closest["prim"] >= 0)
    del C2


def _cudart():
    import ctypes.util
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            lib = C.CDLL(name)
            break
        except OSError:
            lib = None
    if lib is None:
        import glob
        for p in glob.glob("/usr/local/cuda*/lib64/libcudart.so*"):
            try:
                lib = C.CDLL(p)
                break
            except OSError:
                pass
    assert lib is not None, "libcudart not found"
    lib.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    lib.cudaFree.argtypes = [C.c_void_p]
    return lib


def _dev_alloc(rt, nbytes):
    p = C.c_void_p()
    assert rt.cudaMalloc(C.byref(p), nbytes) == 0
    return p


def _h2d(rt, dst, arr):
    assert rt.cudaMemcpy(dst, arr.ctypes.data, arr.nbytes, 1) == 0


def _d2h(rt, arr, src):
    assert rt.cudaMemcpy(arr.ctypes.data, src, arr.nbytes, 2) == 0


def test_raycast_renderer_matches_oracle(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=64, h=64)
    scene.build()
    r = lm.load_renderer("rc", "raycast", scene=scene, output=film)
    r.render()
    img = film.buffer()
    S = oracle_mod.from_lm_scene(scene, double=False)
    S.build(robust=True)
    ref, _ = S.render_raycast(64, 64)
    assert np.abs(img - ref).max() < 1e-4
    # visualize_normal and a background color on a scene with misses
    r2 = lm.load_renderer("rc2", "raycast", scene=scene, output=film, visualize_normal=True)
    r2.render()
    ref2, _ = S.render_raycast(64, 64, visualize_normal=True)
    assert np.abs(film.buffer() - ref2).max() < 1e-4


def _pt_pair(lm, oracle_mod, scene, film, w, h, spp, max_verts, mode="mis", primary="pixel", seed=9):
    scene.build()
    r = lm.load_renderer("pt", "pt", scene=scene, output=film, max_verts=max_verts, seed=seed, sampling_mode=mode,
                         primary_ray_sampling_mode=primary, scheduler="sample", spp=spp)
    out = r.render()
    gpu = film.buffer()
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, _, rays, _ = S.render_pt(w, h, spp, max_verts, seed=seed, sampling_mode=mode, primary_mode=primary, rng="philox")
    return gpu, ref, out, rays


def _rel_l1(a, b):
    return np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-12)


@pytest.mark.parametrize("mode", ["mis", "nee", "naive"])
def test_pt_matched_stream_box(lm, oracle_mod, mode):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=32, h=32)
    gpu, ref, out, rays = _pt_pair(lm, oracle_mod, scene, film, 32, 32, 16, 9, mode=mode)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 2e-3, _rel_l1(gpu, ref)
    assert out["rays"] > 0


def test_pt_matched_stream_spheres(lm, oracle_mod):
    """Diffuse, GGX glossy and dielectric spheres, six area lights and a constant environment."""
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.spheres_scene(n_spheres=6, subdiv=3, ground_quads=16, w=48, h=27)
    gpu, ref, _, _ = _pt_pair(lm, oracle_mod, scene, film, 48, 27, 8, 11)
    assert _rel_l1(gpu, ref) < 2e-3, _rel_l1(gpu, ref)


def test_pt_matched_stream_env_map_and_mirror(lm, oracle_mod):
    """light::env (lat-long map with Dist2 importance sampling) and material::mirror."""
    from lightmetrica import synthetic as syn
    film = lm.load_film("film", "bitmap", w=40, h=30)
    cam = lm.load_camera("cam", "pinhole", position=[0, 1.5, 5], center=[0, 0.5, 0], up=[0, 1, 0], vfov=45, aspect=4 / 3)
    scene = lm.load_scene("scene", "default", accel=lm.load_accel("accel", "sahbvh"))
    scene.add_primitive(camera=cam)
    v, f = syn.icosphere(3)
    for k, (mat, cx) in enumerate([(lm.load_material("d", "diffuse", Kd=[0.8, 0.6, 0.4]), -1.2),
                                   (lm.load_material("mir", "mirror"), 1.2),
                                   (lm.load_material("gl", "glossy", Ks=[0.9, 0.9, 0.9], ax=0.2, ay=0.35), 0.0)]):
        p = (v * 0.5 + [cx, 0.5, 0]).astype(np.float32)
        mesh = lm.load_mesh(f"s{k}", "raw", ps=p, ns=v.astype(np.float32), ts=[0, 0],
                            fs={"p": f.ravel(), "n": f.ravel(), "t": np.zeros(f.size, int)})
        scene.add_primitive(mesh=mesh, material=mat)
    gp, gn, gf = syn.ground_grid(4, 4.0)
    ground = lm.load_mesh("ground", "raw", ps=gp, ns=gn, ts=[0, 0],
                          fs={"p": gf.ravel(), "n": np.zeros(gf.size, int), "t": np.zeros(gf.size, int)})
    scene.add_primitive(mesh=ground, material=lm.load_material("gm", "diffuse", Kd=[0.5, 0.5, 0.5]))
    scene.add_primitive(light=lm.load_light("env", "env", envmap=syn.env_texture(), rot=30, scale=1.5))
    gpu, ref, _, _ = _pt_pair(lm, oracle_mod, scene, film, 40, 30, 8, 6)
    assert ref.sum() > 0
    assert _rel_l1(gpu, ref) < 3e-3, _rel_l1(gpu, ref)


def test_pt_env_map_with_black_rows(lm, oracle_mod):
    """An env map with rows of zero luminance. The reference's Dist2 normalizes such a row by its
    zero sum (math.h Dist::init), so a BSDF-sampled direction into it has a NaN pdf_direct and
    renderer::pt with MIS writes NaN (the fp64 restatement reproduces it, pinned to the
    reference's own code). The GPU gives those rows zero density: its MIS weight is 1 there and
    the black texels add nothing. Every GPU pixel is finite, and the pixels the restatement
    renders finite agree on the matched stream."""
    from lightmetrica import synthetic as syn
    film = lm.load_film("film", "bitmap", w=40, h=30)
    cam = lm.load_camera("cam", "pinhole", position=[0, 1.5, 5], center=[0, 0.5, 0], up=[0, 1, 0], vfov=45, aspect=4 / 3)
    scene = lm.load_scene("scene", "default", accel=lm.load_accel("accel", "sahbvh"))
    scene.add_primitive(camera=cam)
    v, f = syn.icosphere(3)
    for k, (mat, cx) in enumerate([(lm.load_material("d", "diffuse", Kd=[0.8, 0.6, 0.4]), -1.2),
                                   (lm.load_material("gl", "glossy", Ks=[0.9, 0.9, 0.9], ax=0.2, ay=0.35), 1.2)]):
        p = (v * 0.5 + [cx, 0.5, 0]).astype(np.float32)
        mesh = lm.load_mesh(f"s{k}", "raw", ps=p, ns=v.astype(np.float32), ts=[0, 0],
                            fs={"p": f.ravel(), "n": f.ravel(), "t": np.zeros(f.size, int)})
        scene.add_primitive(mesh=mesh, material=mat)
    env = syn.env_texture().copy()
    env[: env.shape[0] // 4] = 0.0      # the lowest quarter of the sphere black
    env[env.shape[0] // 2] = 0.0        # and the row at the horizon
    scene.add_primitive(light=lm.load_light("env", "env", envmap=env, rot=30, scale=1.5))
    gpu, ref, _, _ = _pt_pair(lm, oracle_mod, scene, film, 40, 30, 8, 6)
    nan = np.isnan(ref).any(axis=2)
    assert nan.sum() > 10                # the case occurs on this scene
    assert np.isfinite(gpu).all()
    ok = ~nan
    assert _rel_l1(gpu[ok], ref[ok]) < 3e-3, _rel_l1(gpu[ok], ref[ok])


def test_pt_matched_stream_image_mode(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=24, h=24)
    gpu, ref, _, _ = _pt_pair(lm, oracle_mod, scene, film, 24, 24, 8, 6, primary="image")
    assert _rel_l1(gpu, ref) < 3e-3, _rel_l1(gpu, ref)


@pytest.mark.parametrize("material", ["diffuse", "glass"])
def test_pt_white_furnace(lm, material):
    from lightmetrica import synthetic as syn
    scene, film = syn.furnace_scene(material, w=32, h=32)
    scene.build()
    r = lm.load_renderer("pt", "pt", scene=scene, output=film, max_verts=64 if material == "glass" else 8, seed=1,
                         scheduler="sample", spp=256)
    r.render()
    assert abs(film.buffer().mean() - 1.0) < 0.01


def test_pt_ztest_against_reference_stream(lm, oracle_mod):
    """GPU (Philox) against the oracle with the reference's mt19937 stream, both at 256 spp: the
    per-pixel z statistic is approximately standard normal."""
    from lightmetrica import synthetic as syn
    W = H = 32
    scene, film = syn.box_scene(w=W, h=H)
    scene.build()
    reps = []
    for k in range(4):
        r = lm.load_renderer("pt", "pt", scene=scene, output=film, max_verts=9, seed=100 + k, scheduler="sample", spp=64)
        r.render()
        reps.append(film.buffer())
    gpu = np.mean(reps, 0)
    S = oracle_mod.from_lm_scene(scene, double=True)
    S.build()
    ref, m2, _, _ = S.render_pt(W, H, 256, 9, seed=77, rng="mt19937", with_m2=True)
    var = np.maximum(m2 / 256 - ref * ref, 0)
    z = (gpu - ref) / np.sqrt(2 * var / 256 + 1e-12)
    zz = z[var > 0]
    assert abs(zz.mean()) < 0.1, zz.mean()
    assert np.mean(np.abs(zz) > 4) < 0.005


def test_pt_relmse_vs_16k_reference(lm):
    import json
    import os
    gdir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    ref = np.load(os.path.join(gdir, "box_ref_16k.npy"))
    meta = json.load(open(os.path.join(gdir, "box_ref_16k.json")))
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(seed=1234, w=meta["w"], h=meta["h"])
    scene.build()
    r = lm.load_renderer("pt", "pt", scene=scene, output=film, max_verts=meta["max_verts"], seed=3, scheduler="sample",
                         spp=1024)
    r.render()
    img = film.buffer()
    rel_mse = np.sum((img - ref) ** 2) / np.sum(ref ** 2)
    assert rel_mse <= 1e-3, rel_mse


def test_pt_progressive_accumulation(lm):
    """Two 8-spp passes accumulated on the device equal the mean of the two separate renders."""
    from lightmetrica import synthetic as syn
    from lightmetrica import _native as N
    scene, film = syn.box_scene(w=16, h=16)
    scene.build()
    L = N.lib()
    imgs = []
    for seed in (5, 6):
        p = N.PTParams(); p.spp = 8; p.max_verts = 9; p.seed = seed; p.sampling_mode = 2
        N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(p), None, None))
        imgs.append(film.buffer())
    p = N.PTParams(); p.spp = 8; p.max_verts = 9; p.seed = 5; p.sampling_mode = 2
    N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(p), None, None))
    p.seed = 6; p.accumulate = 1
    N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(p), None, None))
    assert np.allclose(film.buffer(), 0.5 * (imgs[0] + imgs[1]), rtol=1e-5, atol=1e-6)


def test_pt_wave_size_invariance(lm):
    """The estimate does not depend on how many paths are in flight (RNG keyed per path)."""
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=16, h=16)
    scene.build()
    outs = []
    for wave in (0, 1000):
        r = lm.load_renderer("pt", "pt", scene=scene, output=film, max_verts=9, seed=4, scheduler="sample", spp=16,
                             wave_paths=wave)
        r.render()
        outs.append(film.buffer())
    assert np.allclose(outs[0], outs[1], rtol=1e-5, atol=1e-6)


def test_pt_engines_agree(lm, native_lib):
    """An instrumented render (fixed waves, one launch per bounce) and a plain one (the shared
    wavefront regenerating paths) give the same image: the same paths, summed in another order."""
    import ctypes as C
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    scene, film, _ = syn.spheres_scene(n_spheres=4, subdiv=3, ground_quads=8, w=40, h=24, prefix="eng_")
    scene.build()
    imgs = []
    for inst in (0, 1):
        p = N.PTParams()
        p.spp, p.max_verts, p.seed, p.sampling_mode, p.instrument = 12, 11, 21, 2, inst
        st = N.RenderStats()
        N.check(native_lib.lmgpu_render_pt(scene._h, film._h, C.byref(p), None, C.byref(st)))
        assert st.rays > 0 and st.extend_ms > 0
        imgs.append(film.buffer_f32().copy())
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-6)


def test_render_errors(lm):
    from lightmetrica import synthetic as syn
    scene, film = syn.box_scene(w=8, h=8)
    r = lm.load_renderer("pt", "pt", scene=scene, output=film, max_verts=5, scheduler="sample", spp=1)
    with pytest.raises(lm.LmGpuError):
        r.render()  # scene not built


def test_axis_aligned_rays_visit_few_nodes(lm):
    """Rays with exactly-zero direction components (straight down from a light, along a wall) are
    culled like any other ray: counted on the GPU, they visit a handful of nodes, not the tree."""
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    scene, film, info = syn.spheres_scene(n_spheres=6, subdiv=4, ground_quads=64, w=32, h=18)
    scene._accel.build(scene)
    rng = np.random.default_rng(9)
    n = 4096
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0] = rng.uniform(-10, 10, n)
    rays[:, 1] = 7.0
    rays[:, 2] = rng.uniform(-10, 10, n)
    rays[:, 3] = 1e-3
    rays[:, 5] = -1.0            # d = (0, -1, 0) exactly
    rays[:, 7] = 1e10
    rays[n // 2:, 1] = 0.5       # second half: horizontal rays d = (1, 0, 0) exactly
    rays[n // 2:, 4:7] = [1.0, 0.0, 0.0]
    rt = _cudart()
    d_rays = _dev_alloc(rt, rays.nbytes)
    try:
        _h2d(rt, d_rays, rays)
        mn, mt = C.c_double(), C.c_double()
        N.check(N.lib().lmgpu_accel_trace_counts(scene._accel._h, d_rays, n, 0, 1, C.byref(mn), C.byref(mt)))
    finally:
        rt.cudaFree(d_rays)
    st = scene._accel.stats()
    assert mn.value < 40, (mn.value, st["num_nodes"])
    hits = scene._accel.intersect_batch(rays)
    assert (hits["prim"][: n // 2] >= 0).all()  # every downward ray hits the ground


def test_intersect_host_buffers_pinned_and_pageable(lm):
    """Accel::intersect over host buffers (lmgpu_accel_intersect): page-locked buffers of more
    than 2^21 rays go in chunks over two streams (the last one short), pageable ones in one copy
    each way; both give the device-buffer call's hits exactly."""
    import numpy as np
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    scene, _, _ = syn.spheres_scene(n_spheres=8, subdiv=5, ground_quads=64, w=32, h=18, prefix="hb_")
    scene.build()
    acc = scene.accel()
    n = 5 * (1 << 20) + 12345
    rays = syn.sphere_rays(n, [0.0, 1.0, 0.5], seed=21)
    L = N.lib()
    rt = _cudart()
    rt.cudaMallocHost.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFreeHost.argtypes = [C.c_void_p]
    d_rays = _dev_alloc(rt, rays.nbytes)
    d_hits = _dev_alloc(rt, n * 16)
    h_rays, h_hits = C.c_void_p(), C.c_void_p()
    assert rt.cudaMallocHost(C.byref(h_rays), rays.nbytes) == 0
    assert rt.cudaMallocHost(C.byref(h_hits), n * 16) == 0
    try:
        _h2d(rt, d_rays, rays)
        N.check(L.lmgpu_accel_intersect_device(acc._h, d_rays, n, d_hits, None))
        dev = np.zeros(n * 4, np.float32)
        _d2h(rt, dev, d_hits)
        C.memmove(h_rays, rays.ctypes.data, rays.nbytes)
        N.check(L.lmgpu_accel_intersect(acc._h, C.cast(h_rays, C.POINTER(C.c_float)), n, C.cast(h_hits, C.POINTER(N.Hit))))
        pinned = np.frombuffer((C.c_char * (n * 16)).from_address(h_hits.value), dtype=np.float32).copy()
        pageable = np.zeros(n * 4, np.float32)
        N.check(L.lmgpu_accel_intersect(acc._h, rays.ctypes.data_as(C.POINTER(C.c_float)), n,
                                        pageable.ctypes.data_as(C.POINTER(N.Hit))))
        assert (dev.view(np.int32)[3::4] >= 0).mean() > 0.2
        assert np.array_equal(pinned.view(np.uint32), dev.view(np.uint32))
        assert np.array_equal(pageable.view(np.uint32), dev.view(np.uint32))
    finally:
        rt.cudaFreeHost(h_rays)
        rt.cudaFreeHost(h_hits)
        rt.cudaFree(d_rays)
        rt.cudaFree(d_hits)
