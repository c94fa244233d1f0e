"""The GPU builder of the 8-wide tree (LMGPU_BUILDER_GPU_PLOC: Morton order, PLOC clustering,
SAH-optimal collapse, quantization on the device) against the layout's invariants and against the
host builder. Closest hits do not depend on the tree (the traversal's tie rule is the smaller
triangle index), so a tree from either builder must give bit-identical hits, and the same images.
Reference: the accel's build step, accel_sahbvh.cpp:127-267."""
import numpy as np
import pytest

import bvh8_sim as sim
from test_bvh_host import _check_structure, _rays, _soup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device(native_lib):
    from lightmetrica import _native as N
    N.check(native_lib.lmgpu_set_device(0))


@pytest.mark.parametrize("n,scale", [(1, 1.0), (2, 1.0), (3, 1.0), (5, 1.0), (700, 1.0), (2000, 1000.0)])
def test_gpu_tree_structure(native_lib, n, scale):
    tri_p = _soup(n, n + 3, scale)
    nodes, tris, depth = sim.build_gpu(native_lib, tri_p)
    assert depth >= 1 and len(nodes) >= 1
    _check_structure(nodes, tris, tri_p)


def test_gpu_tree_replica_matches_exhaustive(native_lib, oracle_mod):
    """The kernel's traversal (replicated in Python) over the GPU-built arrays returns the
    exhaustive fp32 closest hit, bit for bit."""
    tri_p = _soup(400, 9)
    nodes, tris, depth = sim.build_gpu(native_lib, tri_p)
    S = oracle_mod.OracleScene(False)
    n = len(tri_p)
    m = S.add_mesh(tri_p.reshape(-1, 3), [[0, 0, 1]], np.arange(3 * n, dtype=np.int32), np.zeros(3 * n, np.int32))
    S.add_child(0, S.primitive(m, S.add_material(0, [1, 1, 1])))
    S.build(robust=True)
    rays = _rays(300, 10)
    t_ref, uv_ref, id_ref, _ = S.intersect(rays, brute=True)
    for i, r in enumerate(rays):
        t, u, v, tid, _ = sim.trace(nodes, tris, depth, r)
        assert tid == id_ref[i], (i, tid, id_ref[i])
        if tid >= 0:
            assert np.float32(t) == np.float32(t_ref[i])
            assert np.float32(u) == np.float32(uv_ref[i, 0]) and np.float32(v) == np.float32(uv_ref[i, 1])


def test_gpu_builder_rejects_bad_input(native_lib):
    from lightmetrica import _native as N
    import ctypes as C
    tri = _soup(10, 1)
    tri[3, 4] = np.nan
    nodes = np.zeros(20 * 10, np.uint32)
    tris = np.zeros(12 * 10, np.float32)
    nn, depth = C.c_int64(), C.c_int32()
    rc = native_lib.lmgpu_bvh8_build_gpu(N.fptr(tri), 10, nodes.ctypes.data_as(C.POINTER(C.c_uint32)), N.fptr(tris),
                                         C.byref(nn), C.byref(depth))
    assert rc == 1 and b"non-finite" in native_lib.lmgpu_last_error()
    rc = native_lib.lmgpu_bvh8_build_gpu(N.fptr(tri), 0, nodes.ctypes.data_as(C.POINTER(C.c_uint32)), N.fptr(tris),
                                         C.byref(nn), C.byref(depth))
    assert rc == 1


def _hits_both(lm, scene, rays):
    out = {}
    for b in ("sah", "ploc"):
        acc = lm.load_accel(f"acc_{b}_{id(scene)}", "sahbvh", builder=b)
        acc.build(scene)
        out[b] = acc.intersect_batch(rays)
        out[b + "_stats"] = acc.stats()
        acc._release()
    return out


def test_gpu_builder_same_hits_as_host_builder(lm):
    """Bit-identical hits (triangle, t, u, v) from the two builders on a triangle soup and on the
    displaced-sphere scene (grazing rays, shared edges)."""
    from lightmetrica import synthetic as syn
    scene, _, _ = syn.spheres_scene(n_spheres=6, subdiv=5, ground_quads=64, w=64, h=36, prefix="bg_")
    rays = syn.sphere_rays(400000, [0.0, 1.0, 0.5], seed=5)
    h = _hits_both(lm, scene, rays)
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(h["sah"][k], h["ploc"][k]), k
    print("SAH cost: host", h["sah_stats"]["sah_cost"], "gpu", h["ploc_stats"]["sah_cost"])


def test_gpu_builder_same_image(lm):
    """renderer::pt on a tree from either builder: the same paths and hits, so the same image up to
    the order of fp32 film additions."""
    from lightmetrica import synthetic as syn
    imgs = []
    for b in ("sah", "ploc"):
        scene, film, _ = syn.spheres_scene(n_spheres=4, subdiv=3, ground_quads=8, w=40, h=24, prefix=f"bi_{b}_")
        scene._accel.builder = b
        scene.build()
        r = lm.load_renderer(f"pt_{b}", "pt", scene=scene, output=film, max_verts=11, seed=3, scheduler="sample", spp=8)
        r.render()
        imgs.append(film.buffer_f32().copy())
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-6)


def test_gpu_builder_plain_drop_in_scene(lm):
    """The full displaced-sphere scene (3,801,100 triangles): the GPU build's hits equal the host
    build's on 2^20 probe rays; the build times are printed."""
    import time
    from lightmetrica import synthetic as syn
    scene, _, info = syn.spheres_scene(prefix="bg2_")
    rays = syn.sphere_rays(1 << 20, syn.RAYCAST_PROBE_ORIGIN, seed=syn.RAYCAST_PROBE_SEED)
    tri_p = scene._flatten()["positions"]
    hits = {}
    for b in ("sah", "ploc"):
        acc = lm.load_accel(f"acc2_{b}", "sahbvh", builder=b)
        t = time.perf_counter()
        acc.build_triangles(tri_p)
        secs = time.perf_counter() - t
        st = acc.stats()
        print(f"{b}: {info['triangles']} triangles built in {secs:.3f} s, {st['num_nodes']} nodes, depth "
              f"{st['max_depth']}, SAH cost {st['sah_cost']:.2f}")
        hits[b] = acc.intersect_batch(rays)
        acc._release()
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(hits["sah"][k], hits["ploc"][k]), k


def test_gpu_builder_instanced_same_hits(lm):
    """Two-level trees whose bottom levels come from either builder give bit-identical hits."""
    from lightmetrica import synthetic as syn
    rays = syn.sphere_rays(100000, [0.0, 2.0, 0.0], seed=8)
    hits = []
    for b in ("sah", "ploc"):
        scene, _, _ = syn.instanced_scene(n_instances=6, n_lat=10, n_lon=14, n_lights=2, w=16, h=12, env_w=16, env_h=8,
                                          seed=11, spread=3.0, prefix=f"ib_{b}_")
        scene._accel.builder = b
        scene._accel.build(scene)
        assert scene._accel.stats()["num_instances"] > 1
        hits.append(scene._accel.intersect_batch(rays))
    assert (hits[0]["prim"] >= 0).mean() > 0.05
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(hits[0][k], hits[1][k]), k


def test_transformed_scene_against_reference_fixture(lm, oracle_mod):
    """Nested group transforms, shared edges, duplicated and degenerate triangles, axis-parallel
    and vertex-aimed rays (tests/ref_scenes.py): the hits of trees from either builder against the
    reference's own hits (accel_sahbvh.cpp compiled from its sources, committed as
    tests/golden/ref_transformed_hits.npz) within fp32's error bounds, and bit for bit against the
    fp32 restatement's exhaustive test (exact-t ties exempt). Exhaustive, because rays aimed exactly
    at a triangle's corner can be accepted by the fp32 Moller-Trumbore test a rounding error outside
    the triangle's bounding box: the restated binary BVH's slab test culls some of those hits, the
    kernel's outward-rounded boxes do not."""
    import os

    import ref_scenes as RS
    from parity_util import check_against_fp64, compare_bitexact
    desc = RS.transformed_scene()
    scene = RS.to_lm(lm, desc, "rfx_")
    rays = RS.pin_rays(desc)
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_transformed_hits.npz"))
    S32 = RS.to_oracle(oracle_mod, desc, double=False)
    S32.build(robust=True)
    t32, uv32, ids32, _ = S32.intersect(rays, brute=True, refine_t=True)
    tri32 = S32.triangles()
    tri = scene._flatten()["positions"].reshape(-1, 3, 3).astype(np.float64)
    h = _hits_both(lm, scene, rays)
    for b in ("sah", "ploc"):
        hits, mism, near, graze = check_against_fp64(h[b], fx["t"], fx["uv"], fx["tri"], rays, tri, b)
        ties = compare_bitexact(h[b], t32, uv32, ids32, rays, tri32)
        print(f"{b}: {hits} reference hits, {mism} index mismatches ({near} near-ties, {graze} grazing); "
              f"{ties} exact-t ties against fp32")
        assert hits > 8000
