"""Instancing: the two-level accel (accel::embreeinstanced semantics, accel_embree_instanced.cpp:
84-297) against the same scene flattened into one tree (accel::sahbvh semantics,
accel_sahbvh.cpp:132-151).

CPU: the instanced flattening (BLAS per instance group, one instance per path to it, identity
instance for the rest) reproduces the flattened world triangles; the C entry point refuses bad
arguments before touching the device. GPU: closest hits through the two-level tree agree with the
fp32 oracle on the flattened scene (same primitive node, face and t up to the rounding of the ray
transform); path-traced and raycast images agree with the flattened build; an instanced job renders
the same alone and inside a shared wavefront."""
import ctypes as C

import numpy as np
import pytest


def _scene(lm, n_instances=6, n_lat=10, n_lon=14, w=32, h=24, accel="embreeinstanced", prefix="inst_"):
    from lightmetrica import synthetic as syn
    return syn.instanced_scene(n_instances=n_instances, n_lat=n_lat, n_lon=n_lon, n_lights=3, w=w, h=h, env_w=32,
                               env_h=16, seed=11, spread=3.0, accel=accel, prefix=prefix)


def _world_of_instanced(g):
    """World-space triangles of an instanced flattening, in hit-index order (float64)."""
    out = []
    for b, m in g["instances"]:
        p = g["positions"][g["blas_offsets"][b]:g["blas_offsets"][b + 1]].reshape(-1, 3).astype(np.float64)
        out.append((p @ m[:3, :3].T + m[:3, 3]).reshape(-1, 9))
    return np.concatenate(out)


def test_instanced_flattening_matches_flat(lm):
    scene, _, info = _scene(lm)
    g = scene._flatten_instanced()
    f = scene._flatten()
    world = _world_of_instanced(g)
    assert world.shape == f["positions"].shape
    assert len(g["instances"]) == info["instances"] + 1          # + the identity instance
    assert g["instances"][0][0] == 0 and np.array_equal(g["instances"][0][1], np.eye(4))
    assert len(g["blas_offsets"]) - 1 <= 4                       # root + at most 3 shared groups
    # the same triangles (as a set): sort rows of both
    a = world[np.lexsort(world.T[::-1])]
    b = f["positions"].astype(np.float64)
    b = b[np.lexsort(b.T[::-1])]
    assert np.allclose(a, b, rtol=0, atol=2e-5)
    # BLAS records stay in the group's frame: 2 * n_lon * (n_lat - 1) triangles per shared mesh
    sizes = np.diff(g["blas_offsets"])
    assert (sizes[1:] == info["mesh_triangles"]).all()


def test_build_instanced_refuses_bad_input(native_lib):
    from lightmetrica import _native as N
    L = native_lib
    a = C.c_void_p()
    assert L.lmgpu_accel_create(C.byref(a)) == 0
    tri = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    offs = np.array([0, 1], np.int64)
    inst = (N.Instance * 1)()
    inst[0].blas = 0
    inst[0].transform[:] = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    fp = tri.ctypes.data_as(C.POINTER(C.c_float))
    op = offs.ctypes.data_as(C.POINTER(C.c_int64))
    assert L.lmgpu_accel_build_instanced(a, None, op, 1, inst, 1) == 1
    assert L.lmgpu_accel_build_instanced(a, fp, op, 0, inst, 1) == 1
    bad = np.array([0, 0], np.int64)
    assert L.lmgpu_accel_build_instanced(a, fp, bad.ctypes.data_as(C.POINTER(C.c_int64)), 1, inst, 1) == 1
    assert b"every BLAS" in L.lmgpu_last_error()
    inst[0].blas = 3
    assert L.lmgpu_accel_build_instanced(a, fp, op, 1, inst, 1) == 1
    assert b"missing BLAS" in L.lmgpu_last_error()
    inst[0].blas = 0
    inst[0].transform[:] = [1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0]
    assert L.lmgpu_accel_build_instanced(a, fp, op, 1, inst, 1) == 1
    assert b"singular" in L.lmgpu_last_error()
    inst[0].transform[:] = [float("nan"), 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    assert L.lmgpu_accel_build_instanced(a, fp, op, 1, inst, 1) == 1
    assert b"non-finite" in L.lmgpu_last_error()
    assert L.lmgpu_accel_destroy(a) == 0


# ---------------------------------------------------------------------------------------------
# GPU

def _node_face(tri_prim, prim_node):
    """(primitive node, face) of every triangle of a flattening in index order."""
    node = prim_node[tri_prim]
    first = np.zeros(len(tri_prim), np.int64)
    starts = np.r_[0, np.nonzero(np.diff(tri_prim))[0] + 1]
    for s, e in zip(starts, np.r_[starts[1:], len(tri_prim)]):
        first[s:e] = s
    return node, np.arange(len(tri_prim)) - first


@pytest.mark.gpu
def test_instanced_hits_match_flattened_oracle(lm, oracle_mod):
    from lightmetrica import synthetic as syn
    scene, _, _ = _scene(lm)
    scene.build()
    acc = scene.accel()
    st = acc.stats()
    assert st["num_instances"] == 7
    g = scene._flatten_instanced()
    f = scene._flatten()
    rays = syn.sphere_rays(60000, (0.3, 1.4, 0.2), seed=4)
    gpu = acc.intersect_batch(rays)
    S = oracle_mod.from_lm_scene(scene, double=False)
    S.build(robust=True)
    t_ref, _, r_id, _ = S.intersect(rays)
    g_id = gpu["prim"]
    assert ((g_id >= 0) == (r_id >= 0)).mean() > 0.999
    both = (g_id >= 0) & (r_id >= 0)
    # (node, face) of both sides; faces of a primitive are numbered from 0 in both orders
    n_i, f_i = _node_face(g["tri_prim"], g["prim_node"])
    offs = g["blas_offsets"]
    inst_node, inst_face = [], []
    for b, _ in g["instances"]:
        inst_node.append(n_i[offs[b]:offs[b + 1]])
        inst_face.append(f_i[offs[b]:offs[b + 1]])
    inst_node = np.concatenate(inst_node)
    inst_face = np.concatenate(inst_face)
    n_f, f_f = _node_face(f["tri_prim"], f["prim_node"])
    same = (inst_node[g_id[both]] == n_f[r_id[both]]) & (inst_face[g_id[both]] == f_f[r_id[both]])
    t_g, t_r = gpu["t"][both].astype(np.float64), t_ref[both].astype(np.float64)
    close = np.abs(t_g - t_r) <= 2e-5 * np.maximum(t_r, 1.0)
    assert close[same].all()
    # a different triangle only where the two hits are at (nearly) the same distance: an edge or a
    # near-tie resolved differently by the rounding of the ray transform
    assert (same | close).all()
    assert same.mean() > 0.995


@pytest.mark.gpu
def test_instanced_images_match_flattened(lm):
    s1, f1, _ = _scene(lm, accel="embreeinstanced", prefix="ia_")
    s1.build()
    s2, f2, _ = _scene(lm, accel="sahbvh", prefix="ib_")
    s2.build()
    assert s1.accel().stats()["num_instances"] > 0 and s2.accel().stats()["num_instances"] == 0
    assert s1.accel().stats()["device_bytes"] < s2.accel().stats()["device_bytes"]
    for s, f in ((s1, f1), (s2, f2)):
        lm.load_renderer(f"r_{id(f)}", "pt", scene=s, output=f, max_verts=8, spp=16, seed=3, scheduler="sample").render()
    a, b = f1.buffer_f32(), f2.buffer_f32()
    # the same random streams on geometry that differs only by fp32 rounding: most paths are
    # identical, a few diverge at grazing hits
    assert np.abs(a - b).mean() <= 0.02 * np.abs(b).mean()
    assert abs(a.mean() - b.mean()) <= 0.01 * b.mean()
    for s, f in ((s1, f1), (s2, f2)):
        lm.load_renderer(f"rc_{id(f)}", "raycast", scene=s, output=f).render()
    a, b = f1.buffer_f32(), f2.buffer_f32()
    assert (np.abs(a - b).max(axis=2) > 1e-3).mean() < 0.01


@pytest.mark.gpu
def test_instanced_job_same_alone_and_in_batch(lm):
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import BatchRenderer
    s1, f1, _ = _scene(lm, prefix="ib1_")
    s1.build()
    s2, f2 = syn.box_scene(w=20, h=20, prefix="ib2_")
    s2.build()
    alone = []
    for s, f, kw in ((s1, f1, dict(max_verts=8, spp=6, seed=5)), (s2, f2, dict(max_verts=7, spp=4, seed=9))):
        lm.load_renderer(f"ra_{id(f)}", "pt", scene=s, output=f, scheduler="sample", **kw).render()
        alone.append(f.buffer_f32().copy())
    b = BatchRenderer(queue_paths=700)
    b.render([dict(scene=s1, film=f1, max_verts=8, spp=6, seed=5), dict(scene=s2, film=f2, max_verts=7, spp=4, seed=9)])
    np.testing.assert_allclose(f1.buffer_f32(), alone[0], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(f2.buffer_f32(), alone[1], rtol=1e-5, atol=1e-6)
    b.close()
