"""CPU checks of the product's 8-wide BVH (built by liblmgpu's host builder, no GPU needed):
structural invariants, conservative quantization, and a Python replica of the kernel's traversal
compared bit for bit with the oracle's exhaustive fp32 triangle test."""
import numpy as np
import pytest

import bvh8_sim as sim


def _soup(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)) * scale
    e = rng.uniform(-0.03, 0.03, (n, 2, 3)) * scale
    return np.stack([c, c + e[:, 0], c + e[:, 1]], 1).astype(np.float32).reshape(-1, 9)


def _subtree_ids(nodes, tris, i, memo):
    if i in memo:
        return memo[i]
    nd = sim.decode(nodes[i])
    internal = [s for s in range(8) if (nd["imask"] >> s) & 1]
    out = {}
    for s in range(8):
        if nd["meta"][s] == 0:
            continue
        if (nd["imask"] >> s) & 1:
            child = nd["child_base"] + internal.index(s)
            assert child > i, "children are stored after their parent"
            ids = [t for v in _subtree_ids(nodes, tris, child, memo).values() for t in v]
        else:
            cnt, off = nd["meta"][s] >> 5, nd["meta"][s] & 31
            assert 1 <= cnt <= 3
            ids = [int(tris[nd["tri_base"] + off + j][9:10].view(np.uint32)[0]) for j in range(cnt)]
        out[s] = ids
    memo[i] = out
    return out


def _check_structure(nodes, tris, tri_p):
    """Every triangle stored once with p1, e1 = p2 - p1, e2 = p3 - p1 rounded in fp32; every slot's
    dequantized box encloses the exact bounds of all triangles beneath it (quantized boxes of
    different levels are rounded in different frames and need not nest)."""
    n = tri_p.shape[0]
    ids = tris[:, 9].view(np.uint32).astype(np.int64)
    assert sorted(ids.tolist()) == list(range(n)), "every triangle exactly once"
    for rec in tris:
        v = tri_p[int(rec[9:10].view(np.uint32)[0])].reshape(3, 3)
        assert np.array_equal(rec[0:3], v[0])
        assert np.array_equal(rec[3:6], (v[1] - v[0]).astype(np.float32))
        assert np.array_equal(rec[6:9], (v[2] - v[0]).astype(np.float32))
    memo = {}
    for i in range(len(nodes)):
        nd = sim.decode(nodes[i])
        for s, tids in _subtree_ids(nodes, tris, i, memo).items():
            lo, hi = sim.child_box(nd, s)
            v = tri_p[tids].reshape(-1, 3)
            assert np.all(v.min(0) >= np.array(lo, np.float32)) and np.all(v.max(0) <= np.array(hi, np.float32))
            # the exact planes p + q*s sit at least one quantum outside the exact bounds
            for a in range(3):
                sc = float(nd["scale"][a])
                plo = float(nd["origin"][a]) + nd["qlo"][a][s] * sc
                phi = float(nd["origin"][a]) + nd["qhi"][a][s] * sc
                assert plo + sc <= float(v[:, a].min()) and phi - sc >= float(v[:, a].max())
        for s in range(8):
            if nd["meta"][s] == 0:
                assert not (nd["imask"] >> s) & 1


@pytest.mark.parametrize("n,scale", [(1, 1.0), (2, 1.0), (3, 1.0), (5, 1.0), (700, 1.0), (2000, 1000.0)])
def test_bvh8_structure(native_lib, n, scale):
    tri_p = _soup(n, n, scale)
    nodes, tris, depth = sim.build_host(native_lib, tri_p)
    assert depth >= 1 and len(nodes) >= 1
    _check_structure(nodes, tris, tri_p)


def test_bvh8_degenerate_inputs(native_lib):
    """Coincident triangles and a zero-extent axis still build a valid tree."""
    one = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    tri_p = np.tile(one, (50, 1))
    nodes, tris, depth = sim.build_host(native_lib, tri_p)
    _check_structure(nodes, tris, tri_p)
    flat = _soup(300, 4)
    flat[:, 2::3] = 0.5  # all z equal
    nodes, tris, depth = sim.build_host(native_lib, flat)
    _check_structure(nodes, tris, flat)


def test_bvh8_rejects_bad_input(native_lib):
    from lightmetrica import _native as N
    bad = _soup(4, 1)
    bad[2, 3] = np.nan
    with pytest.raises(N.LmGpuError):
        sim.build_host(native_lib, bad)
    with pytest.raises(N.LmGpuError):
        sim.build_host(native_lib, np.zeros((0, 9), np.float32))


def _rays(n, seed, lo=-0.2, hi=1.2):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.concatenate([o, np.full((n, 1), 1e-3), d, np.full((n, 1), 1e10)], 1).astype(np.float32)
    # a few axis-aligned and zero-component directions
    r[:8, 4:7] = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [0, -0.0, 1], [0.6, 0.8, 0]]
    return r


def test_traversal_replica_matches_exhaustive(native_lib, oracle_mod):
    """The kernel's traversal logic (replicated in Python) returns exactly the exhaustive fp32
    closest hit: same triangle (smallest index among equal t) and the same t, u, v bits."""
    tri_p = _soup(400, 9)
    nodes, tris, depth = sim.build_host(native_lib, tri_p)
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
        # any-hit agrees on occlusion
        occ = sim.trace(nodes, tris, depth, r, any_hit=True)[3] >= 0
        assert occ == (id_ref[i] >= 0)


def test_axis_aligned_rays_stay_cheap(native_lib):
    """Rays with exactly-zero direction components must be culled like any other ray: a straight-
    down ray over a ground grid visits a handful of nodes, not the whole tree."""
    from lightmetrica import synthetic as syn
    ps, ns, f = syn.ground_grid(64, 1.0)
    tri_p = ps[f].reshape(-1, 9).astype(np.float32)
    nodes, tris, depth = sim.build_host(native_lib, tri_p)
    rng = np.random.default_rng(0)
    for d in ([0, -1, 0], [1, 0, 0], [0, 0, -1], [0.6, 0, 0.8]):
        for _ in range(5):
            o = [rng.uniform(-0.9, 0.9), 0.5 if d[1] else 0.0, rng.uniform(-0.9, 0.9)]
            if d[1] == 0:
                o[1] = 0.25  # above the grid, parallel to it: must not touch every node
            ray = np.array([*o, 1e-3, *d, 1e10], np.float32)
            t, u, v, tid, visited = sim.trace(nodes, tris, depth, ray)
            assert visited <= 4 * depth + 16, (d, visited, len(nodes))


@pytest.mark.parametrize("width", [2, 4, 6])
def test_narrower_trees(native_lib, oracle_mod, width):
    """The "node_width" tuning key: the collapse uses at most `width` of a node's 8 slots; the
    layout's invariants hold and the traversal (replayed in Python) still returns the exhaustive
    closest hit."""
    from lightmetrica import _native as N
    N.check(native_lib.lmgpu_tune_set(b"node_width", width))
    try:
        tri_p = _soup(600, 21)
        nodes, tris, depth = sim.build_host(native_lib, tri_p)
    finally:
        N.check(native_lib.lmgpu_tune_set(b"node_width", 8))
    used = [sum(1 for m in sim.decode(w)["meta"] if m) for w in nodes]
    assert max(used) <= width and max(used) == width
    _check_structure(nodes, tris, tri_p)
    S = oracle_mod.OracleScene(False)
    n = len(tri_p)
    m = S.add_mesh(tri_p.reshape(-1, 3), [[0, 0, 1]], np.arange(3 * n, dtype=np.int32), np.zeros(3 * n, np.int32))
    S.add_child(0, S.primitive(m, S.add_material(0, [1, 1, 1])))
    S.build(robust=True)
    rays = _rays(150, 12)
    t_ref, _, id_ref, _ = S.intersect(rays, brute=True)
    for i, r in enumerate(rays):
        t, u, v, tid, _ = sim.trace(nodes, tris, depth, r)
        assert tid == id_ref[i]
        if tid >= 0:
            assert np.float32(t) == np.float32(t_ref[i])
    with pytest.raises(Exception):
        N.check(native_lib.lmgpu_tune_set(b"node_width", 9))
