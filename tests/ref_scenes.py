"""Scene and ray sets for pinning the accel path to the reference's own code (test
infrastructure).

`transformed_scene` is a scene graph with nested group transforms (rotations, non-uniform
scales, translations) over a ground grid (shared edges, an axis-aligned plane), displaced
spheres, a triangle soup with duplicated triangles (exact-t ties) and degenerate ones, and an
axis-aligned cube (rays along its edges and faces). `pin_rays` mixes random rays with the cases a
slab test and a triangle test are sensitive to: directions with zero components, origins on
bounding planes, rays aimed at vertices and edge midpoints, and narrow [tmin, tmax] windows.

The description is plain data so that the reference library (oracle/ref.py), the oracle and the
`lightmetrica` scene graph are built from the same nodes in the same order.
"""
from __future__ import annotations

import math

import numpy as np


def _rot(angle, axis):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    c, s = math.cos(angle), math.sin(angle)
    x, y, z = a
    m = np.eye(4)
    m[:3, :3] = [[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                 [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                 [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]]
    return m


def _tr(v):
    m = np.eye(4)
    m[:3, 3] = v
    return m


def _sc(v):
    return np.diag([v[0], v[1], v[2], 1.0])


def _cube():
    p = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)], np.float32)
    q = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    f = []
    for a, b, c, d in q:
        f += [(a, b, c), (a, c, d)]
    return p, np.asarray(f, np.int32)


def transformed_scene(seed: int = 3) -> dict:
    """{"meshes": [(ps float32 (n,3), faces int32 (m,3))], "nodes": [...]} with nodes in creation
    order after the root group 0: ("group", m4 row-major or None, parent) or ("prim", mesh, parent)."""
    from lightmetrica import synthetic as syn
    rng = np.random.default_rng(seed)
    meshes = []
    gp, _, gf = syn.ground_grid(16, 4.0)
    meshes.append((gp, gf))
    sp, _, sf = syn.displaced_sphere(3, (0.0, 0.0, 0.0), 0.8, 0.05, seed)
    meshes.append((sp, sf.astype(np.int32)))
    soup, _ = syn.random_triangles(400, rng)
    soup = soup.reshape(400, 3, 3)
    soup[360:400] = soup[0:40]                               # exact duplicates: exact-t ties
    soup[350:360, 2] = 2 * soup[350:360, 1] - soup[350:360, 0]  # collinear corners: degenerate
    meshes.append((soup.reshape(-1, 3), np.arange(1200, dtype=np.int32).reshape(-1, 3)))
    meshes.append(_cube())
    nodes = [
        ("group", _tr([0.0, 1.0, 0.0]) @ _rot(math.radians(30), [1, 1, 0]), 0),  # 1
        ("prim", 1, 1),                                                          # 2: sphere
        ("group", _sc([2.0, 0.5, 1.0]), 0),                                      # 3
        ("group", _tr([-1.0, 1.5, -0.5]), 3),                                    # 4
        ("prim", 2, 4),                                                          # 5: soup
        ("prim", 0, 0),                                                          # 6: ground
        ("group", _tr([2.0, 0.5, 1.0]) @ _rot(math.radians(90), [0, 1, 0]), 0),  # 7
        ("prim", 3, 7),                                                          # 8: cube
        ("group", _tr([-2.5, 1.2, 2.0]) @ _sc([0.7, 1.3, 0.7]), 0),              # 9
        ("prim", 1, 9),                                                          # 10: sphere again
    ]
    return {"meshes": meshes, "nodes": nodes}


def world_triangles(desc: dict) -> np.ndarray:
    """(n, 3, 3) float64 world-space corners in the flattening order (depth first from the
    root, children in insertion order), as the reference's traversal visits them."""
    children = {0: []}
    kinds = {0: ("group", None)}
    for i, (kind, a, parent) in enumerate(desc["nodes"], start=1):
        kinds[i] = (kind, a)
        children.setdefault(i, [])
        children[parent].append(i)
    out = []

    def visit(i, M):
        kind, a = kinds[i]
        if kind == "prim":
            ps, f = desc["meshes"][a]
            p = np.c_[ps.astype(np.float64), np.ones(len(ps))] @ M.T
            out.append(p[:, :3][f])
            return
        L = M @ a if a is not None else M
        for c in children[i]:
            visit(c, L)

    visit(0, np.eye(4))
    return np.concatenate(out)


def to_ref(desc: dict):
    from oracle import ref as R
    S = R.RefScene()
    mesh_ids = [S.add_mesh(ps, f) for ps, f in desc["meshes"]]
    for kind, a, parent in desc["nodes"]:
        n = S.group(a) if kind == "group" else S.primitive(mesh_ids[a])
        S.add_child(parent, n)
    return S


def to_oracle(oracle_mod, desc: dict, double: bool = True):
    O = oracle_mod.OracleScene(double)
    mat = O.add_material(oracle_mod.MAT["material::diffuse"], [0.5, 0.5, 0.5])
    nrm = np.array([[0, 1, 0]], np.float32)
    mesh_ids = [O.add_mesh(ps, nrm, f.reshape(-1), np.zeros(f.size, np.int32)) for ps, f in desc["meshes"]]
    for kind, a, parent in desc["nodes"]:
        n = O.group(a) if kind == "group" else O.primitive(mesh_ids[a], mat, -1, -1)
        O.add_child(parent, n)
    return O


def to_lm(lm, desc: dict, prefix: str):
    """The same graph as a `lightmetrica` scene (groups through create_group_node)."""
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", "sahbvh"))
    mat = lm.load_material(prefix + "mat", "diffuse", Kd=[0.5, 0.5, 0.5])
    meshes = []
    for k, (ps, f) in enumerate(desc["meshes"]):
        fl = f.reshape(-1).astype(np.int32)
        meshes.append(lm.load_mesh(f"{prefix}mesh{k}", "raw", ps=ps, ns=np.array([[0, 1, 0]], np.float32),
                                   ts=np.zeros((1, 2), np.float32),
                                   fs={"p": fl, "t": np.zeros_like(fl), "n": np.zeros_like(fl)}))
    for kind, a, parent in desc["nodes"]:
        n = scene.create_group_node(a) if kind == "group" else scene.create_primitive_node(mesh=meshes[a], material=mat)
        scene.add_child(parent, n)
    return scene


def pin_rays(desc: dict, n: int = 16000, seed: int = 5) -> np.ndarray:
    """n x 8 float32 rays (o, tmin, d, tmax)."""
    rng = np.random.default_rng(seed)
    tri = world_triangles(desc)
    k = n // 8
    o = rng.uniform(-5, 5, (n, 3))
    d = rng.normal(size=(n, 3))
    tmin = np.zeros(n)
    tmax = np.full(n, 1e10)
    # aimed at vertices and at edge midpoints
    pick = rng.integers(0, len(tri), 2 * k)
    corner = rng.integers(0, 3, 2 * k)
    target = tri[pick, corner]
    target[k:] = 0.5 * (target[k:] + tri[pick[k:], (corner[k:] + 1) % 3])
    d[:2 * k] = target - o[:2 * k]
    # axis-parallel directions, half of them from origins on the ground plane (y = 0)
    ax = rng.integers(0, 3, k)
    d[2 * k:3 * k] = 0.0
    d[2 * k + np.arange(k), ax] = rng.choice([-1.0, 1.0], k)
    o[2 * k:2 * k + k // 2, 1] = 0.0
    # rays lying in the cube's face planes and along its edges (cube at (2, 0.5, 1), unit size)
    o[3 * k:4 * k] = [2.0, 0.5, 1.0] + rng.choice([-0.5, 0.5], (k, 3))
    o[3 * k:4 * k, 0] = rng.uniform(-5, 5, k)
    d[3 * k:4 * k] = [1.0, 0.0, 0.0]
    # narrow [tmin, tmax] windows around the distance to a triangle's centroid (some exclude it)
    cen = tri[rng.integers(0, len(tri), k)].mean(axis=1)
    d[4 * k:5 * k] = cen - o[4 * k:5 * k]
    dist = np.linalg.norm(d[4 * k:5 * k], axis=1)
    tmin[4 * k:5 * k] = dist * (1 - rng.uniform(-0.002, 0.01, k))
    tmax[4 * k:5 * k] = dist * (1 + rng.uniform(-0.002, 0.01, k))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.empty((n, 8), np.float32)
    out[:, 0:3] = o
    out[:, 3] = tmin
    out[:, 4:7] = d
    out[:, 7] = tmax
    return out
