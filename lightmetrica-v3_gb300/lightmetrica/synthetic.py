"""Seeded procedural scenes for the benchmark workloads and the parity tests.

The reference measures on external OBJ scenes that are not available; these generators stand in
with the shapes, sizes and value distributions of the benchmark configurations:

* box_scene      -- closed 1x1x1 box: 10 axis-aligned wall quads (20 triangles; red left wall,
                    green right wall, grey others, Lambertian albedo .75), two seed-placed rotated
                    inner boxes of 12 triangles, one 0.25 x 0.25 ceiling area light (Ke = 17),
                    pinhole camera with a 30 degree vertical field of view.
* spheres_scene  -- icospheres (subdivision 6 -> 81,920 triangles each) displaced by 3-octave value
                    noise of amplitude 0.05 on a 512 x 512-quad ground plane; 50 % diffuse, 30 %
                    GGX glossy (roughness ~ U(.05, .5)), 20 % dielectric (ior 1.5); 6 area lights
                    plus a constant environment. With the default 40 spheres the scene holds
                    3,801,088 triangles plus 12 light triangles.
* sphere_rays    -- rays from one point with directions uniform on the sphere (math.h:674-681).

Every scene is created through the `lightmetrica` API (lm.load_* and scene.add_primitive), so the
same objects feed the GPU renderers and, in the tests, the CPU oracle.
"""
from __future__ import annotations

import math

import numpy as np

import lightmetrica as lm


# ---------------------------------------------------------------------------------------------
# Geometry helpers

def quad(p0, p1, p2, p3, normal):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with a flat normal."""
    ps = np.array([p0, p1, p2, p3], dtype=np.float32)
    ns = np.array([normal], dtype=np.float32)
    return ps, ns, np.array([0, 1, 2, 0, 2, 3], np.int32), np.zeros(6, np.int32)


def merge(parts):
    ps, ns, fp, fn = [], [], [], []
    op = on = 0
    for p, n, f, g in parts:
        ps.append(p)
        ns.append(n)
        fp.append(f + op)
        fn.append(g + on)
        op += len(p)
        on += len(n)
    return np.concatenate(ps), np.concatenate(ns), np.concatenate(fp), np.concatenate(fn)


def load_mesh(name, ps, ns, fp, fn):
    return lm.load_mesh(name, "raw", ps=np.asarray(ps, np.float32), ns=np.asarray(ns, np.float32),
                        ts=np.zeros((1, 2), np.float32), fs={"p": fp, "n": fn, "t": np.zeros_like(fp)})


def cuboid(center, size, angle):
    """12-triangle box rotated about +y, outward flat normals."""
    c, s = math.cos(angle), math.sin(angle)
    R = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    hx, hy, hz = np.asarray(size) / 2
    corners = np.array([[x, y, z] for x in (-hx, hx) for y in (-hy, hy) for z in (-hz, hz)])
    idx = lambda x, y, z: (x > 0) * 4 + (y > 0) * 2 + (z > 0)  # noqa: E731
    faces = [  # (corner sign patterns counter-clockwise seen from outside, outward normal)
        ([(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)], (1, 0, 0)),
        ([(-1, -1, 1), (-1, 1, 1), (-1, 1, -1), (-1, -1, -1)], (-1, 0, 0)),
        ([(-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)], (0, 1, 0)),
        ([(-1, -1, 1), (-1, -1, -1), (1, -1, -1), (1, -1, 1)], (0, -1, 0)),
        ([(-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)], (0, 0, 1)),
        ([(1, -1, -1), (-1, -1, -1), (-1, 1, -1), (1, 1, -1)], (0, 0, -1)),
    ]
    parts = []
    for cs, n in faces:
        pts = [R @ corners[idx(*sgn)] + center for sgn in cs]
        parts.append(quad(*pts, normal=R @ np.asarray(n, float)))
    return merge(parts)


# ---------------------------------------------------------------------------------------------
# Box scene

def box_scene(seed: int = 1234, w: int = 256, h: int = 256, accel: str = "sahbvh", prefix: str = ""):
    """Closed Cornell-style box. Returns (scene, film). Asset names start with `prefix`, so several
    scenes can be resident at once (loading an existing name replaces that asset)."""
    rng = np.random.default_rng(seed)
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    camera = lm.load_camera(prefix + "camera", "pinhole", position=[0.5, 0.5, 0.99], center=[0.5, 0.5, 0.0], up=[0, 1, 0],
                            vfov=30, aspect=w / h)
    grey = lm.load_material(prefix + "grey", "diffuse", Kd=[0.75, 0.75, 0.75])
    red = lm.load_material(prefix + "red", "diffuse", Kd=[0.75, 0.25, 0.25])
    green = lm.load_material(prefix + "green", "diffuse", Kd=[0.25, 0.75, 0.25])
    black = lm.load_material(prefix + "black", "diffuse", Kd=[0.0, 0.0, 0.0])
    up, down = (0, 1, 0), (0, -1, 0)
    a, b = 0.375, 0.625
    grey_quads = [
        quad((0, 0, 0), (0, 0, 1), (0.5, 0, 1), (0.5, 0, 0), up),          # floor (two halves)
        quad((0.5, 0, 0), (0.5, 0, 1), (1, 0, 1), (1, 0, 0), up),
        quad((0, 1, 0), (1, 1, 0), (1, 1, a), (0, 1, a), down),            # ceiling frame around the light
        quad((0, 1, b), (1, 1, b), (1, 1, 1), (0, 1, 1), down),
        quad((0, 1, a), (a, 1, a), (a, 1, b), (0, 1, b), down),
        quad((b, 1, a), (1, 1, a), (1, 1, b), (b, 1, b), down),
        quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1)),       # back wall
        quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, -1)),      # front wall
    ]
    scene_accel = lm.load_accel(prefix + "accel", accel)
    scene = lm.load_scene(prefix + "scene", "default", accel=scene_accel)
    scene.add_primitive(camera=camera)
    m = load_mesh(prefix + "walls", *merge(grey_quads))
    scene.add_primitive(mesh=m, material=grey)
    scene.add_primitive(mesh=load_mesh(prefix + "left", *quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0))), material=red)
    scene.add_primitive(mesh=load_mesh(prefix + "right", *quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0), (-1, 0, 0))), material=green)
    # two inner boxes, placed and rotated from the seed
    tall = cuboid((0.33 + rng.uniform(-0.05, 0.05), 0.3, 0.33 + rng.uniform(-0.05, 0.05)), (0.28, 0.6, 0.28), rng.uniform(0.2, 0.5))
    short = cuboid((0.68 + rng.uniform(-0.05, 0.05), 0.15, 0.62 + rng.uniform(-0.05, 0.05)), (0.28, 0.3, 0.28), -rng.uniform(0.2, 0.5))
    scene.add_primitive(mesh=load_mesh(prefix + "tall", *tall), material=grey)
    scene.add_primitive(mesh=load_mesh(prefix + "short", *short), material=grey)
    # ceiling light, slightly below the ceiling plane, facing down
    ly = 1.0 - 1e-4
    lmesh = load_mesh(prefix + "light_mesh", *quad((a, ly, a), (b, ly, a), (b, ly, b), (a, ly, b), down))
    light = lm.load_light(prefix + "light", "area", Ke=[17, 17, 17], mesh=lmesh)
    scene.add_primitive(mesh=lmesh, material=black, light=light)
    return scene, film


# ---------------------------------------------------------------------------------------------
# Spheres on a ground plane

_ICO_V = None


def icosphere(subdiv: int):
    """Unit icosphere: 20 * 4^subdiv faces; returns (ps (n,3) float64, faces (m,3) int32)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
                  [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        a = base + inv[:nf]
        b = base + inv[nf:2 * nf]
        c = base + inv[2 * nf:]
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([f[:, 1], b, a], 1),
                            np.stack([f[:, 2], c, b], 1), np.stack([a, b, c], 1)])
    return v, f.astype(np.int32)


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Trilinearly interpolated lattice noise in [-1, 1] with smoothstep weights."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256).astype(np.int64)
    vals = rng.uniform(-1.0, 1.0, 256)
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    wgt = pf * pf * (3 - 2 * pf)

    def lat(ix, iy, iz):
        return vals[perm[(perm[(perm[ix & 255] + iy) & 255] + iz) & 255]]

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wx = wgt[:, 0] if dx else 1 - wgt[:, 0]
                wy = wgt[:, 1] if dy else 1 - wgt[:, 1]
                wz = wgt[:, 2] if dz else 1 - wgt[:, 2]
                out = out + wx * wy * wz * lat(pi[:, 0] + dx, pi[:, 1] + dy, pi[:, 2] + dz)
    return out


def displaced_sphere(subdiv: int, center, radius: float, amplitude: float, seed: int, freq: float = 3.0):
    v, f = icosphere(subdiv)
    d = np.zeros(len(v))
    for o in range(3):
        d += (0.5 ** o) * value_noise(v * freq * (2 ** o), seed + 17 * o)
    d *= amplitude / 1.75
    p = v * (radius * (1.0 + d))[:, None] + np.asarray(center)[None, :]
    # area-weighted vertex normals of the displaced surface
    fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    vn = np.zeros_like(p)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    return p.astype(np.float32), vn.astype(np.float32), f


def ground_grid(n: int, half: float, y: float = 0.0):
    xs = np.linspace(-half, half, n + 1)
    gx, gz = np.meshgrid(xs, xs, indexing="ij")
    ps = np.stack([gx.reshape(-1), np.full(gx.size, y), gz.reshape(-1)], 1).astype(np.float32)
    i = np.arange(n)[:, None] * (n + 1) + np.arange(n)[None, :]
    i = i.reshape(-1)
    a, b, c, d = i, i + (n + 1), i + (n + 1) + 1, i + 1
    f = np.concatenate([np.stack([a, d, c], 1), np.stack([a, c, b], 1)]).astype(np.int32)
    return ps, np.array([[0, 1, 0]], np.float32), f


SPHERES_CAMERA = dict(position=[0.0, 4.0, 15.0], center=[0.0, 0.6, 0.0], up=[0, 1, 0], vfov=40)


def spheres_parts(seed: int = 7, n_spheres: int = 40, subdiv: int = 6, ground_quads: int = 512, w: int = 1920,
                  h: int = 1080, env_le: float = 0.3, half: float = 12.0) -> dict:
    """The displaced-sphere scene as plain data (no library call): camera props, and primitives
    in scene order, each {"name", "mesh": (ps, ns, fp, fn) or None, "material": (kind, props) or
    None, "light": (kind, props) or None}. spheres_scene builds the `lightmetrica` scene from it;
    a CPU restatement can build its own scene from the same data."""
    rng = np.random.default_rng(seed)
    prims = []
    gp, gn, gf = ground_grid(ground_quads, half)
    prims.append({"name": "ground", "mesh": (gp, gn, gf.reshape(-1), np.zeros(gf.size, np.int32)),
                  "material": ("diffuse", {"Kd": [0.6, 0.6, 0.6]}), "light": None})
    kinds = np.array(["diffuse"] * int(round(0.5 * n_spheres)) + ["glossy"] * int(round(0.3 * n_spheres)))
    kinds = np.concatenate([kinds, np.array(["glass"] * (n_spheres - len(kinds)))])
    rng.shuffle(kinds)
    centers = []
    tris = gf.shape[0]
    for i in range(n_spheres):
        for _ in range(1000):
            r = rng.uniform(0.4, 1.0)
            c = np.array([rng.uniform(-half + 1.5, half - 1.5), r * 1.06, rng.uniform(-half + 1.5, half - 1.5)])
            if all(np.linalg.norm(c - c2) > r + r2 + 0.15 for c2, r2 in centers):
                break
        centers.append((c, r))
        p, n, f = displaced_sphere(subdiv, c, r, 0.05, seed * 1000 + i)
        if kinds[i] == "diffuse":
            mat = ("diffuse", {"Kd": rng.uniform(0.2, 0.9, 3)})
        elif kinds[i] == "glossy":
            rough = rng.uniform(0.05, 0.5)
            mat = ("glossy", {"Ks": rng.uniform(0.5, 0.95, 3), "ax": rough, "ay": rough})
        else:
            mat = ("glass", {"Ni": 1.5})
        prims.append({"name": f"sphere{i}", "mesh": (p, n, f.reshape(-1), f.reshape(-1)), "material": mat,
                      "light": None})
        tris += f.shape[0]
    for k in range(6):
        ang = 2 * math.pi * k / 6 + rng.uniform(-0.2, 0.2)
        cx, cz, y, s = 6.0 * math.cos(ang), 6.0 * math.sin(ang), rng.uniform(6.0, 8.0), 0.75
        prims.append({"name": f"light{k}", "mesh": quad((cx - s, y, cz - s), (cx + s, y, cz - s), (cx + s, y, cz + s),
                                                        (cx - s, y, cz + s), (0, -1, 0)),
                      "material": ("diffuse", {"Kd": [0, 0, 0]}),
                      "light": ("area", {"Ke": list(rng.uniform(8.0, 16.0, 3))})})
        tris += 2
    if env_le > 0:
        prims.append({"name": "env", "mesh": None, "material": None,
                      "light": ("envconst", {"Le": [env_le, env_le, env_le * 1.1]})})
    camera = dict(SPHERES_CAMERA, aspect=w / h)
    return {"camera": camera, "primitives": prims, "w": w, "h": h,
            "info": {"triangles": tris, "spheres": n_spheres, "subdiv": subdiv, "ground_quads": ground_quads}}


def spheres_scene(seed: int = 7, n_spheres: int = 40, subdiv: int = 6, ground_quads: int = 512, w: int = 1920,
                  h: int = 1080, accel: str = "sahbvh", env_le: float = 0.3, half: float = 12.0, prefix: str = ""):
    """Displaced icospheres on a ground plane. Returns (scene, film, info dict). Asset names start
    with `prefix`."""
    d = spheres_parts(seed, n_spheres, subdiv, ground_quads, w, h, env_le, half)
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    camera = lm.load_camera(prefix + "camera", "pinhole", **d["camera"])
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", accel))
    scene.add_primitive(camera=camera)
    mats = {}
    for pr in d["primitives"]:
        mesh = mat = light = None
        if pr["mesh"] is not None:
            ps, ns, fp, fn = pr["mesh"]
            mesh = lm.load_mesh(prefix + pr["name"] + ("_mesh" if pr["light"] else ""), "raw",
                                ps=np.asarray(ps, np.float32), ns=np.asarray(ns, np.float32),
                                ts=np.zeros((1, 2), np.float32),
                                fs={"p": np.asarray(fp, np.int32), "n": np.asarray(fn, np.int32),
                                    "t": np.zeros(len(fp), np.int32)})
        if pr["material"] is not None:
            kind, props = pr["material"]
            if pr["light"] is not None:  # every light quad shares one black material
                if "light_mat" not in mats:
                    mats["light_mat"] = lm.load_material(prefix + "light_mat", kind, **props)
                mat = mats["light_mat"]
            else:
                name = "ground_mat" if pr["name"] == "ground" else "mat" + pr["name"][len("sphere"):]
                mat = lm.load_material(prefix + name, kind, **props)
        if pr["light"] is not None:
            kind, props = pr["light"]
            light = lm.load_light(prefix + pr["name"], kind, **(dict(props, mesh=mesh) if kind == "area" else props))
        scene.add_primitive(mesh=mesh, material=mat, light=light)
    return scene, film, d["info"]


# The raycast probe of the plain drop-in workload: 2^24 rays with directions uniform on the sphere
# from one point inside the displaced-sphere scene's bounding box (above the ground, between the
# spheres).
RAYCAST_PROBE_ORIGIN = (0.0, 1.0, 0.5)
RAYCAST_PROBE_RAYS = 1 << 24
RAYCAST_PROBE_SEED = 11


def sphere_rays(n: int, origin, seed: int = 11, tmin: float = 1e-3, tmax: float = 1e10) -> np.ndarray:
    """n x 8 float32 rays (o, tmin, d, tmax) with directions uniform on the sphere
    (math::sample_uniform_sphere, math.h:674-681), from a fixed origin."""
    rng = np.random.default_rng(seed)
    u = rng.random((n, 2))
    z = 1.0 - 2.0 * u[:, 0]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    t = 2.0 * math.pi * u[:, 1]
    d = np.stack([r * np.cos(t), r * np.sin(t), z], 1)
    out = np.empty((n, 8), np.float32)
    out[:, 0:3] = np.asarray(origin, np.float32)
    out[:, 3] = tmin
    out[:, 4:7] = d.astype(np.float32)
    out[:, 7] = tmax
    return out


def furnace_scene(material: str = "diffuse", w: int = 32, h: int = 32, subdiv: int = 3, prefix: str = ""):
    """White furnace: a unit sphere of albedo 1 (or glass) inside a constant environment of
    radiance 1. Every pixel's expected value is 1 for a convex diffuse sphere."""
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    camera = lm.load_camera(prefix + "camera", "pinhole", position=[0, 0, 4], center=[0, 0, 0], up=[0, 1, 0], vfov=40, aspect=w / h)
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", "sahbvh"))
    scene.add_primitive(camera=camera)
    v, f = icosphere(subdiv)
    mesh = lm.load_mesh(prefix + "sphere", "raw", ps=v.astype(np.float32), ns=v.astype(np.float32), ts=np.zeros((1, 2), np.float32),
                        fs={"p": f.reshape(-1), "n": f.reshape(-1), "t": np.zeros(f.size, np.int32)})
    if material == "diffuse":
        mat = lm.load_material(prefix + "mat", "diffuse", Kd=[1, 1, 1])
    else:
        mat = lm.load_material(prefix + "mat", "glass", Ni=1.5)
    scene.add_primitive(mesh=mesh, material=mat)
    scene.add_primitive(light=lm.load_light(prefix + "env", "envconst", Le=[1, 1, 1]))
    return scene, film


def env_texture(w: int = 64, h: int = 32, seed: int = 5) -> np.ndarray:
    """Procedural lat-long HDR texture with log-normal radiance and a bright sun region."""
    rng = np.random.default_rng(seed)
    base = np.exp(rng.normal(-1.0, 0.7, (h, w, 1))).astype(np.float32) * np.array([0.9, 1.0, 1.1], np.float32)
    base[int(h * 0.75):int(h * 0.85), int(w * 0.2):int(w * 0.3)] *= 40.0
    return np.ascontiguousarray(base.astype(np.float32))


# ---------------------------------------------------------------------------------------------
# Many small independent jobs (the batched and served workloads)

BATCH_RESOLUTIONS = (64, 128, 256, 512)


def random_triangles(n: int, rng) -> tuple[np.ndarray, np.ndarray]:
    """n independent triangles: centres U[0,1]^3, each corner at distance U(.001,.03) from the
    centre in a uniform random direction. Returns (positions (3n,3), flat normals (n,3))."""
    c = rng.random((n, 1, 3))
    d = rng.normal(size=(n, 3, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    r = rng.uniform(0.001, 0.03, (n, 3, 1))
    p = (c + d * r).astype(np.float32)
    gn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]).astype(np.float64)
    ln = np.linalg.norm(gn, axis=1, keepdims=True)
    gn = np.where(ln > 0, gn / np.where(ln > 0, ln, 1), np.array([0.0, 0.0, 1.0]))
    return p.reshape(-1, 3), gn.astype(np.float32)


def triangles_scene(seed: int, n_tris: int, w: int, h: int, accel: str = "sahbvh", prefix: str = ""):
    """One batched-workload scene: `n_tris` random triangles in the unit cube split 50/30/20 %
    over diffuse, GGX glossy and dielectric materials, a 0.5 x 0.5 area light above the cube, a
    constant environment, and a pinhole camera looking at the cube. Returns (scene, film)."""
    rng = np.random.default_rng(seed)
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    camera = lm.load_camera(prefix + "camera", "pinhole", position=[0.5, 0.6, 2.3], center=[0.5, 0.5, 0.5],
                            up=[0, 1, 0], vfov=40, aspect=w / h)
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", accel))
    scene.add_primitive(camera=camera)
    p, gn = random_triangles(n_tris, rng)
    kinds = rng.choice(3, size=n_tris, p=[0.5, 0.3, 0.2])
    rough = rng.uniform(0.05, 0.5)
    mats = [lm.load_material(prefix + "diffuse", "diffuse", Kd=list(rng.uniform(0.2, 0.9, 3))),
            lm.load_material(prefix + "glossy", "glossy", Ks=list(rng.uniform(0.5, 0.95, 3)), ax=rough, ay=rough),
            lm.load_material(prefix + "glass", "glass", Ni=1.5)]
    for k in range(3):
        sel = np.nonzero(kinds == k)[0]
        if len(sel) == 0:
            continue
        ps = p.reshape(-1, 3, 3)[sel].reshape(-1, 3)
        fp = np.arange(3 * len(sel), dtype=np.int32)
        fn = np.repeat(np.arange(len(sel), dtype=np.int32), 3)
        mesh = lm.load_mesh(prefix + f"tris{k}", "raw", ps=ps, ns=gn[sel], ts=np.zeros((1, 2), np.float32),
                            fs={"p": fp, "n": fn, "t": np.zeros_like(fp)})
        scene.add_primitive(mesh=mesh, material=mats[k])
    a, b, y = 0.25, 0.75, 1.3
    lmesh = load_mesh(prefix + "light_mesh", *quad((a, y, a), (b, y, a), (b, y, b), (a, y, b), (0, -1, 0)))
    light = lm.load_light(prefix + "light", "area", Ke=list(rng.uniform(6.0, 12.0, 3)), mesh=lmesh)
    scene.add_primitive(mesh=lmesh, material=lm.load_material(prefix + "light_mat", "diffuse", Kd=[0, 0, 0]), light=light)
    scene.add_primitive(light=lm.load_light(prefix + "env", "envconst", Le=[0.4, 0.45, 0.5]))
    return scene, film


def batch_jobs(n_jobs: int = 256, seed: int = 2024, min_tris: int = 1000, max_tris: int = 200000):
    """Job specs of the batched workload: per job a scene seed, a triangle count log-uniform in
    [min_tris, max_tris], a square resolution from BATCH_RESOLUTIONS, spp U{4..64} and a maximum
    path length U{6..12} (max_verts = length + 1)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n_jobs):
        jobs.append({
            "scene_seed": int(rng.integers(0, 2**31)),
            "tris": int(np.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))),
            "res": int(rng.choice(BATCH_RESOLUTIONS)),
            "spp": int(rng.integers(4, 65)),
            "max_verts": int(rng.integers(6, 13)) + 1,
            "seed": int(rng.integers(0, 2**31)),
        })
    return jobs


def served_requests(n: int, rate: float, n_scenes: int, seed: int = 77, refine_frac: float = 0.3,
                    refine_spp: int = 16):
    """Poisson request stream: `n` requests at `rate` per second. A request renders one of
    `n_scenes` batched-workload scenes (resolution, spp and length drawn as in batch_jobs), or
    with probability `refine_frac` adds `refine_spp` samples to an earlier request's film.
    Returns dicts with arrival (s from the start), scene, res, spp, max_verts, seed, refine."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        fresh = [r for r in out if r["refine"] is None]
        if fresh and rng.random() < refine_frac:
            base = fresh[int(rng.integers(0, len(fresh)))]
            out.append({"rid": i, "arrival": t, "scene": base["scene"], "res": base["res"], "spp": refine_spp,
                        "max_verts": base["max_verts"], "seed": int(rng.integers(0, 2**31)), "refine": base["rid"]})
        else:
            out.append({"rid": i, "arrival": t, "scene": int(rng.integers(0, n_scenes)),
                        "res": int(rng.choice(BATCH_RESOLUTIONS)), "spp": int(rng.integers(4, 65)),
                        "max_verts": int(rng.integers(6, 13)) + 1, "seed": int(rng.integers(0, 2**31)), "refine": None})
    return out


# ---------------------------------------------------------------------------------------------
# Instancing (the instanced stress workload)

def displaced_uv_sphere(n_lat: int, n_lon: int, amplitude: float = 0.05, seed: int = 3):
    """Unit UV sphere of 2 * n_lon * (n_lat - 1) triangles displaced by 3-octave value noise.
    Returns (positions (v, 3), vertex normals (v, 3), faces (f, 3))."""
    th = np.linspace(0.0, math.pi, n_lat + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, n_lon, endpoint=False)
    st, ct = np.sin(th), np.cos(th)
    v = np.stack([np.outer(st, np.cos(ph)), np.repeat(ct[:, None], n_lon, 1), np.outer(st, np.sin(ph))], -1).reshape(-1, 3)
    d = np.zeros(len(v))
    for o in range(3):
        d += (0.5 ** o) * value_noise(v * 3.0 * (2 ** o), seed + 17 * o)
    p = v * (1.0 + d * amplitude / 1.75)[:, None]
    faces = []
    for i in range(n_lat):
        a = i * n_lon + np.arange(n_lon)
        b = i * n_lon + (np.arange(n_lon) + 1) % n_lon
        c, e = a + n_lon, b + n_lon
        if i > 0:
            faces.append(np.stack([a, b, e], 1))
        if i < n_lat - 1:
            faces.append(np.stack([a, e, c], 1))
    f = np.concatenate(faces).astype(np.int64)
    fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    keep = np.linalg.norm(fn, axis=1) > 0  # the pole rows collapse to points
    f, fn = f[keep], fn[keep]
    vn = np.zeros_like(p)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    return p.astype(np.float32), vn.astype(np.float32), f.astype(np.int32)


def random_affine(rng, spread: float) -> np.ndarray:
    """4x4 world-from-local: random rotation, anisotropic scale U(.4, 1.1), translation
    U(-spread, spread) in x/z and U(.5, 2.5) in y."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R @ np.diag(rng.uniform(0.4, 1.1, 3))
    M[:3, 3] = [rng.uniform(-spread, spread), rng.uniform(0.5, 2.5), rng.uniform(-spread, spread)]
    return M


def instanced_scene(n_instances: int = 64, n_lat: int = 500, n_lon: int = 500, n_lights: int = 16, w: int = 4096,
                    h: int = 2160, env_w: int = 1024, env_h: int = 512, seed: int = 5, spread: float = 8.0,
                    accel: str = "embreeinstanced", prefix: str = ""):
    """`n_instances` instances of one displaced UV-sphere mesh (2 * n_lon * (n_lat - 1) triangles,
    about 500k by default) under seed-drawn affine transforms, a ground plane, `n_lights` small
    area lights and a procedural lat-long environment (log-normal radiance) of env_w x env_h texels.
    Each instance is its own instance group (scene.create_instance_group_node); they all share
    the mesh's group. Returns (scene, film, info)."""
    rng = np.random.default_rng(seed)
    film = lm.load_film(prefix + "film", "bitmap", w=w, h=h)
    camera = lm.load_camera(prefix + "camera", "pinhole", position=[0.0, 6.0, 22.0], center=[0.0, 1.0, 0.0],
                            up=[0, 1, 0], vfov=40, aspect=w / h)
    scene = lm.load_scene(prefix + "scene", "default", accel=lm.load_accel(prefix + "accel", accel))
    scene.add_primitive(camera=camera)
    gp, gn, gf = ground_grid(8, spread * 1.6)
    ground = lm.load_mesh(prefix + "ground", "raw", ps=gp, ns=gn, ts=np.zeros((1, 2), np.float32),
                          fs={"p": gf.reshape(-1), "n": np.zeros(gf.size, np.int32), "t": np.zeros(gf.size, np.int32)})
    scene.add_primitive(mesh=ground, material=lm.load_material(prefix + "ground_mat", "diffuse", Kd=[0.55, 0.55, 0.5]))
    p, vn, f = displaced_uv_sphere(n_lat, n_lon, seed=seed)
    mesh = lm.load_mesh(prefix + "inst_mesh", "raw", ps=p, ns=vn, ts=np.zeros((1, 2), np.float32),
                        fs={"p": f.reshape(-1), "n": f.reshape(-1), "t": np.zeros(f.size, np.int32)})
    mats = [lm.load_material(prefix + "inst_diffuse", "diffuse", Kd=[0.7, 0.45, 0.3]),
            lm.load_material(prefix + "inst_glossy", "glossy", Ks=[0.8, 0.8, 0.85], ax=0.15, ay=0.15),
            lm.load_material(prefix + "inst_glass", "glass", Ni=1.5)]
    # one shared group per material, instanced n_instances times in all
    groups = []
    for k, mat in enumerate(mats):
        g = scene.create_instance_group_node()
        scene.add_child(g, scene.create_primitive_node(mesh=mesh, material=mat))
        groups.append(g)
    for i in range(n_instances):
        t = scene.create_group_node(random_affine(rng, spread))
        scene.add_child(t, groups[int(rng.choice(3, p=[0.5, 0.3, 0.2]))])
        scene.add_child(scene.root_node(), t)
    black = lm.load_material(prefix + "light_mat", "diffuse", Kd=[0, 0, 0])
    for k in range(n_lights):
        cx, cz = rng.uniform(-spread, spread, 2)
        y, s = rng.uniform(5.0, 8.0), 0.35
        lmesh = load_mesh(prefix + f"light_mesh{k}", *quad((cx - s, y, cz - s), (cx + s, y, cz - s), (cx + s, y, cz + s),
                                                          (cx - s, y, cz + s), (0, -1, 0)))
        light = lm.load_light(prefix + f"light{k}", "area", Ke=list(rng.uniform(10.0, 30.0, 3)), mesh=lmesh)
        scene.add_primitive(mesh=lmesh, material=black, light=light)
    lm.load_texture(prefix + "env_tex", "bitmap", data=env_texture(env_w, env_h, seed=seed))
    scene.add_primitive(light=lm.load_light(prefix + "env", "env", envmap="$.assets." + prefix + "env_tex", rot=30.0))
    tris = n_instances * f.shape[0] + gf.shape[0] + 2 * n_lights
    return scene, film, {"instances": n_instances, "mesh_triangles": int(f.shape[0]), "triangles": int(tris)}
