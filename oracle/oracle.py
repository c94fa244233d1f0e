"""Oracle (test infrastructure only): ctypes wrapper of the CPU restatement (liblmoracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import this
module, to check or to time against the CUDA path. It builds the oracle's own scene from the
same `lightmetrica` scene graph (meshes in local space, group transforms, lights, camera) so the
oracle flattens and transforms the scene itself, as the reference's Scene_ and Accel_SAHBVH do.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblmoracle.so")

_lib = None


def build() -> str:
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, dp, fp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int)
        L.lmo_last_error.restype = C.c_char_p
        L.lmo_create.restype = vp
        L.lmo_create.argtypes = [C.c_int]
        L.lmo_destroy.argtypes = [vp]
        L.lmo_add_mesh.argtypes = [vp, fp, C.c_int, fp, C.c_int, fp, C.c_int, ip, ip, ip, C.c_int]
        L.lmo_add_material.argtypes = [vp, C.c_int, dp]
        L.lmo_add_texture.argtypes = [vp, fp, C.c_int, C.c_int, C.c_int]
        L.lmo_set_material_textures.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.lmo_add_light_area.argtypes = [vp, dp, C.c_int]
        L.lmo_add_light_envconst.argtypes = [vp, dp]
        L.lmo_add_light_point.argtypes = [vp, dp, dp]
        L.lmo_add_light_directional.argtypes = [vp, dp, dp]
        L.lmo_add_light_env.argtypes = [vp, fp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
        L.lmo_add_camera.argtypes = [vp, dp, dp, dp, C.c_double, C.c_double]
        L.lmo_create_primitive_node.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.lmo_create_group_node.argtypes = [vp, dp]
        L.lmo_create_instance_group_node.argtypes = [vp]
        L.lmo_add_child.argtypes = [vp, C.c_int, C.c_int]
        L.lmo_build.argtypes = [vp, C.c_int, C.c_int, dp]
        L.lmo_num_triangles.argtypes = [vp]
        L.lmo_get_triangles.argtypes = [vp, fp]
        L.lmo_intersect.argtypes = [vp, fp, C.c_longlong, dp, dp, ip, C.c_int, C.c_int, C.c_int, dp]
        L.lmo_render_raycast.argtypes = [vp, C.c_int, C.c_int, dp, C.c_int, C.c_int, dp, dp, C.c_int, dp]
        L.lmo_render_pt.argtypes = [vp, C.c_int, C.c_int, C.c_longlong, C.c_int, C.c_uint, C.c_int, C.c_int, C.c_int,
                                    dp, dp, C.POINTER(C.c_longlong), C.c_int, dp]
        L.lmo_render_lt.argtypes = [vp, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_int, C.c_uint, C.c_int, dp,
                                    C.POINTER(C.c_longlong), C.c_int, dp]
        L.lmo_render_bdpt.argtypes = [vp, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_int, C.c_int, C.c_uint, C.c_int,
                                      C.c_int, dp, C.POINTER(C.c_longlong), C.c_int, dp]
        L.lmo_philox_uniform.restype = C.c_float
        L.lmo_philox_uniform.argtypes = [C.c_uint, C.c_ulonglong, C.c_uint, C.c_uint]
        L.lmo_max_threads.restype = C.c_int
        L.lmo_math_eval.argtypes = [C.c_char_p, dp, C.c_longlong, dp]
        L.lmo_dist2_eval.argtypes = [dp, C.c_int, C.c_int, C.c_longlong, dp, dp, dp, dp]
        L.lmo_rng_mt.argtypes = [C.c_uint, C.c_int, C.c_longlong, dp]
        L.lmo_material_query.argtypes = [C.c_int, dp, dp, C.c_longlong, dp]
        L.lmo_light_query.argtypes = [vp, dp, C.c_longlong, dp]
        L.lmo_scene_material_query.argtypes = [vp, C.c_int, dp, C.c_longlong, dp]
        L.lmo_texture_query.argtypes = [vp, C.c_int, dp, C.c_longlong, dp]
        L.lmo_camera_query.argtypes = [dp, dp, C.c_longlong, dp]
        _lib = L
    return _lib


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def _chk(rc: int) -> int:
    if rc < 0:
        raise RuntimeError("oracle: " + lib().lmo_last_error().decode())
    return rc


MAT = {"material::diffuse": 0, "material::glossy": 1, "material::glass": 2, "material::mirror": 3,
       "material::mixture_wavefrontobj": 4}


class OracleScene:
    """One scene in the CPU restatement; `double=True` is the reference's precision."""

    def __init__(self, double: bool = True):
        self.double = double
        self.h = lib().lmo_create(1 if double else 0)
        self.num_tris = 0
        self.build_seconds = 0.0
        self._keep = []

    def __del__(self):
        try:
            lib().lmo_destroy(self.h)
        except Exception:
            pass

    # -- construction -----------------------------------------------------------------------------
    def add_mesh(self, ps, ns, fp, fn, ts=None, ft=None) -> int:
        ps = np.ascontiguousarray(ps, np.float32).reshape(-1, 3)
        ns = np.ascontiguousarray(ns, np.float32).reshape(-1, 3)
        fp = np.ascontiguousarray(fp, np.int32).reshape(-1)
        fn = np.ascontiguousarray(fn, np.int32).reshape(-1)
        F, I = C.POINTER(C.c_float), C.POINTER(C.c_int)
        ts_ = np.ascontiguousarray(ts if ts is not None else np.zeros((0, 2)), np.float32).reshape(-1, 2)
        ft_ = np.ascontiguousarray(ft if ft is not None else np.zeros_like(fp), np.int32).reshape(-1)
        if ts_.shape[0] == 0:
            ft_ = np.zeros_like(fp)
        return _chk(lib().lmo_add_mesh(self.h, ps.ctypes.data_as(F), ps.shape[0], ns.ctypes.data_as(F), ns.shape[0],
                                       ts_.ctypes.data_as(F), ts_.shape[0], fp.ctypes.data_as(I),
                                       ft_.ctypes.data_as(I), fn.ctypes.data_as(I), fp.size))

    def add_material(self, kind: int, params) -> int:
        p = np.zeros(8)
        p[:len(params)] = params
        return _chk(lib().lmo_add_material(self.h, kind, _dp(p)))

    def add_texture(self, data) -> int:
        """texture::bitmap texels (h, w, 3 or 4), row 0 at the bottom."""
        t = np.ascontiguousarray(data, np.float32)
        self._keep.append(t)
        h, w, c = t.shape
        return _chk(lib().lmo_add_texture(self.h, t.ctypes.data_as(C.POINTER(C.c_float)), w, h, c))

    def set_material_textures(self, mat: int, mapKd: int = -1, mask: int = -1) -> None:
        _chk(lib().lmo_set_material_textures(self.h, mat, mapKd, mask))

    def add_area_light(self, Ke, mesh: int) -> int:
        return _chk(lib().lmo_add_light_area(self.h, _dp(Ke), mesh))

    def add_envconst(self, Le) -> int:
        return _chk(lib().lmo_add_light_envconst(self.h, _dp(Le)))

    def add_point(self, Le, position) -> int:
        return _chk(lib().lmo_add_light_point(self.h, _dp(Le), _dp(position)))

    def add_directional(self, Le, direction) -> int:
        return _chk(lib().lmo_add_light_directional(self.h, _dp(Le), _dp(direction)))

    def add_env(self, texels: np.ndarray, rot: float = 0.0, scale: float = 1.0) -> int:
        t = np.ascontiguousarray(texels, np.float32)
        self._keep.append(t)
        h, w = t.shape[:2]
        return _chk(lib().lmo_add_light_env(self.h, t.ctypes.data_as(C.POINTER(C.c_float)), w, h, 3, rot, scale))

    def add_camera(self, position, center, up, vfov, aspect) -> int:
        return _chk(lib().lmo_add_camera(self.h, _dp(position), _dp(center), _dp(up), vfov, aspect))

    def primitive(self, mesh=-1, material=-1, light=-1, camera=-1) -> int:
        return _chk(lib().lmo_create_primitive_node(self.h, mesh, material, light, camera))

    def group(self, m4: np.ndarray) -> int:
        cm = np.asarray(m4, np.float64).T.reshape(-1)  # column-major
        return _chk(lib().lmo_create_group_node(self.h, _dp(cm)))

    def instance_group(self) -> int:
        return _chk(lib().lmo_create_instance_group_node(self.h))

    def add_child(self, parent: int, child: int) -> None:
        _chk(lib().lmo_add_child(self.h, parent, child))

    def build(self, nthreads: int = 0, robust: bool = False) -> None:
        s = C.c_double()
        _chk(lib().lmo_build(self.h, nthreads, 1 if robust else 0, C.byref(s)))
        self.build_seconds = s.value
        self.num_tris = lib().lmo_num_triangles(self.h)

    # -- queries ----------------------------------------------------------------------------------
    def light_query(self, rec: np.ndarray) -> np.ndarray:
        """Direct and emission sampling of the scene's only light over records of 14 doubles
        (layout as oracle/ref.py's light_query); returns n x 33. Double-precision scenes."""
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 33))
        dp = C.POINTER(C.c_double)
        _chk(lib().lmo_light_query(self.h, rec.ctypes.data_as(dp), rec.shape[0], out.ctypes.data_as(dp)))
        return out

    def material_query(self, mat: int, rec: np.ndarray) -> np.ndarray:
        """Every query of material `mat` with its textures over records of 26 doubles (layout as
        oracle/ref.py's material_query); returns n x 18. Double-precision scenes."""
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 18))
        dp = C.POINTER(C.c_double)
        _chk(lib().lmo_scene_material_query(self.h, mat, rec.ctypes.data_as(dp), rec.shape[0], out.ctypes.data_as(dp)))
        return out

    def texture_query(self, tex: int, uv: np.ndarray) -> np.ndarray:
        """Texture `tex` at texture coordinates uv (n x 2): n x 5 (eval[3], eval_alpha,
        has_alpha). Double-precision scenes."""
        uv = np.ascontiguousarray(uv, np.float64)
        out = np.zeros((uv.shape[0], 5))
        dp = C.POINTER(C.c_double)
        _chk(lib().lmo_texture_query(self.h, tex, uv.ctypes.data_as(dp), uv.shape[0], out.ctypes.data_as(dp)))
        return out

    def triangles(self) -> np.ndarray:
        """(n, 9): p1, e1, e2 of every flattened triangle, as the accel stores them."""
        out = np.empty((self.num_tris, 9), np.float32)
        _chk(lib().lmo_get_triangles(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def intersect(self, rays: np.ndarray, nthreads: int = 0, brute: bool = False, refine_t: bool = False):
        """Returns (t, uv, global triangle index, seconds); index -1 = miss. refine_t (fp32 mode):
        t is the hit triangle's distance recomputed in double and rounded once to float, as the
        GPU's accel API reports it for single-level trees."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        t = np.zeros(n)
        uv = np.zeros((n, 2))
        tri = np.zeros(n, np.int32)
        s = C.c_double()
        _chk(lib().lmo_intersect(self.h, rays.ctypes.data_as(C.POINTER(C.c_float)), n, _dp(t) if False else
                                 t.ctypes.data_as(C.POINTER(C.c_double)), uv.ctypes.data_as(C.POINTER(C.c_double)),
                                 tri.ctypes.data_as(C.POINTER(C.c_int)), nthreads, 1 if brute else 0, 1 if refine_t else 0,
                                 C.byref(s)))
        return t, uv, tri, s.value

    def render_raycast(self, w, h, bg=(0, 0, 0), use_constant_color=False, visualize_normal=False, color=None,
                       nthreads: int = 0):
        out = np.zeros((h, w, 3))
        s = C.c_double()
        col = _dp(color) if color is not None else None
        _chk(lib().lmo_render_raycast(self.h, w, h, _dp(bg), int(use_constant_color), int(visualize_normal), col,
                                      out.ctypes.data_as(C.POINTER(C.c_double)), nthreads, C.byref(s)))
        return out, s.value

    def render_pt(self, w, h, spp, max_verts, seed=0, sampling_mode="mis", primary_mode="pixel", rng="philox",
                  with_m2=False, nthreads: int = 0):
        """Returns (image (h,w,3) scaled as the reference, second moment per pixel or None, rays, seconds).
        rng='mt19937' reproduces the reference's per-thread std::mt19937 stream; 'philox' uses the
        GPU path's per-path stream."""
        out = np.zeros((h, w, 3))
        m2 = np.zeros((h, w, 3)) if with_m2 else None
        rays = C.c_longlong()
        s = C.c_double()
        sm = {"naive": 0, "nee": 1, "mis": 2}[sampling_mode]
        pm = {"pixel": 0, "image": 1}[primary_mode]
        rm = {"mt19937": 0, "philox": 1}[rng]
        _chk(lib().lmo_render_pt(self.h, w, h, spp, max_verts, seed & 0xFFFFFFFF, sm, pm, rm,
                                 out.ctypes.data_as(C.POINTER(C.c_double)),
                                 m2.ctypes.data_as(C.POINTER(C.c_double)) if m2 is not None else None,
                                 C.byref(rays), nthreads, C.byref(s)))
        return out, m2, rays.value, s.value


    def render_lt(self, w, h, num_samples, max_verts, seed=0, first_path=0, rng="philox", nthreads: int = 0):
        """renderer::lt: returns (image (h,w,3) scaled by w*h / num_samples, rays, seconds) for light
        paths [first_path, first_path + num_samples)."""
        out = np.zeros((h, w, 3))
        rays = C.c_longlong()
        s = C.c_double()
        rm = {"mt19937": 0, "philox": 1}[rng]
        _chk(lib().lmo_render_lt(self.h, w, h, num_samples, first_path, max_verts, seed & 0xFFFFFFFF, rm,
                                 out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rays), nthreads, C.byref(s)))
        return out, rays.value, s.value


    BDPT_MODES = {"bdpt": 0, "pt_naive_path": 1, "pt_nee_path": 2, "lt_nee_path": 3, "bdptopt": 4}

    def render_bdpt(self, w, h, num_samples, max_verts, seed=0, min_verts=2, first_path=0, rng="philox", nthreads: int = 0,
                    mode: str = "bdpt"):
        """renderer::bdpt (or, by mode, renderer::pt_naive_path / pt_nee_path / lt_nee_path / bdptopt):
        returns (image (h,w,3) scaled by w*h / num_samples, rays, seconds) for samples
        [first_path, first_path + num_samples), each one eye and one light subpath."""
        out = np.zeros((h, w, 3))
        rays = C.c_longlong()
        s = C.c_double()
        rm = {"mt19937": 0, "philox": 1}[rng]
        _chk(lib().lmo_render_bdpt(self.h, w, h, num_samples, first_path, min_verts, max_verts, seed & 0xFFFFFFFF, rm,
                                   self.BDPT_MODES[mode], out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rays), nthreads,
                                   C.byref(s)))
        return out, rays.value, s.value


def mt32(rays, tri32, idx):
    """fp32 Moller-Trumbore t of triangle idx[k] (records p1, e1, e2 of the oracle's fp32 accel)
    for ray k, in the operation order of accel_sahbvh.cpp:58-75 with glm's dot and cross (every
    numpy float32 op rounds once, as the kernel's IEEE ops do)."""
    f = np.float32
    o = rays[:, 0:3].astype(f)
    d = rays[:, 4:7].astype(f)
    T = tri32[idx]
    p1, e1, e2 = T[:, 0:3], T[:, 3:6], T[:, 6:9]

    def cross(x, y):
        return np.stack([x[:, 1] * y[:, 2] - y[:, 1] * x[:, 2], x[:, 2] * y[:, 0] - y[:, 2] * x[:, 0],
                         x[:, 0] * y[:, 1] - y[:, 0] * x[:, 1]], 1)

    def dot(x, y):
        return (x[:, 0] * y[:, 0] + x[:, 1] * y[:, 1]) + x[:, 2] * y[:, 2]

    p = cross(d, e2)
    q = cross(o - p1, e1)
    with np.errstate(divide="ignore", invalid="ignore"):
        return dot(e2, q) / dot(e1, p)


def philox_uniform(seed: int, path: int, vertex: int, slot: int) -> float:
    return float(lib().lmo_philox_uniform(seed, path, vertex, slot))


def max_threads() -> int:
    return lib().lmo_max_threads()


def math_eval(fn: str, inp: np.ndarray, out_width: int) -> np.ndarray:
    """The restated math.h helper `fn` in double over the rows of `inp` (record layouts as
    oracle/ref.py's math_eval, so the two compare bit for bit)."""
    inp = np.ascontiguousarray(inp, np.float64)
    out = np.zeros((inp.shape[0], out_width))
    _chk(lib().lmo_math_eval(fn.encode(), inp.ctypes.data_as(C.POINTER(C.c_double)), inp.shape[0],
                             out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def dist2_eval(v: np.ndarray, uvq: np.ndarray, u4: np.ndarray):
    """Restated Dist2 over the rows x cols table v: pdf at uvq (n x 2), samples from u4 (n x 4)."""
    v = np.ascontiguousarray(v, np.float64)
    rows, cols = v.shape
    uvq = np.ascontiguousarray(uvq, np.float64)
    u4 = np.ascontiguousarray(u4, np.float64)
    n = uvq.shape[0]
    pdf, smp = np.zeros(n), np.zeros((n, 2))
    dp = C.POINTER(C.c_double)
    _chk(lib().lmo_dist2_eval(v.ctypes.data_as(dp), cols, rows, n, uvq.ctypes.data_as(dp), u4.ctypes.data_as(dp),
                              pdf.ctypes.data_as(dp), smp.ctypes.data_as(dp)))
    return pdf, smp


def material_query(key: str, params, rec: np.ndarray) -> np.ndarray:
    """Every query of the restated material `key` over records of 26 doubles (layout as
    oracle/ref.py's material_query); returns n x 18."""
    prm = np.zeros(8)
    prm[:len(params)] = params
    rec = np.ascontiguousarray(rec, np.float64)
    out = np.zeros((rec.shape[0], 18))
    dp = C.POINTER(C.c_double)
    _chk(lib().lmo_material_query(MAT[key], prm.ctypes.data_as(dp), rec.ctypes.data_as(dp), rec.shape[0],
                                  out.ctypes.data_as(dp)))
    return out


def camera_query(params, rec: np.ndarray) -> np.ndarray:
    """The restated camera::pinhole (position, center, up, vfov, aspect) over records of 11
    doubles (layout as oracle/ref.py's camera_query); returns n x 21."""
    prm = np.ascontiguousarray(params, np.float64)
    rec = np.ascontiguousarray(rec, np.float64)
    out = np.zeros((rec.shape[0], 21))
    dp = C.POINTER(C.c_double)
    _chk(lib().lmo_camera_query(prm.ctypes.data_as(dp), rec.ctypes.data_as(dp), rec.shape[0], out.ctypes.data_as(dp)))
    return out


def rng_mt(seed: int, n: int, as_float: bool = False) -> np.ndarray:
    """n uniforms of the restated reference Rng (mt19937, double or the float flavour)."""
    out = np.zeros(n)
    _chk(lib().lmo_rng_mt(seed, 1 if as_float else 0, n, out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def from_parts(parts: dict, double: bool = True) -> OracleScene:
    """Builds the oracle's scene straight from a plain scene description (synthetic.spheres_parts:
    camera props and primitives in scene order), without the GPU library: the same graph
    from_lm_scene rebuilds from the `lightmetrica` objects."""
    O = OracleScene(double)
    c = parts["camera"]
    cam = O.add_camera(c["position"], c["center"], c["up"], c["vfov"], c["aspect"])
    O.add_child(0, O.primitive(-1, -1, -1, cam))
    for pr in parts["primitives"]:
        me = ma = li = -1
        if pr["mesh"] is not None:
            ps, ns, fp, fn = pr["mesh"]
            me = O.add_mesh(ps, ns, fp, fn)
        if pr["material"] is not None:
            kind, m = pr["material"]
            params = {"diffuse": lambda: list(m["Kd"]), "glossy": lambda: list(m["Ks"]) + [m["ax"], m["ay"]],
                      "glass": lambda: [m["Ni"]], "mirror": lambda: []}[kind]()
            ma = O.add_material(MAT["material::" + kind], params)
        if pr["light"] is not None:
            kind, L = pr["light"]
            li = O.add_area_light(L["Ke"], me) if kind == "area" else O.add_envconst(L["Le"])
        O.add_child(0, O.primitive(me, ma, li, -1))
    return O


def from_lm_scene(scene, double: bool = True) -> OracleScene:
    """Rebuilds a `lightmetrica` scene graph (the GPU mirror's SceneDefault) inside the oracle."""
    O = OracleScene(double)
    mesh_id, mat_id, light_id, cam_id = {}, {}, {}, {}

    tex_id = {}

    def mesh_of(m):
        if id(m) not in mesh_id:
            ts = getattr(m, "ts", None)
            ft = getattr(m, "ft", None)
            fn = m.fn
            geo = getattr(m, "geo_normal_faces", None)
            if double and geo is not None and np.any(geo):
                # faces an OBJ gave no normals: the exact geometric normal, not its float32 copy
                fn = np.array(fn, np.int32).reshape(-1, 3)
                fn[np.asarray(geo, bool)] = -1
            mesh_id[id(m)] = O.add_mesh(m.ps, m.ns, m.fp, fn, ts, ft)
        return mesh_id[id(m)]

    def tex_of(t):
        if t is None:
            return -1
        if id(t) not in tex_id:
            tex_id[id(t)] = O.add_texture(t.texels())
        return tex_id[id(t)]

    node_map = {0: 0}
    for i, n in enumerate(scene.nodes):
        if i == 0:
            continue
        if n["type"] == "group":
            node_map[i] = O.instance_group() if n["instanced"] else O.group(n["transform"])
            continue
        me = mesh_of(n["mesh"]) if n["mesh"] is not None else -1
        ma = -1
        if n["material"] is not None:
            m = n["material"]
            while m.key_name == "material::proxy":   # material_proxy.cpp: every query goes to 'ref'
                m = m.ref
            if id(m) not in mat_id:
                k = MAT[m.key_name]
                params = {0: lambda: list(m.Kd), 1: lambda: list(m.Ks) + [m.ax, m.ay], 2: lambda: [m.Ni], 3: lambda: [],
                          4: lambda: list(m.Kd) + list(m.Ks) + [m.ax, m.ay]}[k]()
                mat_id[id(m)] = O.add_material(k, params)
                mk, mm = tex_of(getattr(m, "mapKd", None)), tex_of(getattr(m, "mask", None))
                if mk >= 0 or mm >= 0:
                    O.set_material_textures(mat_id[id(m)], mk, mm)
            ma = mat_id[id(m)]
        li = -1
        if n["light"] is not None:
            L = n["light"]
            if id(L) not in light_id:
                if L.key_name == "light::area":
                    light_id[id(L)] = O.add_area_light(L.Ke, mesh_of(L.mesh))
                elif L.key_name == "light::envconst":
                    light_id[id(L)] = O.add_envconst(L.Le)
                elif L.key_name == "light::point":
                    light_id[id(L)] = O.add_point(L.Le, L.position)
                elif L.key_name == "light::directional":
                    light_id[id(L)] = O.add_directional(L.Le, L.direction)
                else:
                    light_id[id(L)] = O.add_env(L.data, L.rot, L.scale)
            li = light_id[id(L)]
        ca = -1
        if n["camera"] is not None:
            c = n["camera"]
            if id(c) not in cam_id:
                cam_id[id(c)] = O.add_camera(c.position, c.center, c.up, c.vfov, c.aspect)
            ca = cam_id[id(c)]
        node_map[i] = O.primitive(me, ma, li, ca)
    for i, n in enumerate(scene.nodes):
        if n["type"] == "group":
            for c in n["children"]:
                O.add_child(node_map[i], node_map[c])
    return O
