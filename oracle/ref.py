"""Oracle (test infrastructure only): ctypes wrapper of oracle/_ref/liblmref.so, the reference's
own code compiled unmodified by `make -C oracle ref`: src/scene.cpp, src/accel/accel_sahbvh.cpp,
src/mesh/mesh_raw.cpp, src/material/material_{diffuse,glossy,glass,mirror,proxy}.cpp,
src/light/light_{area,envconst,point,directional,env}.cpp, src/texture/texture_bitmap.cpp,
src/objloader/objloader{,_simple}.cpp, src/model/model_wavefrontobj.cpp (with
material::mixture_wavefrontobj), src/camera/camera_pinhole.cpp, src/film/film_bitmap.cpp,
src/scheduler.cpp, src/renderer/renderer_{raycast,pt,lt,bdpt,bdptopt}.cpp and the headers they include (math.h,
surface.h, scene.h, path.h, bidir.h, ...). stb_image, which texture_bitmap.cpp decodes images
with, is not among the reference's sources: images reach it decoded, through register_image.

Only tests/ and tests/golden/make_ref_fixtures.py use it, to pin the CPU restatement (and,
through committed fixtures, the CUDA path) to the reference itself. The library can be built only
where the reference's sources are present; `available()` says whether it is.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "liblmref.so")
REF_ROOT = os.environ.get("LMREF_ROOT", "/root/reference")

_lib = None


def sources_present() -> bool:
    return os.path.exists(os.path.join(REF_ROOT, "src", "renderer", "renderer_pt.cpp"))


def build() -> str | None:
    """Builds the library when the reference's sources are present; returns its path or None."""
    if not sources_present():
        return None
    r = subprocess.run(["make", "-C", HERE, "ref", f"REF={REF_ROOT}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def available() -> bool:
    if os.path.exists(LIB_PATH):
        return True
    try:
        return build() is not None
    except RuntimeError:
        return False


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("liblmref.so is not built (the reference's sources are absent)")
        L = C.CDLL(LIB_PATH)
        vp, dp, fp, ip, lp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_longlong)
        L.lmref_last_error.restype = C.c_char_p
        L.lmref_scene_create.restype = vp
        L.lmref_scene_destroy.argtypes = [vp]
        L.lmref_scene_add_mesh.argtypes = [vp, fp, C.c_int, ip, C.c_int]
        L.lmref_scene_add_mesh_raw.argtypes = [vp, fp, C.c_int, fp, C.c_int, fp, C.c_int, ip, ip, ip, C.c_int]
        L.lmref_scene_add_material.argtypes = [vp, C.c_char_p, dp]
        L.lmref_scene_add_light.argtypes = [vp, C.c_char_p, dp, C.c_int]
        L.lmref_scene_add_camera.argtypes = [vp, dp]
        L.lmref_scene_add_film.argtypes = [vp, C.c_int, C.c_int]
        L.lmref_scene_primitive_ex.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.lmref_scene_group.argtypes = [vp, dp]
        L.lmref_scene_add_child.argtypes = [vp, C.c_int, C.c_int]
        L.lmref_scene_build.argtypes = [vp, dp]
        L.lmref_accel_intersect.argtypes = [vp, fp, C.c_longlong, dp, dp, ip, ip, lp, C.c_int]
        L.lmref_render_pt.argtypes = [vp, C.c_int, C.c_longlong, C.c_int, C.c_uint, C.c_int, C.c_int, dp]
        L.lmref_render_spi.argtypes = [vp, C.c_char_p, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_uint, dp]
        L.lmref_render_raycast.argtypes = [vp, C.c_int, dp, C.c_int, C.c_int, C.c_int, dp, dp]
        L.lmref_light_query.argtypes = [vp, C.c_int, dp, dp, C.c_longlong, dp]
        L.lmref_register_image.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, fp]
        L.lmref_scene_add_texture.argtypes = [vp, C.c_char_p, C.c_int]
        L.lmref_scene_add_material_tex.argtypes = [vp, C.c_char_p, dp, C.c_int]
        L.lmref_scene_add_light_env.argtypes = [vp, C.c_char_p, C.c_double, C.c_double]
        L.lmref_scene_add_model.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
        L.lmref_scene_add_child_from_model.argtypes = [vp, C.c_int, C.c_int]
        L.lmref_texture_query.argtypes = [vp, C.c_int, dp, C.c_longlong, dp]
        L.lmref_scene_material_query.argtypes = [vp, C.c_int, dp, C.c_longlong, dp]
        L.lmref_material_create.restype = vp
        L.lmref_material_create.argtypes = [C.c_char_p, dp]
        L.lmref_material_destroy.argtypes = [vp]
        L.lmref_material_query.argtypes = [vp, dp, C.c_longlong, dp]
        L.lmref_camera_query.argtypes = [dp, dp, C.c_longlong, dp]
        L.lmref_math_eval.argtypes = [C.c_char_p, dp, C.c_longlong, dp]
        L.lmref_dist2_eval.argtypes = [dp, C.c_int, C.c_int, C.c_longlong, dp, dp, dp, dp]
        L.lmref_rng.argtypes = [C.c_int, C.c_int, C.c_longlong, dp]
        _lib = L
    return _lib


def _chk(rc: int) -> int:
    if rc < 0:
        raise RuntimeError("reference: " + lib().lmref_last_error().decode())
    return rc


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _prm(params, n=11):
    prm = np.zeros(n)
    prm[:len(params)] = params
    return prm


def register_image(path: str, texels_top_first) -> None:
    """Hands texture::bitmap's stb_image stand-in the decoded image it loads from `path`: h x w x c
    (3 or 4) floats, top row first as an image file stores them."""
    t = np.ascontiguousarray(texels_top_first, np.float32)
    if t.ndim != 3:
        raise ValueError("texels must be h x w x c")
    h, w, c = t.shape
    _chk(lib().lmref_register_image(str(path).encode(), w, h, c, _p(t, C.c_float)))


class RefScene:
    """One reference scene (scene::default over accel::sahbvh) with its assets; node 0 is the root
    group. Mesh, material, light, camera and film methods return ids that primitive() takes."""

    def __init__(self):
        self.h = lib().lmref_scene_create()
        if not self.h:
            raise RuntimeError("reference: " + lib().lmref_last_error().decode())
        self.films = {}

    def __del__(self):
        if getattr(self, "h", None):
            lib().lmref_scene_destroy(self.h)
            self.h = None

    def add_mesh(self, ps, fp) -> int:
        """Positions and triangle indices only, for intersection (any size)."""
        ps = np.ascontiguousarray(ps, np.float32).reshape(-1, 3)
        fp = np.ascontiguousarray(fp, np.int32).reshape(-1, 3)
        return _chk(lib().lmref_scene_add_mesh(self.h, _p(ps, C.c_float), ps.shape[0], _p(fp, C.c_int), fp.shape[0]))

    def add_mesh_raw(self, ps, ns, fp, fn, ts=None, ft=None) -> int:
        """mesh::raw with normals and texture coordinates, for rendering."""
        ps = np.ascontiguousarray(ps, np.float32).reshape(-1, 3)
        ns = np.ascontiguousarray(ns, np.float32).reshape(-1, 3)
        ts = np.ascontiguousarray(ts if ts is not None else np.zeros((1, 2)), np.float32).reshape(-1, 2)
        fp = np.ascontiguousarray(fp, np.int32).reshape(-1)
        fn = np.ascontiguousarray(fn, np.int32).reshape(-1)
        ft = np.ascontiguousarray(ft if ft is not None else np.zeros_like(fp), np.int32).reshape(-1)
        return _chk(lib().lmref_scene_add_mesh_raw(self.h, _p(ps, C.c_float), ps.shape[0], _p(ns, C.c_float), ns.shape[0],
                                                   _p(ts, C.c_float), ts.shape[0], _p(fp, C.c_int), _p(ft, C.c_int),
                                                   _p(fn, C.c_int), fp.size))

    def material(self, key: str, params) -> int:
        return _chk(lib().lmref_scene_add_material(self.h, key.encode(), _p(_prm(params), C.c_double)))

    def light(self, key: str, params, mesh: int = -1) -> int:
        return _chk(lib().lmref_scene_add_light(self.h, key.encode(), _p(_prm(params), C.c_double), mesh))

    def texture(self, path: str, flip: bool = True) -> int:
        """texture::bitmap of an image given to register_image under `path`."""
        return _chk(lib().lmref_scene_add_texture(self.h, str(path).encode(), 1 if flip else 0))

    def material_tex(self, key: str, params, map_kd: int = -1) -> int:
        """material::diffuse (Kd) or material::mixture_wavefrontobj (Kd, Ks, ax, ay,
        no_alpha_mask) with texture asset map_kd (-1 = none)."""
        return _chk(lib().lmref_scene_add_material_tex(self.h, key.encode(), _p(_prm(params), C.c_double), map_kd))

    def light_env(self, path: str, rot_deg: float = 0.0, scale: float = 1.0) -> int:
        """light::env over the image registered under `path` (loaded flipped)."""
        return _chk(lib().lmref_scene_add_light_env(self.h, str(path).encode(), rot_deg, scale))

    def model(self, path: str, skip_specular_mat: bool = False, base_material: int = -1) -> int:
        """model::wavefrontobj of an OBJ file (MTL and textures beside it; texture images through
        register_image)."""
        return _chk(lib().lmref_scene_add_model(self.h, str(path).encode(), 1 if skip_specular_mat else 0,
                                                base_material))

    def add_child_from_model(self, parent: int, model: int) -> int:
        """Scene::add_child_from_model; returns the number of primitive nodes it added."""
        return _chk(lib().lmref_scene_add_child_from_model(self.h, parent, model))

    def texture_query(self, tex: int, uv: np.ndarray) -> np.ndarray:
        """n x 5: eval[3], eval_alpha (0 without alpha), has_alpha at texture coordinates uv."""
        uv = np.ascontiguousarray(uv, np.float64)
        out = np.zeros((uv.shape[0], 5))
        _chk(lib().lmref_texture_query(self.h, tex, _p(uv, C.c_double), uv.shape[0], _p(out, C.c_double)))
        return out

    def material_query(self, mat: int, rec: np.ndarray) -> np.ndarray:
        """material_query's records on material asset `mat` of this scene (textured ones too)."""
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 18))
        _chk(lib().lmref_scene_material_query(self.h, mat, _p(rec, C.c_double), rec.shape[0], _p(out, C.c_double)))
        return out

    def camera(self, position, center, up, vfov, aspect) -> int:
        prm = _prm(list(position) + list(center) + list(up) + [vfov, aspect])
        return _chk(lib().lmref_scene_add_camera(self.h, _p(prm, C.c_double)))

    def film(self, w: int, h: int) -> int:
        f = _chk(lib().lmref_scene_add_film(self.h, w, h))
        self.films[f] = (w, h)
        return f

    def primitive(self, mesh: int = -1, material: int = -1, light: int = -1, camera: int = -1) -> int:
        return _chk(lib().lmref_scene_primitive_ex(self.h, mesh, material, light, camera))

    def group(self, m4=None) -> int:
        """m4: 4x4 (row-major numpy, as the lightmetrica API takes it) or None."""
        if m4 is None:
            return _chk(lib().lmref_scene_group(self.h, None))
        cm = np.ascontiguousarray(np.asarray(m4, np.float64).T).reshape(16)
        return _chk(lib().lmref_scene_group(self.h, _p(cm, C.c_double)))

    def add_child(self, parent: int, child: int) -> None:
        _chk(lib().lmref_scene_add_child(self.h, parent, child))

    def build(self) -> float:
        s = C.c_double()
        _chk(lib().lmref_scene_build(self.h, C.byref(s)))
        return s.value

    def intersect(self, rays: np.ndarray, nthreads: int = 0):
        """rays: n x 8 float32 (o, tmin, d, tmax). Returns (t, uv, flattened triangle index) with
        index -1 for a miss, as OracleScene.intersect does."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        t, uv = np.zeros(n), np.zeros((n, 2))
        prim, face, tri = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int64)
        _chk(lib().lmref_accel_intersect(self.h, _p(rays, C.c_float), n, _p(t, C.c_double), _p(uv, C.c_double),
                                         _p(prim, C.c_int), _p(face, C.c_int), _p(tri, C.c_longlong), nthreads))
        return t, uv, tri

    def render_pt(self, film: int, samples: int, max_verts: int, seed: int = 0, sampling_mode: str = "mis",
                  primary_mode: str = "pixel") -> np.ndarray:
        """The reference's renderer::pt on one thread (Rng seeded `seed`), scheduler::spp::sample
        (pixel: `samples` spp) or scheduler::spi::sample (image: `samples` samples). Returns the
        film, (h, w, 3), row 0 at the bottom, as film_bitmap holds it."""
        w, h = self.films[film]
        out = np.zeros((h, w, 3))
        sm = {"naive": 0, "nee": 1, "mis": 2}[sampling_mode]
        pm = {"pixel": 0, "image": 1}[primary_mode]
        _chk(lib().lmref_render_pt(self.h, film, samples, max_verts, seed & 0xFFFFFFFF, sm, pm, _p(out, C.c_double)))
        return out

    def render_spi(self, key: str, film: int, num_samples: int, max_verts: int, seed: int = 0,
                   min_verts: int = 2) -> np.ndarray:
        """The reference's light-tracing renderers on one thread (Rng seeded `seed`) with
        scheduler::spi::sample over `num_samples` samples: "renderer::lt", "renderer::bdpt" or a
        strategy renderer ("renderer::pt_naive_path", "renderer::pt_nee_path",
        "renderer::lt_nee_path"). Returns the film, (h, w, 3), row 0 at the bottom."""
        w, h = self.films[film]
        out = np.zeros((h, w, 3))
        _chk(lib().lmref_render_spi(self.h, key.encode(), film, num_samples, min_verts, max_verts, seed & 0xFFFFFFFF,
                                    _p(out, C.c_double)))
        return out

    def render_raycast(self, film: int, bg=(0, 0, 0), use_constant_color: bool = False, visualize_normal: bool = False,
                       color=None) -> np.ndarray:
        """The reference's renderer::raycast into film asset `film`; returns its h x w x 3 buffer."""
        w, h = self.films[film]
        out = np.zeros((h, w, 3))
        bgv = np.asarray(bg, np.float64)
        col = np.asarray(color if color is not None else (0, 0, 0), np.float64)
        _chk(lib().lmref_render_raycast(self.h, film, _p(bgv, C.c_double), int(use_constant_color), int(visualize_normal),
                                        int(color is not None), _p(col, C.c_double), _p(out, C.c_double)))
        return out

    def light_query(self, light: int, m4, rec: np.ndarray) -> np.ndarray:
        """Light asset `light` (built scene: it holds the scene bound) under the 4x4 transform m4
        (row-major), over records of 14 doubles: p n gn of the shading point, up upc ud. Returns
        n x 33: sample_direct (valid, geomL p n wo, wo, weight), its pdf_direct, eval, sample_ray
        (valid, geomL p n, wo, weight)."""
        cm = np.ascontiguousarray(np.asarray(m4, np.float64).T).reshape(16)
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 33))
        _chk(lib().lmref_light_query(self.h, light, _p(cm, C.c_double), _p(rec, C.c_double), rec.shape[0],
                                     _p(out, C.c_double)))
        return out


def from_parts(parts: dict, renderable: bool = False) -> RefScene:
    """The reference's scene from a plain scene description (synthetic.spheres_parts), with the node
    order oracle.from_parts uses (camera primitive first, then the primitives). renderable=False
    keeps positions only (any size, intersection only); True builds mesh::raw meshes, materials,
    lights and the camera, for renderer::pt."""
    S = RefScene()
    c = parts["camera"]
    cam = S.camera(c["position"], c["center"], c["up"], c["vfov"], c["aspect"]) if renderable else -1
    S.add_child(0, S.primitive(camera=cam))
    for pr in parts["primitives"]:
        me = ma = li = -1
        if pr["mesh"] is not None:
            ps, ns, fp, fn = pr["mesh"]
            me = S.add_mesh_raw(ps, ns, fp, fn) if renderable else S.add_mesh(ps, np.asarray(fp).reshape(-1, 3))
        if renderable and pr["material"] is not None:
            kind, m = pr["material"]
            params = {"diffuse": lambda: list(m["Kd"]), "glossy": lambda: list(m["Ks"]) + [m["ax"], m["ay"]],
                      "glass": lambda: [m["Ni"]], "mirror": lambda: []}[kind]()
            ma = S.material("material::" + kind, params)
        if renderable and pr["light"] is not None:
            kind, L = pr["light"]
            li = S.light("light::area", L["Ke"], me) if kind == "area" else S.light("light::envconst", L["Le"])
        if me < 0 and ma < 0 and li < 0:
            continue
        S.add_child(0, S.primitive(me, ma, li, -1))
    return S


def material_query(key: str, params, rec: np.ndarray) -> np.ndarray:
    """Every Material query of the reference's `key` component (diffuse Kd; glossy Ks, ax, ay;
    glass Ni; mirror none) over records of 26 doubles: p n gn t wi wo comp trans_dir(0 LE, 1 EL)
    eval_delta ud udc uc. Returns n x 18: eval[3], pdf_direction, sample_direction (valid, wo[3],
    weight[3]), sample_component (comp, weight), pdf_component, reflectance[3],
    is_specular_component."""
    m = lib().lmref_material_create(key.encode(), _p(_prm(params), C.c_double))
    if not m:
        raise RuntimeError("reference: " + lib().lmref_last_error().decode())
    try:
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 18))
        _chk(lib().lmref_material_query(m, _p(rec, C.c_double), rec.shape[0], _p(out, C.c_double)))
        return out
    finally:
        lib().lmref_material_destroy(m)


def camera_query(params, rec: np.ndarray) -> np.ndarray:
    """The reference's camera::pinhole (position, center, up, vfov, aspect) over records of 11
    doubles: rp[2], wo[3], a scene point p[3] n[3]. Returns n x 21: primary_ray(rp) (o, d),
    raster_position(wo) (valid, rp), pdf_direction(wo), eval(wo), sample_direct toward the point
    (valid, wo, weight) and its pdf_direct."""
    prm = np.ascontiguousarray(params, np.float64)
    rec = np.ascontiguousarray(rec, np.float64)
    out = np.zeros((rec.shape[0], 21))
    _chk(lib().lmref_camera_query(_p(prm, C.c_double), _p(rec, C.c_double), rec.shape[0], _p(out, C.c_double)))
    return out


def math_eval(fn: str, inp: np.ndarray, out_width: int) -> np.ndarray:
    inp = np.ascontiguousarray(inp, np.float64)
    n = inp.shape[0]
    out = np.zeros((n, out_width))
    _chk(lib().lmref_math_eval(fn.encode(), _p(inp, C.c_double), n, _p(out, C.c_double)))
    return out


def dist2_eval(v: np.ndarray, uvq: np.ndarray, u4: np.ndarray):
    v = np.ascontiguousarray(v, np.float64)
    rows, cols = v.shape
    uvq = np.ascontiguousarray(uvq, np.float64)
    u4 = np.ascontiguousarray(u4, np.float64)
    n = uvq.shape[0]
    pdf, smp = np.zeros(n), np.zeros((n, 2))
    _chk(lib().lmref_dist2_eval(_p(v, C.c_double), cols, rows, n, _p(uvq, C.c_double), _p(u4, C.c_double),
                                _p(pdf, C.c_double), _p(smp, C.c_double)))
    return pdf, smp


def rng(seed: int, n: int, as_float: bool = False) -> np.ndarray:
    out = np.zeros(n)
    _chk(lib().lmref_rng(seed, 1 if as_float else 0, n, _p(out, C.c_double)))
    return out


def from_lm_scene(scene) -> RefScene:
    """The reference's scene from a `lightmetrica` scene graph (the GPU mirror's SceneDefault), node
    for node as oracle.from_lm_scene rebuilds it, for the components compiled into the library
    (mesh::raw, diffuse (textured or not) / glossy / glass / mirror / mixture_wavefrontobj /
    proxy materials, area / envconst / point / directional / env lights, the pinhole camera).
    Texture images go to the stb_image stand-in under names of their own, flipped back to file
    order, and load flipped. Anything else raises NotImplementedError."""
    S = RefScene()
    mesh_id, mat_id, light_id, cam_id, tex_id = {}, {}, {}, {}, {}
    tag = f"lmref_mem/{id(scene):x}"

    def image_of(texels, what):
        path = f"{tag}/{what}.img"
        register_image(path, np.ascontiguousarray(np.asarray(texels, np.float32)[::-1]))
        return path

    def tex_of(t):
        # texture::constant's eval is its colour everywhere; a 1 x 1 bitmap of it answers the same
        if t is None:
            return -1
        if id(t) not in tex_id:
            tex_id[id(t)] = S.texture(image_of(t.texels(), f"tex{len(tex_id)}"), flip=True)
        return tex_id[id(t)]

    def mesh_of(m):
        if id(m) not in mesh_id:
            mesh_id[id(m)] = S.add_mesh_raw(m.ps, m.ns, m.fp, m.fn, getattr(m, "ts", None), getattr(m, "ft", None))
        return mesh_id[id(m)]

    node_map = {0: 0}
    for i, n in enumerate(scene.nodes):
        if i == 0:
            continue
        if n["type"] == "group":
            if n["instanced"]:
                raise NotImplementedError("instance groups")
            node_map[i] = S.group(n["transform"])
            continue
        me = mesh_of(n["mesh"]) if n["mesh"] is not None else -1
        ma = -1
        if n["material"] is not None:
            m = n["material"]
            while m.key_name == "material::proxy":   # material_proxy.cpp: every query goes to 'ref'
                m = m.ref
            if id(m) not in mat_id:
                params = {"material::diffuse": lambda: list(m.Kd), "material::glossy": lambda: list(m.Ks) + [m.ax, m.ay],
                          "material::glass": lambda: [m.Ni], "material::mirror": lambda: []}
                mk = getattr(m, "mapKd", None)
                if m.key_name == "material::mixture_wavefrontobj":
                    # the mask is mapKd's alpha unless no_alpha_mask (model_wavefrontobj.cpp:403-410)
                    no_mask = mk is not None and mk.has_alpha() and m.mask is None
                    mat_id[id(m)] = S.material_tex(m.key_name, list(m.Kd) + list(m.Ks) + [m.ax, m.ay, no_mask],
                                                   tex_of(mk))
                elif m.key_name == "material::diffuse" and mk is not None:
                    mat_id[id(m)] = S.material_tex(m.key_name, list(m.Kd), tex_of(mk))
                elif m.key_name in params and mk is None:
                    mat_id[id(m)] = S.material(m.key_name, params[m.key_name]())
                else:
                    raise NotImplementedError(m.key_name)
            ma = mat_id[id(m)]
        li = -1
        if n["light"] is not None:
            L = n["light"]
            if id(L) not in light_id:
                if L.key_name == "light::area":
                    light_id[id(L)] = S.light("light::area", L.Ke, mesh_of(L.mesh))
                elif L.key_name == "light::envconst":
                    light_id[id(L)] = S.light("light::envconst", L.Le)
                elif L.key_name == "light::point":
                    light_id[id(L)] = S.light("light::point", list(L.Le) + list(L.position))
                elif L.key_name == "light::directional":
                    light_id[id(L)] = S.light("light::directional", list(L.Le) + list(L.direction))
                elif L.key_name == "light::env":
                    light_id[id(L)] = S.light_env(image_of(L.data, f"env{len(light_id)}"), L.rot, L.scale)
                else:
                    raise NotImplementedError(L.key_name)
            li = light_id[id(L)]
        ca = -1
        if n["camera"] is not None:
            c = n["camera"]
            if id(c) not in cam_id:
                cam_id[id(c)] = S.camera(c.position, c.center, c.up, c.vfov, c.aspect)
            ca = cam_id[id(c)]
        node_map[i] = S.primitive(me, ma, li, ca)
    for i, n in enumerate(scene.nodes):
        if n["type"] == "group":
            for c in n["children"]:
                S.add_child(node_map[i], node_map[c])
    return S
