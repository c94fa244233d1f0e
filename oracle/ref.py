"""Oracle (test infrastructure only): ctypes wrapper of oracle/_ref/liblmref.so, the reference's
own accel, material, light, camera and math code (src/accel/accel_sahbvh.cpp,
src/material/material_{diffuse,glossy,glass,mirror}.cpp, src/light/light_{area,envconst,point,
directional}.cpp, src/camera/camera_pinhole.cpp, include/lm/math.h, include/lm/surface.h)
compiled unmodified by
`make -C oracle ref`.

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
    return os.path.exists(os.path.join(REF_ROOT, "src", "accel", "accel_sahbvh.cpp"))


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
        L.lmref_scene_primitive.argtypes = [vp, C.c_int]
        L.lmref_scene_group.argtypes = [vp, dp]
        L.lmref_scene_add_child.argtypes = [vp, C.c_int, C.c_int]
        L.lmref_accel_build.argtypes = [vp, C.c_char_p, dp]
        L.lmref_accel_intersect.argtypes = [vp, fp, C.c_longlong, dp, dp, ip, ip, lp, C.c_int]
        L.lmref_math_eval.argtypes = [C.c_char_p, dp, C.c_longlong, dp]
        L.lmref_dist2_eval.argtypes = [dp, C.c_int, C.c_int, C.c_longlong, dp, dp, dp, dp]
        L.lmref_rng.argtypes = [C.c_int, C.c_int, C.c_longlong, dp]
        L.lmref_material_create.restype = vp
        L.lmref_material_create.argtypes = [C.c_char_p, dp]
        L.lmref_material_destroy.argtypes = [vp]
        L.lmref_material_query.argtypes = [vp, dp, C.c_longlong, dp]
        L.lmref_light_create.restype = vp
        L.lmref_light_create.argtypes = [vp, C.c_char_p, dp, C.c_int]
        L.lmref_light_destroy.argtypes = [vp]
        L.lmref_light_query.argtypes = [vp, dp, dp, C.c_longlong, dp]
        L.lmref_camera_query.argtypes = [dp, dp, C.c_longlong, dp]
        _lib = L
    return _lib


def _chk(rc: int) -> int:
    if rc < 0:
        raise RuntimeError("reference: " + lib().lmref_last_error().decode())
    return rc


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class RefScene:
    """A scene graph for the reference's accel: node 0 is the root group."""

    def __init__(self):
        self.h = lib().lmref_scene_create()

    def __del__(self):
        if getattr(self, "h", None):
            lib().lmref_scene_destroy(self.h)
            self.h = None

    def add_mesh(self, ps, fp) -> int:
        ps = np.ascontiguousarray(ps, np.float32).reshape(-1, 3)
        fp = np.ascontiguousarray(fp, np.int32).reshape(-1, 3)
        return _chk(lib().lmref_scene_add_mesh(self.h, _p(ps, C.c_float), ps.shape[0], _p(fp, C.c_int), fp.shape[0]))

    def primitive(self, mesh: int = -1) -> int:
        return _chk(lib().lmref_scene_primitive(self.h, mesh))

    def group(self, m4=None) -> int:
        """m4: 4x4 (row-major numpy, as the lightmetrica API takes it) or None."""
        if m4 is None:
            return _chk(lib().lmref_scene_group(self.h, None))
        cm = np.ascontiguousarray(np.asarray(m4, np.float64).T).reshape(16)
        return _chk(lib().lmref_scene_group(self.h, _p(cm, C.c_double)))

    def add_child(self, parent: int, child: int) -> None:
        _chk(lib().lmref_scene_add_child(self.h, parent, child))

    def build(self, key: str = "accel::sahbvh") -> float:
        s = C.c_double()
        _chk(lib().lmref_accel_build(self.h, key.encode(), C.byref(s)))
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


def from_parts(parts: dict) -> RefScene:
    """The reference accel's scene from a plain scene description (synthetic.spheres_parts), with
    the node order oracle.from_parts uses (camera primitive first, then the primitives)."""
    S = RefScene()
    S.add_child(0, S.primitive(-1))
    for pr in parts["primitives"]:
        me = -1
        if pr["mesh"] is not None:
            ps, _, fp, _ = pr["mesh"]
            me = S.add_mesh(ps, fp)
        S.add_child(0, S.primitive(me))
    return S


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


def material_query(key: str, params, rec: np.ndarray) -> np.ndarray:
    """Every Material query of the reference's `key` component (diffuse Kd; glossy Ks, ax, ay;
    glass Ni; mirror none) over records of 26 doubles: p n gn t wi wo comp trans_dir(0 LE, 1 EL)
    eval_delta ud udc uc. Returns n x 18: eval[3], pdf_direction, sample_direction (valid, wo[3],
    weight[3]), sample_component (comp, weight), pdf_component, reflectance[3],
    is_specular_component."""
    prm = np.zeros(8)
    prm[:len(params)] = params
    m = lib().lmref_material_create(key.encode(), _p(prm, C.c_double))
    if not m:
        raise RuntimeError("reference: " + lib().lmref_last_error().decode())
    try:
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 18))
        _chk(lib().lmref_material_query(m, _p(rec, C.c_double), rec.shape[0], _p(out, C.c_double)))
        return out
    finally:
        lib().lmref_material_destroy(m)


def light_query(scene: RefScene, key: str, params, mesh: int, m4, rec: np.ndarray) -> np.ndarray:
    """The reference's `key` light (area: Ke over the scene's mesh `mesh`; envconst: Le; point:
    Le, position; directional: Le, direction), bounded by the scene's transformed triangles, under
    the 4x4 transform m4 (row-major), over records of 14 doubles: p n gn of the shading point, up
    upc ud. Returns n x 33: sample_direct (valid, geomL p n wo, wo, weight), its pdf_direct, eval,
    sample_ray (valid, geomL p n, wo, weight)."""
    prm = np.zeros(8)
    prm[:len(params)] = params
    h = lib().lmref_light_create(scene.h, key.encode(), _p(prm, C.c_double), mesh)
    if not h:
        raise RuntimeError("reference: " + lib().lmref_last_error().decode())
    try:
        cm = np.ascontiguousarray(np.asarray(m4, np.float64).T).reshape(16)
        rec = np.ascontiguousarray(rec, np.float64)
        out = np.zeros((rec.shape[0], 33))
        _chk(lib().lmref_light_query(h, _p(cm, C.c_double), _p(rec, C.c_double), rec.shape[0], _p(out, C.c_double)))
        return out
    finally:
        lib().lmref_light_destroy(h)


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


def rng(seed: int, n: int, as_float: bool = False) -> np.ndarray:
    out = np.zeros(n)
    _chk(lib().lmref_rng(seed, 1 if as_float else 0, n, _p(out, C.c_double)))
    return out
