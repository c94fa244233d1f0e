"""Drop-in `lightmetrica` module for the GPU rendering hot path.

Mirrors the part of the reference's Python API (src/pylm.cpp, lightmetrica/__init__.py) that the
functests use to build scenes and render them:

    import lightmetrica as lm
    lm.init()
    film = lm.load_film('film', 'bitmap', w=1920, h=1080)
    camera = lm.load_camera('camera', 'pinhole', position=[..], center=[..], up=[0,1,0], vfov=30, aspect=16/9)
    mesh = lm.load_mesh('mesh', 'raw', ps=[..], ns=[..], ts=[..], fs={'p': [..], 't': [..], 'n': [..]})
    material = lm.load_material('mat', 'diffuse', Kd=[.75, .75, .75])
    accel = lm.load_accel('accel', 'sahbvh')
    scene = lm.load_scene('scene', 'default', accel=accel)
    scene.add_primitive(camera=camera)
    scene.add_primitive(mesh=mesh, material=material)
    scene.build()
    renderer = lm.load_renderer('renderer', 'pt', scene=scene, output=film, max_verts=9, scheduler='sample', spp=16)
    renderer.render()
    img = film.buffer()

Every accel key the reference registers (accel::sahbvh, accel::nanort, accel::embree,
accel::embreeinstanced) and accel::gpu resolve to the GB300 8-wide BVH; renderer::pt,
renderer::lt, renderer::bdpt (and the path-structure renderers of renderer_bdpt.cpp,
renderer::bdptopt) and renderer::raycast resolve to the CUDA renderers. There is no CPU fallback: a
missing liblmgpu.so raises at the first render or build.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time
import zlib
from typing import Any

import numpy as np

from . import _native as N
from . import objloader  # lm.objloader.init / shutdown, and the OBJ/MTL parser
from ._native import LmGpuError

Release = True
Inf = 1e10
Eps = 1e-3

# ---------------------------------------------------------------------------------------------
# Component registry (include/lm/component.h: keys "interface::impl", locators "$.assets.<name>")

_assets: dict[str, "Component"] = {}
_registry: dict[str, type] = {}


def _reg(key: str, *aliases: str):
    def deco(cls):
        _registry[key] = cls
        for a in aliases:
            _registry[a] = cls
        cls.key_name = key
        return cls
    return deco


class Component:
    key_name = ""

    def __init__(self, name: str, prop: dict):
        self._name = name
        self._prop = dict(prop)
        self.construct(self._prop)

    def construct(self, prop: dict) -> None:
        pass

    def key(self) -> str:
        return self.key_name

    def loc(self) -> str:
        return "$.assets." + self._name

    def name(self) -> str:
        return self._name

    @property
    def prop(self) -> dict:
        return self._prop

    def __repr__(self) -> str:
        return f"<{self.key_name} {self.loc()}>"


def _resolve(v: Any) -> Any:
    """A Component argument or its locator string resolves to the component (json.h:225-247)."""
    if isinstance(v, Component) or v is None:
        return v
    if isinstance(v, str):
        if v.startswith("$.assets."):
            name = v[len("$.assets."):]
        else:
            name = v
        if name in _assets:
            return _assets[name]
        head, _, rest = name.partition(".")
        if rest and head in _assets and hasattr(_assets[head], "underlying"):
            return _assets[head].underlying(rest)   # an asset a model owns: $.assets.model.mesh_0
    raise LmGpuError(1, f"Invalid component reference: {v!r}")


def _req(prop: dict, key: str) -> Any:
    if key not in prop:
        raise LmGpuError(1, f"Missing property [name='{key}']")
    return prop[key]


def _vec3(v) -> np.ndarray:
    a = np.asarray(v, dtype=np.float64).reshape(-1)
    if a.size == 1:
        a = np.repeat(a, 3)
    if a.size != 3:
        raise LmGpuError(1, f"Expected a 3-vector, got {v!r}")
    return a


# ---------------------------------------------------------------------------------------------
# Library lifecycle (src/user.cpp:54-112)

def init(prop: dict | None = None, **kwargs) -> None:
    """lm.init: loads liblmgpu.so (raises if it is not built) and clears the asset tree."""
    N.lib()
    reset()


def shutdown() -> None:
    reset()


def reset() -> None:
    for a in list(_assets.values()):
        if hasattr(a, "_release"):
            a._release()
    _assets.clear()


def info() -> None:
    print("lightmetrica (GB300 hot path): liblmgpu", N.lib().lmgpu_version())


def get(loc: str) -> Component:
    return _resolve(loc)


def _load(iface: str, name: str, impl: str, prop: dict | None, kwargs: dict) -> Component:
    p = dict(prop or {})
    p.update(kwargs)
    key = impl if "::" in impl else f"{iface}::{impl}"
    cls = _registry.get(key)
    if cls is None:
        raise LmGpuError(1, f"Missing component [key='{key}']")
    if name in _assets and hasattr(_assets[name], "_release"):
        _assets[name]._release()
    comp = cls(name, p)
    _assets[name] = comp
    return comp


def load_film(name, impl, prop=None, **kw): return _load("film", name, impl, prop, kw)
def load_camera(name, impl, prop=None, **kw): return _load("camera", name, impl, prop, kw)
def load_mesh(name, impl, prop=None, **kw): return _load("mesh", name, impl, prop, kw)
def load_material(name, impl, prop=None, **kw): return _load("material", name, impl, prop, kw)
def load_light(name, impl, prop=None, **kw): return _load("light", name, impl, prop, kw)
def load_texture(name, impl, prop=None, **kw): return _load("texture", name, impl, prop, kw)
def load_model(name, impl, prop=None, **kw): return _load("model", name, impl, prop, kw)
def load_accel(name, impl, prop=None, **kw): return _load("accel", name, impl, prop, kw)
def load_scene(name, impl, prop=None, **kw): return _load("scene", name, impl, prop, kw)
def load_renderer(name, impl, prop=None, **kw): return _load("renderer", name, impl, prop, kw)


def load(name: str, impl_key: str, prop: dict | None = None, **kw) -> Component:
    iface = impl_key.split("::")[0]
    return _load(iface, name, impl_key, prop, kw)


@_reg("asset_group::default")
class AssetGroup(Component):
    """asset_group::default (src/assetgroup.cpp): a named subtree of the asset tree. Assets loaded
    through it get the locator $.assets.<group>.<name>; groups nest. Serialization of a subtree
    (save_to_file) is not part of the GPU path."""

    def _child(self, iface: str, name: str, impl: str, prop: dict | None, kw: dict) -> Component:
        return _load(iface, f"{self._name}.{name}", impl, prop, kw)

    def load_film(self, name, impl, prop=None, **kw): return self._child("film", name, impl, prop, kw)
    def load_camera(self, name, impl, prop=None, **kw): return self._child("camera", name, impl, prop, kw)
    def load_mesh(self, name, impl, prop=None, **kw): return self._child("mesh", name, impl, prop, kw)
    def load_material(self, name, impl, prop=None, **kw): return self._child("material", name, impl, prop, kw)
    def load_light(self, name, impl, prop=None, **kw): return self._child("light", name, impl, prop, kw)
    def load_texture(self, name, impl, prop=None, **kw): return self._child("texture", name, impl, prop, kw)
    def load_model(self, name, impl, prop=None, **kw): return self._child("model", name, impl, prop, kw)
    def load_accel(self, name, impl, prop=None, **kw): return self._child("accel", name, impl, prop, kw)
    def load_scene(self, name, impl, prop=None, **kw): return self._child("scene", name, impl, prop, kw)
    def load_renderer(self, name, impl, prop=None, **kw): return self._child("renderer", name, impl, prop, kw)
    def load_asset_group(self, name, impl="default", prop=None, **kw): return self._child("asset_group", name, impl, prop, kw)

    def save_to_file(self, path: str) -> None:
        raise LmGpuError(2, "serialization of assets is not part of the GPU path")


def load_asset_group(name, impl="default", prop=None, **kw): return _load("asset_group", name, impl, prop, kw)


def get_film(loc: str) -> Component: return _resolve(loc)
def get_renderer(loc: str) -> Component: return _resolve(loc)
def get_scene(loc: str) -> Component: return _resolve(loc)
def get_accel(loc: str) -> Component: return _resolve(loc)


class _Namespace:
    pass


comp = _Namespace()
comp.get = get
comp.load_plugin = lambda path: None          # accel/renderer plugins are built in
comp.load_plugin_directory = lambda path: None
comp.unload_plugin = lambda path: None
comp.unload_all_plugins = lambda: None
comp.foreach_registered = lambda f: [f(k) for k in sorted(_registry)]

# Subsystems of the reference that have no work to do on the GPU path.
log = _Namespace()
log.init = lambda *a, **k: None
log.shutdown = lambda: None
progress = _Namespace()
progress.init = lambda *a, **k: None
progress.shutdown = lambda: None
parallel = _Namespace()
parallel.init = lambda *a, **k: None
parallel.shutdown = lambda: None
debug = _Namespace()
debug.attach_to_debugger = lambda: None
debug.print_asset_tree = lambda *a, **k: None
attach_to_debugger = debug.attach_to_debugger


class _Enum:
    def __init__(self, **kw):
        self.__dict__.update(kw)


log.LogLevel = _Enum(Debug=-10, Info=10, Warn=20, Err=30, Progress=100, ProgressEnd=101)
log.LoggerContext = type("LoggerContext", (), {})
progress.ProgressMode = _Enum(Samples=0, Time=1)
progress.ProgressContext = type("ProgressContext", (), {})
# Floating-point type of the reference's build (lm::Float, double by default); the GPU path
# computes in fp32 (FloatT says so, for scripts that pick tolerances by it)
Float32, Float64 = "float32", "float64"
FloatT = Float32


def registered_components() -> list[str]:
    return sorted(_registry)


def pylm_component(name: str):
    def deco(cls):
        _registry[name] = cls
        return cls
    return deco


def array(*args, **kwargs):
    kwargs.setdefault("dtype", np.float32)
    return np.array(*args, **kwargs)


# ---------------------------------------------------------------------------------------------
# Transforms (src/pylm.cpp:88-99): 4x4 numpy matrices acting on column vectors.

def identity() -> np.ndarray:
    return np.eye(4)


def translate(v) -> np.ndarray:
    m = np.eye(4)
    m[:3, 3] = _vec3(v)
    return m


def scale(v) -> np.ndarray:
    m = np.eye(4)
    m[0, 0], m[1, 1], m[2, 2] = _vec3(v)
    return m


def rotate(angle: float, axis) -> np.ndarray:
    a = _vec3(axis)
    a = a / np.linalg.norm(a)
    c, s = math.cos(angle), math.sin(angle)
    x, y, z = a
    r = np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                  [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                  [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])
    m = np.eye(4)
    m[:3, :3] = r
    return m


def rad(deg: float) -> float:
    return deg * math.pi / 180.0


def v3(a, b, c) -> np.ndarray:
    return np.array([a, b, c], dtype=np.float64)


# ---------------------------------------------------------------------------------------------
# Assets

@_reg("film::bitmap")
class FilmBitmap(Component):
    """film::bitmap (src/film/film_bitmap.cpp) backed by a device fp32 accumulator."""

    def construct(self, prop):
        self.w = int(_req(prop, "w"))
        self.h = int(_req(prop, "h"))
        h = C.c_void_p()
        N.check(N.lib().lmgpu_film_create(C.byref(h), self.w, self.h))
        self._h = h

    def _release(self):
        if getattr(self, "_h", None):
            N.lib().lmgpu_film_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    def size(self):
        return (self.w, self.h)

    def num_pixels(self) -> int:
        return self.w * self.h

    def aspect(self) -> float:
        return self.w / self.h

    def clear(self):
        N.check(N.lib().lmgpu_film_clear(self._h))

    def buffer_f32(self) -> np.ndarray:
        out = np.empty((self.h, self.w, 3), dtype=np.float32)
        N.check(N.lib().lmgpu_film_read(self._h, N.fptr(out)))
        return out

    def buffer(self) -> np.ndarray:
        """Film::buffer: (h, w, 3) pixels, row 0 at the bottom (film.h:166-171)."""
        return self.buffer_f32().astype(np.float64)

    def rel_mse(self, eps: float = 1e-2) -> float:
        """Relative MSE of the film's estimate from its even- and odd-pass accumulators (renders
        with split passes; no reference counterpart): mean over pixels and channels of
        Var(I) / (I^2 + eps)."""
        v = C.c_double()
        N.check(N.lib().lmgpu_film_rel_mse(self._h, float(eps), C.byref(v)))
        return v.value

    def save(self, path: str) -> bool:
        """Film::save (film_bitmap.cpp:156-210): .png (flipped, gamma 1/2.2, 8 bits), .hdr
        (flipped, RGBE), .pfm (unflipped) or .npy; missing parent directories are created."""
        from . import imageio
        img = self.buffer_f32()
        if path.endswith(".pfm"):
            imageio.write_pfm(path, img)
        elif path.endswith(".hdr"):
            imageio.write_hdr(path, img)
        elif path.endswith(".png"):
            imageio.write_png(path, img)
        elif path.endswith(".npy"):
            imageio._parent(path)
            np.save(path, img)
        else:
            raise LmGpuError(2, f"Invalid extension [path='{path}']")
        return True


@_reg("camera::pinhole")
class CameraPinhole(Component):
    def construct(self, prop):
        if "matrix" in prop:
            raise LmGpuError(2, "camera::pinhole 'matrix' prop is not supported on the GPU path")
        self.position = _vec3(_req(prop, "position"))
        self.center = _vec3(_req(prop, "center"))
        self.up = _vec3(_req(prop, "up"))
        self.vfov = float(_req(prop, "vfov"))
        self.aspect = float(_req(prop, "aspect"))

    def set_aspect_ratio(self, aspect: float) -> None:
        self.aspect = float(aspect)


@_reg("mesh::raw")
class MeshRaw(Component):
    """mesh::raw (src/mesh/mesh_raw.cpp:50-68). ps/ns/ts flat lists or arrays; fs {'p','t','n'}."""

    def construct(self, prop):
        self.ps = np.asarray(_req(prop, "ps"), dtype=np.float32).reshape(-1, 3)
        self.ns = np.asarray(prop.get("ns", []), dtype=np.float32).reshape(-1, 3)
        self.ts = np.asarray(prop.get("ts", []), dtype=np.float32).reshape(-1, 2)
        fs = _req(prop, "fs")
        self.fp = np.asarray(fs["p"], dtype=np.int32).reshape(-1)
        self.fn = np.asarray(fs.get("n", fs["p"]), dtype=np.int32).reshape(-1)
        self.ft = np.asarray(fs.get("t", fs["p"]), dtype=np.int32).reshape(-1)
        if self.fp.size % 3 != 0:
            raise LmGpuError(1, "mesh::raw: face index count is not a multiple of 3")
        if self.fp.size and (self.fp.min() < 0 or self.fp.max() >= len(self.ps)):
            raise LmGpuError(1, "mesh::raw: position index out of range")
        if self.ns.size == 0:
            raise LmGpuError(1, "mesh::raw: normals are required")
        if self.ts.size == 0:  # no texture coordinates: every corner at (0, 0)
            self.ts = np.zeros((1, 2), np.float32)
            self.ft = np.zeros_like(self.fp)
        if self.ft.size != self.fp.size or (self.ft.size and (self.ft.min() < 0 or self.ft.max() >= len(self.ts))):
            raise LmGpuError(1, "mesh::raw: texture coordinate index out of range")
        if self.fn.size and (self.fn.min() < 0 or self.fn.max() >= len(self.ns)):
            raise LmGpuError(1, "mesh::raw: normal index out of range")

    def num_triangles(self) -> int:
        return self.fp.size // 3

    def tri_positions(self) -> np.ndarray:
        return self.ps[self.fp].reshape(-1, 3, 3)

    def tri_normals(self) -> np.ndarray:
        return self.ns[self.fn].reshape(-1, 3, 3)


_MAT_TYPES = {"material::diffuse": 0, "material::glossy": 1, "material::glass": 2, "material::mirror": 3,
              "material::mixture_wavefrontobj": 4}


class _Material(Component):
    def native(self) -> N.Material:
        m = N.Material()
        m.type = _MAT_TYPES[self.key_name]
        return m


@_reg("material::diffuse")
class MaterialDiffuse(_Material):
    """material::diffuse (material_diffuse.cpp:55-95): Kd, or mapKd, which has priority. A mapKd
    that is a texture::constant evaluates to its color everywhere, so it becomes Kd; a
    texture::bitmap is looked up at the shaded point's texture coordinate (renderer::pt and
    renderer::raycast)."""

    def construct(self, prop):
        self.Kd = _vec3(prop.get("Kd", [1, 1, 1]))
        self.mapKd = None
        if prop.get("mapKd"):
            tex = _resolve(prop["mapKd"])
            if isinstance(tex, TextureConstant):
                self.Kd = np.asarray(tex.color, np.float64)
            elif isinstance(tex, TextureBitmap):
                self.mapKd = tex
            else:
                raise LmGpuError(1, f"material::diffuse: mapKd is not a texture [{prop['mapKd']!r}]")

    def native(self):
        m = super().native()
        m.color[:] = [float(x) for x in self.Kd]
        return m


@_reg("material::glossy")
class MaterialGlossy(_Material):
    def construct(self, prop):
        self.Ks = _vec3(_req(prop, "Ks"))
        self.ax = float(_req(prop, "ax"))
        self.ay = float(_req(prop, "ay"))

    def native(self):
        m = super().native()
        m.color[:] = [float(x) for x in self.Ks]
        m.ax, m.ay = self.ax, self.ay
        return m


@_reg("material::glass")
class MaterialGlass(_Material):
    def construct(self, prop):
        self.Ni = float(_req(prop, "Ni"))

    def native(self):
        m = super().native()
        m.ni = self.Ni
        return m


@_reg("material::mirror")
class MaterialMirror(_Material):
    pass


@_reg("material::proxy")
class MaterialProxy(_Material):
    """material::proxy (material_proxy.cpp:25-76): every query goes to the material 'ref' names,
    so it renders as that material."""

    def construct(self, prop):
        self.ref = _resolve(_req(prop, "ref"))
        if not isinstance(self.ref, _Material):
            raise LmGpuError(1, f"Invalid material reference {prop['ref']!r}")

    def underlying(self) -> "_Material":
        m = self.ref
        while isinstance(m, MaterialProxy):
            m = m.ref
        return m

    def native(self):
        return self.underlying().native()


@_reg("material::mixture_wavefrontobj")
class MaterialMixtureWavefrontObj(_Material):
    """material::mixture_wavefrontobj (src/model/model_wavefrontobj.cpp:361-517): the sum of a
    diffuse (Kd, or the texel of mapKd) and a GGX glossy (Ks, ax, ay) lobe, one lobe sampled with
    probability max(Kd) / (max(Kd) + max(Ks)); when mapKd has an alpha channel (and no_alpha_mask
    is false) it is also the alpha mask: the surface with probability alpha, else a pass-through."""

    def construct(self, prop):
        self.mapKd = None
        self.mask = None
        if prop.get("mapKd"):
            tex = _resolve(prop["mapKd"])
            if not isinstance(tex, (TextureBitmap, TextureConstant)):
                raise LmGpuError(1, f"material::mixture_wavefrontobj: mapKd is not a texture [{prop['mapKd']!r}]")
            self.mapKd = tex
            if not bool(prop.get("no_alpha_mask", False)) and tex.has_alpha():
                self.mask = tex
        self.Kd = _vec3(_req(prop, "Kd"))
        self.Ks = _vec3(_req(prop, "Ks"))
        self.ax = float(_req(prop, "ax"))
        self.ay = float(_req(prop, "ay"))

    def native(self):
        m = super().native()
        m.color[:] = [float(x) for x in self.Kd]
        m.ks[:] = [float(x) for x in self.Ks]
        m.ax, m.ay = self.ax, self.ay
        return m


@_reg("model::wavefrontobj")
class ModelWavefrontObj(Component):
    """model::wavefrontobj (src/model/model_wavefrontobj.cpp:73-235). Props: path; light (the
    light key for materials with Ke > 0, default light::area); skip_specular_mat; base_material
    (a material used for every group instead of the MTL ones).

    Materials: illum 5 -> material::mirror, illum 7 -> material::glass (Ni), otherwise
    material::mixture_wavefrontobj with r = 2 / (2 + Ns), a = sqrt(1 - 0.9 aniso), ax =
    max(1e-3, r / a), ay = max(1e-3, r * a). One mesh per OBJ primitive, named mesh_<k> with k the
    number of assets created before it; a material with Ke > 0 adds an area light mesh_<k>_light
    on that mesh. Faces without normals use the geometric normal."""

    def construct(self, prop):
        from . import objloader
        path = _req(prop, "path")
        try:
            obj = objloader.load_obj(path)
        except OSError as e:
            raise LmGpuError(4, f"Missing OBJ or MTL file: {e}") from None
        except ValueError as e:
            raise LmGpuError(4, str(e)) from None
        self.assets: dict[str, Component] = {}
        self.groups: list[tuple] = []
        light_key = prop.get("light", "light::area")
        skip_spec = bool(prop.get("skip_specular_mat", False))
        base = _resolve(prop["base_material"]) if prop.get("base_material") is not None else None
        mat_of: list[Component] = []
        tex_key = prop.get("texture", "texture::bitmap")
        for m in obj.materials:
            # map_Kd: one texture per file stem, texture_<stem>, path relative to the OBJ
            # (model_wavefrontobj.cpp:133-154)
            tex = None
            if m.map_Kd and base is None:
                tid = "texture_" + os.path.splitext(os.path.basename(m.map_Kd))[0]
                if tid not in self.assets:
                    cls = _registry.get(tex_key if "::" in tex_key else f"texture::{tex_key}")
                    if cls is None:
                        raise LmGpuError(1, f"Missing component [key='{tex_key}']")
                    self.assets[tid] = cls(tid, {"path": os.path.join(os.path.dirname(path), m.map_Kd)})
                tex = self.assets[tid]
            if base is not None:
                mat = base
            elif m.illum in (5, 7):
                if skip_spec:
                    mat = MaterialDiffuse(m.name, {"Kd": [0, 0, 0]})
                elif m.illum == 7:
                    mat = MaterialGlass(m.name, {"Ni": m.Ni})
                else:
                    mat = MaterialMirror(m.name, {})
            else:
                r = 2.0 / (2.0 + m.Ns)
                a = math.sqrt(max(0.0, 1.0 - m.an * 0.9))
                if a == 0.0:
                    raise LmGpuError(1, f"aniso >= 1/0.9 gives an infinite roughness [material='{m.name}']")
                mat = MaterialMixtureWavefrontObj(m.name, {"Kd": list(m.Kd), "Ks": list(m.Ks), "ax": max(1e-3, r / a),
                                                          "ay": max(1e-3, r * a), "mapKd": tex,
                                                          "no_alpha_mask": skip_spec})
            self.assets[m.name] = mat
            mat_of.append(mat)
        n_ps, n_ns = len(obj.ps), len(obj.ns)
        for prim in obj.primitives:
            name = f"mesh_{len(self.assets)}"
            faces = np.asarray(prim.faces, dtype=np.int64).reshape(-1, 3) if prim.faces else np.zeros((0, 3), np.int64)
            fp = faces[:, 0]
            if fp.size and (fp.min() < 0 or fp.max() >= n_ps):
                raise LmGpuError(1, f"OBJ face refers to a missing position [{name}]")
            tri = fp.reshape(-1, 3)
            # the first corner's normal index decides per face (model_wavefrontobj.cpp:299-305)
            has_n = faces[0::3, 2] >= 0 if faces.size else np.zeros(0, bool)
            fn = faces[:, 2].copy()
            if has_n.size and np.any(faces[:, 2].reshape(-1, 3)[has_n] >= n_ns):
                raise LmGpuError(1, f"OBJ face refers to a missing normal [{name}]")
            extra = []
            if (~has_n).any():
                p = obj.ps[tri[~has_n]]
                g = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
                g /= np.maximum(np.linalg.norm(g, axis=1, keepdims=True), 1e-300)
                extra = g
                idx = n_ns + np.arange(len(g))
                fn.reshape(-1, 3)[~has_n] = idx[:, None]
            ns = np.concatenate([obj.ns, extra]) if len(extra) else obj.ns
            # texture coordinates: a face whose first corner has none reads (0, 0) everywhere
            # (model_wavefrontobj.cpp:318-320); the entry after the file's vt lines is that (0, 0)
            n_ts = len(obj.ts)
            ft = faces[:, 1].copy()
            no_t = (ft.reshape(-1, 3)[:, 0] < 0) if ft.size else np.zeros(0, bool)
            ft.reshape(-1, 3)[no_t] = n_ts
            ft[ft < 0] = n_ts
            if ft.size and ft.max() > n_ts:
                raise LmGpuError(1, f"OBJ face refers to a missing texture coordinate [{name}]")
            ts = np.concatenate([np.asarray(obj.ts, np.float32).reshape(-1, 2), np.zeros((1, 2), np.float32)])
            mesh = MeshRaw(name, {"ps": obj.ps.astype(np.float32), "ns": (ns if len(ns) else np.zeros((1, 3))).astype(np.float32),
                                  "ts": ts,
                                  "fs": {"p": fp.astype(np.int32), "n": fn.astype(np.int32), "t": ft.astype(np.int32)}})
            # the faces whose shading normal is the geometric one, computed exactly by the
            # reference; the float32 copy above serves the GPU
            mesh.geo_normal_faces = ~has_n
            self.assets[name] = mesh
            mtl = obj.materials[prim.material]
            light = None
            if max(mtl.Ke) > 0:
                cls = _registry.get(light_key if "::" in light_key else f"light::{light_key}")
                if cls is None:
                    raise LmGpuError(1, f"Missing component [key='{light_key}']")
                light = cls(name + "_light", {"Ke": list(mtl.Ke), "mesh": mesh})
                self.assets[name + "_light"] = light
            self.groups.append((mesh, mat_of[prim.material], light))

    def underlying(self, name: str) -> Component:
        if name not in self.assets:
            raise LmGpuError(1, f"Invalid component reference: {name!r}")
        return self.assets[name]

    def create_primitives(self, fn) -> None:
        """Model::create_primitives: fn(mesh, material, light) per group, in file order."""
        for mesh, mat, light in self.groups:
            fn(mesh, mat, light)


@_reg("texture::constant")
class TextureConstant(Component):
    """texture::constant (texture_constant.cpp:22-56): one color (and an optional alpha) for
    every texture coordinate; a 1 x 1 image where an image is needed (light::env's envmap)."""

    def construct(self, prop):
        self.color = _vec3(_req(prop, "color"))
        self.alpha = float(prop["alpha"]) if prop.get("alpha") is not None else None
        self.data = np.asarray(self.color, np.float32).reshape(1, 1, 3)
        self.h, self.w = 1, 1

    def has_alpha(self) -> bool:
        return self.alpha is not None

    def texels(self) -> np.ndarray:
        """1 x 1 x (3 or 4) texels for a material's texture table."""
        c = list(self.color) + ([self.alpha] if self.alpha is not None else [])
        return np.asarray(c, np.float32).reshape(1, 1, -1)


@_reg("texture::bitmap")
class TextureBitmap(Component):
    """texture::bitmap (texture_bitmap.cpp:40-85) with an in-memory array ('data': h x w x 3 or 4,
    row 0 at the bottom) or an image 'path' (.png, .hdr, .pfm, .npy; flipped on load unless
    flip=False). Three channels serve light::env; a fourth is the alpha has_alpha() reports."""

    def construct(self, prop):
        if "data" in prop:
            full = np.asarray(prop["data"], dtype=np.float32)
        else:
            path = _req(prop, "path")
            full = _read_image(path, flip=bool(prop.get("flip", True)), keep_alpha=True)
        if full.ndim == 2:
            full = full[..., None]
        if full.shape[2] == 1:      # gray: widened to RGB
            full = np.repeat(full, 3, axis=2)
        elif full.shape[2] == 2:    # gray + alpha
            full = np.concatenate([np.repeat(full[..., :1], 3, axis=2), full[..., 1:2]], axis=2)
        self.rgba = np.ascontiguousarray(full[..., :4])
        self.data = np.ascontiguousarray(self.rgba[..., :3])
        self.h, self.w = self.data.shape[:2]

    def has_alpha(self) -> bool:
        return self.rgba.shape[2] == 4

    def texels(self) -> np.ndarray:
        return self.rgba


def _read_image(path: str, flip: bool = True, keep_alpha: bool = False) -> np.ndarray:
    """texture::bitmap's image (texture_bitmap.cpp:49-66), row 0 at the bottom: .hdr and .png
    (flipped on load unless flip=False; a .png becomes linear as stbi_loadf makes it), .pfm
    (stored bottom row first), .npy (as stored). Three channels are kept."""
    from . import imageio
    try:
        nc = 4 if keep_alpha else 3
        if path.endswith(".npy"):
            return np.ascontiguousarray(np.load(path).astype(np.float32)[..., :nc])
        if path.endswith(".pfm"):
            return imageio.read_pfm(path)
        if path.endswith(".hdr"):
            return imageio.read_hdr(path, flip=flip)
        if path.endswith(".png"):
            return np.ascontiguousarray(imageio.read_png(path, flip=flip)[..., :nc])
    except (OSError, ValueError, zlib.error) as e:
        raise LmGpuError(4, f"Failed to load image [path='{path}']: {e}") from None
    raise LmGpuError(2, f"Unsupported image format [path='{path}'] (use .hdr, .png, .pfm or .npy)")


class _Light(Component):
    pass


@_reg("light::area")
class LightArea(_Light):
    def construct(self, prop):
        self.Ke = _vec3(_req(prop, "Ke"))
        self.mesh = _resolve(_req(prop, "mesh"))


@_reg("light::envconst")
class LightEnvConst(_Light):
    def construct(self, prop):
        self.Le = _vec3(_req(prop, "Le"))


@_reg("light::point")
class LightPoint(_Light):
    """light::point (light_point.cpp:34-37): Le and a world-space position; the transform of the
    primitive node that holds it is not applied, as in the reference."""

    def construct(self, prop):
        self.Le = _vec3(_req(prop, "Le"))
        self.position = _vec3(_req(prop, "position"))


@_reg("light::directional")
class LightDirectional(_Light):
    """light::directional (light_directional.cpp:34-37): Le and the direction the light travels,
    normalized."""

    def construct(self, prop):
        self.Le = _vec3(_req(prop, "Le"))
        d = _vec3(_req(prop, "direction"))
        n = float(np.linalg.norm(d))
        if not n > 0:
            raise LmGpuError(1, f"Invalid direction {prop['direction']!r}")
        self.direction = d / n


@_reg("light::env")
class LightEnv(_Light):
    """light::env. The reference loads envmap_path through texture::bitmap; here 'envmap_path'
    may be a .pfm/.npy file, or 'envmap' an in-memory (h, w, 3) array or texture component."""

    def construct(self, prop):
        if "envmap" in prop:
            e = prop["envmap"]
            self.data = _resolve(e).data if isinstance(e, (str, Component)) else np.ascontiguousarray(np.asarray(e, np.float32)[..., :3])
        else:
            self.data = _read_image(_req(prop, "envmap_path"))
        self.rot = float(prop.get("rot", 0.0))
        self.scale = float(prop.get("scale", 1.0))


@_reg("accel::sahbvh", "accel::nanort", "accel::embree")
class AccelGpu(Component):
    """The accel slot (include/lm/accel.h): an 8-wide quantized BVH traced on the GPU. Registered
    under every key the reference's accels use. Like accel::sahbvh, nanort and embree it flattens
    instance groups into one tree; prop `instancing=True` (the default of accel::embreeinstanced
    and accel::gpu) builds the two-level form instead. GPU extra: prop `builder` -- 'sah' (binned
    SAH on the host threads, the default) or 'ploc' (built on the GPU: Morton order, PLOC
    clustering, the same 8-wide collapse); hits are the same either way."""

    default_instancing = False
    BUILDERS = {"sah": 0, "ploc": 1}

    def construct(self, prop):
        h = C.c_void_p()
        N.check(N.lib().lmgpu_accel_create(C.byref(h)))
        self._h = h
        self.num_tris = 0
        self.instancing = bool(prop.get("instancing", self.default_instancing))
        b = prop.get("builder", "sah")
        if b not in self.BUILDERS:
            raise LmGpuError(1, f"Invalid builder '{b}' (sah or ploc)")
        self.builder = b

    def _release(self):
        if getattr(self, "_h", None):
            N.lib().lmgpu_accel_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    def build_triangles(self, tri_p: np.ndarray) -> None:
        tri_p = np.ascontiguousarray(tri_p, dtype=np.float32).reshape(-1, 9)
        N.check(N.lib().lmgpu_accel_build_ex(self._h, N.fptr(tri_p), tri_p.shape[0], self.BUILDERS[self.builder]))
        self.num_tris = tri_p.shape[0]

    def build_instanced(self, tri_p: np.ndarray, blas_offsets, instances) -> None:
        """Two-level build: tri_p holds every BLAS's triangles back to back (each in its own frame),
        blas_offsets the BLAS boundaries (len = number of BLAS + 1), instances a list of
        (blas index, 4x4 world-from-local matrix)."""
        tri_p = np.ascontiguousarray(tri_p, dtype=np.float32).reshape(-1, 9)
        offs = np.ascontiguousarray(blas_offsets, dtype=np.int64)
        arr = (N.Instance * len(instances))()
        for k, (b, m) in enumerate(instances):
            arr[k].blas = int(b)
            arr[k].transform[:] = [float(x) for x in np.asarray(m, np.float64)[:3, :4].reshape(-1)]
        N.check(N.lib().lmgpu_accel_build_instanced_ex(self._h, N.fptr(tri_p), offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                                        len(offs) - 1, arr, len(instances), self.BUILDERS[self.builder]))
        self.num_tris = self.stats()["num_tris"]

    def build(self, scene: "SceneDefault") -> None:
        """Accel::build(const Scene&): flattens the scene (two-level when `instancing` and the
        scene has instance groups) and builds over its triangles."""
        if self.instancing and scene._has_instances():
            g = scene._flatten_instanced()
            self.build_instanced(g["positions"], g["blas_offsets"], g["instances"])
        else:
            self.build_triangles(scene._flatten()["positions"])

    def stats(self) -> dict:
        s = N.AccelStats()
        N.check(N.lib().lmgpu_accel_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.AccelStats._fields_}

    def intersect_batch(self, rays: np.ndarray) -> np.ndarray:
        """Batched Accel::intersect. rays: (n, 8) float32 (o, tmin, d, tmax). Returns a structured
        array with fields t, u, v, prim (flattened triangle index, -1 = miss)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.zeros(rays.shape[0], dtype=[("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<i4")])
        N.check(N.lib().lmgpu_accel_intersect(self._h, N.fptr(rays), rays.shape[0],
                                              out.ctypes.data_as(C.POINTER(N.Hit))))
        return out

    def intersect(self, ray_o, ray_d, tmin: float = Eps, tmax: float = Inf):
        """Single-ray Accel::intersect; returns (t, (u, v), flattened triangle index) or None."""
        r = np.array([[*_vec3(ray_o), tmin, *_vec3(ray_d), tmax]], dtype=np.float32)
        h = self.intersect_batch(r)[0]
        if h["prim"] < 0:
            return None
        return float(h["t"]), (float(h["u"]), float(h["v"])), int(h["prim"])


@_reg("accel::embreeinstanced", "accel::gpu")
class AccelGpuInstanced(AccelGpu):
    default_instancing = True


# ---------------------------------------------------------------------------------------------
# Scene (src/scene.cpp, include/lm/scene.h)

def _f32_matmul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """4x4 product in fp32 with glm's order: column i = ((A0*B0i + A1*B1i) + A2*B2i) + A3*B3i."""
    a = a.astype(np.float32)
    b = b.astype(np.float32)
    out = np.empty((4, 4), dtype=np.float32)
    for i in range(4):
        for k in range(4):
            out[k, i] = ((a[k, 0] * b[0, i] + a[k, 1] * b[1, i]) + a[k, 2] * b[2, i]) + a[k, 3] * b[3, i]
    return out


def _f32_xform(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    """M * vec4(p, 1) in fp32 with glm's pairing: (m0*x + m1*y) + (m2*z + m3*1)."""
    m = m.astype(np.float32)
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    one = np.float32(1)
    out = np.empty(p.shape, dtype=np.float32)
    for i in range(3):
        out[..., i] = (m[i, 0] * x + m[i, 1] * y) + (m[i, 2] * z + m[i, 3] * one)
    return out


def _tri_texcoords(mesh) -> np.ndarray:
    """Per triangle the three corners' texture coordinates (k, 6), in the mesh's face order."""
    ts = getattr(mesh, "ts", None)
    ft = getattr(mesh, "ft", None)
    n = mesh.num_triangles()
    if ts is None or ft is None or len(ts) == 0:
        return np.zeros((n, 6), np.float32)
    return np.asarray(ts, np.float32)[np.asarray(ft)].reshape(n, 6)


def _is_identity(m: np.ndarray) -> bool:
    return bool(np.array_equal(m, np.eye(4, dtype=m.dtype)))


@_reg("scene::default")
class SceneDefault(Component):
    def construct(self, prop):
        self._accel = _resolve(prop["accel"]) if prop.get("accel") is not None else None
        self._h = None
        self._flat = None
        self.reset()

    def _release(self):
        if getattr(self, "_h", None):
            N.lib().lmgpu_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    # -- graph (scene.cpp:54-230) --------------------------------------------------------------
    def reset(self) -> None:
        self._release()
        self._flat = None
        self.nodes: list[dict] = [{"type": "group", "children": [], "transform": None, "instanced": False}]
        self._camera: int | None = None
        self._env: int | None = None

    def root_node(self) -> int:
        return 0

    def num_nodes(self) -> int:
        return len(self.nodes)

    def create_primitive_node(self, prop: dict | None = None, **kw) -> int:
        p = dict(prop or {})
        p.update(kw)
        mesh = _resolve(p.get("mesh"))
        material = _resolve(p.get("material"))
        light = _resolve(p.get("light"))
        camera = _resolve(p.get("camera"))
        if "medium" in p:
            raise LmGpuError(2, "media are not supported on the GPU path")
        if not any([mesh, material, light, camera]):
            raise LmGpuError(1, "Invalid primitive node. Given assets are invalid.")
        if camera is not None and light is not None:
            raise LmGpuError(1, "Primitive cannot be both camera and light.")
        if (mesh is None) != (material is None):
            raise LmGpuError(1, "You must specify both mesh and material.")
        idx = len(self.nodes)
        if camera is not None:
            self._camera = idx
        if light is not None and isinstance(light, (LightEnvConst, LightEnv)):
            if self._env is not None:
                raise LmGpuError(1, "Environment light is already registered. You can register only one environment light in the scene.")
            self._env = idx
        self.nodes.append({"type": "primitive", "mesh": mesh, "material": material, "light": light, "camera": camera})
        return idx

    def create_group_node(self, transform) -> int:
        self.nodes.append({"type": "group", "children": [], "transform": np.asarray(transform, dtype=np.float64),
                           "instanced": False})
        return len(self.nodes) - 1

    def create_instance_group_node(self) -> int:
        self.nodes.append({"type": "group", "children": [], "transform": None, "instanced": True})
        return len(self.nodes) - 1

    def add_child(self, parent: int, child: int) -> None:
        if parent < 0 or parent >= len(self.nodes) or self.nodes[parent]["type"] != "group":
            return
        self.nodes[parent]["children"].append(child)

    def add_primitive(self, prop: dict | None = None, **kw) -> None:
        self.add_transformed_primitive(np.eye(4), prop, **kw)

    def add_transformed_primitive(self, transform, prop: dict | None = None, **kw) -> None:
        p = dict(prop or {})
        p.update(kw)
        t = self.create_group_node(transform)
        if "model" in p:
            self.add_child_from_model(t, p["model"])   # scene.h:141-152
        else:
            self.add_child(t, self.create_primitive_node(p))
        self.add_child(0, t)

    def add_child_from_model(self, parent: int, model) -> None:
        """scene.cpp:158-180: one primitive node per (mesh, material, light) of the model."""
        m = _resolve(model)
        if not hasattr(m, "create_primitives"):
            raise LmGpuError(1, f"Invalid model [loc={model!r}]")
        m.create_primitives(lambda mesh, mat, light: self.add_child(
            parent, self.create_primitive_node(mesh=mesh, material=mat, light=light)))

    def traverse_primitive_nodes(self, fn) -> None:
        """Depth-first traversal with fp32 global transforms (scene.cpp:216-230)."""
        def visit(i: int, m: np.ndarray):
            n = self.nodes[i]
            fn(i, n, m)
            if n["type"] == "group":
                mm = _f32_matmul(m, n["transform"]) if n["transform"] is not None else m
                for c in n["children"]:
                    visit(c, mm)
        visit(0, np.eye(4, dtype=np.float32))

    def camera_node(self) -> int:
        return -1 if self._camera is None else self._camera

    def env_light_node(self) -> int:
        return -1 if self._env is None else self._env

    def num_lights(self) -> int:
        return sum(1 for n in self.nodes if n["type"] == "primitive" and n["light"] is not None)

    def accel(self):
        return self._accel

    def set_accel(self, loc) -> None:
        self._accel = _resolve(loc)

    # -- flatten + build (scene.cpp:274-317, accel_sahbvh.cpp:132-151) ------------------------
    @staticmethod
    def _prim_geometry(mesh, m: np.ndarray):
        """One primitive's triangles under transform m (fp32, glm order): positions (k, 9),
        shading normals (k, 9) and normalized geometric normals (k, 3)."""
        tp = mesh.tri_positions()
        tn = mesh.tri_normals()
        ident = _is_identity(m)
        if ident:
            wp = tp.astype(np.float32)
            wn = tn.astype(np.float32)
            nm = np.eye(3, dtype=np.float32)
        else:
            wp = _f32_xform(m, tp)
            nm = np.linalg.inv(m.astype(np.float64)).T[:3, :3].astype(np.float32)
            wn = (tn @ nm.T).astype(np.float32)
        lp = tp.astype(np.float32)
        # a zero-area triangle's normal is NaN, as glm::normalize of a zero vector makes it
        with np.errstate(invalid="ignore", divide="ignore"):
            g = np.cross(lp[:, 1] - lp[:, 0], lp[:, 2] - lp[:, 0]).astype(np.float32)
            g = g / np.sqrt(np.sum(g * g, axis=1, keepdims=True)).astype(np.float32)
            if not ident:
                g = (g @ nm.T).astype(np.float32)
                g = g / np.sqrt(np.sum(g * g, axis=1, keepdims=True)).astype(np.float32)
        return wp.reshape(-1, 9), wn.reshape(-1, 9), g.reshape(-1, 3)

    def _has_instances(self) -> bool:
        return any(n["type"] == "group" and n["instanced"] for n in self.nodes)

    def _flatten_instanced(self) -> dict:
        """Two-level flattening as accel::embreeinstanced does it (accel_embree_instanced.cpp:
        84-181): primitives outside instance groups go, in world space, to BLAS 0 (an identity
        instance); each instance group reached from the root is flattened once, in its own frame
        and with nested instance groups treated as plain groups, into its own BLAS, and every
        path to it adds an instance with the global transform at the group. Hit indices count the
        instances' triangles in instance order."""
        prim_mat, prim_light, prim_node = [], [], []
        mats: list = []
        light_index_of_node: dict[int, int] = {}
        nl = [0]

        def collect_lights(i, n, m):
            if n["type"] == "primitive" and n["light"] is not None:
                light_index_of_node[i] = nl[0]
                nl[0] += 1
        self.traverse_primitive_nodes(collect_lights)
        blas: list[dict] = [{"pos": [], "nrm": [], "gn": [], "prim": [], "tc": []}]
        blas_of_group: dict[int, int] = {}
        instances: list = []

        def add_prim(b, i, n, m):
            wp, wn, g = self._prim_geometry(n["mesh"], m)
            mat = n["material"]
            if mat not in mats:
                mats.append(mat)
            pi = len(prim_mat)
            prim_mat.append(mats.index(mat))
            prim_light.append(light_index_of_node.get(i, -1))
            prim_node.append(i)
            blas[b]["pos"].append(wp)
            blas[b]["nrm"].append(wn)
            blas[b]["gn"].append(g)
            blas[b]["prim"].append(np.full(wp.shape[0], pi, dtype=np.int32))
            blas[b]["tc"].append(_tri_texcoords(n["mesh"]))

        def visit_local(i, m, b):  # inside an instance group: plain flattening into BLAS b
            n = self.nodes[i]
            if n["type"] == "primitive":
                if n["mesh"] is not None:
                    add_prim(b, i, n, m)
                return
            mm = _f32_matmul(m, n["transform"]) if n["transform"] is not None else m
            for c in n["children"]:
                visit_local(c, mm, b)

        def visit_root(i, m):
            n = self.nodes[i]
            if n["type"] == "primitive":
                if n["mesh"] is not None:
                    add_prim(0, i, n, m)
                return
            if n["instanced"]:
                if i not in blas_of_group:
                    blas_of_group[i] = len(blas)
                    blas.append({"pos": [], "nrm": [], "gn": [], "prim": [], "tc": []})
                    visit_local(i, np.eye(4, dtype=np.float32), blas_of_group[i])
                instances.append((blas_of_group[i], m.astype(np.float64)))
                return
            mm = _f32_matmul(m, n["transform"]) if n["transform"] is not None else m
            for c in n["children"]:
                visit_root(c, mm)
        visit_root(0, np.eye(4, dtype=np.float32))
        if blas[0]["pos"]:
            instances.insert(0, (0, np.eye(4)))
        # drop empty BLAS (the root one without primitives, or groups without meshes)
        keep = [b for b in range(len(blas)) if blas[b]["pos"]]
        remap = {b: k for k, b in enumerate(keep)}
        instances = [(remap[b], m) for b, m in instances if b in remap]
        pos = [np.concatenate(blas[b]["pos"]) for b in keep]
        offs = np.zeros(len(keep) + 1, np.int64)
        for k, p_ in enumerate(pos):
            offs[k + 1] = offs[k] + p_.shape[0]

        def cat(key, width, dt):
            parts = [np.concatenate(blas[b][key]) for b in keep]
            return np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros((0, width), dt), dtype=dt)
        return {"positions": cat("pos", 9, np.float32), "normals": cat("nrm", 9, np.float32),
                "geo_normals": cat("gn", 3, np.float32), "tri_prim": cat("prim", 1, np.int32).reshape(-1),
                "blas_offsets": offs, "instances": instances,
                "prim_material": np.asarray(prim_mat, np.int32), "prim_light": np.asarray(prim_light, np.int32),
                "prim_node": np.asarray(prim_node, np.int32), "materials": mats,
                "texcoords": cat("tc", 6, np.float32)}

    def _flatten(self, geometry: bool = True) -> dict:
        """Flattened scene: world-space triangles with shading data (unless geometry=False, which
        gives the light tables alone), primitive and material tables, lights in traversal order."""
        pos, nrm, gns, tri_prim, tcs = [], [], [], [], []
        prim_mat, prim_light, prim_node = [], [], []
        mats: list[_Material] = []
        lights: list[tuple] = []        # (light component, global transform, node index)
        light_index_of_node: dict[int, int] = {}

        def collect_lights(i, n, m):
            if n["type"] == "primitive" and n["light"] is not None:
                light_index_of_node[i] = len(lights)
                lights.append((n["light"], m, i))
        self.traverse_primitive_nodes(collect_lights)

        def collect_geometry(i, n, m):
            if n["type"] != "primitive" or n["mesh"] is None:
                return
            wp, wn, g = self._prim_geometry(n["mesh"], m)
            mat = n["material"]
            if mat not in mats:
                mats.append(mat)
            pi = len(prim_mat)
            prim_mat.append(mats.index(mat))
            prim_light.append(light_index_of_node.get(i, -1))
            prim_node.append(i)
            pos.append(wp)
            nrm.append(wn)
            gns.append(g)
            tri_prim.append(np.full(wp.shape[0], pi, dtype=np.int32))
            tcs.append(_tri_texcoords(n["mesh"]))
        if geometry:
            self.traverse_primitive_nodes(collect_geometry)

        if pos:
            positions = np.ascontiguousarray(np.concatenate(pos), dtype=np.float32)
            normals = np.ascontiguousarray(np.concatenate(nrm), dtype=np.float32)
            geo = np.ascontiguousarray(np.concatenate(gns), dtype=np.float32)
            tprim = np.ascontiguousarray(np.concatenate(tri_prim), dtype=np.int32)
            texcoords = np.ascontiguousarray(np.concatenate(tcs), dtype=np.float32)
        else:
            texcoords = np.zeros((0, 6), np.float32)
            positions = np.zeros((0, 9), np.float32)
            normals = np.zeros((0, 9), np.float32)
            geo = np.zeros((0, 3), np.float32)
            tprim = np.zeros(0, np.int32)

        # lights (light_area.cpp:68-80; light_env.cpp:55-72)
        nl = []
        ltp, ltg, lta = [], [], []
        env_tex = []
        env_off = 0
        ltri_off = 0
        for comp_, m, node in lights:
            L = N.Light()
            if isinstance(comp_, LightArea):
                L.type = 0
                L.ke[:] = [float(x) for x in comp_.Ke]
                lm_ = comp_.mesh
                lp = lm_.tri_positions().astype(np.float32)
                cr = np.cross((lp[:, 1] - lp[:, 0]).astype(np.float64), (lp[:, 2] - lp[:, 0]).astype(np.float64))
                area = 0.5 * np.sqrt(np.sum(cr * cr, axis=1))
                gl = cr / np.linalg.norm(cr, axis=1, keepdims=True)
                if _is_identity(m):
                    wp = lp
                    gw = gl
                    J = 1.0
                else:
                    wp = _f32_xform(m, lp)
                    nm = np.linalg.inv(m.astype(np.float64)).T[:3, :3]
                    gw = gl @ nm.T
                    gw = gw / np.linalg.norm(gw, axis=1, keepdims=True)
                    J = abs(float(np.linalg.det(m.astype(np.float64)[:3, :3])))
                L.tri_offset = ltri_off
                L.tri_count = lp.shape[0]
                L.transform_j = J
                ltri_off += lp.shape[0]
                ltp.append(np.asarray(wp, np.float32).reshape(-1, 9))
                ltg.append(np.asarray(gw, np.float32).reshape(-1, 3))
                lta.append(np.asarray(area, np.float32))
            elif isinstance(comp_, LightEnvConst):
                L.type = 1
                L.ke[:] = [float(x) for x in comp_.Le]
            elif isinstance(comp_, LightPoint):
                L.type = 3
                L.ke[:] = [float(x) for x in comp_.Le]
                L.vec[:] = [float(x) for x in comp_.position]
            elif isinstance(comp_, LightDirectional):
                L.type = 4
                L.ke[:] = [float(x) for x in comp_.Le]
                L.vec[:] = [float(x) for x in comp_.direction]
            elif isinstance(comp_, LightEnv):
                L.type = 2
                L.env_w, L.env_h = comp_.data.shape[1], comp_.data.shape[0]
                L.env_offset = env_off
                L.rot_deg = comp_.rot
                L.scale = comp_.scale
                env_tex.append(comp_.data.reshape(-1).astype(np.float32))
                env_off += comp_.data.size
            else:
                raise LmGpuError(2, f"Unsupported light {comp_!r}")
            nl.append(L)
        return {
            "positions": positions, "normals": normals, "geo_normals": geo, "tri_prim": tprim,
            "prim_material": np.asarray(prim_mat, np.int32), "prim_light": np.asarray(prim_light, np.int32),
            "prim_node": np.asarray(prim_node, np.int32), "materials": mats, "lights": nl,
            "light_tri_p": np.concatenate(ltp) if ltp else np.zeros((0, 9), np.float32),
            "light_tri_gn": np.concatenate(ltg) if ltg else np.zeros((0, 3), np.float32),
            "light_tri_area": np.concatenate(lta) if lta else np.zeros(0, np.float32),
            "env_texels": np.concatenate(env_tex) if env_tex else np.zeros(0, np.float32),
            "texcoords": texcoords,
        }

    def build(self) -> None:
        """Scene::build: flattens the graph, builds the accel and uploads shading data."""
        if self._accel is None:
            raise LmGpuError(2, "Missing acceleration structure.")
        self._release()
        instanced = getattr(self._accel, "instancing", False) and self._has_instances()
        flat = self._flatten(geometry=not instanced)
        if instanced:
            # shading data per BLAS in its own frame; lights stay as flattened in world space
            g = self._flatten_instanced()
            for k in ("positions", "normals", "geo_normals", "tri_prim", "prim_material", "prim_light", "prim_node",
                      "materials", "blas_offsets", "instances", "texcoords"):
                flat[k] = g[k]
        if flat["positions"].shape[0] == 0:
            raise LmGpuError(2, "Missing primitives. Use lm::primitive() function to add primitives.")
        if instanced:
            self._accel.build_instanced(flat["positions"], flat["blas_offsets"], flat["instances"])
        else:
            self._accel.build_triangles(flat["positions"])
        d = N.SceneDesc()
        keep = []

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a
        d.num_tris = flat["positions"].shape[0]
        d.positions = N.fptr(arr(flat["positions"], np.float32))
        d.normals = N.fptr(arr(flat["normals"], np.float32))
        d.geo_normals = N.fptr(arr(flat["geo_normals"], np.float32))
        d.tri_prim = N.iptr(arr(flat["tri_prim"], np.int32))
        d.num_prims = len(flat["prim_material"])
        d.prim_material = N.iptr(arr(flat["prim_material"], np.int32))
        d.prim_light = N.iptr(arr(flat["prim_light"], np.int32))
        # image textures: each distinct texture once; materials refer to them by index
        textures, tex_index = [], {}

        def tex_of(t):
            if t is None:
                return -1
            if id(t) not in tex_index:
                tex_index[id(t)] = len(textures)
                textures.append(t)
            return tex_index[id(t)]
        natives = []
        for m in flat["materials"]:
            nm = m.native()
            u = m.underlying() if hasattr(m, "underlying") else m
            nm.map_kd = tex_of(getattr(u, "mapKd", None))
            nm.mask = tex_of(getattr(u, "mask", None))
            natives.append(nm)
        mats = (N.Material * max(1, len(natives)))(*natives)
        d.num_materials = len(flat["materials"])
        if textures:
            tables = (N.Texture * len(textures))()
            parts, off = [], 0
            for k, t in enumerate(textures):
                tx = t.texels()
                tables[k].w, tables[k].h, tables[k].c, tables[k].offset = tx.shape[1], tx.shape[0], tx.shape[2], off
                parts.append(tx.reshape(-1))
                off += tx.size
            texels = arr(np.concatenate(parts), np.float32)
            keep.append(tables)
            d.num_textures = len(textures)
            d.textures = C.cast(tables, C.POINTER(N.Texture))
            d.num_texels = texels.size
            d.texels = N.fptr(texels)
            d.texcoords = N.fptr(arr(flat["texcoords"], np.float32))
        d.materials = C.cast(mats, C.POINTER(N.Material))
        lights = (N.Light * max(1, len(flat["lights"])))(*flat["lights"])
        d.num_lights = len(flat["lights"])
        d.lights = C.cast(lights, C.POINTER(N.Light))
        d.num_light_tris = flat["light_tri_p"].shape[0]
        d.light_tri_p = N.fptr(arr(flat["light_tri_p"], np.float32))
        d.light_tri_gn = N.fptr(arr(flat["light_tri_gn"], np.float32))
        d.light_tri_area = N.fptr(arr(flat["light_tri_area"], np.float32))
        d.num_env_texels = flat["env_texels"].size
        d.env_texels = N.fptr(arr(flat["env_texels"], np.float32))
        if self._camera is not None:
            cam = self.nodes[self._camera]["camera"]
            d.has_camera = 1
            d.camera.position[:] = [float(x) for x in cam.position]
            d.camera.center[:] = [float(x) for x in cam.center]
            d.camera.up[:] = [float(x) for x in cam.up]
            d.camera.vfov = cam.vfov
            d.camera.aspect = cam.aspect
        h = C.c_void_p()
        N.check(N.lib().lmgpu_scene_create(C.byref(h), self._accel._h, C.byref(d)))
        self._h = h
        self._flat = flat

    def flattened(self) -> dict:
        if self._flat is None:
            raise LmGpuError(3, "scene is not built")
        return self._flat

    # -- requirements (scene.h:247-300) -----------------------------------------------------------
    def require_primitive(self):
        if len(self.nodes) <= 1:
            raise LmGpuError(2, "Missing primitives. Use lm::primitive() function to add primitives.")

    def require_camera(self):
        if self._camera is None:
            raise LmGpuError(2, "Missing camera primitive. Use lm::primitive() function to add camera primitive.")

    def require_light(self):
        if self.num_lights() == 0:
            raise LmGpuError(2, "No light in the scene. Add at least one light sources to the scene.")

    def require_accel(self):
        if self._accel is None:
            raise LmGpuError(2, "Missing acceleration structure. Use lm::build() function before rendering.")

    def require_renderable(self):
        self.require_primitive()
        self.require_camera()
        self.require_light()
        self.require_accel()

    def _require_built(self):
        if self._h is None:
            raise LmGpuError(3, "Scene is not built. Call scene.build() before rendering.")


# ---------------------------------------------------------------------------------------------
# Renderers

_SAMPLING = {"naive": 0, "nee": 1, "mis": 2}
_PRIMARY = {"pixel": 0, "image": 1}


@_reg("renderer::blank")
class RendererBlank(Component):
    """renderer::blank (src/renderer/renderer_blank.cpp:14-47): every pixel of the output film
    set to `color`."""

    def construct(self, prop):
        self.color = [float(x) for x in _vec3(_req(prop, "color"))]
        self.film = _resolve(_req(prop, "output"))

    def render(self) -> dict:
        N.check(N.lib().lmgpu_film_fill(self.film._h, (C.c_float * 3)(*self.color)))
        return {}


@_reg("renderer::raycast", "renderer::raycast_gpu")
class RendererRaycast(Component):
    """renderer::raycast (src/renderer/renderer_raycast.cpp:48-101)."""

    def construct(self, prop):
        self.scene = _resolve(_req(prop, "scene"))
        self.film = _resolve(_req(prop, "output"))
        self.params = N.RaycastParams()
        self.params.bg_color[:] = [float(x) for x in _vec3(prop.get("bg_color", [0, 0, 0]))]
        self.params.use_constant_color = int(bool(prop.get("use_constant_color", False)))
        self.params.visualize_normal = int(bool(prop.get("visualize_normal", False)))
        if prop.get("color") is not None:
            self.params.has_color = 1
            self.params.color[:] = [float(x) for x in _vec3(prop["color"])]

    def render(self) -> dict:
        self.scene.require_primitive()
        self.scene.require_accel()
        self.scene.require_camera()
        self.scene._require_built()
        t0 = time.perf_counter()
        N.check(N.lib().lmgpu_render_raycast(self.scene._h, self.film._h, C.byref(self.params), None))
        return {"elapsed": time.perf_counter() - t0}


def next_spp_for_error(spp: int, rel_mse: float, target: float, margin: float = 1.05) -> int:
    """Samples per pixel an estimate needs to reach `target` relative MSE, from `rel_mse` measured
    after `spp`: the variance of the mean falls as 1/N (a few percent of margin for the
    estimate's own noise)."""
    return int(math.ceil(spp * rel_mse / target * margin))


@_reg("renderer::pt", "renderer::pt_gpu")
class RendererPT(Component):
    """renderer::pt (src/renderer/renderer_pt.cpp:51-315) as a wavefront on the GPU.

    Props as the reference: scene, output, max_verts, seed, sampling_mode (naive|nee|mis),
    primary_ray_sampling_mode (pixel|image), scheduler ('sample' with spp; 'time' with
    render_time renders progressively in rounds of `spp_per_round` until the time is spent).
    GPU extras: wave_paths (paths in flight per wave); scheduler 'error' with target_rel_mse and
    spp (the most it renders) renders progressively until the film's relative-MSE estimate
    (lmgpu_film_rel_mse over even / odd passes, eps rel_mse_eps = 0.01) is at or below the target:
    a first round of spp_first (8) passes, then rounds sized from the estimate's 1/N fall-off."""

    def construct(self, prop):
        self.scene = _resolve(_req(prop, "scene"))
        self.film = _resolve(_req(prop, "output"))
        self.max_verts = int(_req(prop, "max_verts"))
        seed = prop.get("seed")
        self.seed = int(seed) if seed is not None else int(time.time_ns() & 0xFFFFFFFF)
        sm = prop.get("sampling_mode", "mis")
        if sm not in _SAMPLING:
            raise LmGpuError(1, f"Invalid sampling_mode '{sm}'")
        self.sampling_mode = _SAMPLING[sm]
        pm = prop.get("primary_ray_sampling_mode", "pixel")
        if pm not in _PRIMARY:
            raise LmGpuError(1, f"Invalid primary_ray_sampling_mode '{pm}'")
        self.primary_mode = _PRIMARY[pm]
        self.scheduler = _req(prop, "scheduler")
        npix = self.film.w * self.film.h
        if self.scheduler == "sample":
            if self.primary_mode == _PRIMARY["image"] and "num_samples" in prop:
                # scheduler::spi::sample counts paths (renderer_pt.cpp:71-75); the wavefront takes
                # whole passes of w*h paths, so num_samples is rounded up to a multiple of w*h
                self.spp = max(1, -(-int(prop["num_samples"]) // npix))
            else:
                self.spp = int(_req(prop, "spp"))
        elif self.scheduler == "time":
            self.render_time = float(_req(prop, "render_time"))
            self.spp_per_round = int(prop.get("spp_per_round", 1))
        elif self.scheduler == "error":
            self.target_rel_mse = float(_req(prop, "target_rel_mse"))
            self.spp = int(_req(prop, "spp"))
            self.spp_first = max(2, int(prop.get("spp_first", 8)))
            self.rel_mse_eps = float(prop.get("rel_mse_eps", 1e-2))
            if self.target_rel_mse <= 0 or self.spp < 2:
                raise LmGpuError(1, "scheduler 'error' needs target_rel_mse > 0 and spp >= 2")
        else:
            raise LmGpuError(1, f"Invalid scheduler '{self.scheduler}'")
        # processed samples as the reference's scheduler reports them: passes in pixel mode
        # (scheduler::spp), paths in image mode (scheduler::spi)
        self._per_pass = npix if self.primary_mode == _PRIMARY["image"] else 1
        self.wave_paths = int(prop.get("wave_paths", 0))
        self.last_stats: dict = {}

    def _params(self, spp: int, accumulate: bool, seed: int) -> N.PTParams:
        p = N.PTParams()
        p.spp = spp
        p.max_verts = self.max_verts
        p.seed = seed & 0xFFFFFFFF
        p.sampling_mode = self.sampling_mode
        p.primary_mode = self.primary_mode
        p.wave_paths = self.wave_paths
        p.accumulate = int(accumulate)
        return p

    def render(self) -> dict:
        self.scene.require_renderable()
        self.scene._require_built()
        t0 = time.perf_counter()
        st = N.RenderStats()
        if self.scheduler == "sample":
            N.check(N.lib().lmgpu_render_pt(self.scene._h, self.film._h, C.byref(self._params(self.spp, False, self.seed)),
                                            None, C.byref(st)))
            processed = self.spp * self._per_pass
            rays, dev_ms = st.rays, st.elapsed_ms
        elif self.scheduler == "error":
            processed, rays, dev_ms, k, done_spp = 0, 0, 0.0, 0, 0
            nxt = min(self.spp, self.spp_first)
            while True:
                p = self._params(nxt, k > 0, self.seed + 7919 * k)
                p.split_passes = 1
                N.check(N.lib().lmgpu_render_pt(self.scene._h, self.film._h, C.byref(p), None, C.byref(st)))
                done_spp += nxt
                processed += nxt * self._per_pass
                rays += st.rays
                dev_ms += st.elapsed_ms
                k += 1
                err = self.film.rel_mse(self.rel_mse_eps)
                if err <= self.target_rel_mse or done_spp >= self.spp:
                    break
                nxt = min(self.spp, max(next_spp_for_error(done_spp, err, self.target_rel_mse), done_spp + 1)) - done_spp
            self.last_rel_mse = err
            self.last_spp = done_spp
        else:
            processed, rays, dev_ms, k = 0, 0, 0.0, 0
            while True:
                N.check(N.lib().lmgpu_render_pt(self.scene._h, self.film._h,
                                                C.byref(self._params(self.spp_per_round, k > 0, self.seed + 7919 * k)),
                                                None, C.byref(st)))
                processed += self.spp_per_round * self._per_pass
                rays += st.rays
                dev_ms += st.elapsed_ms
                k += 1
                if time.perf_counter() - t0 >= self.render_time:
                    break
        elapsed = time.perf_counter() - t0
        self.last_stats = {"rays": rays, "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
                           "device_ms": dev_ms, "trace_ms": st.trace_ms}
        return {"processed": processed, "elapsed": elapsed, "rays": rays,
                "Mrays_per_s": rays / max(dev_ms, 1e-9) / 1e3}


class _SpiRenderer(Component):
    """Renderers scheduled per sample (scheduler::spi::*, src/scheduler.cpp:113-183): 'sample' with
    num_samples; 'time' with render_time and samples_per_iter (default 100000), rounds of
    samples_per_iter consecutive samples until the time is spent. The film is rescaled by
    w*h / (samples processed). `_call(n, first, accumulate, stats)` renders samples
    [first, first + n) on the GPU."""

    def _spi_construct(self, prop):
        self.scene = _resolve(_req(prop, "scene"))
        self.film = _resolve(_req(prop, "output"))
        self.max_verts = int(_req(prop, "max_verts"))
        seed = prop.get("seed")
        self.seed = int(seed) if seed is not None else int(time.time_ns() & 0xFFFFFFFF)
        self.scheduler = _req(prop, "scheduler")
        if self.scheduler == "sample":
            self.num_samples = int(_req(prop, "num_samples"))
        elif self.scheduler == "time":
            self.render_time = float(_req(prop, "render_time"))
            self.samples_per_iter = int(prop.get("samples_per_iter", 100000))
        else:
            raise LmGpuError(1, f"Invalid scheduler '{self.scheduler}'")
        self.wave_paths = int(prop.get("wave_paths", 0))
        self.last_stats: dict = {}

    def _call(self, n: int, first: int, accumulate: bool, st) -> None:
        raise NotImplementedError

    def render(self) -> dict:
        self.scene.require_renderable()
        self.scene._require_built()
        t0 = time.perf_counter()
        st = N.RenderStats()
        if self.scheduler == "sample":
            self._call(self.num_samples, 0, False, st)
            processed, rays, dev_ms = self.num_samples, st.rays, st.elapsed_ms
        else:
            # consecutive samples per round, so the rounds together are one longer render
            processed, rays, dev_ms = 0, 0, 0.0
            while True:
                self._call(self.samples_per_iter, processed, processed > 0, st)
                processed += self.samples_per_iter
                rays += st.rays
                dev_ms += st.elapsed_ms
                if time.perf_counter() - t0 > self.render_time:
                    break
        elapsed = time.perf_counter() - t0
        self.last_stats = {"rays": rays, "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
                           "device_ms": dev_ms, "trace_ms": st.trace_ms}
        return {"processed": processed, "elapsed": elapsed, "rays": rays,
                "Mrays_per_s": rays / max(dev_ms, 1e-9) / 1e3}


@_reg("renderer::bdpt", "renderer::bdpt_gpu")
class RendererBDPT(_SpiRenderer):
    """renderer::bdpt (src/renderer/renderer_bdpt.cpp:20-62, 297-413): bidirectional path tracing
    with every strategy weighted by the power heuristic (include/lm/bidir.h). Props as the
    reference: scene, output, min_verts (default 2), max_verts, seed, scheduler ('sample' with
    num_samples, or 'time'). GPU extra: wave_paths (samples per wave)."""

    strategy = 0  # LMGPU_BDPT_ALL

    def construct(self, prop):
        self._spi_construct(prop)
        self.min_verts = int(prop.get("min_verts", 2))

    def _call(self, n, first, accumulate, st):
        p = N.BDPTParams()
        p.num_samples, p.first_path, p.min_verts, p.max_verts = n, first, self.min_verts, self.max_verts
        p.seed, p.accumulate, p.wave_paths = self.seed & 0xFFFFFFFF, int(accumulate), self.wave_paths
        p.strategy = self.strategy
        N.check(N.lib().lmgpu_render_bdpt(self.scene._h, self.film._h, C.byref(p), None, C.byref(st)))


@_reg("renderer::pt_naive_path")
class RendererPTNaivePath(RendererBDPT):
    """renderer::pt_naive_path (renderer_bdpt.cpp:63-124): path tracing through the path
    structure, the eye subpath's hits on lights only (s = 0), unweighted."""
    strategy = 1


@_reg("renderer::pt_nee_path")
class RendererPTNEEPath(RendererBDPT):
    """renderer::pt_nee_path (renderer_bdpt.cpp:129-200): per path length the light endpoint
    connected to the eye subpath (s = 1), or the eye subpath's own hit on a light when that eye
    vertex is specular (s = 0), unweighted."""
    strategy = 2


@_reg("renderer::lt_nee_path")
class RendererLTNEEPath(RendererBDPT):
    """renderer::lt_nee_path (renderer_bdpt.cpp:205-288): light subpath vertices connected to the
    camera (t = 1), unweighted."""
    strategy = 3


@_reg("renderer::bdptopt")
class RendererBDPTOpt(RendererBDPT):
    """renderer::bdptopt (renderer_bdptopt.cpp:419-535): every strategy, weighted by the balance
    heuristic over pdfs without component pdfs (renderer_bdptopt.cpp:315-400)."""
    strategy = 4


@_reg("renderer::lt", "renderer::lt_gpu")
class RendererLT(_SpiRenderer):
    """renderer::lt (src/renderer/renderer_lt.cpp:18-160): light tracing with next-event
    connections to the camera, on the GPU wavefront. Props as the reference: scene, output,
    max_verts, seed, and the scheduler, which counts light paths ('sample' with num_samples, or
    'time'). GPU extra: wave_paths (light paths per wave)."""

    def construct(self, prop):
        self._spi_construct(prop)

    def _call(self, n, first, accumulate, st):
        p = N.LTParams()
        p.num_samples, p.first_path, p.max_verts = n, first, self.max_verts
        p.seed, p.wave_paths, p.accumulate = self.seed & 0xFFFFFFFF, self.wave_paths, int(accumulate)
        N.check(N.lib().lmgpu_render_lt(self.scene._h, self.film._h, C.byref(p), None, C.byref(st)))
