"""ctypes binding of liblmgpu.so (include/lmgpu.h).

The library is the product's only compute path: if it cannot be loaded, every renderer and accel
call raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblmgpu.so")

c_float_p = C.POINTER(C.c_float)
c_int32_p = C.POINTER(C.c_int32)


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("prim", C.c_int32)]


class Instance(C.Structure):
    _fields_ = [("blas", C.c_int32), ("reserved", C.c_int32), ("transform", C.c_float * 12)]


class AccelStats(C.Structure):
    _fields_ = [("num_tris", C.c_int64), ("num_nodes", C.c_int64), ("max_depth", C.c_int32), ("num_instances", C.c_int32),
                ("build_seconds", C.c_double), ("sah_cost", C.c_double), ("device_bytes", C.c_int64)]


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("color", C.c_float * 3), ("ax", C.c_float), ("ay", C.c_float), ("ni", C.c_float),
                ("ks", C.c_float * 3), ("map_kd", C.c_int32), ("mask", C.c_int32)]

    def __init__(self, *a, **kw):
        super().__init__(*a, **kw)
        if "map_kd" not in kw:
            self.map_kd = -1
        if "mask" not in kw:
            self.mask = -1


class Texture(C.Structure):
    _fields_ = [("w", C.c_int32), ("h", C.c_int32), ("c", C.c_int32), ("reserved", C.c_int32), ("offset", C.c_int64)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("ke", C.c_float * 3), ("tri_offset", C.c_int64), ("tri_count", C.c_int64),
                ("transform_j", C.c_float), ("env_w", C.c_int32), ("env_h", C.c_int32), ("env_offset", C.c_int64),
                ("rot_deg", C.c_float), ("scale", C.c_float), ("vec", C.c_float * 3)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("center", C.c_float * 3), ("up", C.c_float * 3), ("vfov", C.c_float),
                ("aspect", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("num_tris", C.c_int64), ("positions", c_float_p), ("normals", c_float_p), ("geo_normals", c_float_p),
                ("tri_prim", c_int32_p), ("num_prims", C.c_int32), ("prim_material", c_int32_p),
                ("prim_light", c_int32_p), ("num_materials", C.c_int32), ("materials", C.POINTER(Material)),
                ("num_lights", C.c_int32), ("lights", C.POINTER(Light)), ("num_light_tris", C.c_int64),
                ("light_tri_p", c_float_p), ("light_tri_gn", c_float_p), ("light_tri_area", c_float_p),
                ("num_env_texels", C.c_int64), ("env_texels", c_float_p), ("has_camera", C.c_int32),
                ("camera", Camera), ("texcoords", c_float_p), ("num_textures", C.c_int32),
                ("textures", C.POINTER(Texture)), ("num_texels", C.c_int64), ("texels", c_float_p)]


class RaycastParams(C.Structure):
    _fields_ = [("bg_color", C.c_float * 3), ("use_constant_color", C.c_int32), ("visualize_normal", C.c_int32),
                ("has_color", C.c_int32), ("color", C.c_float * 3)]


class PTParams(C.Structure):
    _fields_ = [("spp", C.c_int64), ("max_verts", C.c_int32), ("seed", C.c_uint32), ("sampling_mode", C.c_int32),
                ("primary_mode", C.c_int32), ("wave_paths", C.c_int64), ("accumulate", C.c_int32),
                ("instrument", C.c_int32), ("split_passes", C.c_int32), ("reserved", C.c_int32)]


class LTParams(C.Structure):
    _fields_ = [("num_samples", C.c_int64), ("first_path", C.c_int64), ("max_verts", C.c_int32), ("seed", C.c_uint32),
                ("wave_paths", C.c_int64), ("accumulate", C.c_int32), ("reserved", C.c_int32)]


class BDPTParams(C.Structure):
    _fields_ = [("num_samples", C.c_int64), ("first_path", C.c_int64), ("min_verts", C.c_int32), ("max_verts", C.c_int32),
                ("seed", C.c_uint32), ("accumulate", C.c_int32), ("wave_paths", C.c_int64), ("strategy", C.c_int32),
                ("reserved", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("rays", C.c_int64), ("extension_rays", C.c_int64), ("shadow_rays", C.c_int64),
                ("elapsed_ms", C.c_double), ("trace_ms", C.c_double), ("extend_ms", C.c_double),
                ("shade_ms", C.c_double), ("shadow_ms", C.c_double), ("generate_ms", C.c_double),
                ("extend_launches", C.c_int64), ("shadow_launches", C.c_int64), ("ext_nodes", C.c_double),
                ("ext_tris", C.c_double), ("shadow_nodes", C.c_double), ("shadow_tris", C.c_double),
                ("ext_max_nodes", C.c_int64), ("shadow_max_nodes", C.c_int64), ("ext_worst_ray", C.c_float * 8),
                ("shadow_worst_ray", C.c_float * 8)]


# (name, restype, argtypes) of every entry point include/lmgpu.h declares
SIGNATURES = [
    ("lmgpu_last_error", C.c_char_p, []),
    ("lmgpu_version", C.c_int, []),
    ("lmgpu_tune_set", C.c_int, [C.c_char_p, C.c_int64]),
    ("lmgpu_tune_get", C.c_int, [C.c_char_p, C.POINTER(C.c_int64)]),
    ("lmgpu_set_device", C.c_int, [C.c_int]),
    ("lmgpu_accel_create", C.c_int, [C.POINTER(C.c_void_p)]),
    ("lmgpu_accel_destroy", C.c_int, [C.c_void_p]),
    ("lmgpu_accel_build", C.c_int, [C.c_void_p, c_float_p, C.c_int64]),
    ("lmgpu_accel_build_ex", C.c_int, [C.c_void_p, c_float_p, C.c_int64, C.c_int32]),
    ("lmgpu_accel_build_instanced", C.c_int, [C.c_void_p, c_float_p, C.POINTER(C.c_int64), C.c_int32,
                                              C.POINTER(Instance), C.c_int32]),
    ("lmgpu_accel_build_instanced_ex", C.c_int, [C.c_void_p, c_float_p, C.POINTER(C.c_int64), C.c_int32,
                                                 C.POINTER(Instance), C.c_int32, C.c_int32]),
    ("lmgpu_accel_intersect", C.c_int, [C.c_void_p, c_float_p, C.c_int64, C.POINTER(Hit)]),
    ("lmgpu_accel_intersect_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("lmgpu_accel_occluded_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("lmgpu_accel_get_stats", C.c_int, [C.c_void_p, C.POINTER(AccelStats)]),
    ("lmgpu_accel_trace_counts", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("lmgpu_bvh8_build_host", C.c_int, [c_float_p, C.c_int64, C.POINTER(C.c_uint32), c_float_p,
                                        C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    ("lmgpu_bvh8_build_gpu", C.c_int, [c_float_p, C.c_int64, C.POINTER(C.c_uint32), c_float_p,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    ("lmgpu_scene_create", C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.POINTER(SceneDesc)]),
    ("lmgpu_scene_destroy", C.c_int, [C.c_void_p]),
    ("lmgpu_scene_device_bytes", C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    ("lmgpu_film_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_int32]),
    ("lmgpu_film_destroy", C.c_int, [C.c_void_p]),
    ("lmgpu_film_clear", C.c_int, [C.c_void_p]),
    ("lmgpu_probe_l2_bandwidth", C.c_int, [C.c_int64, C.c_int32, C.POINTER(C.c_double)]),
    ("lmgpu_film_fill", C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    ("lmgpu_film_read", C.c_int, [C.c_void_p, c_float_p]),
    ("lmgpu_film_device_ptr", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("lmgpu_film_rel_mse", C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_double)]),
    ("lmgpu_render_raycast", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RaycastParams), C.c_void_p]),
    ("lmgpu_render_pt", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(PTParams), C.c_void_p, C.POINTER(RenderStats)]),
    ("lmgpu_render_lt", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(LTParams), C.c_void_p, C.POINTER(RenderStats)]),
    ("lmgpu_render_bdpt", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(BDPTParams), C.c_void_p, C.POINTER(RenderStats)]),
    ("lmgpu_batch_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int64]),
    ("lmgpu_batch_destroy", C.c_int, [C.c_void_p]),
    ("lmgpu_batch_submit", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(PTParams), C.POINTER(C.c_int32)]),
    ("lmgpu_batch_run", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_int64)]),
    ("lmgpu_batch_job_status", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("lmgpu_batch_job_set_spp", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    ("lmgpu_batch_resolve", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    ("lmgpu_batch_get_stats", C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    ("lmgpu_batch_reset", C.c_int, [C.c_void_p]),
    ("lmgpu_batch_set_timing", C.c_int, [C.c_void_p, C.c_int32]),
    ("lmgpu_render_pt_noalloc", C.c_int, [C.c_void_p, c_float_p, C.c_int32, C.c_int32, C.POINTER(PTParams), C.c_void_p]),
]

ERROR_NAMES = {1: "InvalidArgument", 2: "Unsupported", 3: "Uninitialized", 4: "CUDA", 5: "OutOfMemory",
               6: "Timeout", 7: "Internal"}


class LmGpuError(RuntimeError):
    """A non-zero status from liblmgpu; `code` is the LMGPU_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERROR_NAMES.get(code, code)}] {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Loads liblmgpu.so once; raises if it is missing (build it with build_native.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"liblmgpu.so is not built ({LIB_PATH}); run lightmetrica-v3_gb300/build_native.py")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != 0:
        raise LmGpuError(code, lib().lmgpu_last_error().decode(errors="replace"))


def fptr(a) -> C.POINTER(C.c_float):
    return a.ctypes.data_as(c_float_p)


def iptr(a) -> C.POINTER(C.c_int32):
    return a.ctypes.data_as(c_int32_p)
