"""The C-ABI library loads and exports every entry point include/lmgpu.h declares; error codes and
messages come back without a GPU (no compute call is made here)."""
import ctypes as C
import os
import re

import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "lmgpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(lmgpu_\w+)\s*\(", text, flags=re.M)))


def test_header_parses():
    names = declared_functions()
    assert "lmgpu_accel_intersect" in names and "lmgpu_render_pt" in names
    assert len(names) >= 20


def test_every_declared_symbol_is_exported(native_lib):
    missing = [n for n in declared_functions() if not hasattr(native_lib, n)]
    assert not missing, missing


def test_binding_covers_header(native_lib):
    from lightmetrica import _native as N
    bound = {name for name, _, _ in N.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_errors_without_device(native_lib):
    from lightmetrica import _native as N
    L = native_lib
    f = C.c_void_p()
    assert L.lmgpu_film_create(C.byref(f), 0, 4) == 1  # LMGPU_ERR_INVALID_ARGUMENT
    assert b"film size" in L.lmgpu_last_error()
    a = C.c_void_p()
    assert L.lmgpu_accel_create(C.byref(a)) == 0
    hits = (N.Hit * 1)()
    rays = (C.c_float * 8)()
    assert L.lmgpu_accel_intersect(a, rays, 1, hits) == 3  # LMGPU_ERR_UNINITIALIZED
    assert b"not built" in L.lmgpu_last_error()
    assert L.lmgpu_accel_destroy(a) == 0
    st = N.AccelStats()
    assert L.lmgpu_accel_get_stats(None, C.byref(st)) == 1
    assert L.lmgpu_scene_create(None, None, None) == 1


def test_version(native_lib):
    assert native_lib.lmgpu_version() >= 1


def test_oracle_library_loads(oracle_mod):
    assert oracle_mod.max_threads() >= 1


def test_tuning_keys(native_lib):
    """lmgpu_tune_set/get: known keys round-trip, bad keys and out-of-range values are refused."""
    L = native_lib
    v = C.c_int64()
    assert L.lmgpu_tune_get(b"trace_refill", C.byref(v)) == 0
    old = v.value
    assert 0 <= old <= 32
    try:
        assert L.lmgpu_tune_set(b"trace_refill", 7) == 0
        assert L.lmgpu_tune_get(b"trace_refill", C.byref(v)) == 0 and v.value == 7
        assert L.lmgpu_tune_set(b"trace_refill", 33) == 1
        assert b"trace_refill" in L.lmgpu_last_error()
        assert L.lmgpu_tune_set(b"no_such_key", 1) == 1
        assert b"unknown tuning key" in L.lmgpu_last_error()
        assert L.lmgpu_tune_get(b"no_such_key", C.byref(v)) == 1
        assert L.lmgpu_tune_set(None, 1) == 1
        assert L.lmgpu_tune_get(b"batch_first_pass", C.byref(v)) == 0 and v.value in (0, 1)
        assert L.lmgpu_tune_set(b"batch_first_pass", 2) == 1
        assert L.lmgpu_tune_set(b"shade_minblocks", 5) == 1
    finally:
        assert L.lmgpu_tune_set(b"trace_refill", old) == 0


_STRUCTS = {"Hit": "lmgpu_hit", "Instance": "lmgpu_instance", "AccelStats": "lmgpu_accel_stats", "Material": "lmgpu_material",
            "Light": "lmgpu_light", "Camera": "lmgpu_camera", "SceneDesc": "lmgpu_scene_desc", "Texture": "lmgpu_texture",
            "RaycastParams": "lmgpu_raycast_params", "PTParams": "lmgpu_pt_params", "LTParams": "lmgpu_lt_params",
            "BDPTParams": "lmgpu_bdpt_params", "RenderStats": "lmgpu_render_stats"}


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes mirror of a header struct has the C compiler's size and field offsets (the
    layout a binding in another language must reproduce)."""
    import shutil
    import subprocess
    from lightmetrica import _native as N
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lmgpu.h"', "int main(void) {"]
    for py, c in _STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in getattr(N, py)._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = {}
    for row in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        py, field, v = row.split()
        got[(py, field)] = int(v)
    for py in _STRUCTS:
        cls = getattr(N, py)
        assert got[(py, "size")] == C.sizeof(cls), py
        for name, _ in cls._fields_:
            assert got[(py, name)] == getattr(cls, name).offset, (py, name)
