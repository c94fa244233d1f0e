"""lmgpu_render_pt_noalloc: path tracing for callers that cannot allocate device memory.

Some hosts cannot let the library call cudaMalloc: a framework whose pool allocator reserves all
of HBM at start-up (a library allocation would fail or go unaccounted), or a loop that must stay
free of allocations once it runs (cudaMalloc synchronizes the device and can fail mid-run). The
no-allocation entry point keeps its wavefront queues in a fixed device array and writes into a
film buffer the caller provides. This test calls it through the C-ABI twice in a row and checks
both results against lmgpu_render_pt on the same scene, seed and spp, within the tolerance the
wave-size invariance test uses (rtol 1e-5, atol 1e-6: only the order of fp32 film additions
differs): in pixel and image primary-ray modes, on a one-level box scene and on a two-level
(instanced) scene. It also checks that a wave above the fixed maximum is rejected. The test
allocates the film buffer itself; the entry point allocates nothing.
"""
import ctypes as C
import glob

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    for c in ["libcudart.so", "libcudart.so.13"] + sorted(glob.glob("/usr/local/cuda*/lib64/libcudart.so*")):
        try:
            lib = C.CDLL(c)
        except OSError:
            continue
        lib.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        lib.cudaFree.argtypes = [C.c_void_p]
        return lib
    pytest.fail("libcudart not found")


def _scene(lm, kind, W, H):
    from lightmetrica import synthetic as syn
    if kind == "box":
        scene, film = syn.box_scene(w=W, h=H, prefix="na_")
    else:
        scene, film, _ = syn.instanced_scene(n_instances=5, n_lat=8, n_lon=12, n_lights=2, w=W, h=H, env_w=16,
                                             env_h=8, seed=11, spread=3.0, prefix="nai_")
    scene.build()
    return scene, film


@pytest.mark.parametrize("kind,primary", [("box", "pixel"), ("box", "image"), ("instanced", "pixel")])
def test_noalloc_matches_render_pt(lm, kind, primary):
    from lightmetrica import _native as N
    L = N.lib()
    N.check(L.lmgpu_set_device(0))
    W, H = 32, 24
    scene, film = _scene(lm, kind, W, H)
    if kind == "instanced":
        assert scene._accel.stats()["num_instances"] > 1  # a two-level tree: the two-level kernels run

    p = N.PTParams()
    p.spp = 16
    p.max_verts = 9
    p.seed = 21
    p.sampling_mode = 2
    p.primary_mode = 1 if primary == "image" else 0
    N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(p), None, None))
    ref = film.buffer_f32().copy()
    assert ref.sum() > 0

    rt = _cudart()
    d_film = C.c_void_p()
    nbytes = W * H * 3 * 4
    assert rt.cudaMalloc(C.byref(d_film), nbytes) == 0
    try:
        for _ in range(2):
            N.check(L.lmgpu_render_pt_noalloc(scene._h, C.cast(d_film, N.c_float_p), W, H, C.byref(p), None))
            out = np.zeros((H, W, 3), np.float32)
            assert rt.cudaMemcpy(out.ctypes.data, d_film, nbytes, 2) == 0
            np.testing.assert_allclose(out, ref, rtol=1e-5, atol=1e-6)

        big = N.PTParams()
        C.memmove(C.byref(big), C.byref(p), C.sizeof(p))
        big.wave_paths = 32768 + 1
        rc = L.lmgpu_render_pt_noalloc(scene._h, C.cast(d_film, N.c_float_p), W, H, C.byref(big), None)
        assert rc == 1  # LMGPU_ERR_INVALID_ARGUMENT
        assert b"LMGPU_NOALLOC_MAX_WAVE" in L.lmgpu_last_error()
    finally:
        rt.cudaFree(d_film)
