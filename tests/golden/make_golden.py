"""Generates the committed golden images under tests/golden/ with the CPU oracle.

    python tests/golden/make_golden.py [box32|box256|spheres480|all]

Every image is rendered by the fp64 restatement of renderer::pt with the reference's own random
stream (std::mt19937 per thread, seed + thread id), MIS, pixel sampling. They are the high-spp
references that GPU renders are scored against by relative MSE and per-pixel z statistics.

box_ref_16k.npy -- the benchmark box scene (lightmetrica.synthetic.box_scene, seed 1234) at 32 x 32,
    16384 spp, max_verts = 9 (path length 8). fp64.
box256_ref_16k.npz -- the same box scene at its benchmark size, 256 x 256, 16384 spp, max_verts = 9:
    `img` (the estimate) and `var` (the per-sample variance of every pixel and channel), float16.
spheres480_ref_4k.npz -- the displaced-sphere scene of the plain drop-in benchmark
    (lightmetrica.synthetic.spheres_scene, 3,801,100 triangles) at 1/16 of its 1920 x 1080 pixels
    (480 x 270, the same camera), 4096 spp, max_verts = 11 (path length 10): `img` and `var`,
    float16.

float16 keeps the files small: its rounding (2^-11 relative) adds about 1e-7 to a relative MSE,
four orders below the 1e-3 bars. Each .json beside an image records its parameters, the oracle's
ray count and time, and the sums a test needs to predict the MSE of an N-spp render.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "lightmetrica-v3_gb300"))

import lightmetrica as lm  # noqa: E402
from lightmetrica import synthetic as syn  # noqa: E402
from oracle import oracle as O  # noqa: E402

SEED = 1234


def _render(scene, w, h, spp, max_verts, seed):
    S = O.from_lm_scene(scene, double=True)
    S.build()
    img, m2, rays, secs = S.render_pt(w, h, spp, max_verts, seed=seed, sampling_mode="mis", rng="mt19937", with_m2=True)
    var = np.maximum(m2 / spp - img * img, 0.0)  # per-sample variance per pixel and channel
    return img, var, rays, secs


def _f16(a):
    """float16 where every value fits (|a| < 60000), float32 otherwise."""
    return a.astype(np.float16) if np.abs(a).max() < 6.0e4 else a.astype(np.float32)


def _meta(name, scene_desc, w, h, spp, max_verts, seed, img, var, rays, secs):
    return {"scene": scene_desc, "w": w, "h": h, "spp": spp, "max_verts": max_verts, "seed": seed,
            "sampling_mode": "mis", "rng": "mt19937 per thread (reference stream)", "oracle": "fp64",
            "rays": int(rays), "seconds": secs, "mean": float(img.mean()),
            "mean_sample_variance": float(var.mean()),
            # sum of squares of the image and of the per-sample variance: an unbiased N-spp render
            # has E[sum (x - img)^2] = sum_var / N + sum_var / spp (the golden's own noise)
            "sum_img2": float(np.sum(img * img)), "sum_var": float(np.sum(var)),
            "threads": O.max_threads(), "file": name}


def box32():
    W = H = 32
    SPP, MAX_VERTS = 16384, 9
    lm.init()
    scene, _ = syn.box_scene(seed=1234, w=W, h=H)
    img, var, rays, secs = _render(scene, W, H, SPP, MAX_VERTS, SEED)
    np.save(os.path.join(HERE, "box_ref_16k.npy"), img.astype(np.float64))
    meta = _meta("box_ref_16k.npy", "synthetic.box_scene(seed=1234)", W, H, SPP, MAX_VERTS, SEED, img, var, rays, secs)
    with open(os.path.join(HERE, "box_ref_16k.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta)


def box256():
    W = H = 256
    SPP, MAX_VERTS = 16384, 9
    lm.init()
    scene, _ = syn.box_scene(seed=1234, w=W, h=H)
    img, var, rays, secs = _render(scene, W, H, SPP, MAX_VERTS, SEED)
    np.savez(os.path.join(HERE, "box256_ref_16k.npz"), img=_f16(img), var=_f16(var))
    meta = _meta("box256_ref_16k.npz", "synthetic.box_scene(seed=1234)", W, H, SPP, MAX_VERTS, SEED, img, var, rays,
                 secs)
    with open(os.path.join(HERE, "box256_ref_16k.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta)


def spheres480():
    W, H = 480, 270
    SPP, MAX_VERTS = 4096, 11
    lm.init()
    scene, _, info = syn.spheres_scene(w=W, h=H)
    img, var, rays, secs = _render(scene, W, H, SPP, MAX_VERTS, SEED)
    np.savez(os.path.join(HERE, "spheres480_ref_4k.npz"), img=_f16(img), var=_f16(var))
    meta = _meta("spheres480_ref_4k.npz", "synthetic.spheres_scene() at 480x270", W, H, SPP, MAX_VERTS, SEED, img,
                 var, rays, secs)
    meta["triangles"] = info["triangles"]
    with open(os.path.join(HERE, "spheres480_ref_4k.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta)


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    for name, fn in (("box32", box32), ("box256", box256), ("spheres480", spheres480)):
        if which in (name, "all"):
            fn()
