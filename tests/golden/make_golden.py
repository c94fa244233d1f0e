"""Generates the committed golden images under tests/golden/ with the CPU oracle.

    python tests/golden/make_golden.py

box_ref_16k.npy -- the benchmark box scene (lightmetrica.synthetic.box_scene, seed 1234) at 32 x 32,
16384 samples per pixel, max_verts = 9 (path length 8), MIS, pixel sampling, rendered by the fp64
restatement of renderer::pt with the reference's own random stream (std::mt19937 per thread,
seed + thread id). It is the high-spp reference that GPU renders are scored against by relative
MSE. box_ref_16k.json records the parameters and the oracle's per-pixel variance estimate.
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

W = H = 32
SPP = 16384
MAX_VERTS = 9
SEED = 1234


def main():
    lm.init()
    scene, _ = syn.box_scene(seed=1234, w=W, h=H)
    S = O.from_lm_scene(scene, double=True)
    S.build()
    img, m2, rays, secs = S.render_pt(W, H, SPP, MAX_VERTS, seed=SEED, sampling_mode="mis", rng="mt19937", with_m2=True)
    var = m2 / SPP - img * img  # per-sample variance per pixel and channel
    np.save(os.path.join(HERE, "box_ref_16k.npy"), img.astype(np.float64))
    meta = {"scene": "synthetic.box_scene(seed=1234)", "w": W, "h": H, "spp": SPP, "max_verts": MAX_VERTS,
            "seed": SEED, "sampling_mode": "mis", "rng": "mt19937 per thread (reference stream)",
            "oracle": "fp64", "rays": rays, "seconds": secs, "mean": float(img.mean()),
            "mean_sample_variance": float(var.mean()), "threads": O.max_threads()}
    with open(os.path.join(HERE, "box_ref_16k.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(meta)


if __name__ == "__main__":
    main()
