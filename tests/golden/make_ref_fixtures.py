"""Generates the committed hit fixtures under tests/golden/ with the reference's own accel code.

    python tests/golden/make_ref_fixtures.py [c2|transformed|box256|all]

They come from oracle/_ref/liblmref.so, the reference's own sources compiled unmodified by
`make -C oracle ref` (for hits: src/accel/accel_sahbvh.cpp's Tri::intersect, multithreaded
full-sort SAH build and stack traversal with include/lm/math.h's Bound, Float = double; for
images: src/renderer/renderer_pt.cpp with the scene, film and scheduler). So these fixtures are
outputs of the reference itself; machines without the reference's sources (the GPU machine) compare
against them.

ref_c2_probe_hits.npz -- the displaced-sphere scene of the plain drop-in benchmark
    (lightmetrica.synthetic.spheres_parts, seed 7, 3,801,100 triangles) and every 1024th ray of the
    16,777,216-ray uniform-sphere probe (synthetic.sphere_rays from RAYCAST_PROBE_ORIGIN with
    RAYCAST_PROBE_SEED): `ray` (probe ray index), `tri` (flattened triangle index, -1 = miss), `t`,
    `uv` (float64, as Accel::Hit reports them).
ref_transformed_hits.npz -- tests/ref_scenes.transformed_scene() (nested group transforms, shared
    edges, duplicated and degenerate triangles, an axis-aligned cube) with pin_rays(): `tri`, `t`,
    `uv` for every ray.
ref_box256_pt16.npz -- the reference's own renderer::pt (renderer_pt.cpp, path.h, scene.cpp,
    film_bitmap.cpp, scheduler::spp::sample) on the benchmark box scene (synthetic.box_scene,
    seed 1234) at its benchmark configuration: 256 x 256, 16 spp, max_verts 9, MIS, pixel
    sampling, one thread with Rng seed 77. `img`, float32, as the film holds it (row 0 at the
    bottom).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "lightmetrica-v3_gb300"))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref as R  # noqa: E402
import ref_scenes as RS  # noqa: E402
from lightmetrica import synthetic as syn  # noqa: E402

C2_STRIDE = 1024


def c2_probe():
    parts = syn.spheres_parts(seed=7)
    S = R.from_parts(parts)
    build_s = S.build()
    rays = syn.sphere_rays(syn.RAYCAST_PROBE_RAYS, syn.RAYCAST_PROBE_ORIGIN, seed=syn.RAYCAST_PROBE_SEED)
    sel = np.arange(0, len(rays), C2_STRIDE)
    t, uv, tri = S.intersect(rays[sel])
    np.savez_compressed(os.path.join(HERE, "ref_c2_probe_hits.npz"), ray=sel.astype(np.int32),
                        tri=tri.astype(np.int32), t=t, uv=uv)
    meta = {"scene": "synthetic.spheres_parts(seed=7)", "triangles": 3801100, "probe_rays": len(rays),
            "stride": C2_STRIDE, "rays": int(len(sel)), "hits": int((tri >= 0).sum()),
            "reference": "src/accel/accel_sahbvh.cpp + include/lm/math.h (Float = double)",
            "reference_build_seconds": round(build_s, 2)}
    json.dump(meta, open(os.path.join(HERE, "ref_c2_probe_hits.json"), "w"), indent=1)
    print(meta)


def transformed():
    desc = RS.transformed_scene()
    S = RS.to_ref(desc)
    S.build()
    rays = RS.pin_rays(desc)
    t, uv, tri = S.intersect(rays)
    np.savez_compressed(os.path.join(HERE, "ref_transformed_hits.npz"), tri=tri.astype(np.int32), t=t, uv=uv)
    print({"rays": len(rays), "hits": int((tri >= 0).sum())})


def box256_pt16():
    import lightmetrica as lm
    lm.init()
    scene, _ = syn.box_scene(seed=1234, w=256, h=256, prefix="fx_")
    S = R.from_lm_scene(scene)
    f = S.film(256, 256)
    S.build()
    img = S.render_pt(f, 16, 9, seed=77, sampling_mode="mis", primary_mode="pixel")
    np.savez_compressed(os.path.join(HERE, "ref_box256_pt16.npz"), img=img.astype(np.float32))
    print({"box256_pt16_mean": float(img.mean())})


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    if not R.available():
        sys.exit("the reference's sources are needed to build oracle/_ref/liblmref.so")
    if which in ("c2", "all"):
        c2_probe()
    if which in ("transformed", "all"):
        transformed()
    if which in ("box256", "all"):
        box256_pt16()
