"""Command-line path tracer with the reference's example/pt.cpp interface (example/pt.cpp:18-112):

    python -m lightmetrica.pt <obj> <out> <spp> <max_verts> <w> <h> <eye x y z> <lookat x y z> <vfov>

Loads the OBJ as model::wavefrontobj (lights for Ke > 0), a pinhole camera (up = +y, aspect w/h),
accel::sahbvh and renderer::pt with the 'sample' scheduler, renders on the GPU and saves the film
(.png, .hdr, .pfm or .npy by extension, as film::bitmap saves it).
"""
from __future__ import annotations

import sys

USAGE = "usage: python -m lightmetrica.pt <obj> <out> <spp> <max_verts> <w> <h> <eye x y z> <lookat x y z> <vfov>"


def parse(argv: list[str]) -> dict:
    """The 13 positional arguments of example/pt.cpp:31-41 as typed values."""
    if len(argv) != 13:
        raise ValueError(f"expected 13 arguments, got {len(argv)}")
    return {"obj": argv[0], "out": argv[1], "spp": int(argv[2]), "max_verts": int(argv[3]), "w": int(argv[4]),
            "h": int(argv[5]), "eye": [float(x) for x in argv[6:9]], "lookat": [float(x) for x in argv[9:12]],
            "vfov": float(argv[12])}


def run(opt: dict) -> dict:
    import lightmetrica as lm
    lm.init()
    film = lm.load_film("film1", "bitmap", w=opt["w"], h=opt["h"])
    camera = lm.load_camera("camera1", "pinhole", film=film, position=opt["eye"], center=opt["lookat"], up=[0, 1, 0],
                            vfov=opt["vfov"], aspect=opt["w"] / opt["h"])
    model = lm.load_model("obj1", "wavefrontobj", path=opt["obj"])
    accel = lm.load_accel("accel", "sahbvh")
    scene = lm.load_scene("scene", "default", accel=accel)
    scene.add_primitive(camera=camera)
    scene.add_primitive(model=model)
    scene.build()
    renderer = lm.load_renderer("renderer", "pt", output=film, scene=scene, scheduler="sample", spp=opt["spp"],
                                max_verts=opt["max_verts"])
    out = renderer.render()
    film.save(opt["out"])
    return out


def main(argv: list[str] | None = None) -> int:
    try:
        opt = parse(sys.argv[1:] if argv is None else argv)
    except ValueError as e:
        print(f"{e}\n{USAGE}", file=sys.stderr)
        return 2
    try:
        out = run(opt)
    except Exception as e:  # example/pt.cpp:106-108 logs the error
        print(f"Runtime error: {e}", file=sys.stderr)
        return 1
    print(out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
