"""example/pt.cpp's command line (lightmetrica/pt.py) and renderer::blank (renderer_blank.cpp)."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OBJ = os.path.join(ROOT, "tests", "data", "cornell_quads.obj")


def test_cli_arguments():
    from lightmetrica import pt
    opt = pt.parse([OBJ, "o.pfm", "4", "6", "32", "24", "0.5", "0.5", "2.6", "0.5", "0.5", "0", "30"])
    assert opt["spp"] == 4 and opt["max_verts"] == 6 and (opt["w"], opt["h"]) == (32, 24)
    assert opt["eye"] == [0.5, 0.5, 2.6] and opt["lookat"] == [0.5, 0.5, 0.0] and opt["vfov"] == 30.0
    with pytest.raises(ValueError):
        pt.parse([OBJ, "o.pfm", "4"])
    assert pt.main(["only", "two"]) == 2   # usage error, no GPU needed


@pytest.mark.gpu
def test_cli_renders_obj(tmp_path):
    from lightmetrica import imageio
    out = str(tmp_path / "cornell.pfm")
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([os.path.join(ROOT, "lightmetrica-v3_gb300"), ROOT]))
    r = subprocess.run([sys.executable, "-m", "lightmetrica.pt", OBJ, out, "8", "6", "32", "24", "0.5", "0.5", "2.6",
                        "0.5", "0.5", "0", "30"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    img = imageio.read_pfm(out)
    assert img.shape == (24, 32, 3) and np.isfinite(img).all() and img.mean() > 0


@pytest.mark.gpu
def test_renderer_blank(lm):
    film = lm.load_film("blank_film", "bitmap", w=7, h=5)
    r = lm.load_renderer("blank_r", "blank", output=film, color=[0.25, 0.5, 1.0])
    assert r.render() == {}
    img = film.buffer()
    assert img.shape == (5, 7, 3) and np.array_equal(img, np.broadcast_to([0.25, 0.5, 1.0], (5, 7, 3)))
