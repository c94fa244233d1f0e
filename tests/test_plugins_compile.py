"""The plugin sources a maintainer adds to the reference (lightmetrica-v3_gb300/plugin/:
accel::gpu and renderer::pt_gpu) compile against the reference's own interface headers (CPU).

The headers are the reference's include/lm/*.h as oracle/_ref/include/lm links them, with the
component framework (nlohmann_json, cereal, the registry) and glm taken from the checker's
stand-ins (oracle/ref_shim/). So every override, signature and call in the plugins is checked
against the reference's real Accel, Renderer, Scene, Film, Material and Light interfaces. Only
where the reference's sources are present."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLUGINS = ["accel_gpu.cpp", "renderer_pt_gpu.cpp"]


@pytest.mark.parametrize("src", PLUGINS)
def test_plugin_compiles_against_reference_headers(ref_mod, src):
    oracle = os.path.join(ROOT, "oracle")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wno-unknown-pragmas",
           "-I", os.path.join(oracle, "ref_shim"), "-I", os.path.join(oracle, "_ref", "include"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "lightmetrica-v3_gb300", "plugin", src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
