"""The oracle's procedural scenes equal the library's, array for array.

The benchmark's CPU legs (cpu_baseline and the reference arm) build their
scene with the oracle alone (oracle/hm_oracle_scene.cpp: procedural hair,
head ellipsoid, Preetham sky, the reference's environment sampling tables,
the camera and the scene scale), so they render exactly the scene the GPU
arm renders.  Checked here bit for bit against the library's scene parser
(host code only, no GPU).
"""
import numpy as np
import pytest

from oracle import pyoracle as po

NAMES = ["control_points", "segments", "vertices", "normals", "triangles", "env", "env_cpdf", "env_ccdf",
         "env_mpdf", "env_mcdf", "dir_lights", "camera", "materials"]


def _same(a, b):
    a, b = np.ascontiguousarray(a).ravel(), np.ascontiguousarray(b).ravel()
    if a.dtype == np.float32:
        return b.dtype == np.float32 and np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)


def configs():
    from hairmsnn_gb300 import render as R
    small = R.straight_hair_scene(64, 64, strands=500)
    curly = R.straight_hair_scene(128, 128, strands=300, control_points=48, triangles=3000, sky_w=128, sky_h=64)
    curly["hair"]["procedural"].update(type="curly", helix_radius=0.04, helix_pitch=0.12, seed=7)
    curly["integrator"]["MIS"] = False
    full = R.straight_hair_scene(512, 512)
    return [("small", small), ("curly", curly), ("bench_512", full)]


@pytest.mark.parametrize("name", ["small", "curly", "bench_512"])
def test_oracle_procedural_scene_equals_library(name):
    from hairmsnn_gb300 import render as R
    cfg = dict(configs())[name]
    s = R.Scene(cfg)
    o = po.procedural_scene(cfg)
    for k in NAMES:
        assert _same(s.export(k), o._keep[k]), k
    i = s.info()
    assert np.float32(i.scene_scale) == np.float32(o.scene_scale)
    assert list(o.settings) == [i.width, i.height, i.path_v1, i.path_v2, i.mis, i.env_pdf, i.has_env,
                                i.shading_catrom, i.segment_splits]
    assert tuple(o.env_wh) == (i.env_width, i.env_height)
