"""The scene set-up pinned to the reference's own scene.cpp.

oracle/_ref/libhmref_scene.so is the reference's scene.cpp (parseScene,
LoadCemYuksel, Scene::extractHairData, generateEnvSamplingTables) compiled
unmodified on the host, with stand-ins for its absent libraries (cyHairFile,
nlohmann::json; oracle/ref_shim/).  Against it, bit for bit:
* the environment sampling tables of the library (hm_scene_create, for baked
  skies and decoded EXR maps) and of the oracle's two restatements
  (oracle/pyoracle.py env_tables, oracle/hm_oracle_scene.cpp), including
  all-zero rows and an all-zero map;
* the hair curves the library loads from a HAIR file (control points with
  the phantom points, 0.2 x thickness radii, segment starts, strand count,
  scene scale);
* the values the library parses from scene files that parseScene accepts
  (camera position, hair material, environment scale and rotation,
  directional lights, integrator settings), and the rejections both make.
Where the reference checkout is absent, tests/golden/ref_scene_golden.npz
(tests/golden/make_ref_scene_golden.py) holds its outputs for the oracle
restatements.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import refscene as rs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_scene_golden.npz")
needs_ref = pytest.mark.skipif(not rs.available(), reason="reference checkout absent (live reference build)")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def env_maps():
    """Seeded maps: smooth, with all-zero rows, all zero (no normalisation)."""
    rng = np.random.default_rng(5)
    smooth = rng.uniform(0.0, 3.0, (24, 48, 4)).astype(np.float32)
    rows = rng.uniform(0.0, 1.0, (16, 32, 4)).astype(np.float32)
    rows[[0, 3, 15]] = 0.0
    zero = np.zeros((8, 16, 4), np.float32)
    return {"smooth": smooth, "zero_rows": rows, "zero": zero}


def oracle_c_tables(env):
    h, w = env.shape[:2]
    L = po.lib()
    i32 = po.ctypes.c_int
    L.hmo_env_tables.restype = None
    L.hmo_env_tables.argtypes = [po.F32P, i32, i32, po.F32P, po.F32P, po.F32P, po.F32P]
    out = [np.zeros((h, w + 1), np.float32), np.zeros((h, w + 1), np.float32), np.zeros(h + 1, np.float32),
           np.zeros(h + 1, np.float32)]
    L.hmo_env_tables(np.ascontiguousarray(env, np.float32).ravel(), w, h, out[0].ravel(), out[1].ravel(), out[2],
                     out[3])
    return out


def check_tables(env, ref):
    h, w = env.shape[:2]
    for got in (po.env_tables(env.reshape(-1, 4), w, h), oracle_c_tables(env)):
        for k, g in zip(("cpdf", "ccdf", "mpdf", "mcdf"), got):
            assert np.array_equal(bits(np.asarray(g).reshape(ref[k].shape)), bits(ref[k])), k


# ------------------------------------------------------------------ golden
@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", ["smooth", "zero_rows", "zero"])
def test_oracle_env_tables_match_reference_golden(gold, name):
    env = env_maps()[name]
    check_tables(env, {k: gold[f"env_{name}_{k}"] for k in ("cpdf", "ccdf", "mpdf", "mcdf")})


def test_golden_hair_extraction_matches_oracle_restatement(gold):
    """The reference's extractHairData of the golden HAIR file against the
    restatement the loader tests use (tests/test_scene_loaders.py)."""
    from test_scene_loaders import extract_hair_data
    segs, pts, thick = gold["hair_segs"], gold["hair_points"], gold["hair_thickness"]
    cps, seg = extract_hair_data(list(segs), pts, thick)
    assert np.array_equal(bits(cps), bits(gold["hair_cp"]))
    assert np.array_equal(seg, gold["hair_segments"])


def test_library_hair_file_matches_reference_golden(gold, tmp_path):
    """The library's HAIR loader (host only) on the golden file: control
    points, segment starts and scene scale as the reference extracted them."""
    from hairmsnn_gb300 import render as R
    from test_scene_loaders import scene_json, write_hair
    write_hair(tmp_path / "g.hair", list(gold["hair_segs"]), gold["hair_points"], gold["hair_thickness"])
    s = R.Scene(scene_json(hair={"geometry": "g.hair"}), str(tmp_path))
    assert np.array_equal(bits(s.export("control_points")), bits(gold["hair_cp"]))
    assert np.array_equal(s.export("segments"), gold["hair_segments"])
    assert np.array_equal(bits(np.float32(s.info().scene_scale)), bits(gold["hair_bounds"][6]))


@pytest.mark.parametrize("name", ["smooth", "zero_rows"])
def test_library_env_tables_match_reference_golden(gold, tmp_path, name):
    """The library's tables (host only) for the golden maps decoded from EXR."""
    from test_exr_env import env_scene, write_exr
    env = env_maps()[name].copy()
    env[:, :, 3] = 1.0  # alpha does not enter the tables
    write_exr(tmp_path / "e.exr", {c: env[:, :, i] for i, c in enumerate("RGB")}, "zip")
    s = env_scene(tmp_path, "e.exr")
    for k, arr in (("cpdf", "env_cpdf"), ("ccdf", "env_ccdf"), ("mpdf", "env_mpdf"), ("mcdf", "env_mcdf")):
        ref = gold[f"env_{name}_{k}"]
        assert np.array_equal(bits(s.export(arr).reshape(ref.shape)), bits(ref)), k


# ------------------------------------------------------------------ live
@needs_ref
@pytest.mark.parametrize("name", ["smooth", "zero_rows", "zero"])
def test_env_tables_match_reference(tmp_path, name):
    from test_exr_env import env_scene, write_exr
    env = env_maps()[name]
    ref = rs.env_tables(env)
    check_tables(env, ref)
    if name != "zero":  # the library, through a decoded EXR map (RGB; A = 1)
        env = env.copy()
        env[:, :, 3] = 1.0
        write_exr(tmp_path / "e.exr", {c: env[:, :, i] for i, c in enumerate("RGB")}, "zip")
        s = env_scene(tmp_path, "e.exr")
        ref = rs.env_tables(s.export("env").reshape(env.shape))
        for k, arr in (("cpdf", "env_cpdf"), ("ccdf", "env_ccdf"), ("mpdf", "env_mpdf"), ("mcdf", "env_mcdf")):
            assert np.array_equal(bits(s.export(arr).reshape(ref[k].shape)), bits(ref[k])), k


@needs_ref
def test_sky_env_tables_match_reference():
    from hairmsnn_gb300 import render as R
    s = R.Scene(R.straight_hair_scene(128, 128, strands=100, control_points=8, sky_w=64, sky_h=32))
    env = s.export("env").reshape(32, 64, 4)
    ref = rs.env_tables(env)
    for k, arr in (("cpdf", "env_cpdf"), ("ccdf", "env_ccdf"), ("mpdf", "env_mpdf"), ("mcdf", "env_mcdf")):
        assert np.array_equal(bits(s.export(arr).reshape(ref[k].shape)), bits(ref[k])), k


@needs_ref
@pytest.mark.parametrize("with_segments,with_thickness", [(True, True), (False, False), (True, False)])
def test_hair_file_matches_reference(tmp_path, with_segments, with_thickness):
    from hairmsnn_gb300 import render as R
    from test_scene_loaders import scene_json, write_hair
    rng = np.random.default_rng(7)
    segs = [3, 1, 2, 5, 1] if with_segments else [2, 2, 2, 2]
    n_pts = sum(s + 1 for s in segs)
    pts = np.cumsum(rng.normal(scale=0.1, size=(n_pts, 3)), axis=0).astype(np.float32)
    thick = rng.uniform(0.5, 2.0, n_pts).astype(np.float32) if with_thickness else None
    write_hair(tmp_path / "h.hair", segs, pts, thick, default_segments=None if with_segments else 2,
               default_thickness=0.7)
    ref = rs.hair_file(tmp_path / "h.hair")
    s = R.Scene(scene_json(hair={"geometry": "h.hair"}), str(tmp_path))
    assert np.array_equal(bits(s.export("control_points")), bits(ref["cp"]))
    assert np.array_equal(s.export("segments"), ref["segments"])
    info = s.info()
    assert info.n_strands == ref["strands"]
    assert np.array_equal(bits(np.float32(info.scene_scale)), bits(ref["bounds"][6]))


# ---- parseScene
def base_scene(**over):
    cfg = {"camera": {"from": [0.2, -3.5, 0.4], "to": [0, 0, 0.1], "up": [0, 0, 1], "cos_fovy": 0.61},
           "hair": {"geometry": "h.hair", "type": 1, "sigma_a": [0.11, 0.22, 0.33], "beta_m": 0.25,
                    "beta_n": 0.35, "alpha": 2.5, "Gain R": 0.9, "Gain TT": 1.1, "Gain TRT": 1.2, "Gain TRRT": 0.8},
           "lights": {"directional": [{"from": [3, 2, 1], "emit": [2, 2, 1.5]}, {"from": [-1, 0, 2], "emit": [1, 1, 1]}]},
           "integrator": {"spp": 16, "path_v1": 1, "path_v2": 40, "width": 256, "height": 128, "image_output": "o.exr",
                          "stats_output": "s.json", "MIS": True, "ENV_PDF": False}}
    for k, v in over.items():
        if v is None:
            cfg.pop(k)
        else:
            cfg[k] = v
    return cfg


def parse_cases():
    def without(block, *keys):
        c = base_scene()
        for k in keys:
            c[block].pop(k)
        return c
    def edit(fn):
        c = base_scene()
        fn(c)
        return c
    return {
        "full": base_scene(),
        "material_defaults": without("hair", "sigma_a", "beta_m", "alpha", "Gain TT"),
        "no_material_type": without("hair", "type"),  # parseScene keeps every material default
        "one_light": edit(lambda c: c["lights"]["directional"].pop()),
        "ints_as_numbers": edit(lambda c: c["camera"].update({"cos_fovy": 1})),
        "no_camera": base_scene(camera=None),
        "camera_missing_up": edit(lambda c: c["camera"].pop("up")),
        "too_large": edit(lambda c: c["integrator"].update({"width": 4096, "height": 2048})),
        "not_multiple_of_128": edit(lambda c: c["integrator"].update({"width": 100, "height": 100})),
    }


def library_parse(cfg, tmp_path):
    from hairmsnn_gb300 import render as R
    try:
        s = R.Scene(json.dumps(cfg), str(tmp_path))
    except Exception:
        return None
    i = s.info()
    m = s.export("materials")[0]
    cam = s.export("camera")[0]
    return {"from": cam[:3], "material": m[:10], "env": m[14:16], "lights": s.export("dir_lights"),
            "integrator": (i.spp, i.path_v1, i.path_v2, i.width, i.height, i.mis, i.env_pdf)}


PARSE_HAIR = ([3, 2], np.arange(21, dtype=np.float32).reshape(7, 3) * 0.1)


def check_parse(case, ok, ref, lights, tmp_path):
    cfg = parse_cases()[case]
    got = library_parse(cfg, tmp_path)
    assert (ok == 1) == (got is not None), (case, ok)
    if got is None:
        return
    assert np.array_equal(bits(got["from"]), bits([ref["from_x"], ref["from_y"], ref["from_z"]]))
    want = [ref["sigma_a_r"], ref["sigma_a_g"], ref["sigma_a_b"], ref["beta_m"], ref["beta_n"], ref["alpha"],
            ref["gain_r"], ref["gain_tt"], ref["gain_trt"], ref["gain_trrt"]]
    assert np.array_equal(bits(got["material"]), bits(want)), (got["material"], want)
    assert np.array_equal(bits(got["lights"].reshape(-1, 6)), bits(lights))
    assert got["integrator"] == (int(ref["spp"]), int(ref["path_v1"]), int(ref["path_v2"]), int(ref["width"]),
                                 int(ref["height"]), int(ref["mis"]), int(ref["env_pdf"]))
    assert ref["has_hair"] == 1


@pytest.mark.parametrize("case", list(parse_cases()))
def test_library_parse_matches_reference_golden(gold, tmp_path, case):
    from test_scene_loaders import write_hair
    write_hair(tmp_path / "h.hair", *PARSE_HAIR)
    vals = gold[f"parse_{case}_vals"]
    check_parse(case, int(gold[f"parse_{case}_ok"]), {k: float(vals[i]) for i, k in enumerate(rs.PARSE_FIELDS)},
                gold[f"parse_{case}_lights"], tmp_path)


@needs_ref
@pytest.mark.parametrize("case", list(parse_cases()))
def test_parse_scene_matches_reference(tmp_path, case):
    """Scene files parseScene accepts give the library the same values, and
    the files it rejects the library rejects too.  (The library is more
    lenient than parseScene in two places, by design: a missing integrator
    key takes its default instead of failing the file, and a scene must have
    a light, where parseScene accepts none.)"""
    from test_scene_loaders import write_hair
    write_hair(tmp_path / "h.hair", *PARSE_HAIR)
    (tmp_path / "scene.json").write_text(json.dumps(parse_cases()[case]))
    ok, ref, lights = rs.parse_scene(tmp_path / "scene.json")
    check_parse(case, ok, ref, lights, tmp_path)
