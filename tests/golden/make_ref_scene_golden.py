"""Generate tests/golden/ref_scene_golden.npz from the reference's OWN scene.cpp.

The reference's scene.cpp (generateEnvSamplingTables, LoadCemYuksel,
Scene::extractHairData, parseScene) is compiled unmodified on the host by
oracle/build.py (build_ref) through oracle/ref_shim/.  This script runs it
on the seeded environment maps of tests/test_ref_scene.py, on one seeded
HAIR file and on that test's scene files, and stores inputs and outputs, so the oracle restatements can be
pinned against them wherever the reference checkout is absent
(tests/test_ref_scene.py).  Needs the reference checkout (HM_REF_DIR); run:
python tests/golden/make_ref_scene_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
OUT = os.path.join(HERE, "ref_scene_golden.npz")


def main():
    from oracle import refscene as rs
    from test_ref_scene import env_maps
    from test_scene_loaders import write_hair
    data = {}
    for name, env in env_maps().items():
        for k, v in rs.env_tables(env).items():
            data[f"env_{name}_{k}"] = v
    rng = np.random.default_rng(21)
    segs = np.array([4, 1, 3, 2, 6], np.int32)
    pts = np.cumsum(rng.normal(scale=0.1, size=(int((segs + 1).sum()), 3)), axis=0).astype(np.float32)
    thick = rng.uniform(0.5, 2.0, len(pts)).astype(np.float32)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "g.hair")
        write_hair(path, list(segs), pts, thick)
        ref = rs.hair_file(path)
    data.update(hair_segs=segs, hair_points=pts, hair_thickness=thick, hair_cp=ref["cp"],
                hair_segments=ref["segments"], hair_bounds=ref["bounds"])
    # parseScene on the scene files of tests/test_ref_scene.py
    import json
    from test_ref_scene import PARSE_HAIR, parse_cases
    for name, cfg in parse_cases().items():
        with tempfile.TemporaryDirectory() as d:
            write_hair(os.path.join(d, "h.hair"), *PARSE_HAIR)
            path = os.path.join(d, "scene.json")
            with open(path, "w") as f:
                json.dump(cfg, f)
            ok, vals, lights = rs.parse_scene(path)
        data[f"parse_{name}_ok"] = np.int32(ok)
        data[f"parse_{name}_vals"] = np.array([vals[k] for k in rs.PARSE_FIELDS], np.float32)
        data[f"parse_{name}_lights"] = lights
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
