"""Generate tests/golden/ref_path_golden.npz from the reference's OWN integrator.

The reference's cuda/hair_msnn.cu and cuda/path_tracing.cu (with
optix_common.cuh and the BSDF headers) are compiled unmodified on the host by
oracle/build.py (build_ref) through oracle/ref_shim/; their traceRay is
answered by the oracle's BVH.  This script renders one small seeded scene
with them (the HairMSNN G_BUFFER pass at BETA 1 and 3, the RENDER pass over
a seeded cache output, the scene-sample training pass, the NRC G_BUFFER pass
and the plain path tracer) and stores the scene's
arrays with the outputs, so the oracle restatement can be pinned against
them wherever the reference checkout is absent
(tests/test_ref_integrator.py).  Needs the reference checkout (HM_REF_DIR);
run:  python tests/golden/make_ref_path_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_path_golden.npz")
RES = 32
TRAIN = 256
ACCUM = 3
MAX_EV = 48
ARRAYS = ["control_points", "segments", "vertices", "normals", "triangles", "env", "env_cpdf", "env_ccdf",
          "env_mpdf", "env_mcdf", "dir_lights", "camera", "materials"]


def scene_cfg():
    from hairmsnn_gb300 import render as R
    cfg = R.straight_hair_scene(RES, RES, strands=2000, control_points=12, sky_w=64, sky_h=32, triangles=2000)
    cfg["integrator"]["shade_catmull_rom"] = True
    # framing: the head's top with the hair standing out of it
    cfg["camera"].update({"from": [0.0, -3.8, 1.0], "to": [0.0, 0.0, 0.6], "cos_fovy": 0.5})
    return cfg


def main():
    from hairmsnn_gb300 import render as R
    from oracle import pyoracle as po
    from oracle import refpath as rp
    event_digest = po.event_digest
    s = R.Scene(scene_cfg())
    o = po.OracleScene.from_library(s)
    i = s.info()
    data = {k: s.export(k) for k in ARRAYS}
    data["settings"] = o.settings
    data["env_wh"] = np.array(o.env_wh, np.int32)
    data["scene_scale"] = np.float32(i.scene_scale)
    every_nth = RES * RES // TRAIN
    data["every_nth"] = np.int32(every_nth)
    ref = rp.RefIntegrator(o, "path")
    for beta in (1, 3):
        r = ref.msnn_gbuffer(beta=beta, accum_id=ACCUM, every_nth=every_nth, n_train=TRAIN, max_events=MAX_EV)
        data[f"msnn_b{beta}_gbuf"] = r["gbuf"]
        data[f"msnn_b{beta}_nn_in"] = r["nn_in"]
        data[f"msnn_b{beta}_train_out"] = r["train_out"]
        data[f"msnn_b{beta}_n_events"] = r["n_events"]
        data[f"msnn_b{beta}_events"] = event_digest(r["events"], r["n_events"])
        if beta == 1:
            nn_out = np.random.default_rng(5).normal(0.0, 0.3, (RES * RES, 3)).astype(np.float32)
            acc = {k: np.random.default_rng(6 + j).uniform(0, 2, (RES * RES, 4)).astype(np.float32)
                   for j, k in enumerate(("pt", "nn", "final"))}
            data["render_nn_out"] = nn_out
            for a_id, tag in ((0, "first"), (ACCUM, "later")):
                rr = ref.msnn_render(r["gbuf"], nn_out, accum_id=a_id, acc=None if a_id == 0 else acc)
                for k in ("pt", "nn", "final"):
                    data[f"render_{tag}_acc_{k}"] = rr["acc"][k]
                    data[f"render_{tag}_avg_{k}"] = rr["avg"][k]
            for k in ("pt", "nn", "final"):
                data[f"render_acc_in_{k}"] = acc[k]
    nrc = rp.RefIntegrator(o, "nrc").nrc_gbuffer(accum_id=ACCUM, every_nth=every_nth, n_train=TRAIN, c=0.01,
                                                  max_events=MAX_EV)
    for k in ("gbuf", "query", "tinfo", "n_events"):
        data[f"nrc_{k}"] = nrc[k]
    tp = np.array([t * every_nth + po.feistel_perm(t, TRAIN, ACCUM) % every_nth for t in range(TRAIN)])
    data["nrc_train_pixels"] = tp
    data["nrc_train"] = nrc["train"][tp]
    data["nrc_events"] = event_digest(nrc["events"], nrc["n_events"])
    # the NRC RENDER pass and training data over that G-buffer
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_ref_integrator import nrc_cache_outputs
    nn = nrc_cache_outputs(RES * RES, TRAIN, 4)
    rr = rp.RefIntegrator(o, "nrc").nrc_render(nrc, nn, accum_id=ACCUM, every_nth=every_nth, n_train=TRAIN)
    data["nrc_render_nn"] = nn
    data["nrc_render_color"] = rr["accum"][:, :3]
    data["nrc_render_train_in"] = rr["train_in"]
    data["nrc_render_train_gt"] = rr["train_gt"]
    # the scene-sample training pass: 512 records on a 32-wide grid aiming at hair points
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_ref_integrator import hair_points
    pts = hair_points(o, 512, 11)
    tg = ref.msnn_traingen(pts, np.arange(512, dtype=np.int32), 32, beta=1, accum_id=ACCUM, max_events=MAX_EV)
    data["traingen_points"] = pts
    data["traingen_train_in"] = tg["train_in"]
    data["traingen_train_out"] = tg["train_out"]
    data["traingen_n_events"] = tg["n_events"]
    data["traingen_events"] = event_digest(tg["events"], tg["n_events"])
    pt = rp.RefIntegrator(o, "pt").pt_frame(accum_id=ACCUM, max_events=MAX_EV)
    data["pt_accum"] = pt["accum"]
    data["pt_n_events"] = pt["n_events"]
    data["pt_events"] = event_digest(pt["events"], pt["n_events"])
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
