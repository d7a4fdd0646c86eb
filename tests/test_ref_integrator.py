"""The oracle's integrator pinned to the reference's own integrator.

The reference's cuda/hair_msnn.cu, cuda/path_tracing.cu and cuda/nrc.cu (rayGenCam,
msnnPathTrace, msnnTrainingPath, msnnNextPathVertex, pathTrace, and through
optix_common.cuh directLighting, sampleLights, sampleBSDF, the environment
light, hairCH, triangleMeshCH, miss) are compiled unmodified on the host
(oracle/ref_shim/ref_path_entry.cpp, ref_pt_entry.cpp); owl::traceRay is
answered by the oracle's BVH, the one closed piece (OptiX's intersector).
The oracle restatement (oracle/hm_oracle_render.cpp), which the GPU tests
compare the wavefront kernels with, must reproduce it bit for bit: every
ray each path traces (kind, hit primitive or visibility, t, u, origin,
direction), every path colour, cache-input row and training target, and the
RENDER pass's six float4 buffers.

Two ways: live against the reference-compiled libraries (where the
reference checkout is present), and against tests/golden/ref_path_golden.npz
(tests/golden/make_ref_path_golden.py), which carries its scene's arrays and
so needs neither the reference nor the library.  The scene shades curves
with the reference's Catmull-Rom interpolator (curve_utils.cuh:226-234).
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_path_golden.npz")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def events_as_reference(ev):
    """The oracle logs light / BSDF shadow rays as kinds 1 / 2 and the RNG
    state of radiance rays; the reference's trace hook sees a shadow ray
    type only and no RNG."""
    ev = np.array(ev, np.float32, copy=True)
    k = ev[:, :, 0].view(np.int32)
    k[k == 2] = 1
    ev[:, :, 10] = 0.0
    return ev


@pytest.fixture(autouse=True)
def _reference_fp32_mode():
    po.set_mp_force_fp32(True)  # the reference keeps M_p's log branch in FP32
    yield
    po.set_mp_force_fp32(False)


# ------------------------------------------------------------------ golden
@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def gold_scene(gold):
    names = ["control_points", "segments", "vertices", "normals", "triangles", "env", "env_cpdf", "env_ccdf",
             "env_mpdf", "env_mcdf", "dir_lights", "camera", "materials"]
    s = gold["settings"]
    settings = dict(width=s[0], height=s[1], path_v1=s[2], path_v2=s[3], mis=s[4], env_pdf=s[5], has_env=s[6],
                    catrom=s[7], seg_split=s[8], env_w=gold["env_wh"][0], env_h=gold["env_wh"][1])
    return po.OracleScene({k: gold[k] for k in names}, settings, float(gold["scene_scale"]))


def digest(ev, n_ev):
    return po.event_digest(ev, n_ev)


@pytest.mark.parametrize("beta", [1, 3])
def test_oracle_msnn_gbuffer_matches_reference_golden(gold, gold_scene, beta):
    en = int(gold["every_nth"])
    P = gold_scene.width * gold_scene.height
    col, nn_in, train, flags, ev, nev, _ = gold_scene.render_pixels_ev(1, beta=beta, accum_id=3, every_nth=en,
                                                                       n_train=P // en, max_events=48)
    g = gold[f"msnn_b{beta}_gbuf"]
    assert np.array_equal(bits(col), bits(g[:, 5:8]))
    assert np.array_equal(flags & 1, g[:, 0].astype(np.int32))
    assert np.array_equal((flags >> 1) & 1, (g[:, 1] * g[:, 0]).astype(np.int32))
    assert np.array_equal(bits(nn_in), bits(gold[f"msnn_b{beta}_nn_in"]))
    tp = np.nonzero(flags & 4)[0]
    assert len(tp) == P // en
    assert np.array_equal(bits(train[tp]), bits(gold[f"msnn_b{beta}_train_out"][tp // en]))
    assert np.array_equal(nev, gold[f"msnn_b{beta}_n_events"])
    assert nev.max() <= 48
    assert np.array_equal(digest(ev, nev), gold[f"msnn_b{beta}_events"])


def test_oracle_pt_matches_reference_golden(gold, gold_scene):
    col, _, _, _, ev, nev, _ = gold_scene.render_pixels_ev(0, accum_id=3, max_events=48)
    assert np.array_equal(bits(col), bits(gold["pt_accum"][:, :3]))
    assert np.array_equal(nev, gold["pt_n_events"])
    assert np.array_equal(digest(ev, nev), gold["pt_events"])


def test_oracle_render_pass_matches_reference_golden(gold):
    for a_id, tag in ((0, "first"), (3, "later")):
        acc = None if a_id == 0 else {k: gold[f"render_acc_in_{k}"] for k in ("pt", "nn", "final")}
        out = po.msnn_render(gold["msnn_b1_gbuf"], gold["render_nn_out"], accum_id=a_id, acc=acc)
        for k in ("pt", "nn", "final"):
            assert np.array_equal(bits(out["acc"][k]), bits(gold[f"render_{tag}_acc_{k}"]))
            assert np.array_equal(bits(out["avg"][k]), bits(gold[f"render_{tag}_avg_{k}"]))


def test_oracle_nrc_matches_reference_golden(gold, gold_scene):
    """nrcTracePaths / rayGenCam of cuda/nrc.cu: G-buffer, the pixels' and
    training suffixes' cache queries, the training pixels' train buffers."""
    en = int(gold["every_nth"])
    P = gold_scene.width * gold_scene.height
    o = gold_scene.render_nrc(accum_id=3, every_nth=en, n_train=P // en, c=0.01, max_events=48)
    g = gold["nrc_gbuf"]
    assert np.array_equal(o["gbuf"][:, 6], g[:, 0])
    assert np.array_equal(bits(o["gbuf"][:, 0:6]), bits(g[:, 1:7]))
    assert np.array_equal(bits(o["query"]), bits(gold["nrc_query"][:P]))
    tp = gold["nrc_train_pixels"]
    assert np.array_equal(np.nonzero(o["tinfo"][:, 3])[0], np.sort(tp))
    assert np.array_equal(bits(o["suffix_query"][tp]), bits(gold["nrc_query"][P + tp // en]))
    assert np.array_equal(o["tinfo"][tp, :2], gold["nrc_tinfo"][tp])
    assert np.array_equal(bits(o["records"][tp]), bits(gold["nrc_train"]))
    assert np.array_equal(o["n_events"], gold["nrc_n_events"])
    assert np.array_equal(digest(o["events"], o["n_events"]), gold["nrc_events"])


def test_oracle_traingen_matches_reference_golden(gold, gold_scene):
    """The scene-sample training pass (TRAIN_DATA_GEN) on the golden scene:
    records aiming at stored hair points, a 32-wide launch grid."""
    pts = gold["traingen_points"]
    tin, tout, flags, ev, nev, _ = gold_scene.render_traingen_ev(pts, beta=1, accum_id=3, rec_x=32, max_events=48)
    assert np.array_equal(bits(tin), bits(gold["traingen_train_in"]))
    assert np.array_equal(bits(tout), bits(gold["traingen_train_out"]))
    assert np.array_equal(nev, gold["traingen_n_events"])
    assert np.array_equal(digest(ev, nev), gold["traingen_events"])


def test_oracle_nrc_render_matches_reference_golden(gold):
    """The NRC RENDER pass and training data of the oracle against the
    reference's on the golden G-buffer."""
    en = int(gold["every_nth"])
    P = len(gold["nrc_gbuf"])
    T = P // en
    tp = gold["nrc_train_pixels"]
    g = gold["nrc_gbuf"]
    color, tin, tgt = po.nrc_render(rad=g[:, 1:4], beta=g[:, 4:7], hit=g[:, 0] != 0, cache=gold["nrc_render_nn"],
                                    train_px=tp, unbiased=np.arange(T) % 16 == 0, t_bounces=gold["nrc_tinfo"][tp, 0],
                                    t_hit=gold["nrc_tinfo"][tp, 1], records=gold["nrc_train"])
    assert np.array_equal(bits(color), bits(gold["nrc_render_color"]))
    assert np.array_equal(bits(tin), bits(gold["nrc_render_train_in"]))
    assert np.array_equal(bits(tgt), bits(gold["nrc_render_train_gt"]))


def test_golden_scene_exercises_the_branches(gold):
    """The fixture reaches the branches a frame bar would hide: head-surface
    (GGX) vertices, hair vertices, misses, training pixels, multi-bounce paths."""
    g = gold["msnn_b3_gbuf"]
    assert (g[:, 0] == 0).sum() > 20          # camera misses
    assert ((g[:, 0] == 1) & (g[:, 1] == 1)).sum() > 20  # head surface
    assert ((g[:, 0] == 1) & (g[:, 1] == 0)).sum() > 100  # hair
    assert gold["msnn_b3_n_events"].max() >= 10


# ------------------------------------------------------------------ live
refpath = pytest.importorskip("oracle.refpath")


def _live_scene(strands, v1=1, mis=True, res=48):
    from hairmsnn_gb300 import render as R
    cfg = R.straight_hair_scene(res, res, strands=strands, control_points=32, sky_w=128, sky_h=64, triangles=4000)
    cfg["integrator"]["shade_catmull_rom"] = True
    cfg["integrator"]["path_v1"] = v1
    cfg["integrator"]["MIS"] = mis
    s = R.Scene(cfg)
    return po.OracleScene.from_library(s)


needs_ref = pytest.mark.skipif(not refpath.available(), reason="reference checkout absent (live reference build)")


@needs_ref
@pytest.mark.parametrize("beta,strands,mis", [(1, 2000, True), (2, 4000, True), (4, 2000, False)])
def test_oracle_msnn_matches_reference_live(beta, strands, mis):
    o = _live_scene(strands, mis=mis)
    P = o.width * o.height
    en = 4
    ref = refpath.RefIntegrator(o, "path").msnn_gbuffer(beta=beta, accum_id=7, every_nth=en, n_train=P // en,
                                                         max_events=96)
    col, nn_in, train, flags, ev, nev, _ = o.render_pixels_ev(1, beta=beta, accum_id=7, every_nth=en,
                                                              n_train=P // en, max_events=96)
    assert np.array_equal(bits(col), bits(ref["gbuf"][:, 5:8]))
    assert np.array_equal(bits(nn_in), bits(ref["nn_in"]))
    tp = np.nonzero(flags & 4)[0]
    assert np.array_equal(bits(train[tp]), bits(ref["train_out"][tp // en]))
    assert np.array_equal(nev, ref["n_events"])
    assert np.array_equal(bits(events_as_reference(ev)), bits(ref["events"]))


@needs_ref
@pytest.mark.parametrize("v1,mis", [(1, True), (2, True), (1, False)])
def test_oracle_pt_matches_reference_live(v1, mis):
    o = _live_scene(3000, v1=v1, mis=mis)
    ref = refpath.RefIntegrator(o, "pt").pt_frame(accum_id=11, max_events=96)
    col, _, _, _, ev, nev, _ = o.render_pixels_ev(0, accum_id=11, max_events=96)
    assert np.array_equal(bits(col), bits(ref["accum"][:, :3]))
    assert np.array_equal(nev, ref["n_events"])
    assert np.array_equal(bits(events_as_reference(ev)), bits(ref["events"]))


@needs_ref
def test_oracle_render_pass_matches_reference_live():
    o = _live_scene(1500, res=32)
    P = o.width * o.height
    ref = refpath.RefIntegrator(o, "path")
    g = ref.msnn_gbuffer(beta=1, accum_id=0, every_nth=4, n_train=P // 4)["gbuf"]
    nn = np.random.default_rng(1).normal(0, 0.5, (P, 3)).astype(np.float32)
    acc = {k: np.random.default_rng(2 + j).uniform(0, 3, (P, 4)).astype(np.float32)
           for j, k in enumerate(("pt", "nn", "final"))}
    for a_id in (0, 5):
        r = ref.msnn_render(g, nn, accum_id=a_id, acc=None if a_id == 0 else acc)
        o_ = po.msnn_render(g, nn, accum_id=a_id, acc=acc)
        for k in ("pt", "nn", "final"):
            assert np.array_equal(bits(o_["acc"][k]), bits(r["acc"][k]))
            assert np.array_equal(bits(o_["avg"][k]), bits(r["avg"][k]))


@needs_ref
@pytest.mark.parametrize("unbiased", [False, True])
def test_oracle_nrc_matches_reference_live(unbiased):
    o = _live_scene(6000)
    P = o.width * o.height
    en = 4
    ref = refpath.RefIntegrator(o, "nrc").nrc_gbuffer(accum_id=5, every_nth=en, n_train=P // en, c=0.01,
                                                      all_unbiased=unbiased, max_events=160)
    on = o.render_nrc(accum_id=5, every_nth=en, n_train=P // en, c=0.01, max_events=160)
    if unbiased:  # the oracle has no all-unbiased switch: compare the unbiased pixels only
        keep = (np.arange(P) // en) % 16 == 0
    else:
        keep = np.ones(P, bool)
    g = ref["gbuf"]
    assert np.array_equal(on["gbuf"][keep, 6], g[keep, 0])
    assert np.array_equal(bits(on["gbuf"][keep, 0:6]), bits(g[keep, 1:7]))
    assert np.array_equal(bits(on["query"][keep]), bits(ref["query"][:P][keep]))
    tp = np.nonzero(on["tinfo"][:, 3] & keep)[0]
    assert len(tp) > 10
    assert np.array_equal(bits(on["suffix_query"][tp]), bits(ref["query"][P + tp // en]))
    assert np.array_equal(on["tinfo"][tp, :2], ref["tinfo"][tp])
    assert np.array_equal(bits(on["records"][tp]), bits(ref["train"][tp]))
    assert np.array_equal(on["n_events"][keep], ref["n_events"][keep])
    assert np.array_equal(bits(events_as_reference(on["events"])[keep]), bits(ref["events"][keep]))


def hair_points(o, n, seed):
    """n points on the scene's hair curves (uniform cubic B-spline segments at
    random u): the targets of the scene-sample pass's rays."""
    cp = np.asarray(o._keep["control_points"], np.float32).reshape(-1, 4)[:, :3]
    seg = np.asarray(o._keep["segments"], np.int64)
    rng = np.random.default_rng(seed)
    k = rng.integers(len(seg), size=n)
    u = rng.random(n).astype(np.float32)[:, None]
    v = 1.0 - u
    q = cp[seg[k][:, None] + np.arange(4)]
    b = np.stack([v * v * v / 6, (3 * u ** 3 - 6 * u * u + 4) / 6, (-3 * u ** 3 + 3 * u * u + 3 * u + 1) / 6,
                  u ** 3 / 6], 1)
    return np.einsum("nk,nkc->nc", b[:, :, 0], q).astype(np.float32)


@needs_ref
@pytest.mark.parametrize("beta,rec_x", [(1, 32), (2, 128)])
def test_oracle_traingen_matches_reference_live(beta, rec_x):
    """The scene-sample training pass (TRAIN_DATA_GEN, hair_msnn.cu:222-233):
    rays from the camera to sampled hair points, RNG seeded by the launch
    index over the frame's width, msnnTrainingPath, nnTrainInput /
    nnTrainOutput at trOfs."""
    from hairmsnn_gb300 import render as Rn
    cfg = Rn.straight_hair_scene(48, 48, strands=6000, control_points=32, sky_w=128, sky_h=64, triangles=4000)
    cfg["integrator"]["shade_catmull_rom"] = True
    cfg["camera"].update({"from": [0.0, -3.8, 1.0], "to": [0.0, 0.0, 0.6], "cos_fovy": 0.5})
    o = po.OracleScene.from_library(Rn.Scene(cfg))
    pts = hair_points(o, 3000, 3)
    R = 1024
    sidx = np.random.default_rng(4).permutation(len(pts))[:R].astype(np.int32)
    ref = refpath.RefIntegrator(o, "path").msnn_traingen(pts, sidx, rec_x, beta=beta, accum_id=2, max_events=96)
    tin, tout, flags, ev, nev, _ = o.render_traingen_ev(pts[sidx], beta=beta, accum_id=2, rec_x=rec_x,
                                                        max_events=96)
    assert (flags & 1).sum() > R // 2 and (flags & 2).sum() > 50  # hair and head-surface records
    assert (np.abs(tout).sum(1) > 0).sum() > 5
    assert np.array_equal(bits(tin), bits(ref["train_in"]))
    assert np.array_equal(bits(tout), bits(ref["train_out"]))
    assert np.array_equal(nev, ref["n_events"])
    assert np.array_equal(bits(events_as_reference(ev)), bits(ref["events"]))


def nrc_render_inputs(g, P, en, n_train, accum_id):
    """oracle nrc_render's arguments from the reference's G_BUFFER output."""
    tp = np.array([t * en + po.feistel_perm(t, n_train, accum_id) % en for t in range(n_train)])
    return dict(rad=g["gbuf"][:, 1:4], beta=g["gbuf"][:, 4:7], hit=g["gbuf"][:, 0] != 0, train_px=tp,
                unbiased=np.arange(n_train) % 16 == 0, t_bounces=g["tinfo"][tp, 0], t_hit=g["tinfo"][tp, 1],
                records=g["train"][tp])


def nrc_cache_outputs(P, n_train, seed):
    """Seeded cache outputs with negative values and NaNs (both handled by
    the RENDER pass)."""
    rng = np.random.default_rng(seed)
    nn = rng.normal(0.3, 0.5, (P + n_train, 3)).astype(np.float32)
    nn[rng.random(len(nn)) < 0.01] = np.nan
    return nn


@needs_ref
def test_oracle_nrc_render_matches_reference_live():
    """The NRC RENDER pass (nrc.cu:365-380: colour = radiance + beta x
    max(cache, 0)) and nrcGenerateTrainingData (nrc.cu:70-133) of the oracle
    against the reference's own, on the reference's G-buffer."""
    o = _live_scene(6000)
    P = o.width * o.height
    en = 4
    ref = refpath.RefIntegrator(o, "nrc")
    g = ref.nrc_gbuffer(accum_id=2, every_nth=en, n_train=P // en, c=0.01, max_events=8)
    nn = nrc_cache_outputs(P, P // en, 3)
    # the same frame as the G-buffer (its trainIdxs); zero running sums: accum = colour
    r = ref.nrc_render(g, nn, accum_id=2, every_nth=en, n_train=P // en)
    color, tin, tgt = po.nrc_render(cache=nn, **nrc_render_inputs(g, P, en, P // en, 2))
    assert (g["tinfo"][:, 0] > 1).sum() > 50  # multi-vertex training paths
    assert np.array_equal(bits(color), bits(r["accum"][:, :3]))
    assert np.array_equal(bits(tin), bits(r["train_in"]))
    assert np.array_equal(bits(tgt), bits(r["train_gt"]))
