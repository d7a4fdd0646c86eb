"""The NRC comparison renderer (HM_MODE_NRC) against the oracle's restatement
of nrcTracePaths (cuda/nrc.cu:136-310), which is pinned bit for bit to the
reference's own nrc.cu compiled on the host (tests/test_ref_integrator.py).

Per path, through the per-path ray logs (tests/pathcheck.py, the criterion
of tests/test_gpu_paths.py): paths whose rays agree with the oracle's must
agree in their G-buffer (radiance gathered before the cache, throughput at
the cache query), their cache-query row and their training suffix's query
row (a query's hair normal points from the fibre axis to the hit point, so
it may turn by the hit point's difference over the fibre radius:
hit_normal_tolerance); training pixels with agreeing paths in their train-buffer records and
bounce counts; the unbiased pixels (every 16th) exactly.  Paths that
separate must be ones the oracle separates itself under last-ulp changes.
Frames with online training give a finite image, lower the training loss,
and are bitwise reproducible, with or without CUDA-graph replay.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    from hairmsnn_gb300 import build, render
    build.build()
    return render


@pytest.mark.parametrize("catrom", [True, False])
def test_nrc_paths_match_oracle(R, catrom):
    from pathcheck import check_paths, color_excess, hit_normal_tolerance, nrc_oracle_runs, spread_of
    res = 64
    cfg = R.straight_hair_scene(res, res, strands=6000)
    cfg["integrator"]["shade_catmull_rom"] = catrom
    s = R.Scene(cfg)
    r = R.Renderer(s, R.NRC, train=False, seed=1, frames_in_flight=1)
    r.set_path_log(40)
    r.frame()
    P = res * res
    st = r.stats()
    gbuf, gbeta, q, tinfo = r.buffer(4), r.buffer(8), r.buffer(0), r.buffer(10)
    T = len(tinfo)  # training pixels: 65536 records / 40 vertices
    assert T == st.train_records // 40
    rec = r.buffer(9).reshape(T, 40, 5, 4)
    runs = nrc_oracle_runs(po.OracleScene.from_library(s), 120, st.every_nth, T)
    o0 = runs[0]
    tp = np.nonzero(o0["tinfo"][:, 3])[0]
    assert len(tp) == T
    tr = tp // st.every_nth
    suffix = np.zeros((P, 9), np.float32)
    suffix[tp] = q[P + tr]
    g_col = np.concatenate([gbuf[:, :3], gbeta[:, :3], q[:P], suffix], 1).astype(np.float64)
    g_log = r.read_path_log()
    # the query rows' normals (columns 12-14, 21-23) turn with the hit point
    extra = np.zeros_like(g_col)
    nt = hit_normal_tolerance(g_log, o0["log"], cfg["hair"]["procedural"]["radius"])
    extra[:, 12:15] = nt[:, None]
    extra[:, 21:24] = nt[:, None]
    # NRC paths run up to 40 vertices without Russian roulette: more of them
    # reach a last-ulp decision (the oracle's own perturbed runs separate ~35%)
    agree = check_paths(g_log, g_col, runs, f"NRC catrom={catrom}", os.environ.get("HM_PATHS_DUMP"), extra,
                        separate_max=0.15)
    assert ((gbuf[:, 3] > 0.5) == (o0["hit"] > 0.5))[agree].all()
    # training pixels: unbiased flags exactly; bounce counts and records where the path agrees
    ot = o0["tinfo"][tp]
    gt = tinfo[tr]
    assert np.array_equal(gt[:, 2], ot[:, 2])
    hitp = o0["hit"][tp] > 0.5
    ok = agree[tp] & hitp
    # training pixels trace their suffixes on (unbiased ones to the end), so
    # more of them separate than of all paths
    assert ok.sum() >= 0.7 * hitp.sum(), (ok.sum(), hitp.sum())
    assert np.array_equal(gt[ok, :2], ot[ok, :2])
    spread = spread_of(runs, "records")
    n_checked = 0
    for k in np.nonzero(ok)[0]:
        b = ot[k, 0]
        if b == 0:
            continue
        g = rec[tr[k], :b, :, :3].reshape(b, 15).astype(np.float64)
        assert color_excess(g, o0["records"][tp[k], :b], spread[tp[k], :b]).max() <= 0, k
        n_checked += 1
    assert n_checked > 20


def test_nrc_training_renders_and_is_reproducible(R):
    cfg = R.straight_hair_scene(64, 64, strands=3000)
    imgs, losses = [], []
    for graphs in (True, False):
        s = R.Scene(cfg)
        r = R.Renderer(s, R.NRC, train=True, seed=2)
        r.set_graphs(graphs)
        ls = []
        for _ in range(24):
            r.frame()
            ls.append(r.stats().last_loss)
        img = r.read()
        assert np.isfinite(img).all() and img.mean() > 0
        imgs.append(img)
        losses.append(ls)
    assert np.array_equal(imgs[0], imgs[1])
    ls = np.array(losses[0])
    assert np.mean(ls[-4:]) < np.mean(ls[:4]), ls


def test_nrc_render_pass_matches_oracle(R):
    """The RENDER pass (colour = radiance + beta x max(cache, 0)) and the
    training data (nrcGenerateTrainingData) of a GPU frame against the
    oracle's restatement (pinned bit for bit to the reference's own nrc.cu,
    tests/test_ref_integrator.py) applied to that frame's own G-buffer,
    train buffers and cache outputs: bit for bit."""
    res = 64
    s = R.Scene(R.straight_hair_scene(res, res, strands=6000))
    r = R.Renderer(s, R.NRC, train=False, seed=3, frames_in_flight=1)
    r.frame()
    P = res * res
    st = r.stats()
    gbuf, gbeta, nn, tinfo = r.buffer(4), r.buffer(8), r.buffer(1), r.buffer(10)
    T = len(tinfo)
    rec = r.buffer(9).reshape(T, 40, 5, 4)[:, :, :, :3].reshape(T, 40, 15)
    tp = np.array([t * st.every_nth + po.feistel_perm(t, T, 0) % st.every_nth for t in range(T)])
    assert np.array_equal(tinfo[:, 3], (gbuf[tp, 3] > 0.5).astype(np.int32))  # primary hit of each training pixel
    color, tin, tgt = po.nrc_render(rad=gbuf[:, :3], beta=gbeta[:, :3], hit=gbuf[:, 3] > 0.5, cache=nn[:P + T],
                                    train_px=tp, unbiased=tinfo[:, 2] != 0, t_bounces=tinfo[:, 0],
                                    t_hit=tinfo[:, 1], records=rec)
    assert (tinfo[:, 0] > 1).sum() > 20
    img = r.read(R.IMAGE_FINAL).reshape(-1, 3)  # first frame: the FP64 sums hold the FP32 colours
    assert np.array_equal(img, color.astype(np.float64))
    # the record buffers hold numTrainingRecords rows; the T x 40 first are the training pixels'
    g_in, g_out = r.buffer(2)[:T * 40].reshape(T, 40, -1), r.buffer(3)[:T * 40].reshape(T, 40, 3)
    assert np.array_equal(g_in[:, :, :9].view(np.uint32), tin.view(np.uint32))
    assert np.array_equal(g_out.view(np.uint32), tgt.view(np.uint32))
