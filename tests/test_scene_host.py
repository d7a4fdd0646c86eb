"""Scene construction on the host (no device): the reference's scene JSON
schema, defaults and errors, the procedural generators, the environment
sampling tables and the camera, against the oracle's restatements."""
import json

import numpy as np
import pytest

from oracle import pyoracle as po


@pytest.fixture(scope="module")
def R():
    from hairmsnn_gb300 import build, render
    build.build()
    return render


def small(**kw):
    from hairmsnn_gb300 import render
    return render.straight_hair_scene(64, 64, strands=200, **kw)


def test_generated_counts_and_bounds(R):
    s = R.Scene(small())
    i = s.info()
    assert i.n_strands == 200 and i.n_control_points == 200 * 64 and i.n_segments == 200 * 61
    assert i.n_triangles == 20000 and i.n_dir_lights == 1 and i.has_env
    cp = s.export("control_points")
    assert np.allclose(cp[:, 3], 4e-4)
    seg = s.export("segments")
    assert seg.min() == 0 and seg.max() + 3 < len(cp)
    # every segment's 4 control points belong to one strand
    assert np.all((seg % 64) <= 60)
    diag = np.linalg.norm(np.array(i.bounds_max) - np.array(i.bounds_min))
    assert abs(i.scene_scale - diag) < 1e-5 * diag
    # strands stay outside the head (radii .85, .95, 1.0 + margin)
    q = cp[:, :3] / np.array([0.85, 0.95, 1.0])
    assert (np.linalg.norm(q, axis=1) > 0.999).mean() > 0.99


def test_env_tables_and_camera_match_restatement(R):
    cfg = small()
    s = R.Scene(cfg)
    i = s.info()
    env = s.export("env")
    cp, cc, mp, mc = po.env_tables(env, i.env_width, i.env_height)
    for name, ref in (("env_cpdf", cp), ("env_ccdf", cc), ("env_mpdf", mp), ("env_mcdf", mc)):
        assert np.array_equal(s.export(name), ref), name
    cam = po.camera_vectors(cfg["camera"]["from"], cfg["camera"]["to"], cfg["camera"]["up"],
                            cfg["camera"]["cos_fovy"], 64, 64)
    assert np.array_equal(s.export("camera").ravel(), np.concatenate(cam))


def test_reference_defaults(R):
    cfg = small()
    del cfg["hair"]["beta_m"], cfg["hair"]["sigma_a"], cfg["hair"]["alpha"]
    s = R.Scene(cfg)
    m = s.export("materials").ravel()
    # scene.cpp:190-205: sigma_a (0.06, 0.1, 0.2), beta_m 0.3, alpha 0 when absent
    assert np.allclose(m[:3], [0.06, 0.1, 0.2]) and abs(m[3] - 0.3) < 1e-7 and m[5] == 0.0
    cfg["hair"]["alpha"] = 2.0
    m = R.Scene(cfg).export("materials").ravel()
    assert m[5] == np.float32(np.float32(3.14159) * np.float32(2.0) / np.float32(180.0))
    dl = s.export("dir_lights")[0]
    assert np.allclose(dl[:3], np.ones(3) / np.sqrt(3), atol=1e-7)


@pytest.mark.parametrize("mutate,status", [
    (lambda c: c.pop("camera"), 6),
    (lambda c: (c.pop("hair"), c.pop("surface")), 6),
    (lambda c: c.pop("lights"), 6),
    (lambda c: c["integrator"].update(width=100, height=100), 6),  # not a multiple of 128 pixels
    (lambda c: c["integrator"].update(width=4096, height=4096), 6),
    (lambda c: c.pop("integrator"), 6),
    (lambda c: c["hair"].update(geometry="wStraight.hair") or c["hair"].pop("procedural"), 1),  # missing file: HM_EINVAL
    (lambda c: c["surface"].update(geometry="head.obj") or c["surface"].pop("procedural"), 1),
])
def test_scene_errors(R, mutate, status):
    from hairmsnn_gb300._ffi import HMError
    cfg = small()
    mutate(cfg)
    with pytest.raises(HMError) as e:
        R.Scene(cfg)
    assert e.value.status == status


def test_malformed_json(R):
    from hairmsnn_gb300._ffi import HMError
    with pytest.raises(HMError) as e:
        R.Scene('{"camera": ')
    assert e.value.status == 6


def test_oracle_bvh_is_a_valid_hierarchy(R):
    """Host-side self-check of the oracle's LBVH: every primitive in exactly
    one leaf; every child box contains its subtree."""
    s = R.Scene(small())
    o = po.OracleScene.from_library(s)
    nodes, leaves = o.bvh()
    assert np.array_equal(np.sort(leaves), np.arange(len(leaves)))
    ch = nodes[:, 12:14].copy().view(np.int32)
    seen = []
    stack = [0]
    while stack:
        v = stack.pop()
        for c in range(2):
            lo, hi = nodes[v, 6 * c:6 * c + 3], nodes[v, 6 * c + 3:6 * c + 6]
            assert np.all(lo <= hi)
            k = ch[v, c]
            if k < 0:
                seen.append(~k)
            else:
                clo = np.minimum(nodes[k, 0:3], nodes[k, 6:9])
                chi = np.maximum(nodes[k, 3:6], nodes[k, 9:12])
                assert np.all(lo <= clo) and np.all(chi <= hi)
                stack.append(k)
    assert sorted(seen) == list(range(len(leaves)))


@pytest.mark.parametrize("strands", [1, 300])
def test_wide_collapse_structure(R, strands):
    """The 8-wide restatement over the oracle's LBVH: every leaf slot in
    exactly one wide slot, child boxes copied bit for bit from the binary
    tree (a wide child box is a binary child box, never a union), wide
    nodes numbered breadth first, and the greedy fill: a node with fewer
    than eight children holds only leaves."""
    cfg = small()
    cfg["hair"]["procedural"]["strands"] = strands
    if strands == 1:
        cfg.pop("surface", None)
    s = R.Scene(cfg)
    nodes, leaves = po.OracleScene.from_library(s).bvh()
    w = po.wide_collapse(nodes)
    codes = w[:, 48:56].view(np.int32)
    empty = np.isinf(w[:, 0:8]) & np.isinf(w[:, 8:16]) & (codes == -1)
    used = ~empty
    n_used = used.sum(1)
    assert np.all(n_used >= 2)
    assert np.all((n_used == 8) | np.all((codes < 0) | ~used, axis=1))
    # every wide child box is one of the binary child boxes, bit for bit
    bbox = np.ascontiguousarray(nodes[:, :12]).reshape(-1, 6).view(np.dtype((np.void, 24))).ravel()
    wbox = np.stack([w[:, 0:8], w[:, 16:24], w[:, 32:40], w[:, 8:16], w[:, 24:32], w[:, 40:48]], -1)
    wbox = np.ascontiguousarray(wbox[used]).view(np.dtype((np.void, 24))).ravel()
    assert np.isin(wbox, bbox).all()
    rows = np.nonzero(used)[0]
    c = codes[used]
    assert np.all((c < 0) | ((c > rows) & (c < len(w))))
    assert np.array_equal(np.sort(~c[c < 0]), np.arange(len(leaves)))
    internal = codes[codes >= 0]
    assert np.array_equal(internal, np.arange(1, len(w)))  # breadth-first numbering


def test_oracle_render_runs_and_is_deterministic(R):
    s = R.Scene(small())
    o = po.OracleScene.from_library(s)
    c1, _, _, f1 = o.render_pixels(0, n=1024, threads=4)
    c2, _, _, f2 = o.render_pixels(0, n=1024, threads=1)
    assert np.array_equal(c1, c2) and np.array_equal(f1, f2)
    assert np.isfinite(c1).all() and (c1 >= 0).all()
    col, nn, tr, fl = o.render_pixels(1, beta=1, accum_id=0, every_nth=4, n_train=1024, n=64 * 64)
    assert ((fl & 4) != 0).sum() == 1024  # one training pixel per block of every_nth pixels
    blocks = ((fl & 4) != 0).reshape(-1, 4).sum(axis=1)
    assert np.all(blocks == 1)
    assert np.isfinite(tr).all()


def test_wide_collapse_expansion_order():
    """A hand-built binary tree: the internal child of largest area is
    opened first, in place (its first child takes its slot, the second is
    appended); equal areas open the earlier slot."""
    def box(lo, hi):
        return list(lo) + list(hi)

    def node(b0, c0, b1, c1):
        return np.array(box(*b0) + box(*b1) + [0.0, 0.0, 0.0, 0.0], np.float32), (c0, c1)

    unit = ((0, 0, 0), (1, 1, 1))
    big = ((0, 0, 0), (4, 4, 4))
    small = ((0, 0, 0), (2, 2, 2))
    # 0: [1 (big), 2 (small)]; 1: [leaf 0, leaf 1]; 2: [3 (small), leaf 2]; 3: [leaf 3, leaf 4]
    spec = [(big, 1, small, 2), (unit, ~0, unit, ~1), (small, 3, unit, ~2), (unit, ~3, unit, ~4)]
    nodes = np.zeros((4, 16), np.float32)
    for i, (b0, c0, b1, c1) in enumerate(spec):
        v, cc = node(b0, c0, b1, c1)
        nodes[i] = v
        nodes[i, 12:14] = np.array(cc, np.int32).view(np.float32)
    w = po.wide_collapse(nodes)
    assert w.shape == (1, 56)
    codes = w[0, 48:56].view(np.int32)
    assert list(codes) == [~0, ~3, ~1, ~2, ~4, -1, -1, -1]
    # equal areas: the earlier slot opens first
    nodes[0, :12] = np.array(box(*small) + box(*small), np.float32)
    w = po.wide_collapse(nodes)
    assert list(w[0, 48:56].view(np.int32)) == [~0, ~3, ~1, ~2, ~4, -1, -1, -1]
    nodes[0, :12] = np.array(box(*small) + box(*big), np.float32)
    w = po.wide_collapse(nodes)
    # node 2 opens first: [1, 3, 2] -> 1 opens -> [0, 3, 2, 1] -> 3 opens -> [0, 3', 2, 1, 4]
    assert list(w[0, 48:56].view(np.int32)) == [~0, ~3, ~2, ~1, ~4, -1, -1, -1]
