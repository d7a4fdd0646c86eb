"""Strand groups (per-group hair materials), host side only.

* hair.groups in the scene JSON: "index" assignment is strand k -> k % count,
  "azimuth" splits the roots' azimuth around their mean into equal wedges;
  materials default to the scene's and take the listed overrides (alpha in
  degrees, stored in radians like the scene material).
* Every segment carries its strand's group (segment_groups export).
* hm_scene_set_strand_groups / _set_group_materials validate their input.
* The oracle's integrator with every group at the scene's material renders
  the ungrouped scene bit for bit, and a changed group changes only pixels.
"""
import numpy as np
import pytest

from hairmsnn_gb300 import render as R
from oracle import pyoracle as po


def grouped_cfg(assign="index", count=3, materials=None, strands=30, res=32):
    cfg = R.straight_hair_scene(res, res, strands=strands, control_points=8, triangles=200, sky_w=32, sky_h=16)
    g = {"count": count, "assign": assign}
    if materials is not None:
        g["materials"] = materials
    cfg["hair"]["groups"] = g
    return cfg


def test_index_groups_and_material_overrides():
    mats = [{"sigma_a": [0.5, 0.4, 0.3], "beta_m": 0.6}, {"alpha": 4.0}]
    s = R.Scene(grouped_cfg("index", 3, mats))
    info = s.info()
    assert info.n_groups == 3
    sg = s.export("strand_groups")
    assert np.array_equal(sg, np.arange(info.n_strands) % 3)
    m = s.export("group_materials")
    base = s.export("materials")[0][:10]
    assert m.shape == (3, 10)
    assert np.allclose(m[0, 0:3], [0.5, 0.4, 0.3]) and m[0, 3] == np.float32(0.6)
    assert np.array_equal(m[0, 4:], base[4:])
    assert m[1, 5] == np.float32(3.14159) * np.float32(4.0) / np.float32(180.0)  # as scene.cpp:207, in float
    assert np.array_equal(m[1, :5], base[:5])
    assert np.array_equal(m[2], base)
    seg_g = s.export("segment_groups")
    per_strand = info.n_segments // info.n_strands
    assert np.array_equal(seg_g, np.repeat(sg, per_strand))


def test_azimuth_groups_split_roots_into_wedges():
    s = R.Scene(grouped_cfg("azimuth", 4, strands=400))
    sg = s.export("strand_groups")
    cp = s.export("control_points")
    seg = s.export("segments")
    info = s.info()
    per_strand = info.n_segments // info.n_strands
    roots = cp[seg[::per_strand] + 1, :2].astype(np.float64)
    c = roots.mean(axis=0)
    ang = np.arctan2(roots[:, 1] - c[1], roots[:, 0] - c[0]) + np.pi
    expect = np.minimum(3, (ang / (2 * np.pi) * 4).astype(int))
    assert (sg == expect).mean() >= 0.99  # float vs double at wedge borders
    counts = np.bincount(sg, minlength=4)
    assert counts.min() > 50


def test_set_strand_groups_and_materials_validate():
    s = R.Scene(R.straight_hair_scene(32, 32, strands=20, control_points=8, triangles=200, sky_w=32, sky_h=16))
    n = s.info().n_strands
    assert s.info().n_groups == 0
    with pytest.raises(Exception):
        s.set_strand_groups(np.zeros(n - 1, np.int32), 2)
    with pytest.raises(Exception):
        s.set_strand_groups(np.full(n, 2, np.int32), 2)
    with pytest.raises(Exception):
        s.set_strand_groups(np.zeros(n, np.int32), 65)
    s.set_strand_groups(np.arange(n) % 2, 2)
    assert s.info().n_groups == 2
    m = s.group_materials()
    assert m.shape == (2, 10)
    m[1, 0] = 0.9
    s.set_group_materials(m)
    assert s.export("group_materials")[1, 0] == np.float32(0.9)
    with pytest.raises(Exception):
        s.set_group_materials(m[:1])


def test_ungrouped_scene_material_replaced_through_groups_call():
    s = R.Scene(R.straight_hair_scene(32, 32, strands=20, control_points=8, triangles=200, sky_w=32, sky_h=16))
    m = s.group_materials()
    m[0, 3] = 0.45
    s.set_group_materials(m)
    assert s.export("materials")[0, 3] == np.float32(0.45)
    assert s.info().n_groups == 0


def test_oracle_groups_with_scene_material_render_the_same_image():
    cfg = grouped_cfg("index", 2, strands=60, res=32)
    s = R.Scene(cfg)
    o_g = po.OracleScene.from_library(s)
    del cfg["hair"]["groups"]
    o_plain = po.OracleScene.from_library(R.Scene(cfg))
    a = o_g.render_pixels(0, threads=4)[0]
    b = o_plain.render_pixels(0, threads=4)[0]
    assert np.array_equal(a, b)
    # a different material in group 1 changes some pixels and keeps the rest
    m = s.group_materials()
    m[1, 0:3] = [2.0, 2.0, 2.0]
    o_g.set_groups(s.export("segment_groups"), m)
    c = o_g.render_pixels(0, threads=4)[0]
    diff = np.any(c != b, axis=1)
    assert 0 < diff.mean() < 1
