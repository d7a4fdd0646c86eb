"""Scene files: Cem Yuksel's HAIR format and Wavefront OBJ (host only).

The control points, segment table and scene scale of a loaded HAIR file are
compared with a restatement of Scene::extractHairData (scene.cpp:10-73):
phantom points before and after each strand, one B-spline segment per
original segment, radius 0.2 x thickness, bounds of the file's own points
and the origin.
"""
import json
import struct

import numpy as np
import pytest

from hairmsnn_gb300 import render as R


def write_hair(path, strands_segments, points, thickness=None, default_segments=None, default_thickness=1.0):
    flags = 2
    if default_segments is None:
        flags |= 1
    if thickness is not None:
        flags |= 4
    header = b"HAIR" + struct.pack("<IIII", len(strands_segments), len(points), flags,
                                   default_segments or 0)
    header += struct.pack("<ff3f", default_thickness, 1.0, 1.0, 1.0, 1.0)
    header += b"\0" * (128 - len(header))
    body = b""
    if default_segments is None:
        body += struct.pack(f"<{len(strands_segments)}H", *strands_segments)
    body += np.asarray(points, "<f4").tobytes()
    if thickness is not None:
        body += np.asarray(thickness, "<f4").tobytes()
    with open(path, "wb") as f:
        f.write(header + body)


def extract_hair_data(segs, points, widths):
    """extractHairData restated: returns control points [n, 4], segment starts."""
    cps, seg_idx = [], []
    strand, left = 0, -1
    pts = np.asarray(points, np.float32)
    for i, p in enumerate(pts):
        first = False
        if left == -1:
            if strand == len(segs):
                break
            left = segs[strand]
            strand += 1
            first = True
        w = np.float32(0.2) * np.float32(widths[i])
        if first:
            q = p + (p - pts[i + 1])
            cps.append([*q, w])
            seg_idx.append(len(cps) - 1)
        cps.append([*p, w])
        if left > 1:
            seg_idx.append(len(cps) - 1)
        elif left == 0:
            q = p + (p - pts[i - 1])
            cps.append([*q, w])
        left -= 1
    return np.asarray(cps, np.float32), np.asarray(seg_idx, np.int32)


def scene_json(**parts):
    cfg = {"camera": {"from": [0, -4, 0], "to": [0, 0, 0], "up": [0, 0, 1], "cos_fovy": 0.66},
           "integrator": {"width": 128, "height": 128},
           "lights": {"directional": [{"from": [3, 3, 3], "emit": [1, 1, 1]}]}}
    cfg.update(parts)
    return cfg


@pytest.mark.parametrize("with_segments,with_thickness", [(True, True), (False, False)])
def test_hair_file_matches_extract_hair_data(tmp_path, with_segments, with_thickness):
    rng = np.random.default_rng(3)
    segs = [3, 1, 2, 4] if with_segments else [2, 2, 2]
    n_pts = sum(s + 1 for s in segs)
    pts = np.cumsum(rng.normal(scale=0.1, size=(n_pts, 3)), axis=0).astype(np.float32)
    thick = rng.uniform(0.5, 2.0, n_pts).astype(np.float32) if with_thickness else None
    path = tmp_path / "h.hair"
    write_hair(path, segs, pts, thick, default_segments=None if with_segments else 2, default_thickness=0.7)
    s = R.Scene(scene_json(hair={"geometry": "h.hair"}), str(tmp_path))
    cps = s.export("control_points")
    seg = s.export("segments")
    widths = thick if with_thickness else np.full(n_pts, 0.7, np.float32)
    ref_cps, ref_seg = extract_hair_data(segs, pts, widths)
    assert np.array_equal(cps, ref_cps)
    assert np.array_equal(seg, ref_seg)
    info = s.info()
    assert info.n_strands == len(segs)
    assert info.n_segments == sum(segs)
    # extractHairData's bounds start at the origin (HairModel's defaults)
    scale = np.float32(np.linalg.norm(np.maximum(pts.max(0), 0) - np.minimum(pts.min(0), 0)))
    assert abs(info.scene_scale - scale) <= 1e-6 * scale


def test_hair_file_errors(tmp_path):
    bad = tmp_path / "bad.hair"
    bad.write_bytes(b"NOPE" + b"\0" * 124)
    with pytest.raises(Exception):
        R.Scene(scene_json(hair={"geometry": "bad.hair"}), str(tmp_path))
    short = tmp_path / "short.hair"
    write_hair(short, [3], np.zeros((4, 3), np.float32))
    short.write_bytes(short.read_bytes()[:140])
    with pytest.raises(Exception):
        R.Scene(scene_json(hair={"geometry": "short.hair"}), str(tmp_path))
    with pytest.raises(Exception):
        R.Scene(scene_json(hair={"geometry": "missing.hair"}), str(tmp_path))


def test_obj_file(tmp_path):
    (tmp_path / "m.obj").write_text(
        "# quad with normals and a bare triangle\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0 0 1\n"
        "vn 0 0 1\n"
        "f 1//1 2//1 3//1 4//1\n"
        "f 1 2 5\n")
    s = R.Scene(scene_json(surface={"geometry": "m.obj", "diffuse": [0.5, 0.4, 0.3]}), str(tmp_path))
    v = s.export("vertices")
    n = s.export("normals")
    t = s.export("triangles")
    assert t.shape == (3, 3)
    assert np.array_equal(t, np.arange(9).reshape(3, 3))
    assert np.array_equal(v[:6], np.float32([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 0, 0], [1, 1, 0], [0, 1, 0]]))
    assert np.array_equal(n[:6], np.tile(np.float32([0, 0, 1]), (6, 1)))
    # the bare triangle gets its geometric normal
    assert np.allclose(n[6:], np.tile(np.float32([0, -1, 0]), (3, 1)))
