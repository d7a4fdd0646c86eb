"""OpenEXR environment maps (lights.environment = {"exr", "scale", "rotation"},
parseScene scene.cpp:234-253, loaded as tinyexr's LoadEXR returns them:
RGBA float rows, first stored line first, A = 1 when absent, Y copied to
R, G, B).  Host only.

The files are written here by an encoder of the format's published layout
(attribute header, scanline offset table, chunks; NONE, RLE, ZIPS and ZIP
compression with the byte predictor and even/odd interleave; HALF and FLOAT
channels), and by the CLI's own EXR writer.  Decoded maps equal the source
pixels bit for bit (half-precision sources through numpy's float16), and
the sampling tables equal the restated generateEnvSamplingTables.
"""
import json
import struct
import zlib

import numpy as np
import pytest

from hairmsnn_gb300 import render as R
from oracle import pyoracle as po

COMP = {"none": 0, "rle": 1, "zips": 2, "zip": 3}
LINES = {0: 1, 1: 1, 2: 1, 3: 16}


def _attr(name, typ, payload):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(payload)) + payload


def _reorder(raw):
    """Interleave (even bytes first, then odd) and the byte predictor."""
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int32)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128 + 256) & 255
    return d.astype(np.uint8).tobytes()


def _rle(data):
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        j = i + 1
        while j < n and data[j] == data[i] and j - i < 128:
            j += 1
        if j - i >= 3:
            out += struct.pack("<bB", j - i - 1, data[i])
            i = j
            continue
        j = i
        while j < n and j - i < 127 and not (j + 2 < n and data[j] == data[j + 1] == data[j + 2]):
            j += 1
        out += struct.pack("<b", -(j - i)) + data[i:j]
        i = j
    return bytes(out)


def write_exr(path, chans, comp="zip", half=False):
    """chans: dict name -> [H, W] float array."""
    names = sorted(chans)
    h, w = chans[names[0]].shape
    ptype = 1 if half else 2
    chl = b"".join(nm.encode() + b"\0" + struct.pack("<iB3xii", ptype, 0, 1, 1) for nm in names) + b"\0"
    c = COMP[comp]
    header = b"".join([
        _attr("channels", "chlist", chl),
        _attr("compression", "compression", bytes([c])),
        _attr("dataWindow", "box2i", struct.pack("<4i", 3, 7, 3 + w - 1, 7 + h - 1)),
        _attr("displayWindow", "box2i", struct.pack("<4i", 3, 7, 3 + w - 1, 7 + h - 1)),
        _attr("lineOrder", "lineOrder", b"\0"),
        _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)),
    ]) + b"\0"
    prefix = struct.pack("<ii", 20000630, 2) + header
    lines = LINES[c]
    chunks = []
    n_packed = 0  # chunks whose compressed form was smaller than the raw lines
    for y0 in range(0, h, lines):
        raw = b""
        for y in range(y0, min(h, y0 + lines)):
            for nm in names:
                row = chans[nm][y]
                raw += row.astype("<f2" if half else "<f4").tobytes()
        if c == 0:
            data = raw
        elif c == 1:
            data = _rle(_reorder(raw))
        else:
            data = zlib.compress(_reorder(raw), 6)
        if len(data) >= len(raw):
            data = raw  # stored when compression does not pay, as the format allows
        elif c != 0:
            n_packed += 1
        chunks.append(struct.pack("<ii", 7 + y0, len(data)) + data)
    first = len(prefix) + 8 * len(chunks)
    offs, o = [], first
    for ch in chunks:
        offs.append(o)
        o += len(ch)
    with open(path, "wb") as f:
        f.write(prefix + struct.pack(f"<{len(offs)}Q", *offs) + b"".join(chunks))
    return n_packed


def env_scene(tmp_path, fname, scale=1.5, rotation=0.25):
    cfg = {"camera": {"from": [0, -4, 0], "to": [0, 0, 0], "up": [0, 0, 1], "cos_fovy": 0.66},
           "integrator": {"width": 128, "height": 128},
           "hair": {"procedural": {"type": "straight", "strands": 10, "control_points": 8}},
           "lights": {"environment": {"exr": fname, "scale": scale, "rotation": rotation}}}
    return R.Scene(json.dumps(cfg), str(tmp_path))


def blocky_sky(h, w):
    """Piecewise-constant values: runs of equal bytes, so RLE and ZIP pay."""
    y, x = np.mgrid[0:h, 0:w]
    base = 0.25 * (1 + (x // 8) % 4) + 0.5 * ((y // 4) % 2)
    return {c: (base * (1.0 + 0.5 * i)).astype(np.float32) for i, c in enumerate("RGB")}


def smooth_sky(h, w, seed=0):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    base = 1.0 + 0.5 * np.sin(x / w * 6.28) * np.cos(y / h * 3.14)
    return {c: (base * (0.8 + 0.2 * i) + 0.05 * rng.random((h, w))).astype(np.float32)
            for i, c in enumerate("RGB")}


@pytest.mark.parametrize("comp", ["none", "rle", "zips", "zip"])
@pytest.mark.parametrize("half", [False, True])
@pytest.mark.parametrize("kind", ["smooth", "blocky"])
def test_exr_environment_decodes_exactly(tmp_path, comp, half, kind):
    h, w = 37, 64  # 37 lines: a partial last ZIP chunk
    ch = smooth_sky(h, w) if kind == "smooth" else blocky_sky(h, w)
    packed = write_exr(tmp_path / "env.exr", ch, comp, half)
    if kind == "blocky" and comp != "none":
        assert packed > 0  # the decoder's decompression path is exercised
    s = env_scene(tmp_path, "env.exr")
    env = s.export("env").reshape(h, w, 4)
    info = s.info()
    assert (info.env_width, info.env_height, info.has_env) == (w, h, 1)
    for i, c in enumerate("RGB"):
        want = ch[c].astype(np.float16).astype(np.float32) if half else ch[c]
        assert np.array_equal(env[:, :, i], want), c
    assert np.all(env[:, :, 3] == 1.0)
    m = s.export("materials")[0]
    assert m[14] == np.float32(1.5) and m[15] == np.float32(0.25)


def test_exr_luminance_alpha_and_tables(tmp_path):
    h, w = 16, 32
    y = smooth_sky(h, w, 3)["R"]
    a = np.full((h, w), 0.5, np.float32)
    write_exr(tmp_path / "y.exr", {"Y": y, "A": a}, "zip")
    s = env_scene(tmp_path, "y.exr")
    env = s.export("env").reshape(h, w, 4)
    for i in range(3):
        assert np.array_equal(env[:, :, i], y)
    assert np.all(env[:, :, 3] == 0.5)
    cpdf, ccdf, mpdf, mcdf = po.env_tables(env.reshape(-1, 4), w, h)
    assert np.array_equal(s.export("env_cpdf"), cpdf)
    assert np.array_equal(s.export("env_mcdf"), mcdf)


def test_cli_exr_writer_round_trips_as_environment(tmp_path):
    from hairmsnn_gb300.__main__ import write_exr as cli_write
    img = np.random.default_rng(4).random((8, 16, 3)).astype(np.float32)
    cli_write(str(tmp_path / "cli.exr"), img)
    s = env_scene(tmp_path, "cli.exr")
    env = s.export("env").reshape(8, 16, 4)
    assert np.array_equal(env[:, :, :3], img[::-1])  # the CLI writes the top row first


def test_exr_errors(tmp_path):
    (tmp_path / "bad.exr").write_bytes(b"\x76\x2f\x31\x01" + b"\x02\x02\x00\x00" + b"\0" * 16)  # tiled
    with pytest.raises(Exception) as e:
        env_scene(tmp_path, "bad.exr")
    assert "tiled" in str(e.value) or "7" in str(e.value)
    (tmp_path / "junk.exr").write_bytes(b"not an exr file at all")
    with pytest.raises(Exception):
        env_scene(tmp_path, "junk.exr")
    ch = smooth_sky(4, 8)
    write_exr(tmp_path / "piz.exr", ch, "zip")
    data = bytearray((tmp_path / "piz.exr").read_bytes())
    k = data.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    data[k] = 4  # PIZ
    (tmp_path / "piz.exr").write_bytes(bytes(data))
    with pytest.raises(Exception) as e:
        env_scene(tmp_path, "piz.exr")
    assert "not supported" in str(e.value)
    with pytest.raises(Exception):
        env_scene(tmp_path, "missing.exr")
