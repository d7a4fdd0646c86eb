"""CLI helpers that run without a GPU: the PFM image writer/reader."""
import numpy as np

from hairmsnn_gb300.__main__ import read_pfm, write_pfm


def test_pfm_roundtrip(tmp_path):
    img = np.random.default_rng(0).uniform(0, 4, (5, 7, 3)).astype(np.float32)
    p = str(tmp_path / "x.pfm")
    write_pfm(p, img)
    assert open(p, "rb").read(3) == b"PF\n"
    assert np.array_equal(read_pfm(p), img)


def test_exr_roundtrip_and_layout(tmp_path):
    import struct
    from hairmsnn_gb300.__main__ import read_exr, write_exr
    rng = np.random.default_rng(1)
    img = rng.uniform(0, 4, (5, 7, 3)).astype(np.float32)
    p = tmp_path / "a.exr"
    write_exr(str(p), img)
    assert np.array_equal(read_exr(str(p)), img)
    data = p.read_bytes()
    assert struct.unpack_from("<ii", data, 0) == (20000630, 2)
    # the first stored scanline is the top row (row H-1 of the bottom-first image), channels B, G, R
    i = data.index(b"\0\0\0\0\x54\x00\x00\x00")  # y = 0, 84 bytes (3 channels x 7 floats)
    first = np.frombuffer(data, "<f4", 21, i + 8).reshape(3, 7)
    assert np.array_equal(first[2], img[-1, :, 0]) and np.array_equal(first[0], img[-1, :, 2])
