"""CLI helpers that run without a GPU: the PFM image writer/reader."""
import numpy as np

from hairmsnn_gb300.__main__ import read_pfm, write_pfm


def test_pfm_roundtrip(tmp_path):
    img = np.random.default_rng(0).uniform(0, 4, (5, 7, 3)).astype(np.float32)
    p = str(tmp_path / "x.pfm")
    write_pfm(p, img)
    assert open(p, "rb").read(3) == b"PF\n"
    assert np.array_equal(read_pfm(p), img)
