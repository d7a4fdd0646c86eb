"""Batched renders (hm_render_create_batch): many scenes in one frame.

* Plain path tracing of a batch gives every scene exactly the image a
  renderer of that scene alone gives (same per-pixel random streams, same
  trees; the paths of other scenes only share the launches).
* HairMSNN batches with per-scene BETA are finite and bitwise reproducible,
  and the shared cache's training loss falls.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    from hairmsnn_gb300 import build, render
    build.build()
    return render


def scenes(R):
    cfgs = [R.straight_hair_scene(64, 64, strands=500, seed=1),
            R.straight_hair_scene(128, 64, strands=1500, seed=2),
            R.straight_hair_scene(64, 128, strands=300, seed=3)]
    cfgs[1]["hair"]["procedural"]["type"] = "curly"
    cfgs[2]["hair"]["sigma_a"] = [0.3, 0.2, 0.1]
    return [R.Scene(c) for c in cfgs]


def test_pt_batch_equals_single_scene_renders(R):
    sc = scenes(R)
    b = R.BatchRenderer(sc, R.PT)
    for _ in range(3):
        b.frame()
    for k, s in enumerate(sc):
        r = R.Renderer(s, R.PT)
        for _ in range(3):
            r.frame()
        assert np.array_equal(b.read_scene(k), r.read(R.IMAGE_FINAL)), k
        r.close()


def test_msnn_batch_reproducible_and_training(R):
    imgs, losses = [], []
    for _ in range(2):
        sc = scenes(R)
        b = R.BatchRenderer(sc, R.MSNN, betas=[0, 1, 3], train_records=2048, seed=4)
        ls = []
        for _ in range(12):
            b.frame()
            ls.append(b.stats().last_loss)
        imgs.append(b.read())
        losses.append(ls)
        b.close()
    assert np.isfinite(imgs[0]).all()
    assert np.array_equal(imgs[0], imgs[1])
    assert np.mean(losses[0][-3:]) < np.mean(losses[0][:3])
