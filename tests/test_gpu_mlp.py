"""GPU parity of the radiance-cache network against the FP64 oracle.

Tolerances (FP32 kernels vs FP64 oracle, same parameters and inputs):
  outputs      |gpu - ref| <= 2e-4 * rms(ref) + 1e-4 * |ref|
  loss         relative 1e-4
  gradients    per weight matrix |gpu - ref| <= 2e-4 * max|ref of that matrix|
  Adam step    |delta_gpu - delta_ref| <= 1e-3 * learning rate
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mlpmod():
    from hairmsnn_gb300 import build, mlp
    build.build()
    return mlp


def c1_inputs(n, seed=0):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 16), np.float32)
    x[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    x[:, 3:7] = rng.uniform(0, 1, (n, 4))
    x[:, 7] = rng.uniform(-1, 1, n)
    x[:, 8:11] = [0.06, 0.1, 0.2]
    x[:, 11:13] = 0.3
    return x


def ref_inputs(n, seed=0):
    """The reference's 12-channel cache input: pos/sceneScale, wo, tangent, 3 unused."""
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 12), np.float32)
    x[:, 0:3] = rng.uniform(-0.5, 0.5, (n, 3))
    for o in (3, 6):
        v = rng.normal(size=(n, 3))
        x[:, o:o + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return x


CASES = [("c1_cache_w64.json", 16, c1_inputs), ("c1_cache_w128.json", 16, c1_inputs),
         ("hairmsnn_cache.json", 12, ref_inputs)]


def out_close(gpu, ref):
    rms = np.sqrt(np.mean(ref ** 2))
    err = np.abs(gpu - ref) - (2e-4 * rms + 1e-4 * np.abs(ref))
    return err.max() <= 0, np.abs(gpu - ref).max() / rms


@pytest.mark.parametrize("cfg,in_ch,gen", CASES)
def test_inference_matches_fp64_oracle(mlpmod, cfg, in_ch, gen):
    net = mlpmod.TinyMLP(cfg, in_ch, 3, seed=3)
    if cfg == "hairmsnn_cache.json":  # give the grid a visible contribution
        p = net.params()
        oc = mo.Config(net.config_text, in_ch, 3)
        p[oc.n_net_params:] = np.random.default_rng(5).uniform(-0.5, 0.5, oc.n_enc_params)
        net.set_params(p)
    n = 4096 + 37  # ragged tail tile
    x = gen(n)
    out = net.inference(torch.from_numpy(x).cuda()).cpu().numpy()
    oc = mo.Config(net.config_text, in_ch, 3)
    ref, _ = mo.forward(oc, net.params().astype(np.float64), x)
    ok, rel = out_close(out, ref[:, :3])
    assert ok, rel


@pytest.mark.parametrize("cfg,in_ch,gen", CASES)
def test_training_gradients_and_adam_match_oracle(mlpmod, cfg, in_ch, gen):
    net = mlpmod.TinyMLP(cfg, in_ch, 3, seed=11)
    oc = mo.Config(net.config_text, in_ch, 3)
    n = 2048 + 64
    x = gen(n, seed=2)
    tgt = np.random.default_rng(9).lognormal(0.0, 1.0, (n, 3)).astype(np.float32)
    p0 = net.params().astype(np.float64)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(tgt).cuda()
    out = net.forward(dx).cpu().numpy()
    ref_out, _ = mo.forward(oc, p0, x)
    assert out_close(out, ref_out[:, :3])[0]
    loss = net.backward(dt).item()
    ref_loss, ref_g = mo.backward(oc, p0, x, tgt)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    g = net.gradients().astype(np.float64)
    for off, fo, fi in oc.layer_shapes:
        gm, rm = g[off:off + fo * fi], ref_g[off:off + fo * fi]
        assert np.abs(gm - rm).max() <= 2e-4 * np.abs(rm).max(), (off, np.abs(gm - rm).max())
    if oc.n_enc_params:
        ge, re = g[oc.n_net_params:], ref_g[oc.n_net_params:]
        assert np.abs(ge - re).max() <= 2e-4 * np.abs(re).max()
    net.optimizer_step()
    p1 = net.params().astype(np.float64)
    adam = mo.Adam(oc)
    ref_p1 = adam.update(p0, g)  # oracle Adam on the GPU's own gradients
    assert np.abs((p1 - p0) - (ref_p1 - p0)).max() <= 1e-3 * oc.lr


@pytest.mark.parametrize("cfg,in_ch,gen", [("c1_cache_w64.json", 16, c1_inputs),
                                           ("hairmsnn_cache.json", 12, ref_inputs)])
def test_training_is_bitwise_deterministic(mlpmod, cfg, in_ch, gen):
    """Fixed-order weight-gradient reduction and fixed-point hash-grid
    gradient atomics: repeated training is bit-identical."""
    x = torch.from_numpy(gen(4096, seed=4)).cuda()
    t = torch.from_numpy(np.random.default_rng(3).uniform(0, 2, (4096, 3)).astype(np.float32)).cuda()
    runs = []
    for _ in range(2):
        net = mlpmod.TinyMLP(cfg, in_ch, 3, seed=1)
        for _ in range(5):
            net.training_step(x, t)
        runs.append(net.params())
    assert np.array_equal(runs[0].view(np.uint32), runs[1].view(np.uint32))


def test_training_reduces_loss_and_state_roundtrip(mlpmod, tmp_path):
    net = mlpmod.TinyMLP("hairmsnn_cache.json", 12, 3, seed=2)
    x = torch.from_numpy(ref_inputs(8192, seed=6)).cuda()
    t = torch.sigmoid(x[:, :3] * 4).contiguous()
    first = net.training_step(x, t).item()
    for _ in range(200):
        last = net.training_step(x, t)
    assert last.item() < 0.2 * first
    path = str(tmp_path / "cache.hmmlp")
    net.save(path)
    y0 = net.inference(x)
    net2 = mlpmod.TinyMLP("hairmsnn_cache.json", 12, 3, seed=99)
    net2.load_weights(path)
    assert torch.equal(net2.inference(x), y0)
    assert net2.info().step == 201
    net2.reset()
    assert not net2.params().any()
    assert not net2.inference(x).any()


def test_zero_and_bad_batches(mlpmod):
    from hairmsnn_gb300._ffi import HMError
    net = mlpmod.TinyMLP("c1_cache_w64.json", 16, 3)
    x = torch.zeros((0, 16), device="cuda")
    assert net.inference(x).shape == (0, 3)
    with pytest.raises(HMError):
        net.backward(torch.zeros((5, 3), device="cuda"))  # no matching forward


def _write_snapshot(path, params, dtype):
    """A tiny-cuda-nn trainer snapshot as JSON text, the form
    TINY_MLP::loadWeights reads (params_binary as {"bytes": [...]})."""
    raw = np.ascontiguousarray(params, dtype).tobytes()
    with open(path, "w") as f:
        f.write('{"n_params": %d, "params_type": "%s", "params_binary": {"bytes": [%s], "subtype": null}, '
                '"optimizer": {"current_step": 7}}\n'
                % (len(params), "float" if dtype == np.float32 else "__half", ",".join(map(str, raw))))


@pytest.mark.parametrize("dtype", [np.float32, np.float16])
def test_loads_tcnn_snapshot(mlpmod, tmp_path, dtype):
    """hm_mlp_load on a tiny-cuda-nn trainer snapshot (float or __half
    parameters) and hm_mlp_save's JSON form: the parameters arrive exactly
    (half -> float exactly), and inference runs on them."""
    net = mlpmod.TinyMLP("hairmsnn_cache.json", 12, 3, seed=3)
    n = net.info().n_params
    p = np.random.default_rng(4).normal(scale=0.05, size=n).astype(dtype)
    path = str(tmp_path / "weights.json")
    _write_snapshot(path, p, dtype)
    net.load_weights(path)
    assert np.array_equal(net.params(), p.astype(np.float32))
    x = torch.from_numpy(ref_inputs(4096)).cuda()
    y = net.inference(x)
    net2 = mlpmod.TinyMLP("hairmsnn_cache.json", 12, 3, seed=9)
    out = str(tmp_path / "again.json")
    net.save(out)
    net2.load_weights(out)
    assert np.array_equal(net2.params(), net.params())
    assert torch.equal(net2.inference(x), y)
    bad = str(tmp_path / "short.json")
    _write_snapshot(bad, p[:-1], dtype)
    with pytest.raises(Exception):
        net2.load_weights(bad)


def test_scene_init_weights_loads_the_cache(tmp_path):
    """tcnn.init_weights of the scene JSON (scene.cpp:330-331) is loaded into
    the render's cache network when the renderer is made
    (render_hair_msnn.cu:109-110)."""
    from hairmsnn_gb300 import build, render as R
    build.build()
    cfg = R.straight_hair_scene(64, 64, strands=200)
    s0 = R.Scene(cfg)
    r0 = R.Renderer(s0, R.MSNN, beta=1, train_records=1024, train=False)
    n = r0.cache().info().n_params
    p = np.random.default_rng(5).normal(scale=0.03, size=n).astype(np.float32)
    _write_snapshot(str(tmp_path / "w.json"), p, np.float32)
    cfg["tcnn"] = {"init_train": False, "init_weights": "w.json"}
    s = R.Scene(cfg, str(tmp_path))
    r = R.Renderer(s, R.MSNN, beta=1, train_records=1024, train=False)
    assert np.array_equal(r.cache().params(), p)
