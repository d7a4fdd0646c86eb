"""Tensor-core (tcgen05) cache inference: FP16 / BF16 / E4M3 operands, FP32
accumulation.

Two references on the same parameters and inputs:
  * an emulation of the kernel's rounding in float64 (operands rounded to the
    type exactly where the kernel rounds them, E4M3 with the kernel's
    per-layer weight and per-query activation scales, Frequency features
    from the exact phase as the kernel's sincospif): the kernel must agree
    up to accumulation order, which can flip the rounding of an activation
    that lies on a rounding boundary;
      FP16/BF16: 99.9% of outputs within 3e-3 * rms + 3e-3 * |ref|, all
                 within 3e-2 * rms
      E4M3:      99% within 3e-2 * rms + 3e-2 * |ref|, all within 0.2 * rms
  * the FP64 oracle (the precision's own error, written per test below).
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

E4M3_MAX = np.float32(448.0)


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
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 12), np.float32)
    x[:, 0:3] = rng.uniform(-0.5, 0.5, (n, 3))
    for o in (3, 6):
        v = rng.normal(size=(n, 3))
        x[:, o:o + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return x


TORCH_DT = {"bf16": torch.bfloat16, "fp16": torch.float16}


def _round(a, dt):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dt).to(torch.float64).numpy()


def _e4m3(a):
    a = np.clip(np.asarray(a, np.float32), -E4M3_MAX, E4M3_MAX)
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.float8_e4m3fn).to(torch.float64).numpy()


def emulate(oc, params, x, prec):
    """The kernel's arithmetic in float64 with its roundings."""
    p64 = np.asarray(params, np.float64)
    X = mo.encode(oc, p64, x, exact_phase=True).astype(np.float32)
    Ws = [w.astype(np.float32) for w in mo.weights(oc, p64)]
    if prec in TORCH_DT:
        dt = TORCH_DT[prec]
        h = _round(X, dt)
        for l in range(oc.n_hidden):
            h = _round(np.maximum(h @ _round(Ws[l], dt).T, 0.0), dt)
        return (h @ _round(Ws[-1], dt).T)[:, :oc.out_ch]
    # E4M3
    inv = [np.float32(np.abs(w).max()) / E4M3_MAX for w in Ws]
    Wq = [_e4m3(w * (np.float32(1.0) / iv)) for w, iv in zip(Ws, inv)]
    bound = np.ones(x.shape[0], np.float32)
    for s in oc.segs:
        if s["type"] == "Identity":
            seg = np.abs(x[:, s["in_off"]:s["in_off"] + s["n_dims"]]).max(axis=1)
            bound = np.maximum(bound, seg)
        elif s["type"] == "HashGrid":
            bound = np.maximum(bound, np.float32(np.abs(p64[oc.n_net_params:]).max()))
    row_inv = bound / E4M3_MAX
    h = _e4m3(X * (E4M3_MAX / bound)[:, None])
    for l in range(oc.n_hidden):
        acc = (h @ Wq[l].T).astype(np.float32)
        v = np.maximum(acc * (row_inv * inv[l])[:, None], np.float32(0))
        amax = v.max(axis=1)
        s = np.where(amax > 0, E4M3_MAX / np.where(amax > 0, amax, 1), np.float32(1)).astype(np.float32)
        row_inv = np.where(amax > 0, amax / E4M3_MAX, np.float32(1)).astype(np.float32)
        h = _e4m3(v * s[:, None])
    acc = (h @ Wq[-1].T).astype(np.float32)
    return (acc * (row_inv * inv[-1])[:, None])[:, :oc.out_ch]


def check_vs_emulation(out, emu, prec):
    rms = np.sqrt(np.mean(emu ** 2))
    err = np.abs(out - emu)
    t = 3e-3 if prec in TORCH_DT else 3e-2
    frac = np.mean(err <= t * rms + t * np.abs(emu))
    need = 0.999 if prec in TORCH_DT else 0.99
    cap = (3e-2 if prec in TORCH_DT else 0.2) * rms
    assert frac >= need, (frac, err.max() / rms)
    assert err.max() <= cap, err.max() / rms


# per-output error against the FP64 oracle: rms(error) / rms(ref) at most
ORACLE_REL = {"fp16": 2e-3, "bf16": 1.5e-2, "fp8": 1.2e-1}

CASES = [("hairmsnn_cache.json", 12, ref_inputs), ("c1_cache_w64.json", 16, c1_inputs),
         ("c1_cache_w128.json", 16, c1_inputs)]  # width 128: layer 0 in two K chunks


@pytest.mark.parametrize("prec", ["bf16", "fp16", "fp8"])
@pytest.mark.parametrize("cfg,in_ch,gen", CASES)
def test_tensor_core_inference(mlpmod, cfg, in_ch, gen, prec):
    net = mlpmod.TinyMLP(cfg, in_ch, 3, precision=prec, seed=3)
    oc = mo.Config(net.config_text, in_ch, 3)
    if oc.n_enc_params:  # give the grid a visible contribution
        p = net.params()
        p[oc.n_net_params:] = np.random.default_rng(5).uniform(-0.5, 0.5, oc.n_enc_params)
        net.set_params(p)
    n = 4096 + 37  # ragged tail tile
    x = gen(n, seed=1)
    out = net.inference(torch.from_numpy(x).cuda()).cpu().numpy().astype(np.float64)
    params = net.params()
    assert np.isfinite(out).all()
    check_vs_emulation(out, emulate(oc, params, x, prec), prec)
    ref, _ = mo.forward(oc, params.astype(np.float64), x)
    ref = ref[:, :3]
    rel = np.sqrt(np.mean((out - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    assert rel <= ORACLE_REL[prec], rel


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
def test_tensor_core_inference_follows_training(mlpmod, prec):
    """Training stays FP32; the next inference repacks the updated weights."""
    net = mlpmod.TinyMLP("c1_cache_w64.json", 16, 3, precision=prec, seed=4)
    oc = mo.Config(net.config_text, 16, 3)
    x = c1_inputs(2048, seed=7)
    tgt = np.random.default_rng(2).lognormal(0.0, 1.0, (2048, 3)).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(tgt).cuda()
    before = net.inference(dx).cpu().numpy()
    for _ in range(3):
        net.training_step(dx, dt)
    after = net.inference(dx).cpu().numpy().astype(np.float64)
    assert not np.array_equal(before, after)
    check_vs_emulation(after, emulate(oc, net.params(), x, prec), prec)


def test_tensor_core_inference_is_deterministic(mlpmod):
    net = mlpmod.TinyMLP("c1_cache_w64.json", 16, 3, precision="bf16", seed=3)
    dx = torch.from_numpy(c1_inputs(10000, seed=2)).cuda()
    a = net.inference(dx)
    b = net.inference(dx)
    assert torch.equal(a, b)
