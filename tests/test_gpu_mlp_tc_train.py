"""Cache training on the tensor cores (FP32 accumulation).

FP16 / BF16 handles run the training forward, the dgrad chain and the weight
gradients on tcgen05 (FP16 with a static loss scale of 128, divided out by
the optimizer and by hm_mlp_get_gradients).  E4M3 handles run the training
forward on E4M3 operands (per-layer weight scales, per-row activation
scales: the inference kernel's arithmetic) and the backward on FP16 operands
with the same loss scale.  Against the FP64 oracle on the same parameters
and batch (rms of the error / rms of the reference, per weight matrix and
for the hash tables):
    loss         FP16 2e-3, BF16 1e-2, E4M3 5e-2 (relative)
    gradients    FP16 2.5e-2, BF16 1e-1, E4M3 3e-1
(the errors scale with the operand precision: BF16 has 3 fewer mantissa
bits than FP16 and its errors are about 4-8x larger; E4M3 rounds every
forward operand to 3 mantissa bits (measured: loss 0.6-2.8%, gradients
3-19%, hash tables 23%); the first layer and the hash tables sit at the end
of the dgrad chain and carry the most) and 60 training steps reduce the
loss as the FP32 kernels do (final loss within 1.5x of FP32's; E4M3
measured 1.09x).
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"fp16": (2e-3, 2.5e-2), "bf16": (1e-2, 1e-1), "fp8": (5e-2, 3e-1)}


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


CASES = [("hairmsnn_cache.json", 12, ref_inputs), ("c1_cache_w64.json", 16, c1_inputs),
         ("c1_cache_w128.json", 16, c1_inputs)]


def rel_rms(a, b):
    return np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30)


@pytest.mark.parametrize("prec", ["fp16", "bf16", "fp8"])
@pytest.mark.parametrize("cfg,in_ch,gen", CASES)
def test_tensor_core_gradients_match_oracle(mlpmod, cfg, in_ch, gen, prec):
    net = mlpmod.TinyMLP(cfg, in_ch, 3, precision=prec, seed=11)
    oc = mo.Config(net.config_text, in_ch, 3)
    if oc.n_enc_params:
        p = net.params()
        p[oc.n_net_params:] = np.random.default_rng(5).uniform(-0.5, 0.5, oc.n_enc_params)
        net.set_params(p)
    n = 2048 + 64
    x = gen(n, seed=2)
    tgt = np.random.default_rng(9).lognormal(0.0, 1.0, (n, 3)).astype(np.float32)
    p0 = net.params().astype(np.float64)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(tgt).cuda()
    net.forward(dx)
    loss = net.backward(dt).item()
    ref_loss, ref_g = mo.backward(oc, p0, x, tgt)
    tl, tg = TOL[prec]
    assert abs(loss - ref_loss) <= tl * abs(ref_loss), (loss, ref_loss)
    g = net.gradients().astype(np.float64)
    for off, fo, fi in oc.layer_shapes:
        e = rel_rms(g[off:off + fo * fi], ref_g[off:off + fo * fi])
        assert e <= tg, (off, e)
    if oc.n_enc_params:
        e = rel_rms(g[oc.n_net_params:], ref_g[oc.n_net_params:])
        assert e <= tg, ("grid", e)


@pytest.mark.parametrize("prec", ["fp16", "bf16", "fp8"])
def test_tensor_core_training_converges(mlpmod, prec):
    x = c1_inputs(1 << 14, seed=4)
    tgt = (np.abs(np.sin(3 * x[:, 0:3])) + 0.1).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(tgt).cuda()
    finals = {}
    for p in ("fp32", prec):
        net = mlpmod.TinyMLP("c1_cache_w64.json", 16, 3, precision=p, seed=3)
        losses = []
        for _ in range(60):
            losses.append(net.training_step(dx, dt, read_loss=True) and net.training_loss)
        assert np.isfinite(losses).all()
        assert np.mean(losses[-5:]) < 0.5 * np.mean(losses[:5])
        finals[p] = np.mean(losses[-5:])
    assert finals[prec] <= 1.5 * finals["fp32"], finals


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16", "fp8"])
@pytest.mark.parametrize("cfg,in_ch,gen", CASES[:2])
def test_output_grad_backward_matches_oracle(mlpmod, cfg, in_ch, gen, prec):
    """hm_mlp_backward_output_grad (tcnn's backward with dL_doutput) against
    the FP64 oracle: FP32 within 1e-4, FP16 within 4e-2, BF16 within
    1.5e-1 and E4M3 within 4.5e-1 (1.5x the loss-gradient bars: a random dL/d(output) is
    uncorrelated with the outputs, so each weight's gradient is a sum with
    more cancellation and its relative error is larger; layer 0 measured
    2.7e-2 in FP16)."""
    net = mlpmod.TinyMLP(cfg, in_ch, 3, precision=prec, seed=13)
    oc = mo.Config(net.config_text, in_ch, 3)
    if oc.n_enc_params:
        p = net.params()
        p[oc.n_net_params:] = np.random.default_rng(6).uniform(-0.5, 0.5, oc.n_enc_params)
        net.set_params(p)
    n = 4096 + 32
    x = gen(n, seed=3)
    dy = (np.random.default_rng(8).normal(size=(n, 3)) / n).astype(np.float32)
    p0 = net.params().astype(np.float64)
    net.forward(torch.from_numpy(x).cuda())
    net.backward_output_grad(torch.from_numpy(dy).cuda())
    ref = mo.backward_output_grad(oc, p0, x, dy)
    g = net.gradients().astype(np.float64)
    tg = 1e-4 if prec == "fp32" else 1.5 * TOL[prec][1]
    for off, fo, fi in oc.layer_shapes:
        assert rel_rms(g[off:off + fo * fi], ref[off:off + fo * fi]) <= tg, (off, prec)
    if oc.n_enc_params:
        assert rel_rms(g[oc.n_net_params:], ref[oc.n_net_params:]) <= tg
