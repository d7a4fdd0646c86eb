"""The forms of 16-bit tensor-core inference give the same bits.

* the warp-specialised kernel: encoding and layers overlapped in one CTA
  per SM (two pipeline lanes, each with its own encoder warps, layer warps,
  operand stages and tensor-memory columns), no workspace;
* the encode kernel, then the layer kernel loading the encoded operands by
  bulk copies (hm_mlp_inference's workspace);
* the layer kernel encoding each tile itself (hm_mlp_inference_noalloc, no
  workspace).

All three round every encoded feature, activation and output the same way
and issue the same MMAs in the same order, so their outputs must be equal
bit for bit.  hm_debug_tc_path selects the form; sizes cover one row, ragged
tiles, fewer tiles than SMs and many tiles per pipeline lane (the barriers'
phases wrap many times).
"""
import ctypes

import numpy as np
import pytest

from oracle import mlp_oracle as mo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HM_EUNSUPPORTED = 7


@pytest.fixture(scope="module")
def mods():
    from hairmsnn_gb300 import _ffi, build, mlp
    build.build()
    lib = _ffi.lib()
    vp = ctypes.c_void_p
    lib.hm_debug_tc_path.argtypes = [ctypes.c_int]
    lib.hm_debug_tc_path.restype = ctypes.c_int
    lib.hm_mlp_inference_noalloc.argtypes = [vp, vp, vp, ctypes.c_int64, vp]
    lib.hm_mlp_inference_noalloc.restype = ctypes.c_int
    lib.hm_mlp_inference.argtypes = [vp, vp, vp, ctypes.c_int64, vp]
    lib.hm_mlp_inference.restype = ctypes.c_int
    yield lib, mlp
    lib.hm_debug_tc_path(0)


def _inputs(n, in_ch, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.rand((n, in_ch), generator=g).mul_(2).sub_(1).to("cuda").contiguous()


def _run(L, h, x, n, path, noalloc=False):
    assert L.hm_debug_tc_path(path) == 0
    out = torch.full((n, 3), float("nan"), device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    call = L.hm_mlp_inference_noalloc if noalloc else L.hm_mlp_inference
    st = call(h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), n, stream)
    torch.cuda.synchronize()
    L.hm_debug_tc_path(0)
    assert st == 0, st
    return out


@pytest.mark.parametrize("n", [1, 127, 129, 4096 + 37, 152 * 128 - 5, (1 << 17) + 77])
@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("cfg,in_ch", [("c1_cache_w64.json", 16), ("hairmsnn_cache.json", 12)])
def test_warp_specialised_inference_equals_the_other_forms(mods, cfg, in_ch, prec, n):
    L, mlp = mods
    net = mlp.TinyMLP(cfg, in_ch, 3, precision=prec, seed=11)
    oc = mo.Config(net.config_text, in_ch, 3)
    if oc.n_enc_params:  # a visible hash-grid contribution
        p = net.params()
        p[oc.n_net_params:] = np.random.default_rng(5).uniform(-0.5, 0.5, oc.n_enc_params)
        net.set_params(p)
    x = _inputs(n, in_ch, 3)
    ws = _run(L, net._h, x, n, 2)
    two = _run(L, net._h, x, n, 1)
    fused = _run(L, net._h, x, n, 1, noalloc=True)
    assert torch.isfinite(ws).all()
    assert torch.equal(ws, two), float((ws - two).abs().max())
    assert torch.equal(ws, fused), float((ws - fused).abs().max())
    net.close()


@pytest.mark.parametrize("cfg,prec", [("c1_cache_w128.json", "fp16"), ("c1_cache_w64.json", "fp8")])
def test_warp_specialised_path_refuses_what_it_does_not_fit(mods, cfg, prec):
    """Width 128 (its weights and two operand stages exceed shared memory)
    and E4M3 operands run the other forms; forcing the warp-specialised
    kernel on them is refused, not run."""
    L, mlp = mods
    net = mlp.TinyMLP(cfg, 16, 3, precision=prec, seed=1)
    x = _inputs(256, 16, 1)
    assert L.hm_debug_tc_path(2) == 0
    out = torch.empty((256, 3), device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = L.hm_mlp_inference(net._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), 256, stream)
    L.hm_debug_tc_path(0)
    assert st == HM_EUNSUPPORTED
    assert L.hm_debug_tc_path(3) != 0
    net.close()
