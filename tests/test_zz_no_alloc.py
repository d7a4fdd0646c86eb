"""hm_mlp_inference_noalloc (static device scratch, no allocation) against
hm_mlp_inference, through the C ABI.

Both run the same encode and forward kernels, so two calls in a row of the
static-scratch entry point must equal the allocating entry point bit for bit,
the device's free memory must not move across them, and a batch larger than
the static scratch must be refused with HM_ECAPACITY.  Kept in its own file,
collected last, so it also runs after every other test of the session.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HM_ECAPACITY = 3
SCRATCH_FLOATS = 1 << 20


@pytest.fixture(scope="module")
def L():
    from hairmsnn_gb300 import _ffi, build
    build.build()
    lib = _ffi.lib()
    vp = ctypes.c_void_p
    lib.hm_mlp_inference_noalloc.argtypes = [vp, vp, vp, ctypes.c_int64, vp]
    lib.hm_mlp_inference_noalloc.restype = ctypes.c_int
    lib.hm_mlp_inference.argtypes = [vp, vp, vp, ctypes.c_int64, vp]
    lib.hm_mlp_inference.restype = ctypes.c_int
    return lib


def _inputs(n, in_ch, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.rand((n, in_ch), generator=g).mul_(2).sub_(1).to("cuda").contiguous()


@pytest.mark.parametrize("cfg,in_ch", [("c1_cache_w64.json", 16), ("hairmsnn_cache.json", 12)])
def test_noalloc_inference_matches_allocating_entry_point(L, cfg, in_ch):
    from hairmsnn_gb300 import mlp
    net = mlp.TinyMLP(cfg, in_ch, 3, seed=7)
    h = net._h
    max_n = SCRATCH_FLOATS // net.info().padded_input_width
    n = min(3000, max_n)
    stream0 = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the largest accepted batch fills the scratch up to its last encoded row
    xm = _inputs(max_n, in_ch, 9)
    om, rm = torch.empty((max_n, 3), device="cuda"), torch.empty((max_n, 3), device="cuda")
    assert L.hm_mlp_inference_noalloc(h, ctypes.c_void_p(xm.data_ptr()), ctypes.c_void_p(om.data_ptr()), max_n,
                                      stream0) == 0
    assert L.hm_mlp_inference(h, ctypes.c_void_p(xm.data_ptr()), ctypes.c_void_p(rm.data_ptr()), max_n,
                              stream0) == 0
    torch.cuda.synchronize()
    assert torch.equal(om, rm)
    xs = [_inputs(n, in_ch, s) for s in (1, 2)]
    outs = [torch.full((n, 3), float("nan"), device="cuda") for _ in range(2)]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    # first call on this device: resolves the scratch address (set-up)
    assert L.hm_mlp_inference_noalloc(h, ctypes.c_void_p(xs[0].data_ptr()), ctypes.c_void_p(outs[0].data_ptr()),
                                      n, stream) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for x, o in zip(xs, outs):  # two calls in a row
        assert L.hm_mlp_inference_noalloc(h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(o.data_ptr()), n,
                                          stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before

    for x, o in zip(xs, outs):
        ref = torch.empty((n, 3), device="cuda")
        assert L.hm_mlp_inference(h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(ref.data_ptr()), n,
                                  stream) == 0
        torch.cuda.synchronize()
        assert torch.isfinite(o).all()
        assert torch.equal(o, ref)
    assert not torch.equal(outs[0], outs[1])

    # beyond the static scratch: refused, output untouched
    big = max_n + 1
    xb = torch.zeros((big, in_ch), device="cuda")
    ob = torch.full((big, 3), 7.0, device="cuda")
    st = L.hm_mlp_inference_noalloc(h, ctypes.c_void_p(xb.data_ptr()), ctypes.c_void_p(ob.data_ptr()), big, stream)
    assert st == HM_ECAPACITY
    assert b"static scratch" in L.hm_last_error()
    torch.cuda.synchronize()
    assert bool((ob == 7.0).all())
    net.close()


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_noalloc_tensor_core_inference_matches_allocating_entry_point(L, precision):
    """FP16 / BF16 handles: the encoding runs inside the tensor-core kernel
    (no scratch, no workspace), while hm_mlp_inference encodes into its
    workspace first.  Same roundings either way; held to the tensor-core
    bar of the other tests, with free device memory unchanged across two
    calls in a row and no size cap."""
    from hairmsnn_gb300 import mlp
    net = mlp.TinyMLP("c1_cache_w64.json", 16, 3, precision=precision, seed=7)
    h = net._h
    n = 20000  # beyond the FP32 path's static-scratch cap: no scratch here
    xs = [_inputs(n, 16, s) for s in (3, 4)]
    outs = [torch.full((n, 3), float("nan"), device="cuda") for _ in range(2)]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.hm_mlp_inference_noalloc(h, ctypes.c_void_p(xs[0].data_ptr()), ctypes.c_void_p(outs[0].data_ptr()),
                                      n, stream) == 0  # first call packs the 16-bit weights (no allocation)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for x, o in zip(xs, outs):
        assert L.hm_mlp_inference_noalloc(h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(o.data_ptr()), n,
                                          stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    for x, o in zip(xs, outs):
        ref = torch.empty((n, 3), device="cuda")
        assert L.hm_mlp_inference(h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(ref.data_ptr()), n,
                                  stream) == 0
        torch.cuda.synchronize()
        assert torch.isfinite(o).all()
        rms = float(ref.pow(2).mean().sqrt())
        err = (o - ref).abs() - (3e-3 * rms + 3e-3 * ref.abs())
        assert float(err.max()) <= 0, float(err.max())
    net.close()
