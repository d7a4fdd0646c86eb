"""Failure detection of the tensor-core kernels' waits, without a GPU fault:
a bounded mbarrier wait that nothing completes expires, the kernel returns,
the host reads HM_ETIMEOUT, and the same context then runs the tensor-core
network normally."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from hairmsnn_gb300 import _ffi, build, mlp
    build.build()
    return _ffi, mlp


def test_bounded_wait_expires_and_the_context_stays_usable(mods):
    ffi, mlp = mods
    L = ffi.lib()
    L.hm_debug_wait_expiry.restype = ctypes.c_int
    L.hm_debug_wait_expiry.argtypes = [ctypes.c_int, ctypes.c_void_p]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for tries in (1, 64, 4096):
        assert L.hm_debug_wait_expiry(tries, stream) == 4  # HM_ETIMEOUT
    assert L.hm_debug_wait_expiry(0, stream) == 1  # HM_EINVAL
    net = mlp.TinyMLP("c1_cache_w64.json", 16, 3, precision="fp16", seed=1)
    x = torch.rand((4096, 16), device="cuda")
    y = net.inference(x)
    torch.cuda.synchronize()
    assert torch.isfinite(y).all()
    y2 = net.inference(x)
    assert torch.equal(y, y2)
