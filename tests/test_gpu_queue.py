"""The wavefront's queue compaction (hm_queue_compact: the kernels that
compact the path queue between bounce rounds) against a host stable
partition, bit for bit: every kept entry, in order, and the count, for
empty, single, block-boundary, ragged and frame-sized queues and for
all-kept / none-kept masks."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from hairmsnn_gb300 import _ffi, build
    build.build()
    lib = _ffi.lib()
    vp = ctypes.c_void_p
    lib.hm_queue_compact.argtypes = [vp, vp, ctypes.c_int64, vp, ctypes.POINTER(ctypes.c_int64), vp]
    lib.hm_queue_compact.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("n,density", [(0, 0.5), (1, 1.0), (1, 0.0), (31, 0.5), (1023, 0.3), (1024, 0.5),
                                       (1025, 0.7), (4097, 0.5), (262144, 0.61), (262144, 0.0), (262144, 1.0),
                                       (1 << 21, 0.02), (3_000_001, 0.5)])
def test_compaction_is_a_stable_partition(L, n, density):
    rng = np.random.default_rng(n + int(density * 100))
    keep = (rng.random(n) < density).astype(np.int32)
    queue = rng.permutation(max(n, 1))[:n].astype(np.int32)
    k, q = torch.from_numpy(keep).cuda(), torch.from_numpy(queue).cuda()
    out = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    cnt = ctypes.c_int64(-1)
    st = torch.cuda.current_stream().cuda_stream
    assert L.hm_queue_compact(ctypes.c_void_p(k.data_ptr()), ctypes.c_void_p(q.data_ptr()), n,
                              ctypes.c_void_p(out.data_ptr()), ctypes.byref(cnt), ctypes.c_void_p(st)) == 0
    ref = queue[keep != 0]
    assert cnt.value == len(ref)
    got = out.cpu().numpy()
    assert np.array_equal(got[:len(ref)], ref)
    assert (got[len(ref):] == -7).all()  # nothing written past the kept entries
