"""HairMSNN per-path-vertex hot path on GB300 (sm_103a).

The compute lives in libhairmsnn.so (hand-written CUDA behind the C ABI in
include/hairmsnn.h).  This package is the host-side mirror of the reference's
interfaces for that path, on torch CUDA tensors:

* bsdf_eval / bsdf_sample   — disney_hair() / sample_disney_hair()
                              (cuda_headers/disney_hair.cuh:186,277), batched.

Nothing here computes on the CPU: a missing library raises.
"""
import ctypes

from . import _ffi
from ._ffi import HMError, check, hm_bsdf_queries, hm_hair_params, lib

__all__ = ["HMError", "lib", "bsdf_eval", "bsdf_sample", "gen_bsdf_queries", "hair_params",
           "C1_HAIR"]

# alpha = 3.14159 * 2 deg / 180 as the scene parser converts it (scene.cpp:207)
C1_HAIR = [0.06, 0.1, 0.2, 0.3, 0.3, 3.14159 * 2.0 / 180.0, 1.0, 1.0, 1.0, 1.0]


def hair_params(hp=None):
    return hm_hair_params.from_array(C1_HAIR if hp is None else hp)


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def bsdf_eval(wo, wi, tangent, h, hp=None, stream=None):
    """Planar float32 CUDA tensors wo/wi/tangent [3,n], h [n] -> f [3,n], pdf [n]."""
    import torch
    n = h.shape[0]
    f = torch.empty((3, n), dtype=torch.float32, device=h.device)
    pdf = torch.empty((n,), dtype=torch.float32, device=h.device)
    q = hm_bsdf_queries(_ptr(wo), _ptr(wi), _ptr(tangent), _ptr(h), None)
    p = hair_params(hp)
    check(lib().hm_bsdf_eval(ctypes.byref(q), _ptr(f), _ptr(pdf), n, ctypes.byref(p), _stream(stream)))
    return f, pdf


def bsdf_eval_grad(wo, wi, tangent, h, hp=None, stream=None):
    """bsdf_eval plus derivatives with respect to (sigma_a r, g, b, beta_m,
    beta_n, alpha): returns f [3,n], pdf [n], df [6,3,n], dpdf [6,n]."""
    import torch
    n = h.shape[0]
    f = torch.empty((3, n), dtype=torch.float32, device=h.device)
    pdf = torch.empty((n,), dtype=torch.float32, device=h.device)
    df = torch.empty((6, 3, n), dtype=torch.float32, device=h.device)
    dpdf = torch.empty((6, n), dtype=torch.float32, device=h.device)
    q = hm_bsdf_queries(_ptr(wo), _ptr(wi), _ptr(tangent), _ptr(h), None)
    p = hair_params(hp)
    check(lib().hm_bsdf_eval_grad(ctypes.byref(q), _ptr(f), _ptr(pdf), _ptr(df), _ptr(dpdf), n, ctypes.byref(p),
                                  _stream(stream)))
    return f, pdf, df, dpdf


def bsdf_sample(wo, tangent, h, u, hp=None, stream=None):
    """wo/tangent [3,n], h [n], u [4,n] -> wi [3,n], f [3,n], pdf [n]."""
    import torch
    n = h.shape[0]
    wi = torch.empty((3, n), dtype=torch.float32, device=h.device)
    f = torch.empty((3, n), dtype=torch.float32, device=h.device)
    pdf = torch.empty((n,), dtype=torch.float32, device=h.device)
    q = hm_bsdf_queries(_ptr(wo), None, _ptr(tangent), _ptr(h), _ptr(u))
    p = hair_params(hp)
    check(lib().hm_bsdf_sample(ctypes.byref(q), _ptr(wi), _ptr(f), _ptr(pdf), n, ctypes.byref(p),
                               _stream(stream)))
    return wi, f, pdf


def gen_bsdf_queries(seed, n, device="cuda", stream=None):
    """Synthetic BSDF workload on the device: wo, wi, tangent [3,n], h [n], u [4,n]."""
    import torch
    kw = dict(dtype=torch.float32, device=device)
    wo, wi, t = (torch.empty((3, n), **kw) for _ in range(3))
    h = torch.empty((n,), **kw)
    u = torch.empty((4, n), **kw)
    check(lib().hm_bsdf_gen_queries(seed, n, _ptr(wo), _ptr(wi), _ptr(t), _ptr(h), _ptr(u),
                                    _stream(stream)))
    return wo, wi, t, h, u
