"""numpy/ctypes front end of the ORACLE (test infrastructure only).

Loads oracle/_build/libhmoracle.so (building it with g++ if needed) and
exposes the restatement's functions on numpy arrays.  Imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")

# sigma_a[3], beta_m, beta_n, alpha(rad), gains R, TT, TRT, TRRT
C1_HAIR = np.array([0.06, 0.1, 0.2, 0.3, 0.3, 3.14159 * 2.0 / 180.0, 1, 1, 1, 1], np.float32)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        i64, i32, u32, f32 = ctypes.c_int64, ctypes.c_int, ctypes.c_uint32, ctypes.c_float
        L.hmo_get_rng.restype = u32
        L.hmo_get_rng.argtypes = [i32, u32, u32, u32, u32]
        L.hmo_lcg_stream.restype = u32
        L.hmo_lcg_stream.argtypes = [u32, i32, F32P]
        L.hmo_query_rng.restype = u32
        L.hmo_query_rng.argtypes = [u32, u32]
        L.hmo_setup_hair.argtypes = [F32P, F32P]
        L.hmo_set_mp_force_fp32.argtypes = [i32]
        L.hmo_hair_eval.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P]
        L.hmo_hair_sample.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P]
        L.hmo_hair_eval_mt.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P, i32]
        L.hmo_hair_sample_mt.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P, i32]
        L.hmo_gen_bsdf_queries.argtypes = [u32, i64, F32P, F32P, F32P, F32P, F32P]
        L.hmo_frostbite_ggx.argtypes = [F32P, F32P, F32P, f32, F32P]
        L.hmo_sample_ggx.argtypes = [F32P, f32, F32P, F32P, F32P]
        L.hmo_pdf_ggx.restype = f32
        L.hmo_pdf_ggx.argtypes = [f32, F32P, F32P]
        L.hmo_curve_eval.argtypes = [i32, F32P, f32, F32P, F32P]
        L.hmo_orthonormal_basis.argtypes = [F32P, F32P]
        L.hmo_uniform_sample_sphere.argtypes = [F32P, F32P]
        for name in ("hmo_power_heuristic",):
            getattr(L, name).restype = f32
            getattr(L, name).argtypes = [f32, f32]
        for name in ("hmo_luminance", "hmo_spherical_theta", "hmo_spherical_phi"):
            getattr(L, name).restype = f32
            getattr(L, name).argtypes = [F32P]
        _lib = L
    return _lib


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def lcg_stream(state, n):
    out = np.zeros(n, np.float32)
    end = lib().hmo_lcg_stream(int(state) & 0xFFFFFFFF, n, out)
    return out, end


def setup_hair(hp):
    out = np.zeros(10, np.float32)
    lib().hmo_setup_hair(f32(hp), out)
    return out


def set_mp_force_fp32(on):
    lib().hmo_set_mp_force_fp32(1 if on else 0)


def hair_eval(wo, wi, t, h, hp=C1_HAIR, threads=1):
    """wo, wi, t: [n,3] world vectors; h: [n].  Returns f [n,3], pdf [n]."""
    wo, wi, t, h = f32(wo), f32(wi), f32(t), f32(h)
    n = h.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    if threads > 1:
        lib().hmo_hair_eval_mt(n, wo, wi, t, h, f32(hp), f, pdf, threads)
    else:
        lib().hmo_hair_eval(n, wo, wi, t, h, f32(hp), f, pdf)
    return f, pdf


def hair_sample(wo, t, h, u, hp=C1_HAIR, threads=1):
    """u: [n,4].  Returns wi [n,3], f [n,3], pdf [n], lobe margin [n]."""
    wo, t, h, u = f32(wo), f32(t), f32(h), f32(u)
    n = h.shape[0]
    wi = np.zeros((n, 3), np.float32)
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    margin = np.zeros(n, np.float32)
    if threads > 1:
        lib().hmo_hair_sample_mt(n, wo, t, h, u, f32(hp), wi, f, pdf, threads)
    else:
        lib().hmo_hair_sample(n, wo, t, h, u, f32(hp), wi, f, pdf, margin)
    return wi, f, pdf, margin


def gen_bsdf_queries(seed, n):
    """Synthetic BSDF workload, planar layouts: wo/wi/t [3,n], h [n], u [4,n]."""
    wo = np.zeros((3, n), np.float32)
    wi = np.zeros((3, n), np.float32)
    t = np.zeros((3, n), np.float32)
    h = np.zeros(n, np.float32)
    u = np.zeros((4, n), np.float32)
    lib().hmo_gen_bsdf_queries(seed, n, wo, wi, t, h, u)
    return wo, wi, t, h, u
