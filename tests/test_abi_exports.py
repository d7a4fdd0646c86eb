"""The C-ABI library loads and exports every symbol include/hairmsnn.h
declares; host-only entry points behave without a GPU."""
import ctypes

import numpy as np
import pytest

import hairmsnn_gb300 as hm
from hairmsnn_gb300 import _ffi


@pytest.fixture(scope="module")
def L():
    from hairmsnn_gb300 import build
    build.build()
    return _ffi.lib()


def test_every_header_symbol_is_exported(L):
    names = _ffi.header_functions()
    assert len(names) >= 7
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(L):
    assert L.hm_status_string(0) == b"ok"
    assert L.hm_status_string(3) == b"capacity exceeded"
    assert b"sm_103a" in L.hm_version()


def test_hair_setup_matches_reference_golden(L, golden):
    """hm_hair_setup is host code: setupHairShading bit for bit."""
    for name in ("c1", "dark", "smooth_gain", "thin"):
        p = hm.hair_params(golden[f"{name}_hp"])
        out = np.zeros(10, np.float32)
        assert L.hm_hair_setup(ctypes.byref(p), out.ctypes.data_as(ctypes.c_void_p)) == 0
        assert np.array_equal(out.view(np.uint32), golden[f"{name}_setup"].view(np.uint32))


def test_bad_arguments_are_rejected_without_touching_the_device(L):
    p = hm.hair_params()
    q = _ffi.hm_bsdf_queries()
    assert L.hm_bsdf_eval(ctypes.byref(q), None, None, -1, ctypes.byref(p), None) == 1
    assert L.hm_bsdf_eval(ctypes.byref(q), None, None, 0, ctypes.byref(p), None) == 0
    assert L.hm_bsdf_eval(ctypes.byref(q), None, None, 16, ctypes.byref(p), None) == 1
    assert b"NULL" in L.hm_last_error()
    bad = hm.hair_params([0.1, 0.1, 0.1, 0.0, 0.3, 0.0, 1, 1, 1, 1])
    assert L.hm_bsdf_eval(ctypes.byref(q), None, None, 0, ctypes.byref(bad), None) == 1
    assert L.hm_hair_setup(None, None) == 1


def test_inference_form_selector_checks_its_range(L):
    """hm_debug_tc_path only sets the form of later inferences: no device
    call, so it runs without a GPU."""
    L.hm_debug_tc_path.argtypes = [ctypes.c_int]
    L.hm_debug_tc_path.restype = ctypes.c_int
    for bad in (-1, 3, 7):
        assert L.hm_debug_tc_path(bad) == 1  # HM_EINVAL
    assert b"out of range" in L.hm_last_error()
    for ok in (2, 1, 0):
        assert L.hm_debug_tc_path(ok) == 0
