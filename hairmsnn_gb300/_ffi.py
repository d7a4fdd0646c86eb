"""ctypes binding of libhairmsnn.so (the C ABI declared in include/hairmsnn.h).

There is no fallback: if the library is missing or fails to load, every entry
point raises.  Build it with hairmsnn_gb300.build.build() (or
__graft_entry__.build()).
"""
import ctypes
import os
import re

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "hairmsnn.h")

_lib = None


class HMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"hairmsnn status {status}: {msg}")
        self.status = status


class hm_hair_params(ctypes.Structure):
    _fields_ = [("sigma_a", ctypes.c_float * 3), ("beta_m", ctypes.c_float),
                ("beta_n", ctypes.c_float), ("alpha", ctypes.c_float),
                ("gain_r", ctypes.c_float), ("gain_tt", ctypes.c_float),
                ("gain_trt", ctypes.c_float), ("gain_trrt", ctypes.c_float)]

    @classmethod
    def from_array(cls, hp):
        """hp: sigma_a[3], beta_m, beta_n, alpha(rad), gains R, TT, TRT, TRRT."""
        hp = [float(x) for x in hp]
        p = cls()
        p.sigma_a[:] = hp[0:3]
        p.beta_m, p.beta_n, p.alpha = hp[3], hp[4], hp[5]
        p.gain_r, p.gain_tt, p.gain_trt, p.gain_trrt = hp[6:10]
        return p


class hm_bsdf_queries(ctypes.Structure):
    _fields_ = [("wo", ctypes.c_void_p), ("wi", ctypes.c_void_p), ("tangent", ctypes.c_void_p),
                ("h", ctypes.c_void_p), ("u", ctypes.c_void_p)]


class hm_mlp_desc(ctypes.Structure):
    _fields_ = [("in_ch", ctypes.c_int), ("out_ch", ctypes.c_int), ("encoded_width", ctypes.c_int),
                ("padded_input_width", ctypes.c_int), ("width", ctypes.c_int),
                ("n_hidden_layers", ctypes.c_int), ("padded_output_width", ctypes.c_int),
                ("n_params", ctypes.c_int64), ("n_network_params", ctypes.c_int64),
                ("precision", ctypes.c_int), ("step", ctypes.c_int),
                ("learning_rate", ctypes.c_float)]


def header_functions():
    """Names of every function declared in include/hairmsnn.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hm_[a-z0-9_]+)\s*\(", text)))


def lib_path():
    return _build.LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.isfile(path):
        raise RuntimeError(f"libhairmsnn.so not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    vp, i64, i32, u32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_uint32
    L.hm_status_string.restype = ctypes.c_char_p
    L.hm_status_string.argtypes = [i32]
    L.hm_last_error.restype = ctypes.c_char_p
    L.hm_version.restype = ctypes.c_char_p
    P = ctypes.POINTER
    L.hm_hair_setup.argtypes = [P(hm_hair_params), vp]
    L.hm_bsdf_eval.argtypes = [P(hm_bsdf_queries), vp, vp, i64, P(hm_hair_params), vp]
    L.hm_bsdf_sample.argtypes = [P(hm_bsdf_queries), vp, vp, vp, i64, P(hm_hair_params), vp]
    L.hm_bsdf_eval_grad.argtypes = [P(hm_bsdf_queries), vp, vp, vp, vp, i64, P(hm_hair_params), vp]
    L.hm_bsdf_gen_queries.argtypes = [u32, i64, vp, vp, vp, vp, vp, vp]
    # radiance-cache network
    L.hm_mlp_create.restype = vp
    L.hm_mlp_create.argtypes = [ctypes.c_char_p, i32, i32, i32, u32, P(i32)]
    L.hm_mlp_destroy.restype = None
    L.hm_mlp_destroy.argtypes = [vp]
    L.hm_mlp_info.argtypes = [vp, P(hm_mlp_desc)]
    L.hm_mlp_describe_config.argtypes = [ctypes.c_char_p, i32, i32, P(hm_mlp_desc)]
    L.hm_mlp_inference.argtypes = [vp, vp, vp, i64, vp]
    L.hm_mlp_forward.argtypes = [vp, vp, vp, i64, vp]
    L.hm_mlp_backward.argtypes = [vp, vp, i64, vp, vp]
    L.hm_mlp_backward_output_grad.argtypes = [vp, vp, i64, vp]
    L.hm_mlp_optimizer_step.argtypes = [vp, ctypes.c_float, vp]
    L.hm_mlp_training_step.argtypes = [vp, vp, vp, i64, vp, vp]
    L.hm_mlp_last_loss.argtypes = [vp, P(ctypes.c_float)]
    L.hm_mlp_reset.argtypes = [vp]
    L.hm_mlp_get_params.argtypes = [vp, vp]
    L.hm_mlp_set_params.argtypes = [vp, vp]
    L.hm_mlp_get_gradients.argtypes = [vp, vp]
    L.hm_mlp_save.argtypes = [vp, ctypes.c_char_p]
    L.hm_mlp_load.argtypes = [vp, ctypes.c_char_p]
    _lib = L
    return L


def check(status):
    if status != 0:
        L = lib()
        raise HMError(status, f"{L.hm_status_string(status).decode()}: {L.hm_last_error().decode()}")
    return status
