"""Host mirror of the reference's TINY_MLP wrapper over the C ABI.

TINY_MLP (cuda_headers/neural_network.cuh:33-50, cuda/neural_network.cu:17-64)
held a tiny-cuda-nn network, optimizer and loss built from a JSON config; the
frame driver called inference(), trainer->training_step() and
trainer->loss() (render_hair_msnn.cu:683-691, :745-748).  TinyMLP keeps those
names and argument meanings on torch CUDA tensors; every call runs in
libhairmsnn.so.
"""
import ctypes
import json
import os

import numpy as np

from . import _ffi
from ._ffi import check, hm_mlp_desc, lib

CONFIG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "configs")
PRECISIONS = {"fp32": 0, "fp16": 1, "bf16": 2, "fp8": 3}


def load_config(path_or_dict):
    if isinstance(path_or_dict, dict):
        return json.dumps(path_or_dict)
    if os.path.isfile(path_or_dict):
        return open(path_or_dict).read()
    cand = os.path.join(CONFIG_DIR, path_or_dict)
    if os.path.isfile(cand):
        return open(cand).read()
    return path_or_dict  # JSON text


def describe(config, in_ch, out_ch):
    d = hm_mlp_desc()
    check(lib().hm_mlp_describe_config(load_config(config).encode(), in_ch, out_ch, ctypes.byref(d)))
    return d


def _vp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


class TinyMLP:
    """TINY_MLP(configPath, inputCh, outputCh) on the GB300 library."""

    def __init__(self, config, input_ch, output_ch, precision="fp32", seed=0):
        self.config_text = load_config(config)
        self.input_ch, self.output_ch = input_ch, output_ch
        st = ctypes.c_int(0)
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = lib().hm_mlp_create(self.config_text.encode(), input_ch, output_ch, prec, seed,
                                ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)
        self.training_loss = 0.0

    @classmethod
    def wrap(cls, handle):
        """A view of a network owned elsewhere (e.g. a renderer's cache)."""
        if not handle:
            raise ValueError("no network")
        net = cls.__new__(cls)
        net._h = ctypes.c_void_p(handle)
        net._borrowed = True
        net.training_loss = 0.0
        d = net.info()
        net.input_ch, net.output_ch = d.in_ch, d.out_ch
        return net

    def close(self):
        if getattr(self, "_h", None):
            if not getattr(self, "_borrowed", False):
                lib().hm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        d = hm_mlp_desc()
        check(lib().hm_mlp_info(self._h, ctypes.byref(d)))
        return d

    @property
    def n_params(self):
        return self.info().n_params

    # TINY_MLP::inference(float* in, float* out, int size)
    def inference(self, d_in, d_out=None, size=None, stream=None):
        import torch
        n = d_in.shape[0] if size is None else size
        if d_out is None:
            d_out = torch.empty((n, self.output_ch), dtype=torch.float32, device=d_in.device)
        check(lib().hm_mlp_inference(self._h, _vp(d_in), _vp(d_out), n, _stream(stream)))
        return d_out

    def forward(self, d_in, stream=None):
        import torch
        n = d_in.shape[0]
        out = torch.empty((n, self.output_ch), dtype=torch.float32, device=d_in.device)
        check(lib().hm_mlp_forward(self._h, _vp(d_in), _vp(out), n, _stream(stream)))
        self._last_in = d_in
        return out

    def backward(self, d_target, stream=None):
        import torch
        loss = torch.zeros(1, dtype=torch.float32, device=d_target.device)
        check(lib().hm_mlp_backward(self._h, _vp(d_target), d_target.shape[0], _vp(loss), _stream(stream)))
        return loss

    def backward_output_grad(self, d_dy, stream=None):
        """Backward of the last forward with dL/d(output) given ([n, out_ch])."""
        check(lib().hm_mlp_backward_output_grad(self._h, _vp(d_dy), d_dy.shape[0], _stream(stream)))

    def optimizer_step(self, loss_scale=1.0, stream=None):
        check(lib().hm_mlp_optimizer_step(self._h, float(loss_scale), _stream(stream)))

    # trainer->training_step(input, target); trainer->loss(ctx)
    def training_step(self, d_in, d_target, stream=None, read_loss=False):
        import torch
        loss = torch.zeros(1, dtype=torch.float32, device=d_in.device)
        check(lib().hm_mlp_training_step(self._h, _vp(d_in), _vp(d_target), d_in.shape[0], _vp(loss),
                                         _stream(stream)))
        if read_loss:
            self.training_loss = float(loss.item())
        return loss

    def loss(self):
        v = ctypes.c_float(0)
        check(lib().hm_mlp_last_loss(self._h, ctypes.byref(v)))
        return v.value

    def reset(self):
        check(lib().hm_mlp_reset(self._h))

    def params(self):
        p = np.zeros(self.n_params, np.float32)
        check(lib().hm_mlp_get_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().hm_mlp_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    def gradients(self):
        g = np.zeros(self.n_params, np.float32)
        check(lib().hm_mlp_get_gradients(self._h, g.ctypes.data_as(ctypes.c_void_p)))
        return g

    def save(self, path):
        check(lib().hm_mlp_save(self._h, path.encode()))

    # TINY_MLP::loadWeights(path)
    def load_weights(self, path):
        check(lib().hm_mlp_load(self._h, path.encode()))
