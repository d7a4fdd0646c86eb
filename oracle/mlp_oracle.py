"""FP64 ORACLE of the radiance-cache network (test infrastructure only).

Restates tiny-cuda-nn's documented semantics for the configuration the
reference feeds it (scenes/*/tcnn_hairmsnn.json, called from
cuda/neural_network.cu:34-64 and render_hair_msnn.cu:683-691).  tiny-cuda-nn
is an empty submodule in the reference checkout, so this restatement is
parity-UNPINNED against tiny-cuda-nn itself; it pins the GPU kernels to the
written semantics:

* Composite encoding, inputs consumed in order; encoded width padded to a
  multiple of 16 with ones.
* Frequency: feature (d, f, s) = sin(2^f * pi * x_d + s * pi/2), s in {0,1}.
* OneBlob: n_bins quartic-kernel blobs of radius one bin, periodic on [0,1):
  bin b = C(b+1) - C(b), C(b) = sum_{k=-1,0,1} Q((b/B - x + k) * B),
  Q(u) = clamp(u (15 - 10u^2 + 3u^4)/16 + 1/2, 0, 1), C(B) := C(0) + 1.
* HashGrid (Mueller et al. 2022): level scale = base * s^l - 1, resolution
  ceil(scale)+1, table size min(2^T, dense rounded up to 8), dense index
  while it fits, else the (1, 2654435761, 805459861) xor hash; trilinear.
* FullyFusedMLP: ReLU hidden layers, linear output padded to 16, no biases,
  weights row-major [out][in]; network params then encoding params.
* Losses averaged over n * out_ch; RelativeL2Luminance uses the
  prediction's luminance (0.299, 0.587, 0.114) as a constant denominator.
* Adam: l2 on network weights only, encoding params with zero gradient
  untouched; bias correction folded into the step size; ExponentialDecay.
"""
import json
import math

import numpy as np

PI = np.float32(3.1415926)


def pad16(x):
    return (x + 15) // 16 * 16


class Config:
    def __init__(self, cfg, in_ch, out_ch):
        if isinstance(cfg, str):
            cfg = json.loads(cfg)
        self.in_ch, self.out_ch = in_ch, out_ch
        self.loss = cfg.get("loss", {}).get("otype", "L2")
        opt = cfg.get("optimizer", {})
        self.decay = None
        if opt.get("otype") == "ExponentialDecay":
            self.decay = (opt.get("decay_start", 10000), opt.get("decay_interval", 10000),
                          opt.get("decay_base", 0.33))
            opt = opt["nested"]
        self.lr = opt.get("learning_rate", 1e-3)
        self.beta1 = opt.get("beta1", 0.9)
        self.beta2 = opt.get("beta2", 0.999)
        self.eps = opt.get("epsilon", 1e-8)
        self.l2 = opt.get("l2_reg", 1e-8)
        enc = cfg.get("encoding", {"otype": "Identity"})
        parts = enc["nested"] if enc.get("otype") == "Composite" else [enc]
        self.segs = []
        in_off = out_off = 0
        enc_params = 0
        for e in parts:
            t = e.get("otype", "Identity")
            nd = e.get("n_dims_to_encode", in_ch - in_off)
            if nd == 0:
                continue
            s = dict(type=t, in_off=in_off, n_dims=nd, out_off=out_off)
            if t == "Identity":
                s["n_out"] = nd
            elif t == "Frequency":
                s["n_freq"] = e.get("n_frequencies", 12)
                s["n_out"] = nd * s["n_freq"] * 2
            elif t == "OneBlob":
                s["n_bins"] = e.get("n_bins", 16)
                s["n_out"] = nd * s["n_bins"]
            elif t in ("HashGrid", "Grid"):
                L = e.get("n_levels", 16)
                F = e.get("n_features_per_level", 2)
                T = 1 << e.get("log2_hashmap_size", 19)
                base = e.get("base_resolution", 16)
                l2s = np.float32(math.log2(e.get("per_level_scale", 2.0)))
                levels = []
                off = 0
                for l in range(L):
                    scale = np.float32(np.exp2(np.float32(l) * l2s) * np.float32(base) - np.float32(1))
                    res = int(np.ceil(scale)) + 1
                    size = min(T, (res ** 3 + 7) // 8 * 8)
                    levels.append((scale, res, size, off))
                    off += size
                s.update(n_levels=L, n_feat=F, levels=levels, param_off=enc_params, n_out=L * F)
                enc_params += off * F
            else:
                raise ValueError(t)
            in_off += nd
            out_off += s["n_out"]
            self.segs.append(s)
        self.n_enc = out_off
        self.in_pad = pad16(out_off)
        self.n_enc_params = enc_params
        net = cfg.get("network", {})
        self.width = net.get("n_neurons", 64)
        self.n_hidden = net.get("n_hidden_layers", 2)
        self.out_pad = 16
        self.layer_shapes = []
        off = 0
        for l in range(self.n_hidden + 1):
            fi = self.in_pad if l == 0 else self.width
            fo = self.out_pad if l == self.n_hidden else self.width
            self.layer_shapes.append((off, fo, fi))
            off += fo * fi
        self.n_net_params = off
        self.n_params = off + enc_params


def quartic_cdf(u, inv_r):
    u = u * inv_r
    u2 = u * u
    return np.clip(u * (15.0 - 10.0 * u2 + 3.0 * u2 * u2) / 16.0 + 0.5, 0.0, 1.0)


def grid_index(res, size, x, y, z):
    """x, y, z: uint64 arrays of (uint32-wrapped) grid coordinates."""
    m = np.uint64(0xFFFFFFFF)
    stride = 1
    index = np.zeros_like(x)
    coords = [x, y, z]
    for c in coords:
        if stride > size:
            break
        index = (index + c * np.uint64(stride)) & m
        stride *= res
    if size < stride:
        index = ((x * np.uint64(1)) & m) ^ ((y * np.uint64(2654435761)) & m) ^ \
            ((z * np.uint64(805459861)) & m)
    return index % np.uint64(size)


def _grid_corners(s, lvl, p):
    scale, res, size, off = s["levels"][lvl]
    # fmaf(scale, x, 0.5): the FP64 product of two floats is exact, one rounding
    f = (p.astype(np.float64) * float(scale) + 0.5).astype(np.float32)
    g = np.floor(f)
    w = (f - g).astype(np.float64)
    gi = g.astype(np.int64).astype(np.uint64) & np.uint64(0xFFFFFFFF)
    corners = []
    for c in range(8):
        b = [(c >> k) & 1 for k in range(3)]
        idx = grid_index(res, size, (gi[:, 0] + np.uint64(b[0])) & np.uint64(0xFFFFFFFF),
                         (gi[:, 1] + np.uint64(b[1])) & np.uint64(0xFFFFFFFF),
                         (gi[:, 2] + np.uint64(b[2])) & np.uint64(0xFFFFFFFF))
        wt = np.ones(len(p))
        for k in range(3):
            wt = wt * (w[:, k] if b[k] else 1.0 - w[:, k])
        corners.append((idx.astype(np.int64) + off, wt))
    return corners


def encode(cfg, params, x, exact_phase=False):
    """x [n, in_ch] -> X [n, in_pad] float64.

    exact_phase: Frequency features as sin / cos of pi * (2^f x) evaluated
    in float64 without the FP32 rounding of the phase (the tensor-core
    kernels' sincospif form); default: the FP32 encode kernel's form."""
    x = np.asarray(x, np.float32)
    n = x.shape[0]
    X = np.ones((n, cfg.in_pad))
    enc = params[cfg.n_net_params:]
    for s in cfg.segs:
        xi = x[:, s["in_off"]:s["in_off"] + s["n_dims"]].astype(np.float64)
        o = s["out_off"]
        if s["type"] == "Identity":
            X[:, o:o + s["n_dims"]] = xi
        elif s["type"] == "Frequency":
            F = s["n_freq"]
            xs = x[:, s["in_off"]:s["in_off"] + s["n_dims"]]
            for d in range(s["n_dims"]):
                for f in range(F):
                    if exact_phase:
                        y = xs[:, d].astype(np.float64) * 2.0 ** f
                        X[:, o + (d * F + f) * 2] = np.sin(np.pi * np.mod(y, 2.0))
                        X[:, o + (d * F + f) * 2 + 1] = np.cos(np.pi * np.mod(y, 2.0))
                        continue
                    # the phase is formed in FP32 exactly as the kernel does;
                    # only the sine itself is evaluated in FP64
                    a = (xs[:, d] * np.float32(2.0 ** f)).astype(np.float32) * PI
                    a2 = a + np.float32(0.5) * PI
                    X[:, o + (d * F + f) * 2] = np.sin(a.astype(np.float64))
                    X[:, o + (d * F + f) * 2 + 1] = np.sin(a2.astype(np.float64))
        elif s["type"] == "OneBlob":
            B = s["n_bins"]
            for d in range(s["n_dims"]):
                xd = xi[:, d]
                C = lambda b: sum(quartic_cdf(b / B - xd + k, B) for k in (-1.0, 0.0, 1.0))
                c0 = C(0.0)
                for b in range(B):
                    right = c0 + 1.0 if b == B - 1 else C(b + 1.0)
                    X[:, o + d * B + b] = right - C(float(b)) if b > 0 else right - c0
        else:
            table = enc[s["param_off"]:].reshape(-1, s["n_feat"])
            p = x[:, s["in_off"]:s["in_off"] + 3]
            for l in range(s["n_levels"]):
                acc = np.zeros((n, s["n_feat"]))
                for idx, wt in _grid_corners(s, l, p):
                    acc += wt[:, None] * table[idx]
                X[:, o + l * s["n_feat"]:o + (l + 1) * s["n_feat"]] = acc
    return X


def weights(cfg, params):
    return [params[off:off + fo * fi].reshape(fo, fi).astype(np.float64)
            for off, fo, fi in cfg.layer_shapes]


def forward(cfg, params, x):
    params = np.asarray(params, np.float64)
    X = encode(cfg, params, x)
    Ws = weights(cfg, params)
    hs = [X]
    h = X
    for l in range(cfg.n_hidden):
        h = np.maximum(h @ Ws[l].T, 0.0)
        hs.append(h)
    out = h @ Ws[-1].T
    return out, hs


def loss_and_grad(cfg, out, target):
    n = out.shape[0]
    oc = cfg.out_ch
    pred = out[:, :oc]
    diff = pred - target
    if cfg.loss == "L2":
        den = np.ones_like(pred)
    elif cfg.loss == "RelativeL2":
        den = pred * pred + 0.01
    else:
        lum = 0.299 * pred[:, 0] + 0.587 * pred[:, 1] + 0.114 * pred[:, 2]
        den = np.repeat((lum * lum + 0.01)[:, None], oc, axis=1)
    total = n * oc
    loss = np.sum(diff * diff / den) / total
    g = np.zeros_like(out)
    g[:, :oc] = 2.0 * diff / den / total
    return loss, g


def backward(cfg, params, x, target):
    """Returns loss, grads [n_params] (FP64)."""
    params = np.asarray(params, np.float64)
    out, hs = forward(cfg, params, x)
    loss, g = loss_and_grad(cfg, out, np.asarray(target, np.float64))
    return loss, _backprop(cfg, params, x, hs, g)


def backward_output_grad(cfg, params, x, dy):
    """Parameter gradients for a given dL/d(output) [n, out_ch] (tcnn's
    backward with dL_doutput; no loss)."""
    params = np.asarray(params, np.float64)
    out, hs = forward(cfg, params, x)
    g = np.zeros_like(out)
    g[:, :cfg.out_ch] = np.asarray(dy, np.float64)
    return _backprop(cfg, params, x, hs, g)


def _backprop(cfg, params, x, hs, g):
    Ws = weights(cfg, params)
    grads = np.zeros(cfg.n_params)
    dz = g
    for l in range(cfg.n_hidden, -1, -1):
        off, fo, fi = cfg.layer_shapes[l]
        grads[off:off + fo * fi] = (dz.T @ hs[l]).ravel()
        dh = dz @ Ws[l]
        if l > 0:
            dz = dh * (hs[l] > 0)
        else:
            dX = dh
    enc_grads = grads[cfg.n_net_params:]
    xf = np.asarray(x, np.float32)
    for s in cfg.segs:
        if s["type"] not in ("HashGrid", "Grid"):
            continue
        F = s["n_feat"]
        tg = enc_grads[s["param_off"]:].reshape(-1, F)
        p = xf[:, s["in_off"]:s["in_off"] + 3]
        for l in range(s["n_levels"]):
            gcol = dX[:, s["out_off"] + l * F:s["out_off"] + (l + 1) * F]
            for idx, wt in _grid_corners(s, l, p):
                np.add.at(tg, idx, wt[:, None] * gcol)
    return grads


class Adam:
    """tcnn Adam + ExponentialDecay, FP64 state."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.m = np.zeros(cfg.n_params)
        self.v = np.zeros(cfg.n_params)
        self.step = 0
        self.lr = cfg.lr

    def update(self, params, grads, loss_scale=1.0):
        c = self.cfg
        if c.decay and self.step >= c.decay[0] and (self.step - c.decay[0]) % c.decay[1] == 0:
            self.lr *= c.decay[2]
        self.step += 1
        lr_t = self.lr * math.sqrt(1 - c.beta2 ** self.step) / (1 - c.beta1 ** self.step)
        p = np.asarray(params, np.float64).copy()
        g = np.asarray(grads, np.float64) / loss_scale
        nm = c.n_net_params
        g[:nm] += c.l2 * p[:nm]
        upd = np.ones(c.n_params, bool)
        upd[nm:] = g[nm:] != 0
        self.m[upd] = c.beta1 * self.m[upd] + (1 - c.beta1) * g[upd]
        self.v[upd] = c.beta2 * self.v[upd] + (1 - c.beta2) * g[upd] ** 2
        p[upd] -= lr_t / (np.sqrt(self.v[upd]) + c.eps) * self.m[upd]
        return p
