"""Command line: the reference's `render_hair_msnn [scene.json] [BETA]`
(render_hair_msnn.cu:1146-1175) without the viewer.

  python -m hairmsnn_gb300 render [scene.json] [BETA] [--frames N] [--mode msnn|pt|nrc]
                                  [--width W --height H] [--out image.pfm] [--stats out.json]

  python -m hairmsnn_gb300 infer [--config c1_cache_w64.json] [--precision fp16]
                                 [--queries N] [--repeat R]

  python -m hairmsnn_gb300 diff [--width W --height H --strands N --groups G --frames F]

`infer` times cache-network inference on N synthetic hair-vertex queries
(16-D: position, angles, h, sigma_a, beta) and prints the time per call.

Without a scene file the built-in straight-hair scene is used.  Frames
accumulate in FP64; --out writes the average as OpenEXR (.exr: float
RGB, uncompressed, top row first as the reference's screenShotEXR) or as a
little-endian PFM (any other name: bottom row first, the renderer's own row
order).  --stats writes per-frame
timings (the reference's renderTime/trainTime/inferTime) and the cache loss
as JSON (the reference parses integrator.stats_output but never writes it).
"""
import argparse
import json
import os
import struct
import sys
import time

import numpy as np


def write_pfm(path, img):
    """img: [H, W, 3] float, row 0 = bottom (PFM stores bottom-to-top)."""
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(img, dtype="<f4").tobytes())


def read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        dt = "<f4" if scale < 0 else ">f4"
        return np.frombuffer(f.read(), dtype=dt).reshape(h, w, 3).astype(np.float32)


def _exr_attr(name, typ, payload):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(payload)) + payload


def write_exr(path, img):
    """img: [H, W, 3] float, row 0 = bottom (the renderer's order), written as
    an uncompressed single-part scanline OpenEXR file with FLOAT channels
    B, G, R (top row first), as the reference's screenShotEXR writes its
    accumulation buffer (model.cpp:366-383) minus the compression."""
    h, w, _ = img.shape
    top_first = np.ascontiguousarray(img[::-1], dtype="<f4")
    chans = b"".join(c.encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for c in "BGR") + b"\0"
    header = b"".join([
        _exr_attr("channels", "chlist", chans),
        _exr_attr("compression", "compression", b"\0"),
        _exr_attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1)),
        _exr_attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1)),
        _exr_attr("lineOrder", "lineOrder", b"\0"),
        _exr_attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)),
        _exr_attr("screenWindowCenter", "v2f", struct.pack("<2f", 0.0, 0.0)),
        _exr_attr("screenWindowWidth", "float", struct.pack("<f", 1.0)),
    ]) + b"\0"
    prefix = struct.pack("<ii", 20000630, 2) + header
    row_bytes = 8 + 3 * w * 4
    first = len(prefix) + 8 * h
    offsets = struct.pack(f"<{h}Q", *(first + y * row_bytes for y in range(h)))
    rows = []
    for y in range(h):
        line = top_first[y]
        rows.append(struct.pack("<ii", y, 3 * w * 4) + line[:, 2].tobytes() + line[:, 1].tobytes() +
                    line[:, 0].tobytes())
    with open(path, "wb") as f:
        f.write(prefix + offsets + b"".join(rows))


def read_exr(path):
    """Reads what write_exr writes (uncompressed FLOAT B, G, R scanlines);
    returns [H, W, 3] float32, row 0 = bottom."""
    data = open(path, "rb").read()
    magic, version = struct.unpack_from("<ii", data, 0)
    assert magic == 20000630 and (version & 0xFF) == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        name = data[pos:e].decode()
        e2 = data.index(b"\0", e + 1)
        size, = struct.unpack_from("<i", data, e2 + 1)
        attrs[name] = data[e2 + 5:e2 + 5 + size]
        pos = e2 + 5 + size
    pos += 1
    assert attrs["compression"] == b"\0"
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    names, c = [], 0
    ch = attrs["channels"]
    while ch[c] != 0:
        e = ch.index(b"\0", c)
        names.append(ch[c:e].decode())
        c = e + 1 + 16
    offsets = struct.unpack_from(f"<{h}Q", data, pos)
    img = np.zeros((h, w, 3), np.float32)
    for off in offsets:
        y, n = struct.unpack_from("<ii", data, off)
        vals = np.frombuffer(data, "<f4", n // 4, off + 8).reshape(len(names), w)
        for k, nm in enumerate(names):
            if nm in "RGB":
                img[y - y0, :, "RGB".index(nm)] = vals[k]
    return img[::-1].copy()


def diff(a):
    """Curly hair with strand groups (render.curly_hair_diff_scene): renders a
    target at the groups' materials, moves sigma_a 50% off, renders again
    (hm_render_diff_forward) and replays the paths (hm_render_diff_backward)
    for dL/d(material) of the L2 image loss; prints the gradient and times."""
    import numpy as np
    import torch
    from . import build, render
    build.build()
    cfg, mats = render.curly_hair_diff_scene(a.width, a.height, strands=a.strands,
                                             control_points=a.control_points, groups=a.groups)
    scene = render.Scene(cfg)
    scene.set_group_materials(mats)
    rd = render.Renderer(scene, render.MSNN, beta=a.beta, train=False)
    rd.diff_forward(a.frames)
    target = rd.device_sums(5).clone() / a.frames
    off = mats.copy()
    off[:, 0:3] *= 1.5
    scene.set_group_materials(off)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rd.diff_forward(a.frames)
    img = rd.device_sums(5) / a.frames
    adj = (2.0 / img.numel()) * (img - target)
    loss = float((adj * (img - target)).sum() / 2.0)
    t1 = time.perf_counter()
    g = rd.diff_backward(adj.float())
    t2 = time.perf_counter()
    print(json.dumps({"loss": loss, "forward_s": round(t1 - t0, 4), "backward_s": round(t2 - t1, 4),
                      "grad_sigma_a": np.round(g[:, 0:3], 8).tolist(),
                      "grad_beta_m_beta_n_alpha": np.round(g[:, 3:6], 8).tolist()}))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m hairmsnn_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("render")
    r.add_argument("scene", nargs="?", default=None)
    r.add_argument("beta", nargs="?", type=int, default=1)
    r.add_argument("--frames", type=int, default=None, help="default: integrator.spp")
    r.add_argument("--mode", choices=["msnn", "pt", "nrc"], default="msnn",
                   help="nrc: the reference's neural-radiance-caching comparison renderer (render_nrc.cu)")
    r.add_argument("--width", type=int, default=None)
    r.add_argument("--height", type=int, default=None)
    r.add_argument("--strands", type=int, default=None, help="built-in scene only")
    r.add_argument("--train-records", type=int, default=16384)
    r.add_argument("--out", default=None)
    r.add_argument("--stats", default=None)
    q = sub.add_parser("infer")
    q.add_argument("--config", default="c1_cache_w64.json")
    q.add_argument("--precision", choices=["fp32", "fp16", "bf16", "fp8"], default="fp16")
    q.add_argument("--queries", type=int, default=1 << 18)
    q.add_argument("--repeat", type=int, default=1)
    d = sub.add_parser("diff", help="one gradient of the differentiable appearance fit")
    d.add_argument("--width", type=int, default=256)
    d.add_argument("--height", type=int, default=256)
    d.add_argument("--strands", type=int, default=20000)
    d.add_argument("--control-points", type=int, default=96)
    d.add_argument("--groups", type=int, default=4)
    d.add_argument("--frames", type=int, default=64)
    d.add_argument("--beta", type=int, default=2)
    a = ap.parse_args(argv)
    if a.cmd == "infer":
        return infer(a)
    if a.cmd == "diff":
        return diff(a)

    from . import build, render
    build.build()
    if a.scene:
        cfg = json.load(open(a.scene))
        base = os.path.dirname(os.path.abspath(a.scene))
    else:
        cfg = render.straight_hair_scene(a.width or 512, a.height or 512,
                                         **({"strands": a.strands} if a.strands else {}))
        base = None
    if a.width:
        cfg.setdefault("integrator", {})["width"] = a.width
    if a.height:
        cfg.setdefault("integrator", {})["height"] = a.height
    scene = render.Scene(cfg, base)
    mode = {"msnn": render.MSNN, "pt": render.PT, "nrc": render.NRC}[a.mode]
    records = a.train_records if (a.mode != "nrc" or a.train_records != 16384) else 65536
    rd = render.Renderer(scene, mode, beta=a.beta, train_records=records,
                         train=cfg.get("tcnn", {}).get("init_train", True))
    rd.instrument(timing=True)
    frames = a.frames if a.frames is not None else scene.info().spp
    log = []
    t0 = time.perf_counter()
    for _ in range(frames):
        rd.frame()
        t = rd.timings().as_dict()
        t["loss"] = rd.stats().last_loss
        log.append(t)
    wall = time.perf_counter() - t0
    img = rd.read(render.IMAGE_FINAL)
    out = a.out or cfg.get("integrator", {}).get("image_output") or None
    if out:
        if out.endswith(".exr"):
            write_exr(out, img)
        else:
            if not out.endswith(".pfm"):
                out = os.path.splitext(out)[0] + ".pfm"
            write_pfm(out, img)
    summary = {"frames": frames, "wall_s": wall, "paths_per_s": frames * img.shape[0] * img.shape[1] / wall,
               "mean_radiance": float(img.mean())}
    print(json.dumps(summary))
    stats_path = a.stats or cfg.get("integrator", {}).get("stats_output") or None
    if stats_path:
        json.dump({"summary": summary, "frames": log}, open(stats_path, "w"), indent=1)
    return 0


def vertex_queries(n, seed=0):
    """Synthetic 16-D cache inputs of hair vertices: position in [-1,1]^3,
    four angles in [0,1], h in [-1,1], sigma_a (0.06, 0.1, 0.2), beta 0.3."""
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 16), np.float32)
    x[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    x[:, 3:7] = rng.uniform(0, 1, (n, 4))
    x[:, 7] = rng.uniform(-1, 1, n)
    x[:, 8:11] = [0.06, 0.1, 0.2]
    x[:, 11:13] = 0.3
    return x


def infer(a):
    import torch
    from . import build, mlp
    build.build()
    d = mlp.describe(a.config, 16, 3)
    net = mlp.TinyMLP(a.config, 16, 3, precision=a.precision, seed=0)
    x = torch.from_numpy(vertex_queries(a.queries)).cuda()
    y = torch.empty((a.queries, 3), device="cuda")
    net.inference(x, y)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(a.repeat):
        net.inference(x, y)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / a.repeat
    print(json.dumps({"config": a.config, "precision": a.precision, "width": d.width, "queries": a.queries,
                      "ms": round(ms, 4), "queries_per_s": round(a.queries / (ms * 1e-3), 1),
                      "mean_abs_out": float(y.abs().mean())}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
