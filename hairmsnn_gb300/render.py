"""Scene, renderer and ray-tracing front end over the C ABI.

Mirrors the reference's frame driver (RenderWindow_HairMSNN, render_hair_msnn.cu)
minus the viewer: a Scene is built from the reference's scene JSON (plus the
procedural-asset keys), a Renderer runs HairMSNN (or plain path tracing) one
sample per pixel per frame() and accumulates in FP64.
"""
import ctypes
import json
import os
import time

import numpy as np

from ._ffi import check, lib

HM_SCENE = dict(control_points=0, segments=1, vertices=2, normals=3, triangles=4, env=5, env_cpdf=6,
                env_ccdf=7, env_mpdf=8, env_mcdf=9, dir_lights=10, bvh_nodes=11, bvh_leaves=12, camera=13,
                materials=14, bvh_wide_nodes=15, strand_groups=16, group_materials=17, segment_groups=18)
DTYPES = dict(control_points=(np.float32, 4), segments=(np.int32, 1), vertices=(np.float32, 3),
              normals=(np.float32, 3), triangles=(np.int32, 3), env=(np.float32, 4), env_cpdf=(np.float32, 1),
              env_ccdf=(np.float32, 1), env_mpdf=(np.float32, 1), env_mcdf=(np.float32, 1),
              dir_lights=(np.float32, 6), bvh_nodes=(np.float32, 16), bvh_leaves=(np.int32, 1),
              camera=(np.float32, 12), materials=(np.float32, 16), bvh_wide_nodes=(np.float32, 56),
              strand_groups=(np.int32, 1), group_materials=(np.float32, 10), segment_groups=(np.int32, 1))
PT, MSNN, NRC = 0, 1, 2
IMAGE_FINAL, IMAGE_SHORT, IMAGE_CACHE = 0, 1, 2


class hm_scene_desc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "n_strands", "n_control_points", "n_segments", "n_vertices", "n_triangles", "n_bvh_nodes", "width",
        "height", "spp", "path_v1", "path_v2", "env_width", "env_height", "n_dir_lights", "mis", "env_pdf",
        "has_env", "shading_catrom")] + [("scene_scale", ctypes.c_float), ("bounds_min", ctypes.c_float * 3),
                       ("bounds_max", ctypes.c_float * 3), ("n_bvh_wide_nodes", ctypes.c_int),
                       ("n_groups", ctypes.c_int), ("segment_splits", ctypes.c_int)]


class hm_render_options(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("beta", ctypes.c_int), ("train_records", ctypes.c_int),
                ("train", ctypes.c_int), ("cache_precision", ctypes.c_int), ("seed", ctypes.c_uint32),
                ("cache_config_json", ctypes.c_char_p), ("frames_in_flight", ctypes.c_int),
                ("nrc_c", ctypes.c_float)]


class hm_render_tuning(ctypes.Structure):
    _fields_ = [("extend_blocks_per_sm", ctypes.c_int), ("shadow_blocks_per_sm", ctypes.c_int),
                ("shade_blocks_per_sm", ctypes.c_int), ("ms_per_frame", ctypes.c_float)]


class hm_render_stats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_int), ("pixels", ctypes.c_int), ("extension_rays", ctypes.c_int64),
                ("last_bounces", ctypes.c_int), ("train_records", ctypes.c_int), ("every_nth", ctypes.c_int),
                ("last_loss", ctypes.c_float)]


class hm_render_timings(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in (
        "total_ms", "camera_ms", "extend_ms", "shade_ms", "shadow_ms", "compact_ms", "finalize_ms", "train_ms",
        "infer_ms", "compose_ms")] + [("bounces", ctypes.c_int), ("kernel_launches", ctypes.c_int)] + [
        (n, ctypes.c_int64) for n in ("extension_rays", "shadow_rays", "extend_nodes", "extend_prims",
                                      "shadow_nodes", "shadow_prims")] + [
        ("paths_by_bounce", ctypes.c_int * 48), ("extend_ms_by_bounce", ctypes.c_float * 48),
        ("shadow_ms_by_bounce", ctypes.c_float * 48)]

    def as_dict(self):
        out = {}
        for k, _ in self._fields_:
            v = getattr(self, k)
            out[k] = list(v)[:max(1, self.bounces)] if k.endswith("_by_bounce") else v
        return out


_declared = False


def _declare():
    global _declared
    if _declared:
        return
    L = lib()
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    P = ctypes.POINTER
    L.hm_scene_create.restype = vp
    L.hm_scene_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P(i32)]
    L.hm_scene_build.argtypes = [vp]
    L.hm_scene_destroy.restype = None
    L.hm_scene_destroy.argtypes = [vp]
    L.hm_scene_info.argtypes = [vp, P(hm_scene_desc)]
    L.hm_scene_export_size.restype = i64
    L.hm_scene_export_size.argtypes = [vp, i32]
    L.hm_scene_export.argtypes = [vp, i32, vp, i64]
    L.hm_trace_rays.argtypes = [vp, vp, vp, i64, ctypes.c_float, ctypes.c_float, i32, vp, vp]
    L.hm_render_create.restype = vp
    L.hm_render_create.argtypes = [vp, P(hm_render_options), P(i32)]
    L.hm_render_destroy.restype = None
    L.hm_render_destroy.argtypes = [vp]
    L.hm_render_frame.argtypes = [vp, vp]
    L.hm_render_wait.argtypes = [vp, vp]
    L.hm_render_frames_in_flight.argtypes = [vp]
    L.hm_render_pretrain.argtypes = [vp, i32, vp]
    L.hm_render_create_batch.restype = vp
    L.hm_render_create_batch.argtypes = [P(vp), P(i32), i32, P(hm_render_options), P(i32)]
    L.hm_render_batch_scene.argtypes = [vp, i32, P(i32), P(i32), P(i32)]
    L.hm_render_autotune.argtypes = [vp, i32, vp, P(hm_render_tuning)]
    L.hm_render_read_async.argtypes = [vp, i32, vp, vp]
    L.hm_render_reset.argtypes = [vp]
    L.hm_render_read.argtypes = [vp, i32, vp]
    L.hm_render_get_stats.argtypes = [vp, P(hm_render_stats)]
    L.hm_render_cache.restype = vp
    L.hm_render_cache.argtypes = [vp]
    L.hm_render_buffer.argtypes = [vp, i32, P(vp), P(i64)]
    L.hm_copy_to_host.argtypes = [vp, vp, i64]
    L.hm_render_set_instrumentation.argtypes = [vp, i32, i32]
    L.hm_render_set_path_log.argtypes = [vp, i32]
    L.hm_render_read_path_log.argtypes = [vp, vp, i64]
    L.hm_render_get_timings.argtypes = [vp, P(hm_render_timings)]
    L.hm_scene_set_strand_groups.argtypes = [vp, P(i32), i32, i32]
    L.hm_scene_set_group_materials.argtypes = [vp, vp, i32]
    L.hm_render_diff_forward.argtypes = [vp, i32, vp, i32, vp]
    L.hm_render_set_graphs.argtypes = [vp, i32]
    L.hm_render_diff_backward.argtypes = [vp, vp, P(ctypes.c_double), i32, vp]
    _declared = True


def _stream(stream):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


class Scene:
    """parseScene + asset generation (host); device build on first use."""

    def __init__(self, config, base_dir=None):
        _declare()
        text = json.dumps(config) if isinstance(config, dict) else config
        st = ctypes.c_int(0)
        h = lib().hm_scene_create(text.encode(), (base_dir or "").encode(), ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)
        self.config = config

    def close(self):
        if getattr(self, "_h", None):
            lib().hm_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self):
        check(lib().hm_scene_build(self._h))

    def info(self):
        d = hm_scene_desc()
        check(lib().hm_scene_info(self._h, ctypes.byref(d)))
        return d

    def export(self, name):
        which = HM_SCENE[name]
        nbytes = lib().hm_scene_export_size(self._h, which)
        dt, width = DTYPES[name]
        out = np.zeros(max(nbytes, 0) // np.dtype(dt).itemsize, dt)
        if nbytes > 0:
            check(lib().hm_scene_export(self._h, which, out.ctypes.data_as(ctypes.c_void_p), nbytes))
        return out.reshape(-1, width) if width > 1 else out

    def set_strand_groups(self, groups, n_groups):
        """Group of every strand (int array [n_strands]); see hm_scene_set_strand_groups."""
        g = np.ascontiguousarray(groups, np.int32)
        check(lib().hm_scene_set_strand_groups(self._h, g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(g),
                                               int(n_groups)))

    def set_group_materials(self, materials):
        """materials [n_groups, 10]: sigma_a rgb, beta_m, beta_n, alpha (rad), gains R, TT, TRT, TRRT."""
        arr = hair_params_array(materials)
        check(lib().hm_scene_set_group_materials(self._h, arr, len(arr)))

    def group_materials(self):
        """[n_groups, 10] (the scene's material alone when it has no groups)."""
        m = self.export("group_materials")
        if len(m):
            return m
        x = self.export("materials")[0]
        return x[:10].reshape(1, 10).copy()

    def trace(self, org, dirs, tmin=0.0, tmax=1e30, any_hit=False, stream=None):
        """org, dirs: CUDA float32 [n, 3] -> hits [n, 4] (t, prim bits, u, v)."""
        import torch
        n = org.shape[0]
        hits = torch.empty((n, 4), dtype=torch.float32, device=org.device)
        check(lib().hm_trace_rays(self._h, ctypes.c_void_p(org.data_ptr()), ctypes.c_void_p(dirs.data_ptr()), n,
                                  tmin, tmax, 1 if any_hit else 0, ctypes.c_void_p(hits.data_ptr()),
                                  _stream(stream)))
        return hits


def hair_params_array(materials):
    """ctypes array of hm_hair_params from rows of 10 floats."""
    from ._ffi import hm_hair_params
    m = np.asarray(materials, np.float64).reshape(-1, 10)
    arr = (hm_hair_params * len(m))()
    for i, row in enumerate(m):
        arr[i] = hm_hair_params.from_array(row)
    return arr


class Renderer:
    """One frame() = one sample per pixel of HairMSNN (mode=MSNN) or plain PT."""

    def __init__(self, scene, mode=MSNN, beta=1, train_records=16384, train=True, precision=0, seed=0,
                 cache_config=None, frames_in_flight=0, nrc_c=0.0):
        _declare()
        self.scene = scene
        if mode == NRC and train_records == 16384:
            train_records = 65536  # the NRC renderer's numTrainingRecords
        o = hm_render_options(mode, beta, train_records, 1 if train else 0, precision, seed,
                              cache_config.encode() if cache_config else None, frames_in_flight, nrc_c)
        st = ctypes.c_int(0)
        h = lib().hm_render_create(scene._h, ctypes.byref(o), ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)
        info = scene.info()
        self.width, self.height = info.width, info.height
        self.mode = mode

    def close(self):
        if getattr(self, "_h", None):
            lib().hm_render_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def frame(self, stream=None):
        """Enqueue one frame (asynchronous; see hm_render_frame)."""
        check(lib().hm_render_frame(self._h, _stream(stream)))

    def autotune(self, frames=4, stream=None):
        """Pick the fastest launch shapes (see hm_render_autotune); returns them."""
        t = hm_render_tuning()
        check(lib().hm_render_autotune(self._h, int(frames), _stream(stream), ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def pretrain(self, passes, stream=None):
        """Scene-sample training of the cache (see hm_render_pretrain)."""
        check(lib().hm_render_pretrain(self._h, int(passes), _stream(stream)))

    def set_graphs(self, on=True):
        """Replay each frame's path tracing as a CUDA graph (default) or launch
        its kernels one by one (see hm_render_set_graphs)."""
        check(lib().hm_render_set_graphs(self._h, 1 if on else 0))

    def depth(self):
        """Frames in flight (hm_render_options.frames_in_flight as resolved)."""
        return int(lib().hm_render_frames_in_flight(self._h))

    def wait(self, stream=None):
        """Make `stream` (default: torch's current stream) wait for all frames in flight."""
        check(lib().hm_render_wait(self._h, _stream(stream)))

    def reset(self):
        check(lib().hm_render_reset(self._h))

    def read(self, which=IMAGE_FINAL):
        img = np.zeros((self.height, self.width, 3), np.float64)
        check(lib().hm_render_read(self._h, which, img.ctypes.data_as(ctypes.c_void_p)))
        return img

    def read_async(self, host_sums, which=IMAGE_FINAL, stream=None):
        """Enqueue a copy of the FP64 running sums (not averaged) of every frame
        enqueued so far into `host_sums` (a pinned float64 torch tensor or numpy
        array of [H, W, 3]) on `stream`; see hm_render_read_async."""
        ptr = host_sums.data_ptr() if hasattr(host_sums, "data_ptr") else host_sums.ctypes.data
        check(lib().hm_render_read_async(self._h, which, ctypes.c_void_p(ptr), _stream(stream)))

    def stats(self):
        s = hm_render_stats()
        check(lib().hm_render_get_stats(self._h, ctypes.byref(s)))
        return s

    def instrument(self, timing=True, counting=False):
        check(lib().hm_render_set_instrumentation(self._h, 1 if timing else 0, 1 if counting else 0))

    def set_path_log(self, vertices):
        """Record every path's rays at its first `vertices` vertices in later
        frames (0: off); see hm_render_set_path_log."""
        self._log_slots = 3 * int(vertices)
        check(lib().hm_render_set_path_log(self._h, int(vertices)))

    def read_path_log(self):
        """The last frame's per-path ray log: [P, 3 * vertices, 12] float32
        (see hm_render_set_path_log for the layout)."""
        P = self.width * self.height
        out = np.zeros((P, self._log_slots, 12), np.float32)
        check(lib().hm_render_read_path_log(self._h, out.ctypes.data_as(ctypes.c_void_p), out.size))
        return out

    def timings(self):
        t = hm_render_timings()
        check(lib().hm_render_get_timings(self._h, ctypes.byref(t)))
        return t

    def diff_forward(self, frames, eval_materials=None, stream=None):
        """Differentiable forward: `frames` frames with the cache frozen (see
        hm_render_diff_forward); eval_materials [n_groups, 10] makes it a
        detached render.  The image is read() afterwards."""
        arr, n = (hair_params_array(eval_materials), 0) if eval_materials is not None else (None, 0)
        if arr is not None:
            n = len(arr)
        check(lib().hm_render_diff_forward(self._h, int(frames), arr, n, _stream(stream)))

    def diff_backward(self, adjoint, stream=None):
        """Path replay for dL/dImage `adjoint` (CUDA float32 [H, W, 3]):
        returns dL/d(material) [n_groups, 6] (sigma_a rgb, beta_m, beta_n,
        alpha); the cache's gradients hold dL/dW afterwards."""
        a = adjoint.contiguous()
        assert a.dtype.is_floating_point and a.element_size() == 4 and a.is_cuda
        n = 6 * 64
        out = (ctypes.c_double * n)()
        check(lib().hm_render_diff_backward(self._h, ctypes.c_void_p(a.data_ptr()), out, n, _stream(stream)))
        g = max(1, self.scene.info().n_groups)
        return np.array(out[:6 * g], np.float64).reshape(g, 6)

    def cache(self):
        """The render's cache network as a TinyMLP view (not owned)."""
        from .mlp import TinyMLP
        return TinyMLP.wrap(lib().hm_render_cache(self._h))

    def device_sums(self, which=5):
        """Zero-copy torch view ([H, W, 3] float64, on the device) of the FP64
        running sums: 5 final image, 6 short paths, 7 cache (divide by the
        frame count; valid while the renderer lives)."""
        import torch
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        check(lib().hm_render_buffer(self._h, which, ctypes.byref(p), ctypes.byref(n)))

        class _Dev:
            __cuda_array_interface__ = {"shape": (self.height, self.width, 3), "typestr": "<f8",
                                        "data": (p.value, False), "version": 2, "strides": None}
        return torch.as_tensor(_Dev(), device="cuda")

    def buffer(self, which):
        """Host copy of a device buffer of the last frame (see hm_render_buffer):
        0 cache inputs [P,12], 1 cache outputs [P,3], 2 training inputs [R,12],
        3 training targets [R,3], 4 G-buffer [P,4]."""
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        check(lib().hm_render_buffer(self._h, which, ctypes.byref(p), ctypes.byref(n)))
        in_ch = 9 if self.mode == NRC else 12
        width = {0: in_ch, 1: 3, 2: in_ch, 3: 3, 4: 4, 8: 4, 9: 20, 10: 4}[which]
        count = n.value * (4 if which in (4, 8, 9, 10) else 1)
        host = np.zeros(count, np.int32 if which == 10 else np.float32)
        check(lib().hm_copy_to_host(host.ctypes.data_as(ctypes.c_void_p), p, count * 4))
        return host.reshape(-1, width)


class BatchRenderer(Renderer):
    """Many scenes rendered as one (hm_render_create_batch): one frame() takes
    one sample per pixel of every scene; one cache network serves them all.
    read_scene(k) returns scene k's image."""

    def __init__(self, scenes, mode=MSNN, betas=None, train_records=16384, train=True, precision=0, seed=0,
                 cache_config=None, frames_in_flight=0):
        _declare()
        self.scenes = list(scenes)
        n = len(self.scenes)
        o = hm_render_options(mode, int(betas[0]) if betas is not None else 1, train_records, 1 if train else 0,
                              precision, seed, cache_config.encode() if cache_config else None, frames_in_flight)
        arr = (ctypes.c_void_p * n)(*[sc._h.value for sc in self.scenes])
        b = (ctypes.c_int * n)(*[int(x) for x in betas]) if betas is not None else None
        st = ctypes.c_int(0)
        h = lib().hm_render_create_batch(arr, b, n, ctypes.byref(o), ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)
        self.mode = mode
        self.layout = []
        for k in range(n):
            off, w, hh = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            check(lib().hm_render_batch_scene(self._h, k, ctypes.byref(off), ctypes.byref(w), ctypes.byref(hh)))
            self.layout.append((off.value, w.value, hh.value))
        self.pixels = sum(w * hh for _, w, hh in self.layout)
        self.width, self.height = self.pixels, 1

    def read(self, which=IMAGE_FINAL):
        img = np.zeros((self.pixels, 3), np.float64)
        check(lib().hm_render_read(self._h, which, img.ctypes.data_as(ctypes.c_void_p)))
        return img

    def read_scene(self, k, which=IMAGE_FINAL):
        off, w, h = self.layout[k]
        return self.read(which)[off:off + w * h].reshape(h, w, 3)


def relmse(img, ref, eps=1e-2):
    """mean((x - ref)^2 / (ref^2 + eps)) over pixels and channels."""
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


# ----------------------------------------------------------------- workloads
def straight_hair_scene(width=512, height=512, strands=10000, control_points=64, spp=16, path_v2=40,
                        seed=1, sky_w=512, sky_h=256, triangles=20000):
    """The full-render workload: straight procedural hair (10k strands x 64
    cubic B-spline control points, 20 cm long, radius 0.04 mm, roots on a
    unit-sphere cap; scene unit = 10 cm), a 20k-triangle head ellipsoid, a
    Preetham sky (turbidity 3) and a directional light from (3,3,3)."""
    return {
        "camera": {"from": [0.0, -3.8, 0.1], "to": [0.0, 0.0, -0.25], "up": [0.0, 0.0, 1.0], "cos_fovy": 0.66},
        "hair": {"alpha": 2.0, "beta_m": 0.3, "beta_n": 0.3, "type": 1, "sigma_a": [0.06, 0.1, 0.2],
                 "procedural": {"type": "straight", "strands": strands, "control_points": control_points,
                                "length": 2.0, "radius": 4e-4, "seed": seed}},
        "surface": {"procedural": {"type": "ellipsoid", "triangles": triangles, "radii": [0.85, 0.95, 1.0],
                                   "diffuse": [0.35, 0.25, 0.2]}},
        "lights": {"sky": {"turbidity": 3.0, "sun": [3, 3, 3], "width": sky_w, "height": sky_h, "scale": 1.0},
                   "directional": [{"from": [3, 3, 3], "emit": [1, 1, 1]}]},
        "integrator": {"ENV_PDF": True, "MIS": True, "width": width, "height": height, "spp": spp,
                       "path_v1": 1, "path_v2": path_v2},
        "tcnn": {"init_train": True},
    }


RAY_RECORD_BYTES = 32 + 16   # ray (origin, direction as float4 pairs) + hit record
NODE_BYTES = 224              # one 8-wide BVH node: eight child boxes + child codes
PRIM_BYTES = 64               # one segment's 4 control points (or a triangle's vertex data)
# DRAM bytes per extension ray of the extension traversal kernel (8-wide
# BVH), from ncu (dram__bytes_read.sum + dram__bytes_write.sum) of the first
# launch of a 256x256 frame of this scene: 42.1 MB for its 65,536 camera
# rays.  ncu runs each launch with cold caches, so this is an upper bound
# for warm frames.
EXTEND_DRAM_BYTES_PER_RAY = 643


class RenderBenchWorkload:
    """bench.py workload: one frame (1 spp) of the full HairMSNN render per
    step, in the chosen form: FP16 cache network on the tensor cores
    (training and inference), frames in flight, graph replay, autotuned
    launch shapes, two BVH leaves per segment."""

    name = "render"
    metric = "paths/s (HairMSNN full wavefront render, 512x512, 1 spp/frame, online cache training 2^16/frame)"
    unit = "paths/s"
    cache_precision = 1  # FP16 (tcgen05); its relMSE equals the FP32 cache's (quality workload)
    dtype = "f32 (traversal, shading, FP64 sums); f16 cache MLP with f32 accumulation"

    def __init__(self, torch, width=512, height=512, train_records=1 << 16, frames_in_flight=0):
        self.torch = torch
        self.width, self.height, self.train_records = width, height, train_records
        self.frames_in_flight = frames_in_flight
        self.cfg = straight_hair_scene(width, height)
        self.scene = Scene(self.cfg)
        self.scene.build()
        self.r = Renderer(self.scene, MSNN, beta=1, train_records=train_records, train=True,
                          precision=self.cache_precision, frames_in_flight=frames_in_flight)
        self.tuning = self.r.autotune(frames=6)
        self.P = width * height
        self.h2d_bytes = 0
        self.d2h_bytes = self.P * 3 * 8
        self.stage_ms = []
        self.launches = []
        self.read_stream = torch.cuda.Stream()
        self.host_sums = [torch.empty((height, width, 3), dtype=torch.float64, pin_memory=True) for _ in range(2)]

    def step(self, events=None):
        """One frame enqueued (frames run pipelined on the renderer's own streams)."""
        self.r.frame()
        self.launches.append(self.r.timings().kernel_launches)

    def timed_region(self, steps, flush):
        """Device time of `steps` pipelined frames: an event on the submitting
        stream before the first frame, the renderer's completion joined back
        (hm_render_wait) before the closing event.  No L2 flush: every frame
        streams its own path state (about 90 MB per frame in flight at
        512x512, several frames in flight) past the 129 MB L2, and a flush
        kernel on the submitting stream would run beside the frames in
        flight rather than between them."""
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for k in range(steps):
            self.step()
        self.r.wait()
        t1.record()
        torch.cuda.synchronize()
        self.last_ms = t0.elapsed_time(t1) / steps
        return self.last_ms

    @property
    def kernels_per_step(self):
        return int(round(np.mean(self.launches[-8:]))) if self.launches else 0

    def e2e_region(self, steps):
        """Wall time per frame through the public API with the result read back
        every frame: hm_render_frame, then hm_render_read_async of the FP64
        image sums into pinned host memory on a separate stream (the next
        frame's accumulation waits for that copy); host synchronisation at
        both ends."""
        import time
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            self.r.frame()
            self.r.read_async(self.host_sums[k & 1], IMAGE_FINAL, stream=self.read_stream)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        self.host_img = self.host_sums[(steps - 1) & 1].numpy() / self.r.stats().frames
        return 1e3 * el / steps

    def e2e_step(self):
        self.r.frame()
        self.r.read_async(self.host_sums[0], IMAGE_FINAL, stream=self.read_stream)

    def n_events(self):
        return 2

    def units_per_step(self):
        return self.P

    def profile_frames(self, n=4):
        """Synchronous instrumented frames (per-stage CUDA events on the frame's
        stream) for the stage breakdown and the roofline."""
        self.r.instrument(timing=True, counting=False)
        for _ in range(n):
            self.r.frame()
            self.stage_ms.append(self.r.timings().as_dict())
        self.r.instrument(timing=False, counting=False)

    def counted_frame(self):
        """One untimed frame with traversal work counters."""
        self.r.instrument(timing=True, counting=True)
        self.r.frame()
        t = self.r.timings()
        self.r.instrument(timing=False, counting=False)
        return t

    def plain_form(self, frames=20):
        """The plain FP32 wavefront form on the same scene and GPU: FP32 cache,
        one frame in flight, kernel-by-kernel launches, default launch
        shapes, one BVH leaf per segment.  Pipelined frame time."""
        torch = self.torch
        cfg = dict(self.cfg)
        cfg["integrator"] = dict(cfg["integrator"], segment_splits=1)
        sc = Scene(cfg)
        r = Renderer(sc, MSNN, beta=1, train_records=self.train_records, train=True, precision=0,
                     frames_in_flight=1)
        r.set_graphs(False)
        for _ in range(3):
            r.frame()
        r.wait()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(frames):
            r.frame()
        r.wait()
        t1.record()
        torch.cuda.synchronize()
        ms = t0.elapsed_time(t1) / frames
        r.close()
        sc.close()
        return ms

    def roofline(self, seg_ms, pk):
        keys = ["extend_ms", "shade_ms", "shadow_ms", "compact_ms", "train_ms", "infer_ms", "compose_ms",
                "camera_ms", "finalize_ms"]
        if not self.stage_ms:
            self.profile_frames()
        n = max(1, min(len(self.stage_ms), 16))
        mean = {k: float(np.mean([s[k] for s in self.stage_ms[-n:]])) for k in keys}
        c = self.counted_frame()
        dominant = max(("extend_ms", "shadow_ms", "shade_ms", "train_ms", "infer_ms"), key=lambda k: mean[k])
        out = {"stage_ms_per_frame": {k: round(v, 4) for k, v in mean.items()},
               "rays_per_frame": {"extension": int(c.extension_rays), "shadow": int(c.shadow_rays)},
               "bvh_work_per_frame": {"extend_nodes": int(c.extend_nodes), "extend_prims": int(c.extend_prims),
                                      "shadow_nodes": int(c.shadow_nodes), "shadow_prims": int(c.shadow_prims)}}
        if dominant in ("extend_ms", "shadow_ms"):
            if dominant == "extend_ms":
                rays, nodes, prims = c.extension_rays, c.extend_nodes, c.extend_prims
            else:
                rays, nodes, prims = c.shadow_rays, c.shadow_nodes, c.shadow_prims
            alg = rays * RAY_RECORD_BYTES + nodes * NODE_BYTES + prims * PRIM_BYTES
            ach = alg / (mean[dominant] * 1e-3) / 1e9
            out.update({"kernel": dominant.replace("_ms", "_kernel"), "bound": "hbm", "achieved": round(ach, 2),
                        "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(ach / pk["hbm_gbs"], 4),
                        "traffic": (int(rays * EXTEND_DRAM_BYTES_PER_RAY) if dominant == "extend_ms" else None),
                        "traffic_basis": "DRAM bytes per frame: ncu cold-cache capture at 256x256 scaled by rays",
                        "algorithmic_bytes_per_frame": int(alg),
                        "note": ("algorithmic bytes = rays x 48 B + 8-wide BVH nodes visited x 224 B + primitives "
                                 "tested x 64 B, counted in an untimed frame; the 90 MB BVH and 10 MB of curves "
                                 "are L2-resident, so this can exceed the HBM copy peak ("
                                 + pk["source"] + ")")})
        else:
            out.update({"kernel": dominant, "bound": "tensor", "achieved": None, "peak": pk["bf16_tflops"],
                        "unit": "TFLOP/s", "frac": None, "traffic": None})
        if type(self) is RenderBenchWorkload:
            plain = self.plain_form()
            chosen = self.last_ms if getattr(self, "last_ms", None) else None
            out["plain_fp32_wavefront_form"] = {
                "ms_per_frame": round(plain, 3), "paths_per_s": round(self.P / (plain * 1e-3), 1),
                "chosen_form_speedup": round(plain / chosen, 3) if chosen else None,
                "what": "FP32 cache, 1 frame in flight, kernel-by-kernel launches, default launch shapes, "
                        "1 BVH leaf per segment; same scene and GPU"}
        return out

    workload_name = ("render: straight procedural hair 10k strands x 64 B-spline CPs (610k segments, 2 BVH "
                     "leaves each), 20k-tri head, Preetham sky T=3 + directional (3,3,3), 512x512, "
                     "path_v1=1, path_v2=40, BETA=1, cache HashGrid/OneBlob MLP 64x2 in FP16 on tcgen05 "
                     "(training and inference; FP32 master weights), 2^16 training records/frame")

    def config(self):
        return {"workload": self.workload_name,
                "cache_precision": "fp16" if self.cache_precision == 1 else "fp32",
                "pixels": self.P, "train_records": self.train_records,
                "l2": "inputs larger than L2: each frame in flight streams its own ~90 MB path state, with "
                      "several frames in flight, past the 129 MB L2 (scene: 8-wide BVH 90 MB + curves 10 MB); "
                      "no flush kernel",
                "frames_in_flight": self.r.depth(),
                "launch_shapes": {k: v for k, v in self.tuning.items() if k != "ms_per_frame"},
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=20.0):
        """The oracle's reference-structured integrator (rayGenCam G-buffer pass,
        msnnPathTrace / msnnTrainingPath) on the host cores, bounded sample of
        pixels of the same scene; the cache's inference and training gradient
        by the oracle's C++ FP32 transcription on the same threads."""
        import time
        from oracle import mlp_oracle as mo
        from oracle import pyoracle as po
        o = po.OracleScene.from_library(self.scene)
        net = self.r
        cfg_text = json.dumps(_default_cache_config())
        oc = mo.Config(cfg_text, 12, 3)
        params = np.random.default_rng(0).normal(scale=0.05, size=oc.n_params)
        every = max(1, self.P // self.train_records)
        n = 4096
        t0 = time.perf_counter()
        done = 0
        p0 = (self.height // 2) * self.width  # a band through the hair
        while True:
            col, nn_in, tr, fl = o.render_pixels(1, beta=1, accum_id=done // self.P, every_nth=every,
                                                 n_train=self.train_records, p0=p0, n=n, threads=threads)
            po.mlp_forward_host(oc, params, nn_in, threads=threads)
            tmask = (fl & 4) != 0
            if tmask.any():
                po.mlp_grad_host(oc, params, nn_in[tmask], tr[tmask], threads=threads)
            done += n
            p0 = (p0 + n) % (self.P - n)
            if time.perf_counter() - t0 > budget_s:
                break
        el = time.perf_counter() - t0
        return {"value": round(done / el, 1), "unit": self.unit, "cores": threads, "kind": "port",
                "sample": f"{done} pixels (1 spp) of the same scene: oracle rayGenCam/msnnPathTrace/"
                          f"msnnTrainingPath on {threads} threads + the cache's inference and training "
                          f"gradient in C++ FP32 on the same threads"}


class RenderQualityWorkload(RenderBenchWorkload):
    """HairMSNN (BETA=1, online cache training) against plain path tracing and
    the reference's NRC comparison renderer (online training, 65536 records
    per frame) on the render workload's scene: relMSE of each at 16 spp against a
    converged PT reference of the same scene, their frame times, and the PT
    sample count (and time) needed to reach HairMSNN's relMSE, assuming PT's
    relMSE falls as 1/spp (it is unbiased).  The reference uses frames
    16 .. 16 + ref_spp of one PT run, so it shares no random numbers with
    the 16-spp estimates (the path RNG is seeded by the frame index, as in
    the reference).  The HairMSNN relMSE is also reported with the cache's
    inference in FP16, BF16 and E4M3 on the tensor cores (training FP32).
    One step = one HairMSNN frame, as the render workload."""

    name = "quality"
    metric = "paths/s at fixed relMSE vs PT (HairMSNN BETA=1, 512x512, 16 spp, online cache training 2^16/frame)"

    def __init__(self, torch, width=512, height=512, train_records=1 << 16, spp=16, ref_spp=1024,
                 pretrain_passes=256):
        super().__init__(torch, width, height, train_records)
        self.spp, self.ref_spp, self.pretrain_passes = spp, ref_spp, pretrain_passes

    def _timed_frames(self, r, n):
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(n):
            r.frame()
        r.wait()
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / n

    def quality(self):
        spp = self.spp
        pt = Renderer(self.scene, PT, frames_in_flight=self.frames_in_flight)
        pt_ms = self._timed_frames(pt, spp)
        pt_img = pt.read(IMAGE_FINAL)
        ref_ms = self._timed_frames(pt, self.ref_spp)
        total = pt.read(IMAGE_FINAL) * (spp + self.ref_spp)
        ref = (total - pt_img * spp) / self.ref_spp
        pt.close()
        by_prec = {}
        for name, prec in (("fp32", 0), ("fp16", 1), ("bf16", 2), ("fp8", 3)):
            ms = Renderer(self.scene, MSNN, beta=1, train_records=self.train_records, train=True,
                          precision=prec, frames_in_flight=self.frames_in_flight)
            t_ms = self._timed_frames(ms, spp)
            img = ms.read(IMAGE_FINAL)
            ms.close()
            by_prec[name] = {"relmse": round(relmse(img, ref), 6), "ms_per_frame": round(t_ms, 3)}
            if name == "fp32":
                ms_ms, ms_img = t_ms, img
        # the reference's initial training before the first frame (one second
        # of scene-sample passes there; a fixed pass count here)
        ms = Renderer(self.scene, MSNN, beta=1, train_records=self.train_records, train=True,
                      frames_in_flight=self.frames_in_flight)
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        ms.pretrain(self.pretrain_passes)
        t1.record()
        torch.cuda.synchronize()
        pre_ms = t0.elapsed_time(t1)
        t_pre = self._timed_frames(ms, spp)
        e_pre = relmse(ms.read(IMAGE_FINAL), ref)
        ms.close()
        # the reference's comparison renderer: NRC with online training
        # (65536 records per frame, c = 0.01), same frames
        nrc = Renderer(self.scene, NRC, train=True, frames_in_flight=self.frames_in_flight)
        nrc_ms = self._timed_frames(nrc, spp)
        e_nrc = relmse(nrc.read(IMAGE_FINAL), ref)
        nrc.close()
        e_pt, e_ms = relmse(pt_img, ref), relmse(ms_img, ref)
        eq_spp = spp * e_pt / e_ms
        return {"spp": spp, "reference_spp": self.ref_spp, "reference_ms_per_frame": round(ref_ms, 3),
                "msnn": {"relmse": round(e_ms, 6), "ms_per_frame": round(ms_ms, 3),
                         "paths_per_s": round(self.P / (ms_ms * 1e-3), 1)},
                "pt": {"relmse": round(e_pt, 6), "ms_per_frame": round(pt_ms, 3),
                       "paths_per_s": round(self.P / (pt_ms * 1e-3), 1)},
                "nrc": {"relmse": round(e_nrc, 6), "ms_per_frame": round(nrc_ms, 3),
                        "paths_per_s": round(self.P / (nrc_ms * 1e-3), 1),
                        "pt_spp_for_same_relmse": round(spp * e_pt / e_nrc, 2),
                        "speedup_at_equal_relmse": round((spp * e_pt / e_nrc) * pt_ms / (spp * nrc_ms), 3)},
                "msnn_by_cache_precision": by_prec,
                "msnn_after_scene_sample_training": {
                    "passes": self.pretrain_passes, "training_ms": round(pre_ms, 1), "relmse": round(e_pre, 6),
                    "ms_per_frame": round(t_pre, 3), "pt_spp_for_same_relmse": round(spp * e_pt / e_pre, 2),
                    "speedup_at_equal_relmse": round((spp * e_pt / e_pre) * pt_ms / (spp * t_pre), 3)},
                "pt_spp_for_msnn_relmse": round(eq_spp, 2),
                "speedup_at_equal_relmse": round(eq_spp * pt_ms / (spp * ms_ms), 3)}

    def roofline(self, seg_ms, pk):
        out = super().roofline(seg_ms, pk)
        out["quality"] = self.quality()
        return out

    def config(self):
        c = super().config()
        c["workload"] = "quality: " + c["workload"] + f"; relMSE at {self.spp} spp vs PT {self.ref_spp} spp"
        return c


def batch_scene_configs(n=64, seed=0):
    """The batched-render workload's scenes (seeded): square images of side
    128, 256, 512 or 1024; log-uniform 2k-50k curly strands (helix radius
    2-8 mm, pitch 5-20 mm, 48-128 control points, 20 cm long); BETA uniform
    in 0..10; sigma_a uniform in [0.02, 0.5]^3.  Returns (configs, betas)."""
    rng = np.random.default_rng(seed)
    cfgs, betas = [], []
    for k in range(n):
        side = int(rng.choice([128, 256, 512, 1024]))
        strands = int(np.exp(rng.uniform(np.log(2000), np.log(50000))))
        cps = int(rng.integers(48, 129))
        cfg = straight_hair_scene(side, side, strands=strands, control_points=cps, seed=1000 + k)
        p = cfg["hair"]["procedural"]
        p["type"] = "curly"
        p["helix_radius"] = float(rng.uniform(0.02, 0.08))   # scene unit = 10 cm
        p["helix_pitch"] = float(rng.uniform(0.05, 0.2))
        cfg["hair"]["sigma_a"] = [float(x) for x in rng.uniform(0.02, 0.5, 3)]
        cfgs.append(cfg)
        betas.append(int(rng.integers(0, 11)))
    return cfgs, betas


class BatchBenchWorkload(RenderBenchWorkload):
    """bench.py workload: one frame (1 spp) of each of 64 uneven scenes,
    rendered as one batch with one shared FP32 cache network (width 64)."""

    dtype = "f32"

    name = "batch"
    metric = "paths/s (64 concurrent HairMSNN scenes, 128^2..1024^2, 2k-50k curly strands, one shared cache)"
    unit = "paths/s"

    def __init__(self, torch, n_scenes=64, train_records=1 << 16):
        import time
        self.torch = torch
        self.train_records = train_records
        t0 = time.perf_counter()
        cfgs, self.betas = batch_scene_configs(n_scenes)
        self.scenes = [Scene(c) for c in cfgs]
        for sc in self.scenes:
            sc.build()
        self.setup_s = time.perf_counter() - t0
        self.r = BatchRenderer(self.scenes, MSNN, betas=self.betas, train_records=train_records, train=True)
        self.tuning = self.r.autotune(frames=1)
        self.P = self.r.pixels
        self.h2d_bytes = 0
        self.d2h_bytes = self.P * 3 * 8
        self.stage_ms = []
        self.launches = []
        self.read_stream = torch.cuda.Stream()
        self.host_sums = [torch.empty((self.P, 3), dtype=torch.float64, pin_memory=True) for _ in range(2)]
        self.n_scenes = n_scenes
        infos = [sc.info() for sc in self.scenes]
        self.stats_scenes = {"pixels": self.P, "segments": int(sum(i.n_segments for i in infos)),
                             "strands": int(sum(i.n_strands for i in infos))}

    def e2e_region(self, steps):
        import time
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            self.r.frame()
            self.r.read_async(self.host_sums[k & 1], IMAGE_FINAL, stream=self.read_stream)
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0) / steps

    def config(self):
        return {"workload": f"batch: {self.n_scenes} scenes (seeded), sides 128/256/512/1024, log-uniform 2k-50k "
                            "curly strands (helix r 2-8 mm, pitch 5-20 mm, 48-128 CPs), BETA 0..10, sigma_a "
                            "U[0.02,0.5]^3, one shared FP32 cache (HashGrid/OneBlob MLP 64x2), 2^16 records/frame",
                **self.stats_scenes, "frames_in_flight": self.r.depth(), "scene_setup_s": round(self.setup_s, 1),
                "launch_shapes": {k: v for k, v in self.tuning.items() if k != "ms_per_frame"},
                "l2": "inputs larger than L2 (path state of tens of millions of paths); no flush kernel",
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=20.0):
        return {"value": None, "unit": self.unit, "cores": threads, "kind": "port",
                "sample": "not run for the batch workload (see the render workload's CPU baseline)"}


def _default_cache_config():
    return {
        "loss": {"otype": "RelativeL2Luminance"},
        "optimizer": {"otype": "ExponentialDecay", "decay_start": 4000, "decay_interval": 4000, "decay_base": 0.33,
                      "nested": {"otype": "Adam", "learning_rate": 1e-2, "beta1": 0.9, "beta2": 0.99,
                                 "epsilon": 1e-15, "l2_reg": 1e-6}},
        "encoding": {"otype": "Composite", "nested": [
            {"n_dims_to_encode": 3, "otype": "HashGrid", "per_level_scale": 2.0, "log2_hashmap_size": 15,
             "base_resolution": 16, "n_levels": 16},
            {"n_dims_to_encode": 6, "otype": "OneBlob", "n_bins": 4}, {"otype": "Identity"}]},
        "network": {"otype": "FullyFusedMLP", "activation": "ReLU", "output_activation": "None",
                    "n_neurons": 64, "n_hidden_layers": 2}}


# ----------------------------------------------------- differentiable rendering
def diff_materials(n, seed=0):
    """Seeded strand-group materials [n, 10]: sigma_a U[0.08, 0.5]^3,
    beta_m U[0.6, 0.75] (every lobe's M_p on its direct branch), beta_n
    U[0.3, 0.6], alpha U[1, 4] degrees (in radians), gains 1."""
    rng = np.random.default_rng(seed)
    m = np.zeros((n, 10), np.float32)
    m[:, 0:3] = rng.uniform(0.08, 0.5, (n, 3))
    m[:, 3] = rng.uniform(0.6, 0.75, n)
    m[:, 4] = rng.uniform(0.3, 0.6, n)
    m[:, 5] = np.deg2rad(rng.uniform(1.0, 4.0, n))
    m[:, 6:10] = 1.0
    return m


def curly_hair_diff_scene(width=256, height=256, strands=20000, control_points=96, groups=4, seed=7):
    """The differentiable-fit workload's scene: 20k curly strands (helix
    radius 5 mm, pitch 10 mm, 96 B-spline control points, 20 cm), head,
    sky + directional light, split by root azimuth into `groups` strand
    groups with seeded materials.  Returns (config, materials)."""
    cfg = straight_hair_scene(width, height, strands=strands, control_points=control_points, seed=seed)
    p = cfg["hair"]["procedural"]
    p["type"] = "curly"
    p["helix_radius"] = 0.05
    p["helix_pitch"] = 0.1
    mats = diff_materials(groups, seed)
    cfg["hair"]["groups"] = {"count": groups, "assign": "azimuth", "materials": [
        {"sigma_a": [float(x) for x in r[0:3]], "beta_m": float(r[3]), "beta_n": float(r[4]),
         "alpha": float(np.rad2deg(r[5]))} for r in mats]}
    return cfg, mats


class DiffBenchWorkload:
    """bench.py workload: one gradient evaluation per step of the
    differentiable appearance fit.  A step renders 64 frames (1 spp each) of
    20k curly strands at 256x256, HairMSNN with BETA=2 and the cache frozen
    (hm_render_diff_forward), forms the L2 image loss against a target
    rendered at the true materials, and replays the paths
    (hm_render_diff_backward) for dL/d(sigma_a, beta_m, beta_n, alpha) of 4
    strand groups and dL/dW of the cache.  The target is rendered once with
    the same frame seeds; the materials start with sigma_a 50% off."""

    name = "diff"
    metric = ("gradient evaluations/s (path replay: dL/d(material) of 4 strand groups + dL/dW, 20k curly strands, "
              "256x256, 64 spp, BETA=2)")
    unit = "gradient evaluations/s"

    def __init__(self, torch, width=256, height=256, spp=64, strands=20000, groups=4, pretrain_passes=64):
        self.torch = torch
        self.width, self.height, self.spp, self.groups = width, height, spp, groups
        self.cfg, self.truth = curly_hair_diff_scene(width, height, strands=strands, groups=groups)
        self.scene = Scene(self.cfg)
        self.scene.build()
        self.scene.set_group_materials(self.truth)
        self.r = Renderer(self.scene, MSNN, beta=2, train_records=1 << 14, train=True)
        self.tuning = self.r.autotune(frames=4)
        self.r.pretrain(pretrain_passes)
        self.P = width * height
        self.n = self.P * 3
        self.r.diff_forward(spp)
        self.target = (self.r.device_sums(5) / spp).clone()
        self.target_host = self.target.cpu().numpy()
        self.start = self.truth.copy()
        self.start[:, 0:3] *= np.where(np.random.default_rng(11).random((groups, 3)) < 0.5, 0.5, 1.5)
        self.scene.set_group_materials(self.start)
        self.h2d_bytes = self.P * 3 * 4
        self.d2h_bytes = self.P * 3 * 8 + groups * 6 * 8
        self.launches = []
        self.adj_host = torch.empty((height, width, 3), dtype=torch.float32, pin_memory=True)
        self.adj_dev = torch.empty((height, width, 3), dtype=torch.float32, device="cuda")

    def gradient(self):
        """One gradient evaluation on the device: forward, adjoint, replay."""
        self.r.diff_forward(self.spp)
        img = self.r.device_sums(5) / self.spp
        adj = ((2.0 / self.n) * (img - self.target)).float()
        return self.r.diff_backward(adj)

    def step(self, events=None):
        self.last_grad = self.gradient()

    def timed_region(self, steps, flush):
        """CUDA events on the submitting stream around `steps` evaluations;
        every evaluation streams 64 frames of path state (about 20 MB per
        frame at 256x256, several in flight) and 4.2M cache queries through
        the backward, far past the 129 MB L2: no flush kernel."""
        torch = self.torch
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(steps):
            self.step()
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / steps

    def e2e_region(self, steps):
        """Through the public API with host buffers: forward, image read to the
        host (FP64), adjoint on the host, copied in from pinned memory,
        replay returning the gradients to the host."""
        import time
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            self.r.diff_forward(self.spp)
            img = self.r.read()
            self.adj_host.numpy()[...] = (2.0 / self.n) * (img - self.target_host)
            self.adj_dev.copy_(self.adj_host, non_blocking=True)
            self.last_grad = self.r.diff_backward(self.adj_dev)
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0) / steps

    @property
    def kernels_per_step(self):
        # forward frames (bounce loop, cache inference, compose) + replay frames
        # (bounce loop, cache adjoint, two gradient sums) + group duals, total,
        # cache forward + backward
        rounds = 3  # BETA + 1 vertices at BETA = 2
        md = self.r.cache().info()
        # cache forward (encode, layers) + backward (fused dgrad, loss sum,
        # per-layer weight-gradient partials and reduction, hash-grid scatter
        # and conversion)
        mlp = 2 + 2 + 2 * (md.n_hidden_layers + 1) + 2
        fwd = 1 + 7 * rounds + 1 + 2 + 1
        rep = 1 + 7 * rounds + 3
        return self.spp * (fwd + rep) + 2 + mlp

    def units_per_step(self):
        return 1

    def paths_per_step(self):
        return 2 * self.P * self.spp

    def fit(self, steps=200, lr=0.05):
        """Adam on log(sigma_a) of every group from the +-50% start; returns
        the final relative error per component (the other materials fixed)."""
        torch = self.torch
        x = torch.tensor(np.log(self.start[:, 0:3].astype(np.float64)), requires_grad=True)
        opt = torch.optim.Adam([x], lr=lr)
        for _ in range(steps):
            m = self.truth.copy()
            m[:, 0:3] = np.exp(x.detach().numpy())
            self.scene.set_group_materials(m)
            g = self.gradient()
            opt.zero_grad()
            x.grad = torch.from_numpy(g[:, 0:3] * m[:, 0:3])
            opt.step()
        self.scene.set_group_materials(self.start)
        got = np.exp(x.detach().numpy())
        return np.abs(got - self.truth[:, 0:3]) / self.truth[:, 0:3]

    def roofline(self, seg_ms, pk):
        """Traversal of the forward frames (instrumented, one frame at a time)
        and the split of an evaluation into forward, replay and cache backward."""
        torch = self.torch
        self.r.instrument(timing=True, counting=False)
        self.r.diff_forward(4)
        t = self.r.timings().as_dict()
        self.r.instrument(timing=True, counting=True)
        self.r.diff_forward(1)
        c = self.r.timings()
        self.r.instrument(timing=False, counting=False)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        self.r.diff_forward(self.spp)
        ev[1].record()
        img = self.r.device_sums(5) / self.spp
        self.r.diff_backward(((2.0 / self.n) * (img - self.target)).float())
        ev[2].record()
        torch.cuda.synchronize()
        dominant = "extend_ms" if t["extend_ms"] >= t["shadow_ms"] else "shadow_ms"
        if dominant == "extend_ms":
            rays, nodes, prims = c.extension_rays, c.extend_nodes, c.extend_prims
        else:
            rays, nodes, prims = c.shadow_rays, c.shadow_nodes, c.shadow_prims
        alg = rays * RAY_RECORD_BYTES + nodes * NODE_BYTES + prims * PRIM_BYTES
        ach = alg / (t[dominant] * 1e-3) / 1e9
        return {"kernel": dominant.replace("_ms", "_kernel") + " (forward frames)", "bound": "hbm",
                "achieved": round(ach, 2), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(ach / pk["hbm_gbs"], 4), "traffic": None,
                "evaluation_split_ms": {"forward_64_frames": round(ev[0].elapsed_time(ev[1]), 3),
                                        "replay_and_cache_backward": round(ev[1].elapsed_time(ev[2]), 3)},
                "stage_ms_per_forward_frame": {k: round(t[k], 4) for k in ("extend_ms", "shade_ms", "shadow_ms",
                                                                           "compact_ms", "infer_ms")},
                "rays_per_forward_frame": {"extension": int(c.extension_rays), "shadow": int(c.shadow_rays)},
                "algorithmic_bytes_per_frame": int(alg),
                "note": ("algorithmic bytes = rays x 48 B + 8-wide BVH nodes visited x 224 B + primitives tested "
                         "x 64 B, counted in an untimed forward frame; the replay re-traces the same rays. "
                         "Peak " + pk["source"])}

    def config(self):
        return {"workload": "diff: 20k curly procedural strands x 96 B-spline CPs (helix r 5 mm, pitch 10 mm), "
                            "20k-tri head, sky + directional light, 256x256, 64 spp per evaluation, HairMSNN BETA=2, "
                            "cache FP32 (frozen, 64 scene-sample training passes), 4 azimuthal strand groups; "
                            "L2 image loss against a target at the true materials (same frame seeds)",
                "pixels": self.P, "spp": self.spp, "groups": self.groups,
                "paths_per_evaluation": self.paths_per_step(),
                "l2": "inputs larger than L2: 64 frames of path state and 4.2M cache queries per evaluation",
                "launch_shapes": {k: v for k, v in self.tuning.items() if k != "ms_per_frame"},
                "parallelism": "replicas"}

    def cpu_baseline(self, threads, budget_s=20.0):
        """The reference has no gradient path.  Baseline: central finite
        differences on the host, the way to differentiate it as it is: one
        gradient of 4 groups x 6 parameters = 49 forward renders of 256x256 x
        64 spp, each timed as the oracle's reference-structured integrator
        (rayGenCam / msnnPathTrace G-buffer pass) on a bounded pixel sample."""
        import time
        from oracle import pyoracle as po
        o = po.OracleScene.from_library(self.scene)
        n = 4096
        t0 = time.perf_counter()
        done = 0
        p0 = (self.height // 2) * self.width
        while True:
            o.render_pixels(1, beta=2, accum_id=done // self.P, every_nth=self.P, n_train=0, p0=p0, n=n,
                            threads=threads)
            done += n
            p0 = (p0 + n) % (self.P - n)
            if time.perf_counter() - t0 > budget_s:
                break
        rate = done / (time.perf_counter() - t0)
        renders = 2 * self.groups * 6 + 1
        value = rate / (self.P * self.spp * renders)
        return {"value": value, "unit": self.unit, "cores": threads, "kind": "port",
                "sample": f"{done} pixels (1 spp) of the oracle's forward integrator on {threads} threads "
                          f"({rate:.0f} paths/s); a finite-difference gradient = {renders} renders of "
                          f"{self.P} pixels x {self.spp} spp; cache not included"}
