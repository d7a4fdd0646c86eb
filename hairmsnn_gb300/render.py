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

    def autotune(self, frames=16, stream=None):
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
        3 training targets [R,3], 4 G-buffer [P,4], 11 scene samples of the
        scene-sample training pass [N,4] (after pretrain)."""
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        check(lib().hm_render_buffer(self._h, which, ctypes.byref(p), ctypes.byref(n)))
        in_ch = 9 if self.mode == NRC else 12
        width = {0: in_ch, 1: 3, 2: in_ch, 3: 3, 4: 4, 8: 4, 9: 20, 10: 4, 11: 4}[which]
        count = n.value * (4 if which in (4, 8, 9, 10, 11) else 1)
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
