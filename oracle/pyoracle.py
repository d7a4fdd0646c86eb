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
        L.hmo_set_ulp_perturb.argtypes = [i32]
        L.hmo_hair_eval.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P]
        L.hmo_hair_sample.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P]
        L.hmo_hair_eval_mt.argtypes = [i64, F32P, F32P, F32P, F32P, F32P, F32P, F32P, i32]
        L.hmo_mlp_forward.restype = None
        L.hmo_mlp_forward.argtypes = [F32P, i64, i32, I32P, i32, i32, i32, F32P, i64, I32P, i32, i32,
                                      F32P, I32P, I32P, I32P, F32P, i32]
        L.hmo_mlp_grad.restype = ctypes.c_double
        L.hmo_mlp_grad.argtypes = [F32P, F32P, i64, i32, I32P, i32, i32, i32, F32P, i64, i64, I32P, i32, i32,
                                   F32P, I32P, I32P, I32P, i32, F32P, i32]
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


def set_ulp_perturb(k):
    """0: libm's transcendentals (default); +1 / -1: every result one ulp up /
    down; k >= 2: a pseudo-random -2..+2 ulps per call (stream k) -- to
    measure a path's sensitivity to last-ulp differences."""
    lib().hmo_set_ulp_perturb(int(k))


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


def _declare_render(L):
    if getattr(L, "_render_declared", False):
        return
    i32, f32, vp = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    L.hmo_scene_new.restype = vp
    L.hmo_scene_new.argtypes = [F32P, i32, I32P, i32, F32P, F32P, i32, I32P, i32, F32P, i32, i32, F32P, F32P,
                                F32P, F32P, F32P, i32, F32P, F32P, I32P, f32]
    L.hmo_scene_free.restype = None
    L.hmo_scene_free.argtypes = [vp]
    L.hmo_bvh_sizes.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.hmo_bvh_export.restype = None
    L.hmo_bvh_export.argtypes = [vp, F32P, I32P]
    L.hmo_trace_rays.restype = None
    L.hmo_trace_rays.argtypes = [vp, F32P, F32P, i32, f32, f32, i32, F32P]
    L.hmo_render_pixels.restype = None
    L.hmo_render_pixels.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, F32P, F32P, F32P, I32P, i32]
    L.hmo_render_pixels_ev.restype = None
    L.hmo_render_pixels_ev.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, F32P, F32P, F32P, I32P, F32P, I32P,
                                       U32P, i32, i32]
    L.hmo_render_traingen_ev.restype = None
    L.hmo_render_traingen_ev.argtypes = [vp, i32, i32, i32, F32P, i32, i32, F32P, F32P, I32P, F32P, I32P, U32P,
                                         i32, i32]
    L.hmo_feistel_perm.restype = ctypes.c_uint32
    L.hmo_feistel_perm.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
    L.hmo_render_nrc.restype = None
    L.hmo_render_nrc.argtypes = [vp, i32, i32, i32, f32, i32, i32, F32P, F32P, F32P, F32P, I32P, i32]
    L.hmo_render_nrc_ev.restype = None
    L.hmo_render_nrc_ev.argtypes = [vp, i32, i32, i32, f32, i32, i32, F32P, F32P, F32P, F32P, I32P, F32P, I32P,
                                    i32, i32]
    L.hmo_scene_set_groups.restype = None
    L.hmo_scene_set_groups.argtypes = [vp, I32P, i32, F32P, i32]
    L._render_declared = True


class OracleScene:
    """The oracle's copy of a scene: same arrays as the library's, its own LBVH."""

    def __init__(self, arrays, settings, scene_scale):
        L = lib()
        _declare_render(L)
        a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        self._keep = a
        env_w, env_h = int(settings["env_w"]), int(settings["env_h"])
        empty = np.zeros(4, np.float32)
        g = lambda k: a[k] if a[k].size else empty
        sets = np.array([settings["width"], settings["height"], settings["path_v1"], settings["path_v2"],
                         settings["mis"], settings["env_pdf"], settings["has_env"], settings["catrom"],
                         settings.get("seg_split", 1)], np.int32)
        self.h = L.hmo_scene_new(
            a["control_points"].astype(np.float32).ravel(), len(a["control_points"]),
            a["segments"].astype(np.int32).ravel(), len(a["segments"]),
            a["vertices"].astype(np.float32).ravel(), a["normals"].astype(np.float32).ravel(), len(a["vertices"]),
            a["triangles"].astype(np.int32).ravel(), len(a["triangles"]),
            g("env").astype(np.float32).ravel(), env_w, env_h,
            g("env_cpdf").ravel(), g("env_ccdf").ravel(), g("env_mpdf").ravel(), g("env_mcdf").ravel(),
            g("dir_lights").astype(np.float32).ravel(), len(a["dir_lights"]),
            a["camera"].astype(np.float32).ravel(), a["materials"].astype(np.float32).ravel(), sets,
            float(scene_scale))
        self.width, self.height = int(settings["width"]), int(settings["height"])
        self.settings = sets
        self.env_wh = (env_w, env_h)
        self.scene_scale = float(scene_scale)

    @classmethod
    def from_library(cls, scene):
        """scene: hairmsnn_gb300.render.Scene (host arrays only, no device)."""
        names = ["control_points", "segments", "vertices", "normals", "triangles", "env", "env_cpdf",
                 "env_ccdf", "env_mpdf", "env_mcdf", "dir_lights", "camera", "materials"]
        arrays = {k: scene.export(k) for k in names}
        i = scene.info()
        settings = dict(width=i.width, height=i.height, path_v1=i.path_v1, path_v2=i.path_v2, mis=i.mis,
                        env_pdf=i.env_pdf, has_env=i.has_env, catrom=i.shading_catrom, env_w=i.env_width,
                        env_h=i.env_height, seg_split=i.segment_splits)
        o = cls(arrays, settings, i.scene_scale)
        if i.n_groups > 0:
            o.set_groups(scene.export("segment_groups"), scene.export("group_materials"))
        return o

    def set_groups(self, seg_group, materials):
        """Strand groups: group of every segment, [n_groups, 10] materials."""
        sg = np.ascontiguousarray(seg_group, np.int32)
        m = f32(np.asarray(materials).reshape(-1, 10))
        self._keep["groups"] = (sg, m)
        lib().hmo_scene_set_groups(self.h, sg, len(sg), m.ravel(), len(m))

    def __del__(self):
        try:
            lib().hmo_scene_free(self.h)
        except Exception:
            pass

    def bvh(self):
        L = lib()
        nn, nl = ctypes.c_int(), ctypes.c_int()
        L.hmo_bvh_sizes(self.h, ctypes.byref(nn), ctypes.byref(nl))
        nodes = np.zeros(nn.value * 16, np.float32)
        leaves = np.zeros(nl.value, np.int32)
        L.hmo_bvh_export(self.h, nodes, leaves)
        return nodes.reshape(-1, 16), leaves

    def trace(self, org, dirs, tmin=0.0, tmax=1e30, any_hit=False):
        org, dirs = f32(org), f32(dirs)
        hits = np.zeros((org.shape[0], 4), np.float32)
        lib().hmo_trace_rays(self.h, org, dirs, org.shape[0], tmin, tmax, 1 if any_hit else 0, hits)
        return hits

    def render_pixels(self, mode, beta=1, accum_id=0, every_nth=1, n_train=0, p0=0, n=None, threads=8):
        """One frame of rayGenCam for pixels [p0, p0+n): mode 0 PT, 1 MSNN G-buffer."""
        n = self.width * self.height - p0 if n is None else n
        color = np.zeros((n, 3), np.float32)
        nn_in = np.zeros((n, 12), np.float32)
        train = np.zeros((n, 3), np.float32)
        flags = np.zeros(n, np.int32)
        lib().hmo_render_pixels(self.h, mode, beta, accum_id, every_nth, n_train, p0, n, color, nn_in, train, flags,
                                threads)
        return color, nn_in, train, flags


# Event log of a path (kEvFloats = 12 floats per traced ray, in order):
# kind (0 radiance, 1 light-sample shadow, 2 BSDF-sample shadow), result
# (radiance: hit primitive or -1; shadow: 1 unoccluded), t, u, origin[3],
# direction[3], RNG state when a radiance ray was traced, 0.
EV_FLOATS = 12


def _render_pixels_ev(self, mode, beta=1, accum_id=0, every_nth=1, n_train=0, max_events=128, threads=8):
    """render_pixels over the whole frame plus every path's ray log:
    (color, nn_in, train, flags, events [P, max_events, 12] float32,
    n_events [P], rng_end [P] uint32)."""
    n = self.width * self.height
    color = np.zeros((n, 3), np.float32)
    nn_in = np.zeros((n, 12), np.float32)
    train = np.zeros((n, 3), np.float32)
    flags = np.zeros(n, np.int32)
    ev = np.zeros((n, max_events, EV_FLOATS), np.float32)
    nev = np.zeros(n, np.int32)
    rng_end = np.zeros(n, np.uint32)
    lib().hmo_render_pixels_ev(self.h, mode, beta, accum_id, every_nth, n_train, 0, n, color, nn_in, train, flags,
                               ev, nev, rng_end, max_events, threads)
    return color, nn_in, train, flags, ev, nev, rng_end


OracleScene.render_pixels_ev = _render_pixels_ev


def _render_traingen_ev(self, points, beta=1, accum_id=0, rec_x=128, max_events=128, threads=8):
    """The scene-sample training pass (TRAIN_DATA_GEN) for len(points)
    records: record r aims at points[r] (float [R, 3]) and sits at launch
    index (r % rec_x, r // rec_x).  Returns (train_in [R, 12], train_out
    [R, 3], flags [R], events [R, max_events, 12], n_events [R], rng_end [R])."""
    pts = np.ascontiguousarray(np.asarray(points, np.float32)[:, :3])
    n = len(pts)
    tin = np.zeros((n, 12), np.float32)
    tout = np.zeros((n, 3), np.float32)
    flags = np.zeros(n, np.int32)
    ev = np.zeros((n, max_events, EV_FLOATS), np.float32)
    nev = np.zeros(n, np.int32)
    rng_end = np.zeros(n, np.uint32)
    lib().hmo_render_traingen_ev(self.h, beta, accum_id, rec_x, pts, 0, n, tin, tout, flags, ev, nev, rng_end,
                                 max_events, threads)
    return tin, tout, flags, ev, nev, rng_end


OracleScene.render_traingen_ev = _render_traingen_ev


def event_digest(ev, n_ev):
    """One 64-bit FNV-1a digest per path over its logged rays, in the form
    the reference's trace hook records them (kinds 1 and 2 both read as
    shadow rays; the RNG word is left out)."""
    ev = np.array(ev, np.float32, copy=True)
    k = ev[:, :, 0].view(np.int32)
    k[k == 2] = 1
    ev[:, :, 10] = 0.0
    raw = ev.view(np.uint8).reshape(len(ev), -1)
    out = np.zeros(len(ev), np.uint64)
    per = ev.shape[2] * 4
    for p in range(len(ev)):
        h = 0xcbf29ce484222325
        for b in raw[p, :min(int(n_ev[p]), ev.shape[1]) * per].tobytes():
            h = ((h ^ b) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
        out[p] = h
    return out


def feistel_perm(i, n, key):
    """The library's training-pixel permutation of [0, n) (keyed by the frame)."""
    return int(lib().hmo_feistel_perm(int(i), int(n), int(key) & 0xFFFFFFFF))


def msnn_render(gbuf, nn_out, accum_id=0, acc=None):
    """The RENDER pass of hair_msnn.cu:314-356 in float32: gbuf [P, 8] (hit,
    isSurface, p, shortPathColor), nn_out [P, 3], acc (dict pt/nn/final of
    [P, 4] float32 running sums, read when accum_id > 0).  Returns
    {"acc": ..., "avg": ...} like the reference's six float4 buffers."""
    f = np.float32
    g = np.asarray(gbuf, f)
    sc = g[:, 5:8].copy()
    nn = np.asarray(nn_out, f).copy()
    other = (g[:, 0] == 0) | (g[:, 1] != 0)  # escaped or hit the surface
    color = (sc + nn).astype(f)
    color[other] = sc[other]
    nn[other] = sc[other]
    if accum_id > 0:
        sc = (sc + np.asarray(acc["pt"], f)[:, :3]).astype(f)
        nn = (nn + np.asarray(acc["nn"], f)[:, :3]).astype(f)
        color = (color + np.asarray(acc["final"], f)[:, :3]).astype(f)
    one = np.ones((len(g), 1), f)
    out = {"acc": {}, "avg": {}}
    w = f(f(1.0) / f(accum_id + 1))
    for k, v in (("pt", sc), ("nn", nn), ("final", color)):
        out["acc"][k] = np.concatenate([v, one], 1)
        out["avg"][k] = np.concatenate([(w * v).astype(f), one], 1)
    return out


def nrc_render(rad, beta, hit, cache, train_px, unbiased, t_bounces, t_hit, records):
    """The NRC RENDER pass (nrc.cu:365-380) and nrcGenerateTrainingData
    (nrc.cu:70-133) in float32, operation by operation.  rad / beta [P, 3]:
    the G-buffer's radiance and throughput, hit [P]; cache [P + T, 3]: the
    cache outputs (pixels, then the T training suffixes); per training pixel
    t: its pixel train_px[t], unbiased[t], its train buffer's bounces and hit
    and records [T, 40, 15] (vert, wo, n, vertRadiance, vertBeta).  Returns
    (color [P, 3] before accumulation, NaN as 0; train_in [T, 40, 9];
    train_gt [T, 40, 3])."""
    f = np.float32
    rad, beta, cache = np.asarray(rad, f), np.asarray(beta, f), np.asarray(cache, f)
    P = len(rad)
    c = cache[:P].copy()
    c[np.isnan(c).any(1)] = 0.0
    color = (rad + (beta * np.maximum(c, f(0.0))).astype(f)).astype(f)
    color[np.isnan(color).any(1)] = 0.0
    T = len(train_px)
    rec = np.asarray(records, f).reshape(T, 40, 15)
    tin = np.zeros((T, 40, 9), f)
    tgt = np.zeros((T, 40, 3), f)
    hit_t = np.asarray(hit, bool)[np.asarray(train_px)]
    bounces = np.where(hit_t, np.asarray(t_bounces), 0)
    suffix = cache[P:P + T].copy()
    use = hit_t & (np.asarray(t_hit) != 0) & ~np.asarray(unbiased, bool)
    suffix[~use] = 0.0
    for b in range(40):
        on = bounces > b
        col = np.zeros((T, 3), f)
        bt = np.ones((T, 3), f)
        for sub in range(b, 40):
            m = on & (bounces > sub)
            col = np.where(m[:, None], (col + (bt * rec[:, sub, 9:12]).astype(f)).astype(f), col)
            bt = np.where(m[:, None], (bt * rec[:, sub, 12:15]).astype(f), bt)
        t = (col + (bt * suffix).astype(f)).astype(f)
        t[np.isnan(t).any(1)] = 0.0
        tin[on, b] = rec[on, b, 0:9]
        tgt[on, b] = t[on]
    return color, tin, tgt


def _render_nrc(self, accum_id=0, every_nth=1, n_train=0, c=0.01, p0=0, n=None, threads=8, max_events=0):
    """One frame of the NRC G_BUFFER pass for pixels [p0, p0+n): dict of
    gbuf [n,7] (radiance, beta, hit), query [n,9], suffix_query [n,9],
    records [n,40,15] (vert, wo, n, direct light, factor), tinfo [n,4]
    (bounces, suffix ended at a query, unbiased, training pixel); with
    max_events > 0 also events [n, max_events, 12] and n_events [n] (the
    ray log of render_pixels_ev)."""
    n = self.width * self.height - p0 if n is None else n
    out = dict(gbuf=np.zeros((n, 7), np.float32), query=np.zeros((n, 9), np.float32),
               suffix_query=np.zeros((n, 9), np.float32), records=np.zeros((n, 40, 15), np.float32),
               tinfo=np.zeros((n, 4), np.int32))
    if max_events > 0:
        out["events"] = np.zeros((n, max_events, EV_FLOATS), np.float32)
        out["n_events"] = np.zeros(n, np.int32)
        lib().hmo_render_nrc_ev(self.h, accum_id, every_nth, n_train, c, p0, n, out["gbuf"], out["query"],
                                out["suffix_query"], out["records"], out["tinfo"], out["events"], out["n_events"],
                                max_events, threads)
    else:
        lib().hmo_render_nrc(self.h, accum_id, every_nth, n_train, c, p0, n, out["gbuf"], out["query"],
                             out["suffix_query"], out["records"], out["tinfo"], threads)
    return out


OracleScene.render_nrc = _render_nrc


def _half_area(lo, hi):
    """Surface area / 2 of float32 boxes, in the library's operation order."""
    ex = hi[..., 0] - lo[..., 0]
    ey = hi[..., 1] - lo[..., 1]
    ez = hi[..., 2] - lo[..., 2]
    return (ex * ey + ey * ez) + ex * ez


def wide_collapse(nodes, width=8):
    """The 8-wide tree the kernels traverse, built from the binary LBVH
    (nodes [n, 16] float32: child-0 box, child-1 box, child codes) the way
    the library collapses it: breadth first, the wide node of binary node r
    starts with r's two children; while it has fewer than 8, its internal
    child of largest surface area (the first of equals) is replaced by that
    child's first child and the second child is appended.  Wide nodes are
    numbered level by level in the order their parents list them.  Returns
    [n_wide, 56] float32: lo.x[8] hi.x[8] lo.y[8] hi.y[8] lo.z[8] hi.z[8]
    child[8] (int bits; >= 0 wide node, < 0 leaf ~slot, -1 in empty slots
    whose box is [+inf, +inf])."""
    nodes = np.ascontiguousarray(nodes, np.float32)
    codes = nodes.view(np.int32)[:, 12:14]
    boxes = nodes[:, :12].reshape(-1, 2, 6)
    out = []
    roots = np.array([0], np.int64)
    base = 0
    while len(roots):
        n = len(roots)
        rows = np.arange(n)
        lo = np.full((n, width, 3), np.inf, np.float32)
        hi = np.full((n, width, 3), np.inf, np.float32)
        kc = np.full((n, width), -1, np.int32)
        area = np.zeros((n, width), np.float32)
        for slot in (0, 1):
            lo[:, slot] = boxes[roots, slot, :3]
            hi[:, slot] = boxes[roots, slot, 3:]
            kc[:, slot] = codes[roots, slot]
            area[:, slot] = _half_area(lo[:, slot], hi[:, slot])
        k = np.full(n, 2, np.int64)
        for _ in range(width - 2):
            cand = (kc >= 0) & (np.arange(width)[None] < k[:, None])
            r = rows[cand.any(1)]
            if not len(r):
                break
            best = np.argmax(np.where(cand[r], area[r], -np.inf), axis=1)
            c = kc[r, best].astype(np.int64)
            for slot, col in ((0, best), (1, k[r])):
                lo[r, col] = boxes[c, slot, :3]
                hi[r, col] = boxes[c, slot, 3:]
                kc[r, col] = codes[c, slot]
                area[r, col] = _half_area(lo[r, col], hi[r, col])
            k[r] += 1
        internal = kc >= 0
        nxt = kc[internal].astype(np.int64)
        kc = kc.copy()
        kc[internal] = base + n + np.arange(len(nxt), dtype=np.int32)
        w = np.zeros((n, 7 * width), np.float32)
        for a in range(3):
            w[:, 2 * a * width:(2 * a + 1) * width] = lo[:, :, a]
            w[:, (2 * a + 1) * width:(2 * a + 2) * width] = hi[:, :, a]
        w[:, 6 * width:] = kc.view(np.float32)
        out.append(w)
        base += n
        roots = nxt
    return np.concatenate(out)


def env_tables(env, w, h):
    """generateEnvSamplingTables (scene.cpp:349-425), single precision, order kept."""
    env = np.asarray(env, np.float32).reshape(h, w, 4)
    cw = w + 1
    cpdf = np.zeros((h, cw), np.float32)
    ccdf = np.zeros((h, cw), np.float32)
    third = np.float32(1.0) / np.float32(3.0)
    for y in range(h):
        s = _sinf(np.float32(3.14159) * (np.float32(y) + np.float32(0.5)) / np.float32(h))
        for x in range(w):
            c = env[y, x]
            avg = np.float32((np.float32(c[0] + c[1]) + c[2]) * third)
            cpdf[y, x] = np.float32(avg * s)
            if x > 0:
                ccdf[y, x] = np.float32(ccdf[y, x - 1] + np.float32(cpdf[y, x - 1] / np.float32(w)))
        total = np.float32(ccdf[y, w - 1] + np.float32(cpdf[y, w - 1] / np.float32(w)))
        cpdf[y, w] = total
        if total > 0:
            inv = np.float32(np.float32(1.0) / total)
            ccdf[y, 1:w] = (ccdf[y, 1:w] * inv).astype(np.float32)
        ccdf[y, w] = 1.0
    mpdf = np.zeros(h + 1, np.float32)
    mcdf = np.zeros(h + 1, np.float32)
    mpdf[0] = cpdf[0, w]
    for i in range(1, h):
        mpdf[i] = cpdf[i, w]
        mcdf[i] = np.float32(mcdf[i - 1] + np.float32(mpdf[i - 1] / np.float32(h)))
    total = np.float32(mcdf[h - 1] + np.float32(mpdf[h - 1] / np.float32(h)))
    mpdf[h] = total
    if total > 0:
        mcdf[1:h] = (mcdf[1:h] / total).astype(np.float32)
    mcdf[h] = 1.0
    return cpdf.ravel(), ccdf.ravel(), mpdf, mcdf


def _sinf(x):
    """C sinf (float in, float out) through the oracle library's libm."""
    return np.float32(_libm().sinf(ctypes.c_float(float(x))))


_libm_h = None


def _libm():
    global _libm_h
    if _libm_h is None:
        _libm_h = ctypes.CDLL("libm.so.6")
        _libm_h.sinf.restype = ctypes.c_float
        _libm_h.sinf.argtypes = [ctypes.c_float]
    return _libm_h


def camera_vectors(frm, at, up, cos_fovy, width, height):
    """cameraChanged (render_hair_msnn.cu:1093-1118) in float32."""
    f = lambda v: np.asarray(v, np.float32)

    def normalize(v):
        v = f(v)
        d = np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
        return (v * np.float32(np.float32(1.0) / np.float32(np.sqrt(d)))).astype(np.float32)

    def cross(a, b):
        return f([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])

    d00 = normalize(f(at) - f(frm))
    aspect = np.float32(np.float32(width) / np.float32(height))
    ddu = (np.float32(cos_fovy) * aspect * normalize(cross(d00, f(up)))).astype(np.float32)
    ddv = (np.float32(cos_fovy) * normalize(cross(ddu, d00))).astype(np.float32)
    d00 = (d00 - np.float32(0.5) * ddu).astype(np.float32)
    d00 = (d00 - np.float32(0.5) * ddv).astype(np.float32)
    return f(frm), d00, ddu, ddv


def _declare_scene(L):
    if getattr(L, "_scene_declared", False):
        return
    i32, f32_, u32 = ctypes.c_int, ctypes.c_float, ctypes.c_uint32
    L.hmo_gen_hair.restype = None
    L.hmo_gen_hair.argtypes = [i32, i32, i32, f32_, f32_, f32_, f32_, f32_, u32, F32P, F32P, I32P]
    L.hmo_gen_ellipsoid.restype = None
    L.hmo_gen_ellipsoid.argtypes = [i32, F32P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.hmo_bake_sky.restype = None
    L.hmo_bake_sky.argtypes = [f32_, F32P, i32, i32, f32_, F32P]
    L.hmo_env_tables.restype = None
    L.hmo_env_tables.argtypes = [F32P, i32, i32, F32P, F32P, F32P, F32P]
    L._scene_declared = True


def _normalize32(v):
    v = np.asarray(v, np.float32)
    d = np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
    return (v * np.float32(np.float32(1.0) / np.float32(np.sqrt(d)))).astype(np.float32)


def _length32(v):
    v = np.asarray(v, np.float32)
    return np.float32(np.sqrt(np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])))


def procedural_scene(cfg):
    """An OracleScene built from a procedural scene config (the keys the
    library's scene parser reads: hair.procedural, surface.procedural,
    lights.sky / directional, camera, integrator), generated by the oracle
    alone (hm_oracle_scene.cpp) -- no shipped library involved.  The arrays
    equal the library's for the same config on the same host."""
    L = lib()
    _declare_scene(L)
    f = np.float32
    hp = cfg["hair"].get("procedural", {})
    sp = cfg.get("surface", {}).get("procedural", {})
    head_r = np.asarray(sp.get("radii", [0.85, 0.95, 1.0]), np.float32)
    arrays = {}
    strands, cps = int(hp.get("strands", 10000)), int(hp.get("control_points", 64))
    cp = np.zeros((strands * cps, 4), np.float32)
    seg = np.zeros(strands * (cps - 3), np.int32)
    L.hmo_gen_hair(1 if hp.get("type", "straight") == "curly" else 0, strands, cps, hp.get("length", 2.0),
                   hp.get("radius", 4e-4), hp.get("root_min_z", 0.25), hp.get("helix_radius", 0.05),
                   hp.get("helix_pitch", 0.1), int(hp.get("seed", 1)), head_r, cp.ravel(), seg)
    arrays["control_points"], arrays["segments"] = cp, seg
    if sp:
        nv, nt = ctypes.c_int(), ctypes.c_int()
        tris = int(sp.get("triangles", 20000))
        L.hmo_gen_ellipsoid(tris, head_r, None, None, None, ctypes.byref(nv), ctypes.byref(nt))
        vtx = np.zeros((nv.value, 3), np.float32)
        nrm = np.zeros((nv.value, 3), np.float32)
        tri = np.zeros((nt.value, 3), np.int32)
        L.hmo_gen_ellipsoid(tris, head_r, vtx.ctypes.data, nrm.ctypes.data, tri.ctypes.data, ctypes.byref(nv),
                            ctypes.byref(nt))
        diffuse, alpha_raw = sp.get("diffuse", [0.35, 0.25, 0.2]), sp.get("alpha", 1.0)
    else:
        vtx, nrm, tri = np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
        diffuse, alpha_raw = [0.35, 0.25, 0.2], 1.0
    arrays.update(vertices=vtx, normals=nrm, triangles=tri)
    lights = cfg.get("lights", {})
    sky = lights.get("sky")
    env_w = env_h = 0
    env_scale, env_rot = f(1.0), f(0.0)
    if sky:
        env_w, env_h = int(sky.get("width", 512)), int(sky.get("height", 256))
        env = np.zeros((env_h, env_w, 4), np.float32)
        L.hmo_bake_sky(sky.get("turbidity", 3.0), np.asarray(sky.get("sun", [3, 3, 3]), np.float32), env_w, env_h,
                       sky.get("radiance_scale", 1.0), env.ravel())
        cpdf = np.zeros((env_h, env_w + 1), np.float32)
        ccdf = np.zeros((env_h, env_w + 1), np.float32)
        mpdf = np.zeros(env_h + 1, np.float32)
        mcdf = np.zeros(env_h + 1, np.float32)
        L.hmo_env_tables(env.ravel(), env_w, env_h, cpdf.ravel(), ccdf.ravel(), mpdf, mcdf)
        env_scale, env_rot = f(sky.get("scale", 1.0)), f(sky.get("rotation", 0.0))
        arrays.update(env=env, env_cpdf=cpdf, env_ccdf=ccdf, env_mpdf=mpdf, env_mcdf=mcdf)
    else:
        z = np.zeros(0, np.float32)
        arrays.update(env=z, env_cpdf=z, env_ccdf=z, env_mpdf=z, env_mcdf=z)
    dl = [np.concatenate([_normalize32(d.get("from", [0, 0, 1])), np.asarray(d.get("emit", [1, 1, 1]), np.float32)])
          for d in lights.get("directional", [])]
    arrays["dir_lights"] = np.asarray(dl, np.float32).reshape(-1, 6)
    it = cfg["integrator"]
    w, h = int(it.get("width", 512)), int(it.get("height", 512))
    c = cfg["camera"]
    pos, d00, du, dv = camera_vectors(c["from"], c["to"], c["up"], c["cos_fovy"], w, h)
    arrays["camera"] = np.concatenate([pos, d00, du, dv]).astype(np.float32)
    hair = cfg["hair"]
    if isinstance(hair.get("type"), (int, float)) and not isinstance(hair.get("type"), bool):
        alpha = f(f(f(3.14159) * f(hair["alpha"])) / f(180.0)) if "alpha" in hair else f(0.0)
    else:  # parseScene reads the material only after hair.type (scene.cpp:188): the Scene defaults
        hair, alpha = {}, f(0.03)
    mat = [*hair.get("sigma_a", [0.06, 0.1, 0.2]), hair.get("beta_m", 0.3), hair.get("beta_n", 0.3), alpha,
           hair.get("Gain R", 1.0), hair.get("Gain TT", 1.0), hair.get("Gain TRT", 1.0), hair.get("Gain TRRT", 1.0),
           *diffuse, alpha_raw, env_scale, env_rot]
    arrays["materials"] = np.asarray(mat, np.float32).reshape(1, 16)
    # bounds and scale (render_hair_msnn.cu:318-357)
    surf_scale = _length32(vtx.max(0) - vtx.min(0)) if len(vtx) else f(0.0)
    hair_scale = _length32(cp[:, :3].max(0) - cp[:, :3].min(0)) if len(cp) else f(0.0)
    settings = dict(width=w, height=h, path_v1=int(it.get("path_v1", 1)), path_v2=int(it.get("path_v2", 40)),
                    mis=int(bool(it.get("MIS", True))), env_pdf=int(bool(it.get("ENV_PDF", True))),
                    has_env=int(bool(sky)), catrom=int(bool(it.get("shade_catmull_rom", False))), env_w=env_w,
                    env_h=env_h, seg_split=int(it.get("segment_splits", 2)))
    return OracleScene(arrays, settings, float(max(hair_scale, surf_scale)))


def gen_bsdf_queries(seed, n):
    """Synthetic BSDF workload, planar layouts: wo/wi/t [3,n], h [n], u [4,n]."""
    wo = np.zeros((3, n), np.float32)
    wi = np.zeros((3, n), np.float32)
    t = np.zeros((3, n), np.float32)
    h = np.zeros(n, np.float32)
    u = np.zeros((4, n), np.float32)
    lib().hmo_gen_bsdf_queries(seed, n, wo, wi, t, h, u)
    return wo, wi, t, h, u


def _mlp_desc(cfg):
    """Segment and hash-grid level tables of an mlp_oracle.Config in the
    layout hm_oracle_mlp.cpp reads."""
    kinds = {"Identity": 0, "Frequency": 1, "OneBlob": 2, "HashGrid": 3, "Grid": 3}
    seg, scale, res, size, off = [], [], [], [], []
    for s in cfg.segs:
        if s["type"] not in kinds:
            raise ValueError("host transcription: %s encoding not supported" % s["type"])
        k = kinds[s["type"]]
        if k == 3:
            seg.append([k, s["in_off"], s["n_dims"], s["out_off"], s["n_levels"], s["n_feat"], len(scale),
                        s["param_off"]])
            for sc, rs, sz, of in s["levels"]:
                scale.append(sc)
                res.append(rs)
                size.append(sz)
                off.append(of)
        else:
            seg.append([k, s["in_off"], s["n_dims"], s["out_off"], s.get("n_freq", s.get("n_bins", 0)), 0, 0, 0])
    shapes = np.ascontiguousarray([[fo, fi] for _, fo, fi in cfg.layer_shapes], np.int32).ravel()
    lv = (f32(scale + [0.0]), np.ascontiguousarray(res + [0], np.int32), np.ascontiguousarray(size + [0], np.int32),
          np.ascontiguousarray(off + [0], np.int32))
    return np.ascontiguousarray(seg, np.int32).ravel(), shapes, lv


def mlp_forward_host(cfg, params, x, threads=1):
    """The cache network's inference as the oracle's C++ FP32 transcription
    on `threads` host threads (hm_oracle_mlp.cpp): cfg an mlp_oracle.Config,
    params the network weights then the encoding parameters, x [n, in_ch]
    -> [n, out_ch] float32."""
    seg, shapes, lv = _mlp_desc(cfg)
    w = f32(np.asarray(params)[:cfg.n_params])
    x = f32(x)
    out = np.zeros((x.shape[0], cfg.out_ch), np.float32)
    lib().hmo_mlp_forward(x, x.shape[0], cfg.in_ch, seg, len(cfg.segs), cfg.n_enc, cfg.in_pad, w,
                          cfg.n_net_params, shapes, len(cfg.layer_shapes), cfg.out_ch, *lv, out, int(threads))
    return out


def mlp_grad_host(cfg, params, x, target, threads=1):
    """The loss (cfg.loss) over the rows and its gradient with respect to
    every parameter, as the C++ FP32 transcription: (loss, grads [n_params]
    float32)."""
    seg, shapes, lv = _mlp_desc(cfg)
    w = f32(np.asarray(params)[:cfg.n_params])
    x, target = f32(x), f32(target)
    grads = np.zeros(cfg.n_params, np.float32)
    kind = {"L2": 0, "RelativeL2": 1}.get(cfg.loss, 2)
    loss = lib().hmo_mlp_grad(x, target, x.shape[0], cfg.in_ch, seg, len(cfg.segs), cfg.n_enc, cfg.in_pad, w,
                              cfg.n_net_params, cfg.n_params, shapes, len(cfg.layer_shapes), cfg.out_ch, *lv, kind,
                              grads, int(threads))
    return loss, grads
