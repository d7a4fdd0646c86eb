"""ctypes front end of the reference's own integrator compiled on the host
(test infrastructure only).

oracle/_ref/libhmref_path.so holds the reference's cuda/hair_msnn.cu (with
optix_common.cuh and the BSDF headers), libhmref_pt.so its
cuda/path_tracing.cu and libhmref_nrc.so its cuda/nrc.cu, all compiled
unmodified through oracle/ref_shim/;
their owl::traceRay is answered by the oracle's BVH (ref_harness.h).  They
exist only where the reference checkout is present (oracle/build.py
build_ref); everything here returns None / raises when they are absent.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from . import pyoracle as po

F32P = po.F32P
I32P = po.I32P

_libs = {}


def available():
    """True when the reference-compiled integrator libraries exist (or can
    be built because the reference checkout is present)."""
    try:
        return _load("path") is not None and _load("pt") is not None
    except OSError:
        return False


def _load(which):
    if which in _libs:
        return _libs[which]
    name = {"path": "libhmref_path.so", "pt": "libhmref_pt.so", "nrc": "libhmref_nrc.so"}[which]
    path = os.path.join(_build.OUT_DIR, name)
    if not os.path.isfile(path):
        if not _build.ref_available():
            _libs[which] = None
            return None
        _build.build_ref()
    po.lib()  # the oracle library (its BVH answers traceRay) first
    L = ctypes.CDLL(path)
    i32, f32, vp = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    scene_args = [vp, F32P, i32, I32P, i32, F32P, F32P, i32, I32P, i32, F32P, i32, i32, F32P, F32P, F32P, F32P,
                  F32P, i32, F32P, I32P]
    if which == "path":
        L.hmr_scene_new.restype = vp
        L.hmr_scene_new.argtypes = scene_args
        L.hmr_scene_free.argtypes = [vp]
        L.hmr_msnn_gbuffer.restype = None
        L.hmr_msnn_gbuffer.argtypes = [vp, F32P, F32P, I32P, f32, i32, i32, i32, I32P, i32, F32P, F32P, F32P, F32P,
                                       F32P, I32P, i32, i32]
        L.hmr_msnn_traingen.restype = None
        L.hmr_msnn_traingen.argtypes = [vp, F32P, F32P, I32P, f32, i32, i32, i32, i32, I32P, F32P, i32, F32P, F32P,
                                        F32P, I32P, i32, i32]
        L.hmr_msnn_render.restype = None
        L.hmr_msnn_render.argtypes = [vp, i32, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P, i32]
    elif which == "nrc":
        L.hmr_nrc_scene_new.restype = vp
        L.hmr_nrc_scene_new.argtypes = scene_args
        L.hmr_nrc_scene_free.argtypes = [vp]
        L.hmr_nrc_render.restype = None
        L.hmr_nrc_render.argtypes = [vp, i32, i32, I32P, i32, i32, F32P, F32P, I32P, F32P, F32P, F32P, F32P, F32P]
        L.hmr_nrc_gbuffer.restype = None
        L.hmr_nrc_gbuffer.argtypes = [vp, F32P, F32P, I32P, f32, i32, i32, I32P, i32, f32, i32, F32P, F32P, F32P,
                                      I32P, F32P, I32P, i32]
    else:
        L.hmr_pt_scene_new.restype = vp
        L.hmr_pt_scene_new.argtypes = scene_args
        L.hmr_pt_scene_free.argtypes = [vp]
        L.hmr_pt_frame.restype = None
        L.hmr_pt_frame.argtypes = [vp, F32P, F32P, I32P, f32, i32, F32P, F32P, F32P, I32P, i32, i32]
    _libs[which] = L
    return L


class RefIntegrator:
    """The reference's rayGenCam programs over an OracleScene's arrays."""

    def __init__(self, osc, which="path"):
        self.osc, self.which = osc, which
        L = _load(which)
        if L is None:
            raise RuntimeError("reference checkout absent: the reference-compiled integrator is not built")
        self.L = L
        a = osc._keep
        env_w, env_h = osc.env_wh
        empty = np.zeros(4, np.float32)
        g = lambda k: np.ascontiguousarray(a[k], np.float32).ravel() if a[k].size else empty
        self._arr = dict(
            cp=np.ascontiguousarray(a["control_points"], np.float32).ravel(),
            seg=np.ascontiguousarray(a["segments"], np.int32).ravel(),
            vtx=np.ascontiguousarray(a["vertices"], np.float32).ravel(),
            nrm=np.ascontiguousarray(a["normals"], np.float32).ravel(),
            tri=np.ascontiguousarray(a["triangles"], np.int32).ravel(),
            env=g("env"), cpdf=g("env_cpdf"), ccdf=g("env_ccdf"), mpdf=g("env_mpdf"), mcdf=g("env_mcdf"),
            dl=np.ascontiguousarray(a["dir_lights"], np.float32).ravel() if a["dir_lights"].size else empty,
            cam=np.ascontiguousarray(a["camera"], np.float32).ravel(),
            mat=np.ascontiguousarray(a["materials"], np.float32).ravel()[:16].copy(),
            sets=np.ascontiguousarray(osc.settings, np.int32))
        r = self._arr
        new = getattr(L, {"path": "hmr_scene_new", "pt": "hmr_pt_scene_new", "nrc": "hmr_nrc_scene_new"}[which])
        self.h = new(osc.h, r["cp"], len(r["cp"]) // 4, r["seg"], len(r["seg"]), r["vtx"], r["nrm"],
                     len(r["vtx"]) // 3, r["tri"], len(r["tri"]) // 3, r["env"], env_w, env_h, r["cpdf"], r["ccdf"],
                     r["mpdf"], r["mcdf"], r["dl"], len(a["dir_lights"]), r["mat"], r["sets"])
        self.P = osc.width * osc.height

    def __del__(self):
        try:
            getattr(self.L, {"path": "hmr_scene_free", "pt": "hmr_pt_scene_free",
                             "nrc": "hmr_nrc_scene_free"}[self.which])(self.h)
        except Exception:
            pass

    def msnn_gbuffer(self, beta=1, accum_id=0, every_nth=1, n_train=0, max_events=128, threads=8):
        """The G_BUFFER pass.  The trainIdxs table is the library's keyed
        permutation of [0, n_train) for this frame (the reference shuffles it
        with thrust::shuffle).  Returns a dict: gbuf [P, 8] (hit, isSurface,
        p, shortPathColor), nn_in [P, 12], train_in [R, 12], train_out
        [R, 3], events [P, max_events, 12], n_events [P]."""
        assert self.which == "path"
        P, r = self.P, self._arr
        ntr = max(n_train, (P + every_nth - 1) // every_nth)
        tidx = np.array([po.feistel_perm(t, n_train, accum_id) if t < n_train else 0 for t in range(ntr)], np.int32)
        out = dict(gbuf=np.zeros((P, 8), np.float32), nn_in=np.zeros((P, 12), np.float32),
                   train_in=np.zeros((ntr, 12), np.float32), train_out=np.zeros((ntr, 3), np.float32),
                   events=np.zeros((P, max_events, po.EV_FLOATS), np.float32), n_events=np.zeros(P, np.int32))
        self.L.hmr_msnn_gbuffer(self.h, r["cam"], r["mat"], r["sets"], self.osc.scene_scale, beta, accum_id,
                                every_nth, tidx, len(tidx), out["gbuf"], out["nn_in"], out["train_in"],
                                out["train_out"], out["events"], out["n_events"], max_events, threads)
        return out

    def msnn_traingen(self, points, scene_indices, rec_x, beta=1, accum_id=0, max_events=128, threads=8):
        """The TRAIN_DATA_GEN pass over a rec_x-wide grid of len(scene_indices)
        records aiming at points[scene_indices[r]] (points float [N, 3]).
        Returns dict train_in [R, 12], train_out [R, 3], events [R,
        max_events, 12], n_events [R]."""
        assert self.which == "path"
        r = self._arr
        sidx = np.ascontiguousarray(scene_indices, np.int32)
        R = len(sidx)
        assert R % rec_x == 0
        pts = np.ascontiguousarray(np.asarray(points, np.float32)[:, :3])
        out = dict(train_in=np.zeros((R, 12), np.float32), train_out=np.zeros((R, 3), np.float32),
                   events=np.zeros((R, max_events, po.EV_FLOATS), np.float32), n_events=np.zeros(R, np.int32))
        self.L.hmr_msnn_traingen(self.h, r["cam"], r["mat"], r["sets"], self.osc.scene_scale, beta, accum_id, rec_x,
                                 R // rec_x, sidx, pts, len(pts), out["train_in"], out["train_out"], out["events"],
                                 out["n_events"], max_events, threads)
        return out

    def msnn_render(self, gbuf, nn_out, accum_id=0, acc=None, threads=8):
        """The RENDER pass over a G-buffer [P, 8] and cache outputs [P, 3];
        acc: the three float4 accumulation buffers of the previous frames
        (dict pt/nn/final [P, 4]) or None.  Returns dict of the accumulation
        and average buffers."""
        assert self.which == "path"
        P = self.P
        acc = acc or {k: np.zeros((P, 4), np.float32) for k in ("pt", "nn", "final")}
        acc = {k: np.ascontiguousarray(v, np.float32).copy() for k, v in acc.items()}
        avg = {k: np.zeros((P, 4), np.float32) for k in ("pt", "nn", "final")}
        self.L.hmr_msnn_render(self.h, accum_id, np.ascontiguousarray(gbuf, np.float32),
                               np.ascontiguousarray(nn_out, np.float32), acc["pt"], acc["nn"], acc["final"],
                               avg["pt"], avg["nn"], avg["final"], threads)
        return {"acc": acc, "avg": avg}

    def pt_frame(self, accum_id=0, accum=None, max_events=128, threads=8):
        """One launch of the path tracer: dict accum [P, 4], avg [P, 4],
        events [P, max_events, 12], n_events [P]."""
        assert self.which == "pt"
        P, r = self.P, self._arr
        accum = np.zeros((P, 4), np.float32) if accum is None else np.ascontiguousarray(accum, np.float32).copy()
        out = dict(accum=accum, avg=np.zeros((P, 4), np.float32),
                   events=np.zeros((P, max_events, po.EV_FLOATS), np.float32), n_events=np.zeros(P, np.int32))
        self.L.hmr_pt_frame(self.h, r["cam"], r["mat"], r["sets"], self.osc.scene_scale, accum_id, out["accum"],
                            out["avg"], out["events"], out["n_events"], max_events, threads)
        return out

    def nrc_render(self, g, nn_out, accum_id=0, every_nth=1, n_train=0, all_unbiased=False, accum=None):
        """The NRC RENDER pass over nrc_gbuffer's output g and cache outputs
        nn_out [P + n_train, 3].  Returns dict accum / avg [P, 4], train_in
        [n_train, 40, 9], train_gt [n_train, 40, 3]."""
        assert self.which == "nrc"
        P = self.P
        tidx = np.array([po.feistel_perm(t, n_train, accum_id) for t in range(n_train)], np.int32)
        out = dict(accum=np.zeros((P, 4), np.float32) if accum is None else np.array(accum, np.float32),
                   avg=np.zeros((P, 4), np.float32), train_in=np.zeros((n_train, 40, 9), np.float32),
                   train_gt=np.zeros((n_train, 40, 3), np.float32))
        self.L.hmr_nrc_render(self.h, accum_id, every_nth, tidx, len(tidx), 1 if all_unbiased else 0,
                              np.ascontiguousarray(g["gbuf"], np.float32), np.ascontiguousarray(g["train"], np.float32),
                              np.ascontiguousarray(g["tinfo"], np.int32), np.ascontiguousarray(nn_out, np.float32),
                              out["accum"], out["avg"], out["train_in"], out["train_gt"])
        return out

    def nrc_gbuffer(self, accum_id=0, every_nth=1, n_train=0, c=0.01, all_unbiased=False, max_events=128):
        """The NRC G_BUFFER pass.  Returns a dict: gbuf [P, 8] (hit,
        pathRadiance, beta, bounces), query [P + n_train, 9], train
        [P, 40, 15] (each pixel's own train buffer), tinfo [P, 2] (bounces,
        hit), events [P, max_events, 12], n_events [P]."""
        assert self.which == "nrc"
        P, r = self.P, self._arr
        tidx = np.array([po.feistel_perm(t, n_train, accum_id) for t in range(n_train)], np.int32)
        out = dict(gbuf=np.zeros((P, 8), np.float32), query=np.zeros((P + n_train, 9), np.float32),
                   train=np.zeros((P, 40, 15), np.float32), tinfo=np.zeros((P, 2), np.int32),
                   events=np.zeros((P, max_events, po.EV_FLOATS), np.float32), n_events=np.zeros(P, np.int32))
        self.L.hmr_nrc_gbuffer(self.h, r["cam"], r["mat"], r["sets"], self.osc.scene_scale, accum_id, every_nth,
                               tidx, len(tidx), c, 1 if all_unbiased else 0, out["gbuf"], out["query"], out["train"],
                               out["tinfo"], out["events"], out["n_events"], max_events)
        return out
